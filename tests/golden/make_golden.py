"""Regenerate tests/golden/scihpc_ref_golden.npz from the REFERENCE implementation itself
(compiled from its own sources by oracle/Makefile; needs the reference sources).

    python tests/golden/make_golden.py

Every case is a seeded input and the reference's output for it, at sizes small enough to
commit.  The restatement (oracle/port) is checked against these bit for bit on the CPU, and
the CUDA library within round-off on the GPU, where the reference itself is not available.
"""
from __future__ import annotations

import os
import sys

os.environ["OMP_NUM_THREADS"] = "1"
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from tests.helpers import bubble_params, bubble_phi, smooth_field  # noqa: E402

OUT = os.path.join(HERE, "scihpc_ref_golden.npz")

GRIDS = {"g2": O.Grid(2, (8, 11), (0.0, 0.0), (1.0, 1.5)), "g3": O.Grid(3, (5, 6, 7), (0.0, 0.0, 0.0), (1.0, 1.2, 1.4))}


def main():
    R = O.Checker("ref")
    data = {}
    for gname, g in GRIDS.items():
        rng = np.random.default_rng(1234 + g.ndim)
        vals = rng.standard_normal(6)
        data[f"{gname}/bc_values"] = vals
        f = rng.standard_normal(g.shape)
        data[f"{gname}/bc_input"] = f
        for loc in range(g.ndim + 1):
            for t in range(5):
                data[f"{gname}/bc_{loc}_{t}"] = R.bc_fill(g, loc, [t] * 6, vals, f)
            data[f"{gname}/flux_{loc}"] = R.flux_extrapolate(g, loc, f)
        data[f"{gname}/zoe"] = R.zero_order_extrapolation(g, f)
        flux = smooth_field(g, rng)
        vel = [rng.standard_normal(g.shape) for _ in range(3)]
        data[f"{gname}/flux_in"] = flux
        for c in range(3):
            data[f"{gname}/vel_{c}"] = vel[c]
        data[f"{gname}/uccd"] = R.uccd(g, flux, *vel)
        data[f"{gname}/ccd"] = R.ccd(g, flux, mixed=True)
        data[f"{gname}/weno5"] = R.weno5(g, flux, *vel)
        phi = 0.2 * smooth_field(g, rng)
        sign = np.sign(rng.standard_normal(g.shape))
        data[f"{gname}/phi"] = phi
        data[f"{gname}/sign"] = sign
        data[f"{gname}/godunov"] = R.godunov(g, phi, sign)
        prm = [0.15, 0.001, 0.01, 0.0]
        data[f"{gname}/lsf_fields"] = R.lsf_fields(g, prm, phi)
        data[f"{gname}/lsf_integrals"] = R.lsf_integrals(g, prm, phi)
    # reference multigrid, Dirichlet operator of multigrid_base.cpp:293-345, 32 x 32
    g = O.Grid(2, (32, 32), (0.0, 0.0), (1.0, 1.0))
    xc = (np.arange(32) + 0.5) / 32
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    rhs = (-2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)).T.ravel()
    sol, cyc, hist = R.mg_poisson(g, rhs, True, 1e-12, 100)
    data["mg32/rhs"] = rhs
    data["mg32/sol"] = sol
    data["mg32/hist"] = hist
    # two time steps of the rising bubble, 16 x 32, projection() every step with a capped SOR
    g = O.Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
    prm = bubble_params(g, 1e-12)
    prm.update(ppe_tol=1e-30, ppe_tol2=0.0, ppe_max_iter=3000)
    s = R.twophase(g, ["no_slip"] * 6, ["neumann"] * 6, prm,
                   dict(scheme=1, n_mpls=5, reinit_every=1, ppe_mode=1, reinit_lambda=1))
    phi = bubble_phi(g, (0.43, 0.57), 0.23)
    data["tp/phi0"] = phi
    s.set("phi", phi)
    s.call("init")
    for k in range(2):
        s.call("step", 1)
        for nm in ("phi", "p", "u", "v", "nu", "nv"):
            data[f"tp/step{k + 1}/{nm}"] = s.get(nm)
        sc = s.scalars()
        data[f"tp/step{k + 1}/scalars"] = np.array([sc[k2] for k2 in ("t", "dt", "dt_old", "stable_CFL")])
    np.savez_compressed(OUT, **data)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
