"""The CPU restatement against golden vectors of the reference (tests/golden/
scihpc_ref_golden.npz, written by tests/golden/make_golden.py from the compiled reference):
bit for bit.  Runs anywhere (no reference sources needed)."""
import os

import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_params

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scihpc_ref_golden.npz")
GRIDS = {"g2": O.Grid(2, (8, 11), (0.0, 0.0), (1.0, 1.5)), "g3": O.Grid(3, (5, 6, 7), (0.0, 0.0, 0.0), (1.0, 1.2, 1.4))}


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def port():
    return O.Checker("port")


@pytest.mark.parametrize("gname", ["g2", "g3"])
def test_kernels_match_golden(port, gold, gname):
    g = GRIDS[gname]
    f = gold[f"{gname}/bc_input"]
    vals = gold[f"{gname}/bc_values"]
    for loc in range(g.ndim + 1):
        for t in range(5):
            assert np.array_equal(port.bc_fill(g, loc, [t] * 6, vals, f), gold[f"{gname}/bc_{loc}_{t}"]), (loc, t)
        assert np.array_equal(port.flux_extrapolate(g, loc, f), gold[f"{gname}/flux_{loc}"])
    assert np.array_equal(port.zero_order_extrapolation(g, f), gold[f"{gname}/zoe"])
    flux = gold[f"{gname}/flux_in"]
    vel = [gold[f"{gname}/vel_{c}"] for c in range(3)]
    assert np.array_equal(port.uccd(g, flux, *vel)[:g.ndim], gold[f"{gname}/uccd"][:g.ndim])
    assert np.array_equal(port.ccd(g, flux), gold[f"{gname}/ccd"])
    assert np.array_equal(port.weno5(g, flux, *vel), gold[f"{gname}/weno5"])
    phi, sign = gold[f"{gname}/phi"], gold[f"{gname}/sign"]
    assert np.array_equal(port.godunov(g, phi, sign), gold[f"{gname}/godunov"])
    prm = [0.15, 0.001, 0.01, 0.0]
    assert np.array_equal(port.lsf_fields(g, prm, phi), gold[f"{gname}/lsf_fields"])
    assert np.array_equal(port.lsf_integrals(g, prm, phi), gold[f"{gname}/lsf_integrals"])


def test_multigrid_matches_golden(port, gold):
    g = O.Grid(2, (32, 32), (0.0, 0.0), (1.0, 1.0))
    sol, cyc, hist = port.mg_poisson(g, gold["mg32/rhs"], True, 1e-12, 100)
    assert cyc == len(gold["mg32/hist"]) - 1
    assert np.abs(sol - gold["mg32/sol"]).max() <= 1e-12 * np.abs(gold["mg32/sol"]).max()


def test_two_phase_matches_golden(port, gold):
    g = O.Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
    prm = bubble_params(g, 1e-12)
    prm.update(ppe_tol=1e-30, ppe_tol2=0.0, ppe_max_iter=3000)
    s = port.twophase(g, ["no_slip"] * 6, ["neumann"] * 6, prm,
                      dict(scheme=1, n_mpls=5, reinit_every=1, ppe_mode=1, reinit_lambda=1))
    s.set("phi", gold["tp/phi0"])
    s.call("init")
    for k in range(2):
        s.call("step", 1)
        for nm in ("phi", "p", "u", "v", "nu", "nv"):
            assert np.array_equal(s.get(nm), gold[f"tp/step{k + 1}/{nm}"]), (k, nm)
        sc = s.scalars()
        assert np.array_equal(np.array([sc[k2] for k2 in ("t", "dt", "dt_old", "stable_CFL")]),
                              gold[f"tp/step{k + 1}/scalars"])
