"""3D dam break (water column [0,1] x [0,2] x [0,1] in a 4 x 2 x 2 tank, gravity -z, slip walls
on all six faces, air/water density and viscosity) on a coarse grid: the GPU step against the
CPU restatement, both precisions of the pressure solve."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

G = O.Grid(3, (16, 8, 8), (0.0, 0.0, 0.0), (4.0, 2.0, 2.0))


def dambreak_params(g, ppe_tol=1e-12):
    """set_parameters(1000, 1.2, 1e-3, 1.8e-5, sigma, 9.81, L = 1) (global.cpp:31-52) without
    surface tension (We = -1, as the reference's dam-break driver sets it), ls_width 1.5h."""
    h = min(g.spacing())
    Uc = np.sqrt(9.81 * 1.0)
    return dict(density_ratio=1.2 / 1000.0, viscosity_ratio=1.8e-5 / 1e-3, Re=1000.0 * Uc * 1.0 / 1e-3,
                Fr=Uc / np.sqrt(9.81 * 1.0), We=-1.0, ls_width=1.5 * h, rdt=0.1 * h, max_CFL=0.1, min_CFL=1e-4,
                positive_ref=1.0, ppe_tol=ppe_tol, ppe_tol2=0.0, ppe_max_iter=400, ppe_omega=1.5, ppe_initer=1,
                dt0=1.0)


def column_phi(g):
    """Signed distance to the water surfaces x = 1 and z = 1 (positive in the water)."""
    c = [g.lo[a] + (np.arange(g.n[a]) + 0.5) * g.spacing()[a] for a in range(3)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    inside = (X < 1.0) & (Z < 1.0)
    d_in = np.minimum(1.0 - X, 1.0 - Z)
    d_out = -np.sqrt(np.maximum(X - 1.0, 0.0) ** 2 + np.maximum(Z - 1.0, 0.0) ** 2)
    phi = np.zeros(g.shape)
    phi[3:-3, 3:-3, 3:-3] = np.where(inside, d_in, d_out)
    return phi


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32_refined"])
def test_dambreak_steps_match_oracle(fp32):
    from scihpc_gb300 import Grid, TwoPhase
    # Density ratio 833: a relative residual r leaves a pressure error of up to ~2e3 r, so the
    # solve runs to its FP64 floor (about 1e-13) for the 1e-9 parity bound.
    prm = dambreak_params(G, ppe_tol=1e-13)
    port = O.Checker("port").twophase(G, ["slip"] * 6, ["neumann"] * 6, prm,
                                      dict(scheme=0, n_mpls=0, reinit_every=1, ppe_mode=2, reinit_lambda=1))
    port.set_exact_tol(1e-14)
    gpu = TwoPhase(Grid(3, tuple(G.n), tuple(G.lo), tuple(G.hi)), ["slip"] * 6, ["neumann"] * 6, prm, scheme=0,
                   n_mpls=0, reinit_every=1, fp32=fp32)
    phi = column_phi(G)
    port.set("phi", phi)
    gpu.set("phi", phi)
    port.call("init")
    gpu.init()
    I = G.interior()

    def errors():
        # velocity components against the norm of the whole velocity (v, across the uniform
        # y direction, is round-off on both sides)
        out = {nm: rel_l2(gpu.get(nm)[I], port.get(nm)[I]) for nm in ("phi", "p")}
        vnorm = np.sqrt(sum(np.linalg.norm(port.get(nm)[I]) ** 2 for nm in ("u", "v", "w")))
        for nm in ("u", "v", "w"):
            out[nm] = np.linalg.norm(gpu.get(nm)[I] - port.get(nm)[I]) / vnorm
        return out

    # step 1 from identical inputs: the reference's parity bounds
    port.call("step", 1)
    gpu.step(1, graph=True)
    e1 = errors()
    assert e1["phi"] <= 1e-10 and all(e1[nm] <= 1e-9 for nm in ("p", "u", "v", "w")), e1
    # step 2 starts from velocities that agree to ~1e-13; its right-hand side div(u*)/dt is a
    # small difference of O(1) face velocities and amplifies that by ~1e5 here (measured:
    # rhs 2.8e-8, p 1.8e-9 with every stage's own error at round-off).  The restatement
    # itself, its velocities perturbed in the last bit after step 1, moves by p 2.5e-9 and
    # u, v, w 8e-9 at this step (test_oracle_sensitivity.py), so the bound is 5e-8
    port.call("step", 1)
    gpu.step(1, graph=True)
    e2 = errors()
    assert e2["phi"] <= 1e-10 and all(e2[nm] <= 5e-8 for nm in ("p", "u", "v", "w")), e2
    sp, sg = port.scalars(), gpu.scalars()
    assert abs(sp["dt"] - sg["dt"]) <= 1e-14 * sp["dt"]
