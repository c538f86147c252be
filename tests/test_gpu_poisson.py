"""Pressure Poisson solver (scihpc_poisson_*) against the CPU checkers.

Converged fields are compared (the iterates differ: red-black Gauss-Seidel multigrid with
CG acceleration here, steepest-descent multigrid / SOR / CG in the checkers).  Both sides
solve to a relative residual far below the parity tolerance, so the difference is the
solution's own round-off: pressure within 1e-9 relative L2."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_phi, rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

PARITY = 1e-9


@pytest.fixture(scope="module")
def port():
    return O.Checker("port")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def native(g):
    from scihpc_gb300 import Grid
    return Grid(g.ndim, tuple(g.n), tuple(g.lo), tuple(g.hi))


def ghosted_from_mg(g, v):
    """x-fastest multigrid vector -> ghosted [Nx][Ny][Nz] field (interior cells)."""
    out = np.zeros(g.shape)
    if g.ndim == 2:
        out[3:-3, 3:-3, 0] = v.reshape(g.n[1], g.n[0]).T
    else:
        out[3:-3, 3:-3, 3:-3] = v.reshape(g.n[2], g.n[1], g.n[0]).transpose(2, 1, 0)
    return out


@pytest.mark.parametrize("n", [32, 64])
@pytest.mark.parametrize("fp32", [False, True])
def test_dirichlet_constant_matches_reference_multigrid(port, n, fp32):
    """cfg-1 problem (-lap p = 2 pi^2 sin sin, the reference's Dirichlet operator with the
    zero at the ghost-cell centre, multigrid_base.cpp:293-345) at a reduced size."""
    from scihpc_gb300 import Poisson
    g = O.Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
    h = 1.0 / n
    xc = (np.arange(n) + 0.5) * h
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    f = 2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
    rhs_mg = (-f).T.ravel()                       # A p = -f, x-fastest
    ref, cyc, hist = port.mg_poisson(g, rhs_mg, True, 1e-14, 400)
    ref = ghosted_from_mg(g, ref)
    rhs = np.zeros(g.shape)
    rhs[3:-3, 3:-3, 0] = -f
    ps = Poisson(native(g), bc=1, density=False, fp32=fp32)
    p = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    it, rr = ps.solve(dev(rhs), p, rel_tol=1e-12, max_iter=100)
    out = p.cpu().numpy()
    I = g.interior()
    assert rr <= 1e-11, rr
    assert rel_l2(out[I], ref[I]) <= PARITY, rel_l2(out[I], ref[I])


def _density_case(g, seed):
    rng = np.random.default_rng(seed)
    if g.ndim == 2:
        phi = bubble_phi(g, (0.5, 0.5 * g.hi[1] / 2 + 0.25), 0.2)
    else:
        c = g.spacing()
        xs = [g.lo[a] + (np.arange(g.n[a]) + 0.5) * c[a] for a in range(3)]
        X, Y, Z = np.meshgrid(*xs, indexing="ij")
        phi = np.zeros(g.shape)
        d = np.full(X.shape, -1e9)
        for s in range(3):
            r = rng.uniform(0.1, 0.2)
            cen = rng.uniform(r, 1 - r, size=3)
            d = np.maximum(d, r - np.sqrt((X - cen[0]) ** 2 + (Y - cen[1]) ** 2 + (Z - cen[2]) ** 2))
        phi[3:-3, 3:-3, 3:-3] = d
    phi = O.Checker("port").bc_fill(g, 0, [1] * 6, [0.0] * 6, phi)
    h = min(g.spacing())
    H = np.where(phi < -1.5 * h, 0.0, np.where(phi > 1.5 * h, 1.0,
                 0.5 * (1 + phi / (1.5 * h) + np.sin(np.pi * phi / (1.5 * h)) / np.pi)))
    rho = (1.0 - H) + H * 0.001
    rhs = np.zeros(g.shape)
    I = g.interior()
    rhs[I] = rng.standard_normal(rhs[I].shape)
    rhs[I] -= rhs[I].mean()
    return rho, rhs


def operator_relres(g, rho, rhs, p):
    """||g - L p|| / ||g|| with g = -(rhs - mean) and L the face-coefficient operator of
    init_ppe_proj_coefficients (1 / mean density / d^2 on interior faces, none on walls),
    evaluated here in numpy, independently of both solvers."""
    I = g.interior()
    pi, ri = p[I], rho[I]
    gv = -(rhs[I] - rhs[I].mean())
    Lp = np.zeros_like(pi)
    d = g.spacing()
    for a in range(g.ndim):
        lo = [slice(None)] * pi.ndim
        hi = [slice(None)] * pi.ndim
        lo[a], hi[a] = slice(0, -1), slice(1, None)
        lo, hi = tuple(lo), tuple(hi)
        C = 1.0 / (0.5 * (ri[lo] + ri[hi])) / d[a] / d[a]
        flux = C * (pi[lo] - pi[hi])
        Lp[lo] += flux
        Lp[hi] -= flux
    return np.linalg.norm(gv - Lp) / np.linalg.norm(gv)


DENSITY_GRIDS = {
    "2d": ((32, 64), (1.0, 2.0)),
    "3d": ((16, 16, 16), (1.0, 1.0, 1.0)),
    # level 0 of these is smoothed by the one-pass fused sweep (>= 65536 cells); the second
    # has partial tiles in j and k
    "3d_fused": ((48, 48, 48), (1.0, 1.0, 1.0)),
    "3d_ragged": ((48, 40, 80), (1.0, 0.8, 1.6)),
}


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("case", list(DENSITY_GRIDS))
def test_variable_density_matches_exact_solve(port, fp32, case):
    """Density ratio 1000 pressure equation of projection() (coefficients of
    init_ppe_proj_coefficients, projection_method.cpp:404-465, Neumann walls, zero mean)."""
    from scihpc_gb300 import Poisson
    n, hi = DENSITY_GRIDS[case]
    g = O.Grid(len(n), n, (0.0,) * len(n), hi)
    rho, rhs = _density_case(g, 5)
    ref, it_ref, rel_ref = port.coef_solve(g, rho, rhs, rel_tol=1e-14, max_iter=200000)
    ps = Poisson(native(g), bc=0, density=True, fp32=fp32)
    rho_d = dev(rho)   # the solver keeps using this buffer: it must outlive the solves
    ps.set_density(rho_d)
    p = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    it, rr = ps.solve(dev(rhs), p, rel_tol=1e-12, max_iter=200)
    out = p.cpu().numpy()
    I = g.interior()
    assert rr <= 1e-11, (rr, it)
    assert operator_relres(g, rho, rhs, out) <= 2e-11
    assert abs(out[I].mean()) <= 1e-12 * np.abs(out[I]).max()
    assert rel_l2(out[I], ref[I]) <= PARITY, rel_l2(out[I], ref[I])


@pytest.mark.parametrize("case", ["3d_fused", "3d_ragged"])
def test_staged_sweep_matches_direct_sweep(case, monkeypatch):
    """The FP32 level-0 kernels with their planes staged in shared memory by TMA (sweeps,
    residual restriction, prolongation fused into the first post-smoothing sweep) perform the
    same updates as the kernels that read global memory directly (SCIHPC_SWEEP_TMA=0): after
    one iteration the pressures agree to FP32 round-off, and converged solves take the same
    number of iterations to the same answer."""
    from scihpc_gb300 import Poisson
    n, hi = DENSITY_GRIDS[case]
    g = O.Grid(len(n), n, (0.0,) * len(n), hi)
    rho, rhs = _density_case(g, 7)
    rho_d, rhs_d = dev(rho), dev(rhs)
    out = {}
    for flag in ("0", "1"):
        monkeypatch.setenv("SCIHPC_SWEEP_TMA", flag)
        ps = Poisson(native(g), bc=0, density=True, fp32=True)
        ps.set_density(rho_d)
        p1 = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        ps.solve(rhs_d, p1, rel_tol=1e-12, max_iter=1)
        p = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        it, rr = ps.solve(rhs_d, p, rel_tol=1e-12, max_iter=200)
        torch.cuda.synchronize()
        out[flag] = (p1.cpu().numpy(), p.cpu().numpy(), it, rr)
        ps.close()
    I = g.interior()
    (a1, a, ita, rra), (b1, b, itb, rrb) = out["0"], out["1"]
    assert rel_l2(b1[I], a1[I]) <= 1e-6, rel_l2(b1[I], a1[I])
    assert rra <= 1e-11 and rrb <= 1e-11, (rra, rrb)
    assert abs(ita - itb) <= 1, (ita, itb)
    assert rel_l2(b[I], a[I]) <= 1e-10, rel_l2(b[I], a[I])


@pytest.mark.parametrize("fp32", [False, True])
def test_dirichlet_constant_3d_fused(port, fp32):
    """Constant-coefficient Dirichlet problem in 3D at 48^3 (fused level-0 sweep, constant
    faces with the zero ghost-centre wall term) against the reference multigrid."""
    from scihpc_gb300 import Poisson
    n = 48
    g = O.Grid(3, (n, n, n), (0.0,) * 3, (1.0,) * 3)
    xc = (np.arange(n) + 0.5) / n
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij")
    f = 3 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
    ref, cyc, hist = port.mg_poisson(g, (-f).transpose(2, 1, 0).ravel(), True, 1e-13, 400)
    ref = ghosted_from_mg(g, ref)
    rhs = np.zeros(g.shape)
    rhs[3:-3, 3:-3, 3:-3] = -f
    ps = Poisson(native(g), bc=1, density=False, fp32=fp32)
    p = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    it, rr = ps.solve(dev(rhs), p, rel_tol=1e-12, max_iter=100)
    out = p.cpu().numpy()
    I = g.interior()
    assert rr <= 1e-11, rr
    assert rel_l2(out[I], ref[I]) <= PARITY, rel_l2(out[I], ref[I])


def test_levels_follow_reference_rule(port):
    from scihpc_gb300 import Poisson
    for nd, n in [(2, (128, 256)), (2, (256, 256)), (3, (128, 64, 64)), (3, (64, 64, 64))]:
        g = O.Grid(nd, n, (0,) * nd, (1,) * nd)
        ps = Poisson(native(g), bc=0, density=True, fp32=False)
        assert [tuple(l[:nd]) for l in ps.levels()] == [tuple(l[:nd]) for l in port.mg_levels(nd, n)]


@pytest.mark.parametrize("fp32", [False, True])
@pytest.mark.parametrize("case", ["2d", "3d_fused"])
def test_repeated_solve_graph_replay(fp32, case):
    """A solve repeated with the same inputs runs as a captured CUDA graph (second call: capture
    and launch; third: replay); it gives bit for bit the answer of the host-driven loop, also
    after set_density changes the coefficients between replays."""
    from scihpc_gb300 import Poisson
    n, hi = DENSITY_GRIDS[case]
    g = O.Grid(len(n), n, (0.0,) * len(n), hi)
    rho, rhs = _density_case(g, 11)
    rho2, _ = _density_case(g, 12)
    rho_d, rhs_d = dev(rho), dev(rhs)
    ps = Poisson(native(g), bc=0, density=True, fp32=fp32)
    ps.set_density(rho_d)
    p = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    runs = []
    for _ in range(3):
        p.zero_()
        it, rr = ps.solve(rhs_d, p, rel_tol=1e-11, max_iter=200)
        runs.append((p.cpu().numpy(), it, rr))
    for out, it, rr in runs[1:]:
        assert it == runs[0][1] and rr == runs[0][2], (it, rr, runs[0][1:])
        assert np.array_equal(out, runs[0][0])
    # new coefficients, same buffers: the replay uses them
    rho_d.copy_(dev(rho2))
    ps.set_density(rho_d)
    p.zero_()
    it2, rr2 = ps.solve(rhs_d, p, rel_tol=1e-11, max_iter=200)
    fresh = Poisson(native(g), bc=0, density=True, fp32=fp32)
    fresh.set_density(rho_d)
    q = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    it3, rr3 = fresh.solve(rhs_d, q, rel_tol=1e-11, max_iter=200)   # first call: host loop
    assert it2 == it3 and rr2 == rr3 and rr2 <= 1e-11, (it2, rr2, it3, rr3)
    assert torch.equal(p, q)
    ps.close()
    fresh.close()
