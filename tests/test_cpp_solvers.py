"""The reference's derivative solver classes and level-set helpers (ccd_solver, uccd_solver,
weno_solver from SharedSolvers_alloc; find_heavyside / find_delta / find_density /
find_viscosity / find_curvature; godunov_gradient; identity_with_extrapolation), called by a
C++ driver through the GPU-backed drop-in headers, against the CPU restatement of the
reference (oracle/port) on the same seeded inputs."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.helpers import grid2, smooth_field

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "solvers_driver.cpp")
TOL, TOL_UCCD = 1e-12, 1e-9   # as in test_gpu_kernels.py


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from scihpc_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "solvers_driver")
    r = subprocess.run(["g++", "-O2", "-Wall", DRIVER, "-o", exe] + build.cxx_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_solvers_driver_compiles_and_links(driver):
    assert os.path.exists(driver)


def near(a, b, tol):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
def test_solver_classes_match_oracle(driver, tmp_path):
    torch = pytest.importorskip("torch")
    g = grid2(24, 40)
    rng = np.random.default_rng(31)
    flux = smooth_field(g, rng)
    u, v = rng.standard_normal(g.shape), rng.standard_normal(g.shape)
    phi = 0.2 * smooth_field(g, rng)
    sign = np.sign(rng.standard_normal(g.shape))
    h = min(g.spacing())
    prm = [1.5 * h, 0.001, 0.01, 0.0]
    fin = tmp_path / "in.bin"
    np.concatenate([a.ravel() for a in (flux, u, v, phi, sign)]).astype(np.float64).tofile(fin)
    fout = tmp_path / "out.bin"
    args = [driver, str(fin), str(fout), str(g.n[0]), str(g.n[1]), repr(g.lo[0]), repr(g.hi[0]), repr(g.lo[1]),
            repr(g.hi[1])] + [repr(x) for x in prm[:3]]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(fout, dtype=np.float64)
    n = int(np.prod(g.shape))
    out = [raw[q * n:(q + 1) * n].reshape(g.shape) for q in range(raw.size // n)]
    assert len(out) == 21
    port = O.Checker("port")
    zeros = np.zeros(g.shape)
    ccd = port.ccd(g, flux, mixed=True)
    for q, k in enumerate((0, 1, 3, 4, 6)):   # fx fy fxx fyy fxy
        assert near(out[q], ccd[k], TOL), ("ccd", q)
    uccd = port.uccd(g, flux, u, v, zeros)
    for q, k in enumerate((0, 1, 3, 4)):
        assert near(out[5 + q], uccd[k], TOL_UCCD), ("uccd", q)
    weno = port.weno5(g, flux, u, v, zeros)
    I = g.interior()
    for q in range(2):
        assert near(out[9 + q][I], weno[q][I], TOL), ("weno", q)
    fields = port.lsf_fields(g, prm + [0.0], phi)
    for q, k in enumerate((0, 1, 3, 4)):   # heaviside delta density viscosity
        assert np.abs(out[11 + q] - fields[k]).max() <= 1e-14 * max(1.0, np.abs(fields[k]).max()), ("fields", q)
    assert near(out[15], port.godunov(g, phi, sign), TOL), "godunov"
    assert np.array_equal(out[16], port.flux_extrapolate(g, 0, phi)), "identity_with_extrapolation"
    # curvature of the drop-in = the library's curvature kernel on the same CCD derivatives
    from scihpc_gb300 import Grid, Workspace
    w = Workspace(Grid(2, tuple(g.n), tuple(g.lo), tuple(g.hi)))
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    derivs = [d(out[0]), d(out[1]), d(zeros), d(out[2]), d(out[3]), d(zeros), d(out[4]), d(zeros), d(zeros)]
    curv = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    w.curvature(d(phi), derivs, curv)
    torch.cuda.synchronize()
    assert np.array_equal(out[17], curv.cpu().numpy())
    ext = port.flux_extrapolate(g, 0, phi)
    assert np.array_equal(out[18], port.guess_from_history(g, phi, ext)), "guess_from_history"
    st_phi, st_grad = port.stabilize(g, phi, sign)
    assert near(out[19], st_phi, TOL), "stabilized_upon_gradient phi"
    assert near(out[20], st_grad, TOL), "stabilized_upon_gradient grad"


@pytest.mark.gpu
def test_projection_stages_compose_to_ab_solve():
    """find_source + find_intermediate_velocity + projection + node_from_face through the C
    ABI give the fields of one ab_solve (the same kernels, run stage by stage)."""
    pytest.importorskip("torch")
    import ctypes
    from scihpc_gb300 import Grid, TwoPhase
    from tests.helpers import bubble_params, bubble_phi
    g = O.Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
    prm = bubble_params(g, ppe_tol=1e-12)
    res = []
    for staged in (False, True):
        tp = TwoPhase(Grid(2, tuple(g.n), tuple(g.lo), tuple(g.hi)), ["no_slip"] * 6, ["neumann"] * 6, prm, scheme=1)
        tp.set("phi", bubble_phi(g, (0.45, 0.55), 0.23))
        tp.init()
        tp.find_dt()
        if staged:
            tp.L.check(tp.L.scihpc_twophase_find_source(tp.h))
            tp.L.check(tp.L.scihpc_twophase_intermediate_velocity(tp.h))
            it, rr = ctypes.c_int(0), ctypes.c_double(0.0)
            tp.L.check(tp.L.scihpc_twophase_projection(tp.h, ctypes.byref(it), ctypes.byref(rr)))
            tp.L.check(tp.L.scihpc_twophase_node_from_face(tp.h))
        else:
            tp.ab_solve()
        res.append({nm: tp.get(nm) for nm in ("p", "u", "v", "nu", "nv")})
        tp.close()
    for nm in res[0]:
        a, b = res[0][nm], res[1][nm]
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(a).max(), 1e-300), nm
