"""The reference's multigrid Poisson drivers (2D Dirichlet and Neumann, 3D Dirichlet), written
against the GPU-backed multigrid / multigrid_base drop-in headers, converge on the GPU to the
reference multigrid's own solution (the restatement in oracle/port)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.helpers import rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "poisson_driver.cpp")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from scihpc_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "poisson_driver")
    r = subprocess.run(["g++", "-O2", "-Wall", DRIVER, "-o", exe] + build.cxx_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_poisson_driver_compiles_and_links(driver):
    assert os.path.exists(driver)


def reference_solution(dim, n, dirichlet):
    """The reference multigrid (v_cycle) converged to 1e-14 on the driver's problem."""
    if dim == 2:
        lo, hi = ((0.0, -0.5), (1.0, 0.5)) if dirichlet else ((-0.5, -0.5), (0.5, 0.5))
    else:
        lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    g = O.Grid(dim, (n,) * dim, lo, hi)
    c = [g.lo[a] + (np.arange(n) + 0.5) * (g.hi[a] - g.lo[a]) / n for a in range(dim)]
    pi = np.pi
    if dim == 3:
        X, Y, Z = np.meshgrid(*c, indexing="ij")
        rhs = -3 * pi ** 2 * np.sin(pi * X) * np.sin(pi * Y) * np.sin(pi * Z)
        flat = rhs.transpose(2, 1, 0).ravel()   # x fastest
    else:
        X, Y = np.meshgrid(*c, indexing="ij")
        if dirichlet:
            rhs = np.sin(pi * X) * np.cos(pi * Y) + np.sin(5 * pi * X) * np.cos(5 * pi * Y)
        else:
            rhs = -2 * pi ** 2 * np.sin(pi * X) * np.sin(pi * Y) - 50 * pi ** 2 * np.sin(5 * pi * X) * np.sin(5 * pi * Y)
        flat = rhs.T.ravel()
    sol, _, _ = O.Checker("port").mg_poisson(g, flat, bool(dirichlet), 1e-14, 400)
    return np.asarray(sol), float(np.linalg.norm(flat))


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,dirichlet", [(2, 64, 1), (2, 48, 0), (3, 16, 1)],
                         ids=["2d_dirichlet", "2d_neumann", "3d_dirichlet"])
def test_poisson_driver_matches_reference_multigrid(driver, tmp_path, dim, n, dirichlet):
    ref, rnorm = reference_solution(dim, n, dirichlet)
    out = tmp_path / "sol.bin"
    r = subprocess.run([driver, str(dim), str(n), str(dirichlet), repr(1e-12 * rnorm), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    info = dict(ln.split(None, 1) for ln in r.stdout.splitlines() if ln.split()[0] in ("cycles", "residual", "error"))
    assert float(info["residual"]) <= 1e-12 * rnorm, r.stdout
    assert int(info["cycles"]) < 60, r.stdout
    sol = np.fromfile(out, dtype=np.float64)
    if not dirichlet:   # defined up to a constant
        sol, ref = sol - sol.mean(), ref - ref.mean()
    assert rel_l2(sol, ref) <= 1e-9, rel_l2(sol, ref)
