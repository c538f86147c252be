"""second_order_solver (second_order_solver.cpp:7-241) through the GPU-backed drop-in: the
shared solvers' secSol on host arrays (tests/cpp/secorder_driver.cpp) against the oracle,
which is pinned bit for bit to the reference; the stencils are the same arithmetic in the same
order, so the GPU's results are bit for bit too."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.helpers import smooth_field

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "secorder_driver.cpp")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from scihpc_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "secorder_driver")
    r = subprocess.run(["g++", "-O2", "-Wall", DRIVER, "-o", exe] + build.cxx_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_secorder_driver_compiles_and_links(driver):
    assert os.path.exists(driver)


@pytest.mark.gpu
@pytest.mark.parametrize("ndim,n", [(2, (12, 17)), (3, (6, 7, 9))])
def test_second_order_solver_through_drop_in(driver, tmp_path, ndim, n):
    g = O.Grid(ndim, n, (-0.5,) * ndim, (1.5,) * ndim)
    rng = np.random.default_rng(90 + ndim)
    flux = smooth_field(g, rng) + 0.01 * rng.standard_normal(g.shape)
    vel = [rng.standard_normal(g.shape) for _ in range(3)]
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    np.concatenate([flux.ravel()] + [v.ravel() for v in vel]).tofile(inp)
    r = subprocess.run([driver, str(ndim)] + [str(k) for k in n] + ["-0.5", "1.5", str(inp), str(out)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.float64).reshape((15,) + g.shape)
    port = O.Checker("port")
    central, upwind = port.sec(g, flux), port.sec(g, flux, *vel)
    for k in range(9):
        if (k % 3) < ndim and (k < 6 or ndim > 2 or k == 6):
            assert np.array_equal(raw[k], central[k]), k
    for k in range(6):
        if (k % 3) < ndim:
            assert np.array_equal(raw[9 + k], upwind[k]), k
