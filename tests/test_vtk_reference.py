"""vtkWriter of the C++ drop-in against the reference's own vtkWriter (vtkWriter.cpp:13-111,
compiled from the reference's sources into oracle/_ref): the same fields written through the
same calls (create, add_scalar of a scalar_data and of a raw array, add_vector of a
vector_data and of three raw arrays) give byte-identical files, in 2D and 3D.  Runs on the
CPU: the drop-in's writer reads host arrays that no GPU session owns."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "vtk_driver.cpp")

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from scihpc_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "vtk_driver")
    r = subprocess.run(["g++", "-O2", "-Wall", DRIVER, "-o", exe] + build.cxx_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("n", [(7, 5), (4, 6, 3)])
def test_vtk_bytes_match_reference(driver, tmp_path, n):
    ndim = len(n)
    shape = tuple(m + 6 for m in n) + ((1,) if ndim == 2 else ())
    rng = np.random.default_rng(5 + ndim)
    fields = [rng.standard_normal(shape) for _ in range(4)]
    fields[0][0, 0, 0] = -0.0        # signed zero and ghost values never reach the file
    fields[1][3, 3, 0] = 1e-300
    src = tmp_path / "in.bin"
    np.concatenate([f.ravel() for f in fields]).tofile(src)
    mine = tmp_path / "mine"
    nn = list(n) + [1] * (3 - ndim)
    r = subprocess.run([driver, str(ndim), *map(str, nn), str(src), str(mine)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ref = tmp_path / "ref"
    lib = O.Checker("ref").lib
    c_n = (ctypes.c_int * 3)(*nn)
    ptrs = [np.ascontiguousarray(f).ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for f in fields]
    assert lib.ref_vtk_write(ndim, c_n, *ptrs, str(ref).encode()) == 0
    a = (tmp_path / "mine0.vtk").read_bytes()
    b = (tmp_path / "ref0.vtk").read_bytes()
    assert len(a) == len(b) and a == b
