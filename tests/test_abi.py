"""C ABI of the CUDA library, checked without a GPU: the library loads, exports every entry
point include/scihpc_gpu.h declares, and its host-side argument checks reject bad input
before any CUDA call."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "scihpc_gpu.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(scihpc_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from scihpc_gb300 import native
    if not os.path.exists(native.LIB_PATH):
        from scihpc_gb300 import build
        build.build()
    return native.Lib()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib.dll, n)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from scihpc_gb300 import native
    assert sorted(native._SIGS) == declared()


def test_version_and_error_strings(lib):
    assert b"sm_103a" in lib.scihpc_version()
    assert lib.scihpc_last_error() is not None


def test_host_argument_checks(lib):
    from scihpc_gb300 import native
    bad = native.Grid(2, (2, 8), (0.0, 0.0), (1.0, 1.0)).c()
    h = ctypes.c_void_p()
    assert lib.scihpc_ctx_create(ctypes.byref(bad), ctypes.byref(h)) == 1
    assert b"n >= 3" in lib.scihpc_last_error()
    g = native.Grid(2, (8, 8), (0.0, 0.0), (1.0, 1.0)).c()
    assert lib.scihpc_poisson_create(ctypes.byref(g), 7, 1, 0, ctypes.byref(h)) == 1
    assert lib.scihpc_poisson_create(ctypes.byref(g), 1, 1, 0, ctypes.byref(h)) == 1   # density + Dirichlet
    vb = (ctypes.c_int * 6)(0, 0, 2, 2, 2, 2)   # periodic walls are not solved by the pressure multigrid
    sb = (ctypes.c_int * 6)(*[1] * 6)
    prm = (ctypes.c_double * 16)(*[1.0] * 16)
    opt = (ctypes.c_int * 5)(1, 5, 1, 0, 1)
    assert lib.scihpc_twophase_create(ctypes.byref(g), vb, sb, prm, opt, ctypes.byref(h)) == 1
    big = native.Grid(3, (200, 200, 200), (0.0,) * 3, (1.0,) * 3).c()
    p4 = (ctypes.c_double * 4)(0.1, 0.001, 0.01, 0.0)
    out = (ctypes.c_double * 2)()
    assert lib.scihpc_lsf_integrals_noalloc(ctypes.byref(big), p4, ctypes.c_void_p(8), out, None) == 1
    assert b"static scratch" in lib.scihpc_last_error()
    # the batched field copies check their arguments before any copy
    names = (ctypes.c_char_p * 1)(b"phi")
    bufs = (ctypes.POINTER(ctypes.c_double) * 1)()
    assert lib.scihpc_twophase_upload_many(None, 1, names, bufs) == 1
    assert b"upload_many" in lib.scihpc_last_error()
    assert lib.scihpc_twophase_download_many(None, -1, names, bufs) == 1
    assert b"download_many" in lib.scihpc_last_error()


def test_build_recipe_targets_sm103a():
    from scihpc_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in build.ARCH
