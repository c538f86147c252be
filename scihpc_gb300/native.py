"""ctypes binding of the C ABI in include/scihpc_gpu.h.

Device arrays are passed as raw pointers (``int``) -- callers typically hold them in
``torch`` CUDA tensors of dtype float64 and shape ``Grid.shape`` -- and streams as raw
``cudaStream_t`` values (0 = legacy default stream).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libscihpc_gb300.so")

BC = {"periodic": 0, "neumann": 1, "no_slip": 2, "slip": 3, "dirichlet": 4}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


class LibraryNotBuilt(RuntimeError):
    pass


class ScihpcError(RuntimeError):
    def __init__(self, rc: int, msg: str):
        super().__init__(f"scihpc status {rc}: {msg}")
        self.rc = rc


class _GridC(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("n", ctypes.c_int * 3), ("lo", ctypes.c_double * 3),
                ("hi", ctypes.c_double * 3)]


@dataclass(frozen=True)
class Grid:
    """Uniform cell-centred grid: n interior cells on [lo, hi] per axis (structured_grid)."""
    ndim: int
    n: tuple
    lo: tuple
    hi: tuple

    @property
    def shape(self) -> tuple:
        return (self.n[0] + 6, self.n[1] + 6 if self.ndim > 1 else 1, self.n[2] + 6 if self.ndim > 2 else 1)

    @property
    def size(self) -> int:
        return int(np.prod(self.shape))

    def spacing(self) -> list:
        return [(self.hi[a] - self.lo[a]) / self.n[a] for a in range(self.ndim)]

    def c(self) -> _GridC:
        g = _GridC()
        g.ndim = self.ndim
        for a in range(3):
            g.n[a] = self.n[a] if a < self.ndim else 1
            g.lo[a] = self.lo[a] if a < self.ndim else 0.0
            g.hi[a] = self.hi[a] if a < self.ndim else 1.0
        return g

    def interior(self) -> tuple:
        return tuple(slice(3, -3) if a < self.ndim else slice(0, 1) for a in range(3))


_SIGS = {
    "scihpc_last_error": ([], ctypes.c_char_p),
    "scihpc_version": ([], ctypes.c_char_p),
    "scihpc_ctx_create": ([ctypes.POINTER(_GridC), ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_ctx_destroy": ([_vp], ctypes.c_int),
    "scihpc_bc_fill": ([_vp, ctypes.c_int, _ip, _dp, _vp, _vp], ctypes.c_int),
    "scihpc_flux_extrapolate": ([_vp, ctypes.c_int, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_zero_order_extrapolation": ([_vp, _vp, _vp], ctypes.c_int),
    "scihpc_uccd": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_ccd": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_flux_fill": ([_vp, ctypes.c_int, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_sec_derivative": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_sec_mixed": ([_vp, ctypes.c_int, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_rk3_stage": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, _vp, _vp, _vp, _vp, _vp, _vp],
                         ctypes.c_int),
    "scihpc_ccd_mixed": ([_vp, ctypes.c_int, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_weno5": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_godunov_gradient": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_stabilized_upon_gradient": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_guess_from_history": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_lsf_fields": ([_vp, _dp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_curvature": ([_vp, _vp, ctypes.POINTER(_vp), _vp, _vp], ctypes.c_int),
    "scihpc_lsf_integrals": ([_vp, _dp, _vp, _dp, _vp], ctypes.c_int),
    "scihpc_lsf_integrals_noalloc": ([ctypes.POINTER(_GridC), _dp, _vp, _dp, _vp], ctypes.c_int),
    "scihpc_poisson_create": ([ctypes.POINTER(_GridC), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_poisson_destroy": ([_vp], ctypes.c_int),
    "scihpc_poisson_set_density": ([_vp, _vp, _vp], ctypes.c_int),
    "scihpc_poisson_solve": ([_vp, _vp, _vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _ip, _dp, _vp],
                             ctypes.c_int),
    "scihpc_poisson_time_vcycles": ([_vp, _vp, _vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float), _vp],
                                    ctypes.c_int),
    "scihpc_poisson_levels": ([_vp, _ip, ctypes.c_int], ctypes.c_int),
    "scihpc_poisson_residual": ([_vp, _vp, _vp, _dp, _vp], ctypes.c_int),
    "scihpc_poisson_set_inner": ([_vp, ctypes.c_double, ctypes.c_int], ctypes.c_int),
    "scihpc_twophase_create": ([ctypes.POINTER(_GridC), _ip, _ip, _dp, _ip, ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_twophase_destroy": ([_vp], ctypes.c_int),
    "scihpc_twophase_upload": ([_vp, ctypes.c_char_p, _dp], ctypes.c_int),
    "scihpc_twophase_download": ([_vp, ctypes.c_char_p, _dp], ctypes.c_int),
    "scihpc_twophase_upload_many": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_dp)],
                                    ctypes.c_int),
    "scihpc_twophase_download_many": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_dp)],
                                      ctypes.c_int),
    "scihpc_twophase_field": ([_vp, ctypes.c_char_p, ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_twophase_checkpoint": ([_vp, ctypes.c_char_p], ctypes.c_int),
    "scihpc_twophase_restore": ([_vp, ctypes.c_char_p], ctypes.c_int),
    "scihpc_twophase_get_scalars": ([_vp, _dp], ctypes.c_int),
    "scihpc_twophase_set_scalars": ([_vp, _dp], ctypes.c_int),
    "scihpc_twophase_init": ([_vp], ctypes.c_int),
    "scihpc_twophase_find_dt": ([_vp], ctypes.c_int),
    "scihpc_twophase_advect": ([_vp], ctypes.c_int),
    "scihpc_twophase_mpls": ([_vp, ctypes.c_int], ctypes.c_int),
    "scihpc_twophase_reinit": ([_vp, _ip], ctypes.c_int),
    "scihpc_twophase_find_source": ([_vp], ctypes.c_int),
    "scihpc_twophase_find_sign": ([_vp], ctypes.c_int),
    "scihpc_twophase_reinit_step": ([_vp, ctypes.c_int], ctypes.c_int),
    "scihpc_twophase_set_scheme": ([_vp, ctypes.c_int], ctypes.c_int),
    "scihpc_twophase_set_source_scheme": ([_vp, ctypes.c_int], ctypes.c_int),
    "scihpc_conv3x3": ([_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp],
                       ctypes.c_int),
    "scihpc_conv3x3_wgrad": ([_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, _vp], ctypes.c_int),
    "scihpc_unet_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_unet_create3": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_unet_create_coarse": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.POINTER(_vp)],
                                  ctypes.c_int),
    "scihpc_conv3x3x3": ([_vp, _vp, _vp, _vp] + [ctypes.c_int] * 6 + [_vp], ctypes.c_int),
    "scihpc_conv3x3x3_wgrad": ([_vp, _vp, _vp, _vp] + [ctypes.c_int] * 6 + [_vp], ctypes.c_int),
    "scihpc_unet_destroy": ([_vp], ctypes.c_int),
    "scihpc_unet_num_params": ([_vp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "scihpc_unet_set_weights": ([_vp, _vp, ctypes.c_longlong], ctypes.c_int),
    "scihpc_unet_get_weights": ([_vp, _vp, ctypes.c_longlong], ctypes.c_int),
    "scihpc_unet_get_gradient": ([_vp, _vp, ctypes.c_longlong], ctypes.c_int),
    "scihpc_unet_infer": ([_vp, ctypes.POINTER(_GridC), _vp, _vp, _vp, _vp], ctypes.c_int),
    "scihpc_unet_loss_grad": ([_vp, ctypes.POINTER(_GridC), _vp, _vp, _vp, _vp, _dp], ctypes.c_int),
    "scihpc_unet_train_step": ([_vp, ctypes.POINTER(_GridC), _vp, _vp, _vp, _vp, ctypes.c_float, _dp], ctypes.c_int),
    "scihpc_unet_stream": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_twophase_ab_solve": ([_vp, _ip, _dp], ctypes.c_int),
    "scihpc_twophase_intermediate_velocity": ([_vp], ctypes.c_int),
    "scihpc_twophase_projection": ([_vp, _ip, _dp], ctypes.c_int),
    "scihpc_twophase_node_from_face": ([_vp], ctypes.c_int),
    "scihpc_twophase_set_ppe_schedule": ([_vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "scihpc_twophase_time_reinit_gradient": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "scihpc_measure_fp64_peak": ([_dp], ctypes.c_int),
    "scihpc_twophase_pressure_guess": ([_vp], ctypes.c_int),
    "scihpc_twophase_fpc_coefficients": ([_vp], ctypes.c_int),
    "scihpc_twophase_fast_pressure_correction": ([_vp, _ip, _dp], ctypes.c_int),
    "scihpc_twophase_step": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "scihpc_twophase_diagnostics": ([_vp, _dp], ctypes.c_int),
    "scihpc_twophase_stream": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
    "scihpc_twophase_ppe_stats": ([_vp, _dp], ctypes.c_int),
    "scihpc_twophase_graph_stats": ([_vp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
}


class Lib:
    def __init__(self, path: str = LIB_PATH):
        if not os.path.exists(path):
            raise LibraryNotBuilt(f"{path} is missing: run `python -m scihpc_gb300.build` (no CPU fallback exists)")
        self.path = path
        self.dll = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            f = getattr(self.dll, name)
            f.argtypes = args
            f.restype = res

    def __getattr__(self, name):
        return getattr(self.dll, name)

    def check(self, rc: int) -> None:
        if rc != 0:
            raise ScihpcError(rc, self.dll.scihpc_last_error().decode())

    def exported(self) -> list:
        return list(_SIGS)


_LIB = None


def lib() -> Lib:
    global _LIB
    if _LIB is None:
        _LIB = Lib()
    return _LIB


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


class Workspace:
    """scihpc_ctx: per-grid kernel workspace (factored line operators, scratch)."""

    def __init__(self, grid: Grid):
        self.L = lib()
        self.grid = grid
        self.h = _vp()
        self._g = grid.c()
        self.L.check(self.L.scihpc_ctx_create(ctypes.byref(self._g), ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.L.scihpc_ctx_destroy(self.h)
            self.h = _vp()

    __del__ = close

    def bc_fill(self, location, types, values, f, stream=0):
        t = (ctypes.c_int * 6)(*types)
        v = (ctypes.c_double * 6)(*values)
        self.L.check(self.L.scihpc_bc_fill(self.h, location, t, v, _ptr(f), stream))

    def flux_extrapolate(self, location, data, flux, stream=0):
        self.L.check(self.L.scihpc_flux_extrapolate(self.h, location, _ptr(data), _ptr(flux), stream))

    def zero_order_extrapolation(self, f, stream=0):
        self.L.check(self.L.scihpc_zero_order_extrapolation(self.h, _ptr(f), stream))

    def uccd(self, axis, flux, vel, f1, f2, stream=0):
        self.L.check(self.L.scihpc_uccd(self.h, axis, _ptr(flux), _ptr(vel), _ptr(f1), _ptr(f2), stream))

    def ccd(self, axis, flux, f1, f2, stream=0):
        self.L.check(self.L.scihpc_ccd(self.h, axis, _ptr(flux), _ptr(f1), _ptr(f2), stream))

    def ccd_mixed(self, axis, src, out, stream=0):
        self.L.check(self.L.scihpc_ccd_mixed(self.h, axis, _ptr(src), _ptr(out), stream))

    def sec_derivative(self, axis, flux, vel, f1, f2, stream=0):
        """second_order_solver::find_fx/fy/fz: central (vel None) or upwind-biased."""
        self.L.check(self.L.scihpc_sec_derivative(self.h, axis, _ptr(flux), _ptr(vel), _ptr(f1), _ptr(f2), stream))

    def sec_mixed(self, axis, src, out, stream=0):
        self.L.check(self.L.scihpc_sec_mixed(self.h, axis, _ptr(src), _ptr(out), stream))

    def weno5(self, axis, flux, vel, fa, stream=0):
        self.L.check(self.L.scihpc_weno5(self.h, axis, _ptr(flux), _ptr(vel), _ptr(fa), stream))

    def godunov_gradient(self, phi, sign, grad, stream=0):
        self.L.check(self.L.scihpc_godunov_gradient(self.h, _ptr(phi), _ptr(sign), _ptr(grad), stream))

    def stabilized_upon_gradient(self, phi, sign, grad, stream=0):
        """grad = Godunov |grad phi|, then phi /= max(grad) in place (godunov_gradient.cpp:159-181)."""
        self.L.check(self.L.scihpc_stabilized_upon_gradient(self.h, _ptr(phi), _ptr(sign), _ptr(grad), stream))

    def guess_from_history(self, old, old2, flux, stream=0):
        """flux = 2 old - old2 on every cell (flux.cpp:653-662)."""
        self.L.check(self.L.scihpc_guess_from_history(self.h, _ptr(old), _ptr(old2), _ptr(flux), stream))

    def lsf_fields(self, prm, phi, H=None, delta=None, sign=None, rho=None, mu=None, stream=0):
        p = (ctypes.c_double * 4)(*prm)
        self.L.check(self.L.scihpc_lsf_fields(self.h, p, _ptr(phi), _ptr(H), _ptr(delta), _ptr(sign), _ptr(rho),
                                              _ptr(mu), stream))

    def curvature(self, phi, derivs, curv, stream=0):
        arr = (_vp * 9)(*[_ptr(d) for d in derivs])
        self.L.check(self.L.scihpc_curvature(self.h, _ptr(phi), arr, _ptr(curv), stream))

    def lsf_integrals(self, prm, phi, stream=0):
        p = (ctypes.c_double * 4)(*prm)
        out = (ctypes.c_double * 2)()
        self.L.check(self.L.scihpc_lsf_integrals(self.h, p, _ptr(phi), out, stream))
        return out[0], out[1]


def lsf_integrals_noalloc(grid: Grid, prm, phi, stream=0):
    """lsf_mass and lsf_volume without any device allocation (static scratch; see the header)."""
    L = lib()
    g = grid.c()
    p = (ctypes.c_double * 4)(*prm)
    out = (ctypes.c_double * 2)()
    L.check(L.scihpc_lsf_integrals_noalloc(ctypes.byref(g), p, _ptr(phi), out, stream))
    return out[0], out[1]


class Poisson:
    """scihpc_poisson: multigrid-preconditioned pressure solver."""

    def __init__(self, grid: Grid, bc: int = 0, density: bool = True, fp32: bool = False):
        self.L = lib()
        self.grid = grid
        self.h = _vp()
        self._g = grid.c()
        self.L.check(self.L.scihpc_poisson_create(ctypes.byref(self._g), bc, int(density), int(fp32),
                                                  ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.L.scihpc_poisson_destroy(self.h)
            self.h = _vp()

    __del__ = close

    def set_density(self, rho, stream=0):
        self.L.check(self.L.scihpc_poisson_set_density(self.h, _ptr(rho), stream))

    def solve(self, rhs, p, use_guess=False, rel_tol=1e-10, max_iter=200, stream=0):
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        rc = self.L.scihpc_poisson_solve(self.h, _ptr(rhs), _ptr(p), int(use_guess), rel_tol, max_iter,
                                         ctypes.byref(it), ctypes.byref(rr), stream)
        if rc not in (0, 4):
            self.L.check(rc)
        return it.value, rr.value

    def time_vcycles(self, rhs, p, ncycles, stream=0) -> float:
        ms = ctypes.c_float(0.0)
        self.L.check(self.L.scihpc_poisson_time_vcycles(self.h, _ptr(rhs), _ptr(p), ncycles, ctypes.byref(ms), stream))
        return ms.value

    def set_inner(self, inner_tol: float, inner_max: int) -> None:
        """FP32 mode: residual reduction and iteration cap of each inner FP32 solve."""
        self.L.check(self.L.scihpc_poisson_set_inner(self.h, float(inner_tol), int(inner_max)))

    def residual(self, rhs, p, stream=0) -> float:
        """||rhs - A p|| over the interior cells (FP64, on the GPU)."""
        out = ctypes.c_double(0.0)
        self.L.check(self.L.scihpc_poisson_residual(self.h, _ptr(rhs), _ptr(p), ctypes.byref(out), stream))
        return out.value

    def levels(self) -> list:
        buf = (ctypes.c_int * 96)()
        n = self.L.scihpc_poisson_levels(self.h, buf, 32)
        return [tuple(buf[3 * l:3 * l + 3]) for l in range(n)]


PARAM_ORDER = ["density_ratio", "viscosity_ratio", "Re", "Fr", "We", "ls_width", "rdt", "max_CFL", "min_CFL",
               "positive_ref", "ppe_tol", "ppe_tol2", "ppe_max_iter", "ppe_omega", "ppe_initer", "dt0"]
PARAM_DEFAULT = dict(density_ratio=1.0, viscosity_ratio=1.0, Re=1.0, Fr=-1.0, We=-1.0, ls_width=0.0, rdt=0.0,
                     max_CFL=0.01, min_CFL=0.01, positive_ref=1.0, ppe_tol=1e-10, ppe_tol2=0.0, ppe_max_iter=200,
                     ppe_omega=1.5, ppe_initer=1, dt0=1.0)
SCALARS = ["t", "dt", "dt_old", "dt_old2", "iter", "stable_CFL", "lsf_mass0"]


class TwoPhase:
    """scihpc_twophase: one two-phase problem resident on the GPU."""

    def __init__(self, grid: Grid, vel_bc, scalar_bc, prm: dict, scheme=1, n_mpls=5, reinit_every=1, fp32=False,
                 reinit_lambda=True):
        self.L = lib()
        self.grid = grid
        P = dict(PARAM_DEFAULT)
        P.update(prm)
        pa = (ctypes.c_double * 16)(*[float(P[k]) for k in PARAM_ORDER])
        oa = (ctypes.c_int * 5)(scheme, n_mpls, reinit_every, int(fp32), int(reinit_lambda))
        vb = (ctypes.c_int * 6)(*[BC[b] if isinstance(b, str) else b for b in vel_bc])
        sb = (ctypes.c_int * 6)(*[BC[b] if isinstance(b, str) else b for b in scalar_bc])
        self.h = _vp()
        self._g = grid.c()
        self.L.check(self.L.scihpc_twophase_create(ctypes.byref(self._g), vb, sb, pa, oa, ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.L.scihpc_twophase_destroy(self.h)
            self.h = _vp()

    __del__ = close

    def set(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.grid.shape, (a.shape, self.grid.shape)
        self.L.check(self.L.scihpc_twophase_upload(self.h, name.encode(), a.ctypes.data_as(_dp)))

    def get(self, name: str) -> np.ndarray:
        out = np.zeros(self.grid.shape)
        self.L.check(self.L.scihpc_twophase_download(self.h, name.encode(), out.ctypes.data_as(_dp)))
        return out

    def device_ptr(self, name: str) -> int:
        p = _vp()
        self.L.check(self.L.scihpc_twophase_field(self.h, name.encode(), ctypes.byref(p)))
        return p.value

    def checkpoint(self, path: str) -> None:
        self.L.check(self.L.scihpc_twophase_checkpoint(self.h, str(path).encode()))

    def restore(self, path: str) -> None:
        self.L.check(self.L.scihpc_twophase_restore(self.h, str(path).encode()))

    def scalars(self) -> dict:
        out = (ctypes.c_double * 7)()
        self.L.check(self.L.scihpc_twophase_get_scalars(self.h, out))
        return dict(zip(SCALARS, list(out)))

    def set_scalars(self, **kw) -> None:
        s = self.scalars()
        s.update(kw)
        arr = (ctypes.c_double * 7)(*[s[k] for k in SCALARS])
        self.L.check(self.L.scihpc_twophase_set_scalars(self.h, arr))

    def init(self):
        self.L.check(self.L.scihpc_twophase_init(self.h))

    def find_dt(self):
        self.L.check(self.L.scihpc_twophase_find_dt(self.h))

    def advect(self):
        self.L.check(self.L.scihpc_twophase_advect(self.h))

    def mpls(self, count):
        self.L.check(self.L.scihpc_twophase_mpls(self.h, count))

    def reinit(self) -> int:
        n = ctypes.c_int(0)
        self.L.check(self.L.scihpc_twophase_reinit(self.h, ctypes.byref(n)))
        return n.value

    def find_source(self):
        self.L.check(self.L.scihpc_twophase_find_source(self.h))

    def find_sign(self):
        self.L.check(self.L.scihpc_twophase_find_sign(self.h))

    def reinit_step(self, lambda_correction=True):
        self.L.check(self.L.scihpc_twophase_reinit_step(self.h, int(lambda_correction)))

    def set_scheme(self, scheme: int):
        self.L.check(self.L.scihpc_twophase_set_scheme(self.h, scheme))

    def set_source_scheme(self, scheme: int):
        """find_source's derivatives: 0 compact (CCD/UCCD), 1 second order (find_source_sec)."""
        self.L.check(self.L.scihpc_twophase_set_source_scheme(self.h, scheme))

    def ab_solve(self):
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        self.L.check(self.L.scihpc_twophase_ab_solve(self.h, ctypes.byref(it), ctypes.byref(rr)))
        return it.value, rr.value

    def set_ppe_schedule(self, schedule: int, tol_mode: int = 0):
        """0: the projection equation every step; 1: the reference's schedule (projection while
        iter < 5, then the fast pressure correction).  tol_mode 1: ppe_tol is absolute."""
        self.L.check(self.L.scihpc_twophase_set_ppe_schedule(self.h, schedule, tol_mode))

    def pressure_guess(self):
        self.L.check(self.L.scihpc_twophase_pressure_guess(self.h))

    def fpc_coefficients(self):
        self.L.check(self.L.scihpc_twophase_fpc_coefficients(self.h))

    def fast_pressure_correction(self):
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        self.L.check(self.L.scihpc_twophase_fast_pressure_correction(self.h, ctypes.byref(it), ctypes.byref(rr)))
        return it.value, rr.value

    def step(self, nsteps=1, graph=False, sync=True):
        self.L.check(self.L.scihpc_twophase_step(self.h, nsteps, int(graph), int(sync)))

    def diagnostics(self) -> dict:
        out = (ctypes.c_double * 3)()
        self.L.check(self.L.scihpc_twophase_diagnostics(self.h, out))
        return dict(mass=out[0], volume=out[1], div=out[2])

    def stream(self) -> int:
        p = _vp()
        self.L.check(self.L.scihpc_twophase_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    def graph_stats(self) -> dict:
        out = (ctypes.c_longlong * 4)()
        self.L.check(self.L.scihpc_twophase_graph_stats(self.h, out))
        return dict(pre=out[0], body=out[1], post=out[2], ppe_iters_total=out[3])

    def upload_ptr(self, name: str, host_ptr: int) -> None:
        self.L.check(self.L.scihpc_twophase_upload(self.h, name.encode(), ctypes.cast(host_ptr, _dp)))

    def download_ptr(self, name: str, host_ptr: int) -> None:
        self.L.check(self.L.scihpc_twophase_download(self.h, name.encode(), ctypes.cast(host_ptr, _dp)))

    @staticmethod
    def _many(names, host_ptrs):
        n = len(names)
        assert len(host_ptrs) == n
        nm = (ctypes.c_char_p * n)(*[x.encode() for x in names])
        hp = (_dp * n)(*[ctypes.cast(p, _dp) for p in host_ptrs])
        return n, nm, hp

    def upload_many_ptr(self, names, host_ptrs) -> None:
        """Several fields from host memory in one call (one synchronisation)."""
        n, nm, hp = self._many(names, host_ptrs)
        self.L.check(self.L.scihpc_twophase_upload_many(self.h, n, nm, hp))

    def download_many_ptr(self, names, host_ptrs) -> None:
        """Several fields to host memory in one call (one synchronisation)."""
        n, nm, hp = self._many(names, host_ptrs)
        self.L.check(self.L.scihpc_twophase_download_many(self.h, n, nm, hp))

    def time_reinit_gradient(self, n: int = 100) -> float:
        """ms per launch of the reinitialisation's gradient kernel (measurement hook)."""
        ms = ctypes.c_float(0.0)
        self.L.check(self.L.scihpc_twophase_time_reinit_gradient(self.h, n, ctypes.byref(ms)))
        return ms.value

    def ppe_stats(self) -> dict:
        out = (ctypes.c_double * 3)()
        self.L.check(self.L.scihpc_twophase_ppe_stats(self.h, out))
        return dict(iters=out[0], relres=out[1], ms=out[2])


def measure_fp64_peak() -> float:
    """FP64 TFLOP/s of fused multiply-add chains on the current device (measurement hook)."""
    L = lib()
    t = ctypes.c_double(0.0)
    L.check(L.scihpc_measure_fp64_peak(ctypes.byref(t)))
    return t.value


def conv3x3(x, w, bias, out, h: int, wd: int, ci: int, co: int, relu: bool = False):
    """scihpc_conv3x3 on device tensors: x BF16 [h*w][ci], w BF16 [co][9][ci], out FP32."""
    lib().check(lib().scihpc_conv3x3(_ptr(x), _ptr(w), _ptr(bias), _ptr(out), h, wd, ci, co, int(relu), None))


def conv3x3_wgrad(x, dz, dw, partial, splits: int, h: int, wd: int, ci: int, co: int):
    """scihpc_conv3x3_wgrad on device tensors: dw FP32 [co][9][ci]."""
    lib().check(lib().scihpc_conv3x3_wgrad(_ptr(x), _ptr(dz), _ptr(dw), _ptr(partial), splits, h, wd, ci, co, None))


def conv3x3x3(x, w, bias, out, d: int, h: int, wd: int, ci: int, co: int, relu: bool = False):
    """scihpc_conv3x3x3 on device tensors: x BF16 [d*h*w][ci], w BF16 [co][27][ci], out FP32."""
    lib().check(lib().scihpc_conv3x3x3(_ptr(x), _ptr(w), _ptr(bias), _ptr(out), d, h, wd, ci, co, int(relu), None))


def conv3x3x3_wgrad(x, dz, dw, partial, splits: int, d: int, h: int, wd: int, ci: int, co: int):
    """scihpc_conv3x3x3_wgrad on device tensors: dw FP32 [co][27][ci]."""
    lib().check(lib().scihpc_conv3x3x3_wgrad(_ptr(x), _ptr(dz), _ptr(dw), _ptr(partial), splits, d, h, wd, ci, co,
                                             None))


class UNet:
    """scihpc_unet: the learned initial guess of the pressure solve (tensor-core U-Net).
    UNet(h, w) is the 2D network of an h x w grid; UNet(h, w, factor=F) the same network on
    the grid coarsened F x F predicting a coarse correction; UNet(n0, n1, n2) the 3D network
    of an n0 x n1 x n2 grid (run at half resolution)."""

    def __init__(self, h: int, w: int, d: int | None = None, seed: int = 0, factor: int = 1):
        self.L = lib()
        self.h = _vp()
        if d is None and factor > 1:
            self.L.check(self.L.scihpc_unet_create_coarse(h, w, factor, seed, ctypes.byref(self.h)))
        elif d is None:
            self.L.check(self.L.scihpc_unet_create(h, w, seed, ctypes.byref(self.h)))
        else:
            self.L.check(self.L.scihpc_unet_create3(h, w, d, seed, ctypes.byref(self.h)))
        n = ctypes.c_longlong(0)
        self.L.check(self.L.scihpc_unet_num_params(self.h, ctypes.byref(n)))
        self.nparam = n.value

    def close(self):
        if self.h:
            self.L.scihpc_unet_destroy(self.h)
            self.h = _vp()

    __del__ = close

    def weights(self):
        import numpy as np
        a = np.zeros(self.nparam, dtype=np.float32)
        self.L.check(self.L.scihpc_unet_get_weights(self.h, a.ctypes.data, self.nparam))
        return a

    def gradient(self):
        import numpy as np
        a = np.zeros(self.nparam, dtype=np.float32)
        self.L.check(self.L.scihpc_unet_get_gradient(self.h, a.ctypes.data, self.nparam))
        return a

    def set_weights(self, a):
        import numpy as np
        a = np.ascontiguousarray(a, dtype=np.float32)
        self.L.check(self.L.scihpc_unet_set_weights(self.h, a.ctypes.data, self.nparam))

    def infer(self, grid: Grid, rho, rhs, pprev, guess):
        g = grid.c()
        self.L.check(self.L.scihpc_unet_infer(self.h, ctypes.byref(g), _ptr(rho), _ptr(rhs), _ptr(pprev), _ptr(guess)))

    def loss_grad(self, grid: Grid, rho, rhs, pprev, p) -> float:
        g = grid.c()
        loss = ctypes.c_double(0.0)
        self.L.check(self.L.scihpc_unet_loss_grad(self.h, ctypes.byref(g), _ptr(rho), _ptr(rhs), _ptr(pprev), _ptr(p),
                                                  ctypes.byref(loss)))
        return loss.value

    def train_step(self, grid: Grid, rho, rhs, pprev, p, lr: float) -> float:
        g = grid.c()
        loss = ctypes.c_double(0.0)
        self.L.check(self.L.scihpc_unet_train_step(self.h, ctypes.byref(g), _ptr(rho), _ptr(rhs), _ptr(pprev), _ptr(p),
                                                   ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value
