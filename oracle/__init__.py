"""TEST INFRASTRUCTURE: ctypes access to the CPU checkers.

Two libraries expose the same C entry points (``<prefix>_bc_fill``, ``<prefix>_uccd``,
``<prefix>_tp_step`` ...) over flat ``[Nx][Ny][Nz]`` float64 arrays:

* ``port`` -- this project's CPU restatement of the reference's algorithms
  (``oracle/port/*.cpp``), built anywhere from committed sources.  It is the checker on
  machines without the reference sources and the timed CPU baseline.
* ``ref``  -- the reference implementation itself, compiled from its own sources by
  ``oracle/Makefile`` plus ``oracle/ref_shim.cpp``; present only where those sources are.

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU leg of ``bench.py`` use this
module.  The product package ``scihpc_gb300`` never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libscihpc_port.so")
REF_SO = os.path.join(HERE, "_ref", "libscihpc_ref.so")

BC = {"periodic": 0, "neumann": 1, "no_slip": 2, "slip": 3, "dirichlet": 4}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(ref: bool = True) -> None:
    """Compile the restatement (always) and the reference (when its sources exist: the
    recipe in ``oracle/Makefile`` locates them, ``SCIHPC_REFERENCE_DIR`` overrides)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


@dataclass
class Grid:
    ndim: int
    n: tuple
    lo: tuple
    hi: tuple

    @property
    def shape(self):
        nx = self.n[0] + 6
        ny = self.n[1] + 6 if self.ndim > 1 else 1
        nz = self.n[2] + 6 if self.ndim > 2 else 1
        return (nx, ny, nz)

    def c_args(self):
        n = (ctypes.c_int * 3)(*(list(self.n) + [1] * (3 - len(self.n))))
        lo = (ctypes.c_double * 3)(*(list(self.lo) + [0.0] * (3 - len(self.lo))))
        hi = (ctypes.c_double * 3)(*(list(self.hi) + [1.0] * (3 - len(self.hi))))
        return n, lo, hi

    def spacing(self):
        return [(self.hi[a] - self.lo[a]) / self.n[a] for a in range(self.ndim)]

    def interior(self):
        sl = []
        for a in range(3):
            sl.append(slice(3, -3) if a < self.ndim else slice(0, 1))
        return tuple(sl)


class Checker:
    """One of the two CPU libraries ('port' or 'ref')."""

    def __init__(self, which: str = "port"):
        path = PORT_SO if which == "port" else REF_SO
        if not os.path.exists(path):
            build(ref=(which == "ref"))
        self.lib = ctypes.CDLL(path)
        self.pre = which
        self.which = which
        tp_create = getattr(self.lib, f"{which}_tp_create")
        tp_create.restype = ctypes.c_void_p

    def fn(self, name):
        f = getattr(self.lib, f"{self.pre}_{name}")
        return f

    # ---- pointwise / line kernels
    def bc_fill(self, g: Grid, location: int, types, values, f: np.ndarray) -> np.ndarray:
        out = np.ascontiguousarray(f, dtype=np.float64).copy()
        n, lo, hi = g.c_args()
        t = (ctypes.c_int * 6)(*types)
        v = (ctypes.c_double * 6)(*values)
        self.fn("bc_fill")(g.ndim, n, lo, hi, location, t, v, _p(out))
        return out

    def flux_extrapolate(self, g: Grid, location: int, data: np.ndarray) -> np.ndarray:
        data = np.ascontiguousarray(data, dtype=np.float64)
        out = np.zeros_like(data)
        n, _, _ = g.c_args()
        self.fn("flux_extrapolate")(g.ndim, n, location, _p(data), _p(out))
        return out

    def zero_order_extrapolation(self, g: Grid, f: np.ndarray) -> np.ndarray:
        out = np.ascontiguousarray(f, dtype=np.float64).copy()
        n, _, _ = g.c_args()
        self.fn("zero_order_extrapolation")(g.ndim, n, _p(out))
        return out

    def uccd(self, g: Grid, flux, u, v, w) -> np.ndarray:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (flux, u, v, w)]
        out = np.zeros((6,) + g.shape)
        n, lo, hi = g.c_args()
        self.fn("uccd")(g.ndim, n, lo, hi, *[_p(a) for a in arrs], _p(out))
        return out

    def transport_rk3(self, g: Grid, types, values, flux_kind: int, rhs_kind: int, dt: float, nsteps: int, phi, u,
                      v, w, vel_from_phi: bool = False) -> np.ndarray:
        """runge_kutta::tvd_rk3 for nsteps steps with (identity_flux, convection) (kinds 0, 0),
        (burgers_flux, Hamilton_Jacobi) (kinds 1, 1) or convection_sec (rhs kind 2); returns the
        new phi."""
        out = np.ascontiguousarray(phi, dtype=np.float64).copy()
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, w)]
        t = (ctypes.c_int * 6)(*types)
        vals = (ctypes.c_double * 6)(*values)
        n, lo, hi = g.c_args()
        self.fn("transport_rk3")(g.ndim, n, lo, hi, t, vals, flux_kind, rhs_kind, ctypes.c_double(dt), nsteps,
                                 int(vel_from_phi), _p(out), *[_p(a) for a in arrs])
        return out

    def sec(self, g: Grid, flux, u=None, v=None, w=None) -> np.ndarray:
        """second_order_solver: central derivatives and mixed ones (u None) or the upwind-biased
        derivatives; out: fx, fy, fz, fxx, fyy, fzz, fxy, fyz, fzx."""
        z = np.zeros(g.shape)
        arrs = [np.ascontiguousarray(a if a is not None else z, dtype=np.float64) for a in (flux, u, v, w)]
        out = np.zeros((9,) + g.shape)
        n, lo, hi = g.c_args()
        self.fn("sec")(g.ndim, n, lo, hi, int(u is not None), *[_p(a) for a in arrs], _p(out))
        return out

    def ccd(self, g: Grid, flux, mixed: bool = True) -> np.ndarray:
        flux = np.ascontiguousarray(flux, dtype=np.float64)
        out = np.zeros((9,) + g.shape)
        n, lo, hi = g.c_args()
        self.fn("ccd")(g.ndim, n, lo, hi, int(mixed), _p(flux), _p(out))
        return out

    def weno5(self, g: Grid, flux, u, v, w) -> np.ndarray:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (flux, u, v, w)]
        out = np.zeros((3,) + g.shape)
        n, lo, hi = g.c_args()
        self.fn("weno5")(g.ndim, n, lo, hi, *[_p(a) for a in arrs], _p(out))
        return out

    def godunov(self, g: Grid, phi, sign) -> np.ndarray:
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        sign = np.ascontiguousarray(sign, dtype=np.float64)
        out = np.zeros(g.shape)
        n, lo, hi = g.c_args()
        self.fn("godunov")(g.ndim, n, lo, hi, _p(phi), _p(sign), _p(out))
        return out

    def stabilize(self, g: Grid, phi, sign):
        """stabilized_upon_gradient: returns (phi / max grad, grad)."""
        out = np.ascontiguousarray(phi, dtype=np.float64).copy()
        sign = np.ascontiguousarray(sign, dtype=np.float64)
        grad = np.zeros(g.shape)
        n, lo, hi = g.c_args()
        self.fn("stabilize")(g.ndim, n, lo, hi, _p(out), _p(sign), _p(grad))
        return out, grad

    def guess_from_history(self, g: Grid, old, old2) -> np.ndarray:
        old = np.ascontiguousarray(old, dtype=np.float64)
        old2 = np.ascontiguousarray(old2, dtype=np.float64)
        out = np.zeros(g.shape)
        n, _, _ = g.c_args()
        self.fn("guess_from_history")(g.ndim, n, _p(old), _p(old2), _p(out))
        return out

    def lsf_fields(self, g: Grid, prm, phi) -> np.ndarray:
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        p = np.asarray(prm, dtype=np.float64)
        out = np.zeros((6,) + g.shape)
        n, lo, hi = g.c_args()
        self.fn("lsf_fields")(g.ndim, n, lo, hi, _p(p), _p(phi), _p(out))
        return out

    def lsf_integrals(self, g: Grid, prm, phi) -> np.ndarray:
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        p = np.asarray(prm, dtype=np.float64)
        out = np.zeros(2)
        n, lo, hi = g.c_args()
        self.fn("lsf_integrals")(g.ndim, n, lo, hi, _p(p), _p(phi), _p(out))
        return out

    def mg_levels(self, ndim: int, n) -> list:
        buf = (ctypes.c_int * 96)()
        nn = (ctypes.c_int * 3)(*(list(n) + [1] * (3 - len(n))))
        L = self.fn("mg_levels")(ndim, nn, buf, 32)
        return [tuple(buf[3 * l:3 * l + 3]) for l in range(L)]

    def mg_poisson(self, g: Grid, rhs, dirichlet: bool, rel_tol: float, max_cycles: int, full: bool = False):
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        sol = np.zeros_like(rhs)
        hist = np.zeros(max_cycles + 1)
        cyc = ctypes.c_int(0)
        n, lo, hi = g.c_args()
        self.fn("mg_poisson")(g.ndim, n, lo, hi, int(dirichlet), int(full), _p(rhs), _p(sol),
                              ctypes.c_double(rel_tol), max_cycles, ctypes.byref(cyc), _p(hist))
        return sol, cyc.value, hist[: cyc.value + 1]

    def coef_solve(self, g: Grid, rho, rhs, p0=None, rel_tol=1e-13, max_iter=100000):
        assert self.which == "port"
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        p = np.zeros(g.shape) if p0 is None else np.ascontiguousarray(p0, dtype=np.float64).copy()
        rel = ctypes.c_double(0.0)
        n, lo, hi = g.c_args()
        it = self.lib.port_coef_solve(g.ndim, n, lo, hi, _p(rho), _p(rhs), _p(p), ctypes.c_double(rel_tol),
                                      max_iter, ctypes.byref(rel))
        return p, it, rel.value

    def sor_solve(self, g: Grid, rho, rhs, p0=None, omega=1.5, parallel=True, rel_tol=0.0, max_sweeps=1,
                  check_every=0):
        """projection()'s SOR sweeps (port_sor_solve); returns (p, sweeps, relative residual,
        seconds spent in the sweep loop)."""
        assert self.which == "port"
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        p = np.zeros(g.shape) if p0 is None else np.ascontiguousarray(p0, dtype=np.float64).copy()
        rel = ctypes.c_double(1.0)
        sec = ctypes.c_double(0.0)
        n, lo, hi = g.c_args()
        it = self.lib.port_sor_solve(g.ndim, n, lo, hi, _p(rho), _p(rhs), _p(p), ctypes.c_double(omega),
                                     int(parallel), ctypes.c_double(rel_tol), int(max_sweeps), int(check_every),
                                     ctypes.byref(rel), ctypes.byref(sec))
        return p, it, rel.value, sec.value

    def twophase(self, g: Grid, vel_bc, scalar_bc, prm: dict, opt: dict) -> "TwoPhaseState":
        return TwoPhaseState(self, g, vel_bc, scalar_bc, prm, opt)


PARAM_ORDER = ["density_ratio", "viscosity_ratio", "Re", "Fr", "We", "ls_width", "rdt", "max_CFL", "min_CFL",
               "positive_ref", "ppe_tol", "ppe_tol2", "ppe_max_iter", "ppe_omega", "ppe_initer", "dt0"]
PARAM_DEFAULT = dict(density_ratio=1.0, viscosity_ratio=1.0, Re=1.0, Fr=-1.0, We=-1.0, ls_width=0.0, rdt=0.0,
                     max_CFL=0.01, min_CFL=0.01, positive_ref=1.0, ppe_tol=1e-4, ppe_tol2=1e-7,
                     ppe_max_iter=100, ppe_omega=1.5, ppe_initer=10, dt0=1.0)
OPT_ORDER = ["scheme", "n_mpls", "reinit_every", "ppe_mode", "reinit_lambda"]


class TwoPhaseState:
    """A two-phase problem held by one checker library (see ref_tp_create / port_tp_create)."""

    def __init__(self, chk: Checker, g: Grid, vel_bc, scalar_bc, prm: dict, opt: dict):
        self.chk, self.g = chk, g
        P = dict(PARAM_DEFAULT)
        P.update(prm)
        pa = (ctypes.c_double * 16)(*[float(P[k]) for k in PARAM_ORDER])
        oa = (ctypes.c_int * 5)(*[int(opt.get(k, 0)) for k in OPT_ORDER])
        vb = (ctypes.c_int * 6)(*[BC[b] if isinstance(b, str) else b for b in vel_bc])
        sb = (ctypes.c_int * 6)(*[BC[b] if isinstance(b, str) else b for b in scalar_bc])
        n, lo, hi = g.c_args()
        self.h = ctypes.c_void_p(chk.fn("tp_create")(g.ndim, n, lo, hi, vb, sb, pa, oa))

    def set(self, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.g.shape, (a.shape, self.g.shape)
        rc = self.chk.fn("tp_set")(self.h, name.encode(), _p(a))
        assert rc == 0, name

    def get(self, name: str) -> np.ndarray:
        out = np.zeros(self.g.shape)
        rc = self.chk.fn("tp_get")(self.h, name.encode(), _p(out))
        assert rc == 0, name
        return out

    def scalars(self) -> dict:
        out = np.zeros(7)
        self.chk.fn("tp_scalars")(self.h, _p(out))
        return dict(zip(["t", "dt", "dt_old", "dt_old2", "iter", "stable_CFL", "lsf_mass0"], out.tolist()))

    def set_scalars(self, **kw) -> None:
        s = self.scalars()
        s.update(kw)
        arr = np.array([s[k] for k in ["t", "dt", "dt_old", "dt_old2", "iter", "stable_CFL", "lsf_mass0"]])
        self.chk.fn("tp_set_scalars")(self.h, _p(arr))

    def set_exact_tol(self, tol: float) -> None:
        self.chk.lib.port_tp_set_exact_tol(self.h, ctypes.c_double(tol))

    def set_fpc_cycles(self, n: int) -> None:
        """Cycle cap of the restatement's fast pressure correction (the reference's is 100)."""
        self.chk.lib.port_tp_set_fpc_cycles(self.h, int(n))

    def call(self, name: str, *args) -> int:
        return self.chk.fn(f"tp_{name}")(self.h, *args)

    def diagnostics(self) -> dict:
        out = np.zeros(3)
        self.chk.fn("tp_diagnostics")(self.h, _p(out))
        return dict(zip(["mass", "volume", "div"], out.tolist()))
