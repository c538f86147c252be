"""Shared test helpers: seeded inputs and comparisons."""
from __future__ import annotations

import numpy as np

import oracle as O


def grid2(nx=12, ny=17, lo=(0.0, 0.0), hi=(1.0, 2.0)):
    return O.Grid(2, (nx, ny), lo, hi)


def grid3(nx=8, ny=9, nz=10, lo=(0.0, 0.0, 0.0), hi=(1.0, 2.0, 1.5)):
    return O.Grid(3, (nx, ny, nz), lo, hi)


def smooth_field(g, rng, amp=1.0):
    """A smooth seeded field on every cell (ghosts included) of grid g."""
    idx = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in g.shape], indexing="ij")
    f = np.zeros(g.shape)
    for _ in range(3):
        k = rng.uniform(0.2, 0.9, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        term = amp * rng.uniform(0.5, 1.0)
        for a in range(3):
            term = term * np.cos(k[a] * idx[a] + ph[a])
        f += term
    return f


def bubble_phi(g, center=(0.5, 0.5), radius=0.25):
    """phi = radius - distance to the centre, positive inside (benchmarks_2d_bubble_rising.cpp:45-50)."""
    dx, dy = g.spacing()[:2]
    xc = g.lo[0] + (np.arange(g.n[0]) + 0.5) * dx
    yc = g.lo[1] + (np.arange(g.n[1]) + 0.5) * dy
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    phi = np.zeros(g.shape)
    phi[3:-3, 3:-3, 0] = radius - np.sqrt((X - center[0]) ** 2 + (Y - center[1]) ** 2)
    return phi


def bubble_params(g, ppe_tol=1e-12):
    """Rising-bubble parameters: rho 1000/1, mu 10/0.1, sigma 1.96, g 0.98, L = 1
    (set_parameters, global.cpp:31-52), ls_width 1.5h, rdt 0.25h.  CFL 0.2 is the upper bound
    max_CFL; the step follows the reference's stability estimate (find_dt,
    wrapper_func.cpp:335-385) below it, because a fixed CFL of 0.2 violates the explicit
    viscous limit of this density/viscosity ratio and the reference diverges within 3 steps."""
    h = min(g.spacing())
    Uc = np.sqrt(0.98 * 1.0)
    return dict(density_ratio=1.0 / 1000.0, viscosity_ratio=0.1 / 10.0, Re=1000.0 * Uc * 1.0 / 10.0,
                Fr=Uc / np.sqrt(0.98 * 1.0), We=1000.0 * Uc * Uc * 1.0 / 1.96, ls_width=1.5 * h, rdt=0.25 * h,
                max_CFL=0.2, min_CFL=1e-4, positive_ref=0.0, ppe_tol=ppe_tol, ppe_tol2=0.0, ppe_max_iter=400,
                ppe_omega=1.5, ppe_initer=1, dt0=1.0)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def max_rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)
