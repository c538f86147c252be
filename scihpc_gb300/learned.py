"""Learned initial guess for the pressure solve: snapshot generation with the GPU multigrid
solver, training of the tensor-core U-Net (scihpc_unet_*), and the comparison of solver
iterations with and without the guess.

The 2D workload is the Rayleigh-Taylor-type variable-density Poisson equation (density
1 + 2 H(phi), interface y = 0.5 + sum of 8 seeded sinusoids of amplitude <= 0.02, Neumann walls,
zero-mean right-hand side).  Consecutive time steps are imitated by pairs of problems whose
interface phases and right-hand-side modes differ slightly: the solution of the first is the
"previous pressure" of the second, as in a time loop.  The multigrid solve always iterates to
the same relative residual; the network only changes where it starts.  The 3D workload
(sphere_problem) is the spheres problem of the 256^3 pressure benchmark with a smooth
right-hand side, in the same pairs of consecutive steps.
"""
from __future__ import annotations

import math

import numpy as np

from .native import Grid, Poisson, UNet

__all__ = ["rt_problem", "make_snapshots", "cfg4_problem", "make_snapshots_cfg4", "sphere_problem", "make_snapshots3", "train", "train_cfg4_stream", "solve_iterations", "guess_errors"]


def _grid_of(rho):
    """The unit-square (2D) or unit-cube (3D) grid of a ghosted field."""
    n0, n1, n2 = rho.shape[0] - 6, rho.shape[1] - 6, rho.shape[2]
    if n2 == 1:
        return Grid(2, (n0, n1), (0.0, 0.0), (1.0, 1.0))
    return Grid(3, (n0, n1, n2 - 6), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))


def rt_problem(n: int, seed: int, drift: float, torch, device):
    """Density and right-hand side (ghosted FP64 fields on an n x n grid of [0,1]^2) of sample
    `seed`, advanced by `drift` (0 = the previous step, 1 = the current one)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.0, 0.02, 8)
    m = rng.integers(1, 9, 8)
    th = rng.uniform(0.0, 2 * math.pi, 8)
    kx, ky = rng.integers(1, 6, 6), rng.integers(1, 6, 6)
    amp, ph = rng.standard_normal(6), rng.uniform(0.0, 2 * math.pi, 6)
    h = 1.0 / n
    c = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) * h
    X, Y = torch.meshgrid(c, c, indexing="ij")
    iface = 0.5 + sum(float(a[k]) * torch.sin(2 * math.pi * float(m[k]) * X + float(th[k]) + 0.05 * drift)
                      for k in range(8))
    phi = Y - iface
    w = 1.5 * h
    H = torch.where(phi < -w, torch.zeros_like(phi), torch.where(phi > w, torch.ones_like(phi),
                    0.5 * (1 + phi / w + torch.sin(math.pi * phi / w) / math.pi)))
    rho = torch.ones((n + 6, n + 6, 1), dtype=torch.float64, device=device)
    rho[3:-3, 3:-3, 0] = 1.0 + 2.0 * H
    rho[:3], rho[-3:] = rho[3:4].clone(), rho[-4:-3].clone()
    rho[:, :3], rho[:, -3:] = rho[:, 3:4].clone(), rho[:, -4:-3].clone()
    # smooth zero-mean modes (cosines of the Neumann problem), slightly rotated with the drift
    f = torch.zeros_like(X)
    for j in range(6):
        f += float(amp[j]) * (1 + 0.02 * drift) * torch.cos(math.pi * float(kx[j]) * X + 0.03 * drift * j) * \
             torch.cos(math.pi * float(ky[j]) * Y + float(ph[j]) * 0.0)
    rhs = torch.zeros_like(rho)
    rhs[3:-3, 3:-3, 0] = f - f.mean()
    return rho, rhs


def cfg4_problem(n: int, seed: int, drift: float, torch, device, modes: int = 24):
    """The learned-guess workload of the 512^2 benchmark configuration on an n x n grid of
    [0,1]^2 (ghosted FP64 fields), sample `seed` advanced by `drift` (0 = the previous step,
    1 = the current one): density 1 + 2 H(phi) (ratio 3, heavy above) across the interface
    y = 0.5 + sum_{k=1..8} a_k sin(2 pi m_k x + theta_k), a_k ~ U[0, 0.02], m_k ~ U{1..8},
    theta_k ~ U[0, 2 pi) (numpy's default generator seeded with `seed`; the phases advance by
    0.05 per step), and a right-hand side that is the discrete divergence of a seeded random
    face velocity with no flux through the walls: `modes` Fourier modes
    u = A sin(pi p x) cos(pi q y), v = B cos(pi p' x) sin(pi q' y) with p, q ~ U{1..16} and
    amplitudes ~ N(0, 1) / (p + q), perturbed by 5 % of a second draw per step."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.0, 0.02, 8)
    m = rng.integers(1, 9, 8)
    th = rng.uniform(0.0, 2 * math.pi, 8)
    pu, qu, pv, qv = (rng.integers(1, 17, modes) for _ in range(4))
    A = rng.standard_normal(modes) / (pu + qu) + 0.05 * drift * rng.standard_normal(modes) / (pu + qu)
    B = rng.standard_normal(modes) / (pv + qv) + 0.05 * drift * rng.standard_normal(modes) / (pv + qv)
    h = 1.0 / n
    c = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) * h
    f = torch.arange(n + 1, dtype=torch.float64, device=device) * h    # face coordinates
    X, Y = torch.meshgrid(c, c, indexing="ij")
    iface = 0.5 + sum(float(a[k]) * torch.sin(2 * math.pi * float(m[k]) * X + float(th[k]) + 0.05 * drift)
                      for k in range(8))
    phi = Y - iface
    w = 1.5 * h
    H = torch.where(phi < -w, torch.zeros_like(phi), torch.where(phi > w, torch.ones_like(phi),
                    0.5 * (1 + phi / w + torch.sin(math.pi * phi / w) / math.pi)))
    rho = torch.ones((n + 6, n + 6, 1), dtype=torch.float64, device=device)
    rho[3:-3, 3:-3, 0] = 1.0 + 2.0 * H   # the heavy fluid above the interface
    rho[:3], rho[-3:] = rho[3:4].clone(), rho[-4:-3].clone()
    rho[:, :3], rho[:, -3:] = rho[:, 3:4].clone(), rho[:, -4:-3].clone()
    Xu, Yu = torch.meshgrid(f, c, indexing="ij")    # x-faces: (n + 1) x n
    Xv, Yv = torch.meshgrid(c, f, indexing="ij")    # y-faces: n x (n + 1)
    u = sum(float(A[k]) * torch.sin(math.pi * float(pu[k]) * Xu) * torch.cos(math.pi * float(qu[k]) * Yu)
            for k in range(modes))
    v = sum(float(B[k]) * torch.cos(math.pi * float(pv[k]) * Xv) * torch.sin(math.pi * float(qv[k]) * Yv)
            for k in range(modes))
    u[0], u[-1] = 0.0, 0.0
    v[:, 0], v[:, -1] = 0.0, 0.0
    div = (u[1:] - u[:-1]) / h + (v[:, 1:] - v[:, :-1]) / h
    rhs = torch.zeros_like(rho)
    rhs[3:-3, 3:-3, 0] = div - div.mean()
    return rho, rhs


def make_snapshots_cfg4(n: int, seeds, torch, device, rel_tol: float = 1e-10, fp32: bool = True):
    """[(rho, rhs, pprev, p)] of cfg4_problem for the given seeds: pprev solves the drift-0
    problem from zero, p the drift-1 problem from pprev (both to rel_tol, one solver)."""
    g = Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
    ps = Poisson(g, bc=0, density=True, fp32=fp32)
    out = []
    for s in seeds:
        rho0, rhs0 = cfg4_problem(n, s, 0.0, torch, device)
        rho1, rhs1 = cfg4_problem(n, s, 1.0, torch, device)
        p0 = torch.zeros_like(rho0)
        ps.set_density(rho0)
        ps.solve(rhs0, p0, rel_tol=rel_tol, max_iter=200)
        p1 = p0.clone()
        ps.set_density(rho1)
        ps.solve(rhs1, p1, rel_tol=rel_tol, max_iter=200, use_guess=True)
        torch.cuda.synchronize()
        out.append((rho1, rhs1, p0, p1))
    ps.close()
    return out


def make_snapshots(n: int, seeds, torch, device, rel_tol: float = 1e-10, fp32: bool = True):
    """[(rho, rhs, pprev, p)] for the given seeds: pprev solves the drift-0 problem, p the
    drift-1 problem (both to rel_tol)."""
    g = Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
    out = []
    for s in seeds:
        ps = Poisson(g, bc=0, density=True, fp32=fp32)
        rho0, rhs0 = rt_problem(n, s, 0.0, torch, device)
        rho1, rhs1 = rt_problem(n, s, 1.0, torch, device)
        p0 = torch.zeros_like(rho0)
        ps.set_density(rho0)
        ps.solve(rhs0, p0, rel_tol=rel_tol, max_iter=200)
        p1 = p0.clone()
        ps.set_density(rho1)
        ps.solve(rhs1, p1, rel_tol=rel_tol, max_iter=200, use_guess=True)
        torch.cuda.synchronize()
        ps.close()
        out.append((rho1, rhs1, p0, p1))
    return out


def sphere_problem(n: int, seed: int, drift: float, torch, device):
    """Density and right-hand side (ghosted FP64 fields on an n^3 grid of [0,1]^3) of 3D sample
    `seed` advanced by `drift` (0 = the previous step, 1 = the current one): density
    1 + 999 H(phi) with phi the union of 1-12 seeded spheres (radius 0.05-0.2) that move by up
    to one cell per step, and a zero-mean right-hand side -- the divergence of a smooth random
    velocity with no flux through the walls -- made of six Neumann cosine modes that change
    slightly from step to step."""
    rng = np.random.default_rng(seed)
    ns = 1 + seed % 12
    r = rng.uniform(0.05, 0.2, ns)
    cen = [rng.uniform(r[k], 1 - r[k], 3) for k in range(ns)]
    move = [rng.standard_normal(3) for _ in range(ns)]
    ks = rng.integers(1, 5, (6, 3))
    amp = rng.standard_normal(6)
    h = 1.0 / n
    c = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) * h
    X, Y, Z = torch.meshgrid(c, c, c, indexing="ij")
    phi = torch.full((n, n, n), -1e9, dtype=torch.float64, device=device)
    for k in range(ns):
        m = move[k] / np.linalg.norm(move[k]) * h * drift
        cx, cy, cz = (float(cen[k][a] + m[a]) for a in range(3))
        phi = torch.maximum(phi, float(r[k]) - torch.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2))
    w = 1.5 * h
    H = torch.where(phi < -w, torch.zeros_like(phi), torch.where(phi > w, torch.ones_like(phi),
                    0.5 * (1 + phi / w + torch.sin(math.pi * phi / w) / math.pi)))
    del phi
    rho = torch.ones((n + 6, n + 6, n + 6), dtype=torch.float64, device=device)
    rho[3:-3, 3:-3, 3:-3] = 1.0 + 999.0 * H
    del H
    rho[:3], rho[-3:] = rho[3:4].clone(), rho[-4:-3].clone()
    rho[:, :3], rho[:, -3:] = rho[:, 3:4].clone(), rho[:, -4:-3].clone()
    rho[:, :, :3], rho[:, :, -3:] = rho[:, :, 3:4].clone(), rho[:, :, -4:-3].clone()
    f = torch.zeros_like(X)
    for j in range(6):
        f += float(amp[j]) * (1 + 0.02 * drift) * torch.cos(math.pi * float(ks[j, 0]) * X + 0.03 * drift * j) * \
             torch.cos(math.pi * float(ks[j, 1]) * Y) * torch.cos(math.pi * float(ks[j, 2]) * Z)
    del X, Y, Z
    rhs = torch.zeros_like(rho)
    rhs[3:-3, 3:-3, 3:-3] = f - f.mean()
    return rho, rhs


def make_snapshots3(n: int, seeds, torch, device, rel_tol: float = 1e-10, fp32: bool = True):
    """[(rho, rhs, pprev, p)] of sphere_problem for the given seeds: pprev solves the drift-0
    problem, p the drift-1 problem (both to rel_tol)."""
    g = Grid(3, (n, n, n), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    ps = Poisson(g, bc=0, density=True, fp32=fp32)
    out = []
    for s in seeds:
        rho0, rhs0 = sphere_problem(n, s, 0.0, torch, device)
        p0 = torch.zeros_like(rho0)
        ps.set_density(rho0)
        ps.solve(rhs0, p0, rel_tol=rel_tol, max_iter=200)
        del rho0, rhs0
        rho1, rhs1 = sphere_problem(n, s, 1.0, torch, device)
        p1 = p0.clone()
        ps.set_density(rho1)
        ps.solve(rhs1, p1, rel_tol=rel_tol, max_iter=200, use_guess=True)
        torch.cuda.synchronize()
        out.append((rho1, rhs1, p0, p1))
    ps.close()
    return out


def train(net: UNet, snaps, steps: int, lr: float, torch, seed: int = 0, cosine: bool = False):
    """Adam steps over the snapshots in a seeded random order; returns the loss history.
    cosine: the learning rate decays from lr to 0 along a half cosine over the steps."""
    g = _grid_of(snaps[0][0])
    rng = np.random.default_rng(seed)
    losses = []
    torch.cuda.synchronize()
    for k in range(steps):
        rho, rhs, pprev, p = snaps[int(rng.integers(len(snaps)))]
        lr_k = lr * 0.5 * (1.0 + math.cos(math.pi * k / steps)) if cosine else lr
        losses.append(net.train_step(g, rho, rhs, pprev, p, lr_k))
    return losses


def train_cfg4_stream(net: UNet, n: int, seeds, chunk: int, lr: float, torch, device, visits: int = 1,
                      seed: int = 0):
    """Adam training on cfg4_problem snapshots generated chunk by chunk: each chunk of seeds is
    solved (make_snapshots_cfg4), every snapshot of it visited `visits` times in a seeded
    random order, and the chunk dropped, so the number of snapshots is not bounded by device
    memory.  The learning rate decays from lr to 0 along a half cosine over all steps.
    Returns the loss history."""
    seeds = list(seeds)
    steps = len(seeds) * visits
    g = Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
    rng = np.random.default_rng(seed)
    losses = []
    for c0 in range(0, len(seeds), chunk):
        snaps = make_snapshots_cfg4(n, seeds[c0:c0 + chunk], torch, device)
        for i in rng.permutation(np.repeat(np.arange(len(snaps)), visits)):
            k = len(losses)
            rho, rhs, pprev, p = snaps[int(i)]
            losses.append(net.train_step(g, rho, rhs, pprev, p, lr * 0.5 * (1.0 + math.cos(math.pi * k / steps))))
        del snaps
    return losses


def solve_iterations(snaps, torch, net: UNet | None = None, rel_tol: float = 1e-10, fp32: bool = True):
    """Solver iterations (V-cycles) and final residuals for each snapshot, starting from the
    previous pressure (net None) or from the network's guess."""
    g = _grid_of(snaps[0][0])
    its, res = [], []
    for rho, rhs, pprev, _ in snaps:
        ps = Poisson(g, bc=0, density=True, fp32=fp32)
        ps.set_density(rho)
        p = pprev.clone()
        if net is not None:
            torch.cuda.synchronize()
            net.infer(g, rho, rhs, pprev, p)
        it, rr = ps.solve(rhs, p, rel_tol=rel_tol, max_iter=200, use_guess=True)
        torch.cuda.synchronize()
        ps.close()
        its.append(it)
        res.append(rr)
    return its, res


def guess_errors(snaps, torch, net: UNet):
    """For each snapshot, the interior L2 distance of the network's guess to the converged
    pressure over that of the previous pressure, both with their means removed (the Neumann
    problem fixes the pressure up to a constant): below 1 where the network moves the start
    of the solve towards the answer."""
    g = _grid_of(snaps[0][0])
    out = []
    for rho, rhs, pprev, p in snaps:
        guess = pprev.clone()
        torch.cuda.synchronize()
        net.infer(g, rho, rhs, pprev, guess)
        torch.cuda.synchronize()
        if rho.shape[2] == 1:
            I = (slice(3, -3), slice(3, -3), 0)
        else:
            I = (slice(3, -3),) * 3
        e_net = guess[I] - p[I]
        e_prev = pprev[I] - p[I]
        e_net = e_net - e_net.mean()
        e_prev = e_prev - e_prev.mean()
        out.append(float(torch.linalg.vector_norm(e_net) / torch.linalg.vector_norm(e_prev)))
    return out
