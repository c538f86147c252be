#!/usr/bin/env python
"""Benchmark of the two-phase projection time step (rising bubble, 128 x 256) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-poisson]

One JSON line on stdout (rank 0).  Our arm: the CUDA library through its C ABI, one step =
one complete time step replayed as a captured CUDA graph (find_dt, WENO5/TVD-RK3 advection,
5 mass-correction Euler steps, ab_solve with the multigrid pressure solve iterated to a
relative residual of 1e-10 inside the graph, Godunov reinitialisation).  The reference
arm (--impl reference) times the reference algorithm's CPU implementation (the CPU
restatement in oracle/, built from committed sources) on all host cores, on the same
workload.  With N > 1 (torchrun) every rank runs an independent replica: the step does
not shard (one 128 x 256 grid), so scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY = 128, 256
DOMAIN = ((0.0, 0.0), (1.0, 2.0))
BUBBLE = ((0.5, 0.5), 0.25)
PPE_TOL = 1e-10

# Algorithmic FP64 operations per interior cell of the reinitialisation's gradient kernel in
# 2D, counted from the reference formulas (one flop per add, subtract, multiply, divide or
# square root; max/min not counted): per axis the fourth-order central difference (10), the
# five distinct second differences (15), two WENO-JS corrections (47 each: three indicators
# 23, three weights 9, two normalised weights 4, the correction 11), the two one-sided
# derivatives (6) and the square (1) -- 126; both axes, their sum and its root (254); the
# redistance source -sign (g - 1) rdt / dt (4) and the lambda fields a, b (4) -- 262
# (godunov_gradient.cpp:19-198, source.cpp:157-198).
REINIT_FLOPS_2D = 262
# DRAM traffic per launch and share of the step from the committed ncu summaries (None when
# not captured); the command that made each is in the summary file.
REINIT_TRAFFIC_BYTES = 838485   # read 838,485 B, write 0 B (mean of three launches)
REINIT_TRAFFIC_SRC = "profiles/reinit_2d_128x256_traffic.md"
REINIT_SHARE = 0.211   # profiles/twophase_step_128x256_launches.md
VCYCLE_256_TRAFFIC_BYTES = 1436369067   # read 1.088 GB + write 0.348 GB, mean of three V-cycles
VCYCLE_256_TRAFFIC_SRC = "profiles/poisson_256cubed_vcycle_traffic.md"


PPE_DESC = {"fp32": "FP32 V-cycles and conjugate gradients inside FP64 iterative refinement "
                    "(FP64 residual and pressure)",
            "fp64": "FP64 V-cycles inside FP64 conjugate gradients"}


def physics(h: float) -> dict:
    """Hysing TC1 (rho 1000/100, mu 10/1, sigma 24.5, g 0.98, L = 1), nondimensionalised as
    set_parameters does (global.cpp:31-52); ls_width 1.5h, rdt 0.25h; dt from the reference's
    stability estimate (find_dt) capped at CFL 0.2."""
    import math
    r1, r2, m1, m2, sig, g = 1000.0, 100.0, 10.0, 1.0, 24.5, 0.98
    Uc = math.sqrt(g * 1.0)
    return dict(density_ratio=r2 / r1, viscosity_ratio=m2 / m1, Re=r1 * Uc * 1.0 / m1, Fr=Uc / math.sqrt(g * 1.0),
                We=r1 * Uc * Uc * 1.0 / sig, ls_width=1.5 * h, rdt=0.25 * h, max_CFL=0.2, min_CFL=1e-4,
                positive_ref=0.0, ppe_tol=PPE_TOL, ppe_tol2=0.0, ppe_max_iter=200, ppe_omega=1.5, ppe_initer=1,
                dt0=1.0)


def initial_phi(shape):
    import numpy as np
    dx, dy = (DOMAIN[1][0] - DOMAIN[0][0]) / NX, (DOMAIN[1][1] - DOMAIN[0][1]) / NY
    xc = DOMAIN[0][0] + (np.arange(NX) + 0.5) * dx
    yc = DOMAIN[0][1] + (np.arange(NY) + 0.5) * dy
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    phi = np.zeros(shape)
    (cx, cy), r = BUBBLE
    phi[3:-3, 3:-3, 0] = r - np.sqrt((X - cx) ** 2 + (Y - cy) ** 2)
    return phi


def config_block(extra=None) -> dict:
    c = {"workload": "2D rising bubble, one two-phase projection time step",
         "grid": f"{NX}x{NY} cells on [0,1]x[0,2], ghost width 3",
         "physics": "Hysing TC1 (rho 1000/100, mu 10/1, sigma 24.5, g 0.98); the stated "
                    "rho 1000/1, mu 10/0.1 case diverges within 20 steps in the reference scheme",
         "step": "find_dt + WENO5/TVD-RK3 advection + 5 mpls Euler steps + ab_solve "
                 f"(multigrid-PCG pressure to rel. residual {PPE_TOL:g}) + 12-stage-triple reinit",
         "l2": "working set 24 MB < L2; L2 flushed (256 MiB write) before every timed step"}
    if extra:
        c.update(extra)
    return c


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "src": "fallback"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"scihpc_clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}", "--format=csv,noheader",
                                          "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            os.remove(self.path)
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1].split()[0]) for r in rows if len(r) >= 9 and r[1].strip().split()[0].replace(".", "").isdigit()]
        mx = [float(r[2].split()[0]) for r in rows if len(r) >= 9 and r[2].strip().split()[0].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v: float, device) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- CPU legs
# The reference algorithm on the host cores (oracle/port: the restatement, pinned bit for bit
# to the reference compiled from its sources where those are present; the GPU machine has only
# the restatement).  Every figure is the median of three fixed windows, with all host cores
# (the reference's OpenMP loops, SOR's racy in-place sweep included) and with one thread.

def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=20).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def _port(threads: int):
    import oracle as O
    P = O.Checker("port")
    P.lib.port_set_threads(threads)
    return O, P


def _windows(step, nwin: int, nsteps: int) -> list:
    rates = []
    for _ in range(nwin):
        t0 = time.perf_counter()
        for _ in range(nsteps):
            step()
        rates.append(nsteps / (time.perf_counter() - t0))
    return rates


def cpu_bubble(threads: int, win_all: int = 50, win_one: int = 10) -> dict:
    """The bench's workload (128 x 256 rising bubble, TC1 fluid, WENO5, 5 mpls steps, reinit
    every step) under the reference's stock ab_solve schedule and its drivers' solver
    settings (ppe_tol 1e-8, ppe_tol2 1e-7, 100 SOR sweeps at most, ppe_initer 1;
    benchmarks_2d_bubble_rising.cpp:78-79, global.h:49-53), after the five start-up steps
    (SOR while iter < 5, then the first fast pressure correction): steps/s of three windows
    of win_all steps on all cores, then three of win_one steps on one thread (same run)."""
    import numpy as np
    O, P = _port(threads)
    g = O.Grid(2, (NX, NY), DOMAIN[0], DOMAIN[1])
    prm = physics(min((DOMAIN[1][0] - DOMAIN[0][0]) / NX, (DOMAIN[1][1] - DOMAIN[0][1]) / NY))
    prm.update(ppe_tol=1e-8, ppe_tol2=1e-7, ppe_max_iter=100, ppe_initer=1)
    s = P.twophase(g, ["no_slip"] * 6, ["neumann"] * 6, prm,
                   dict(scheme=1, n_mpls=5, reinit_every=1, ppe_mode=0, reinit_lambda=1))
    s.set("phi", initial_phi(g.shape))
    s.call("init")
    for _ in range(5):
        s.call("step", 1)
    step = lambda: s.call("step", 1)
    r_all = _windows(step, 3, win_all)
    P.lib.port_set_threads(1)
    r_one = _windows(step, 3, win_one)
    P.lib.port_set_threads(threads)
    return {"all_cores": {"value": float(np.median(r_all)), "windows": r_all, "steps_per_window": win_all,
                          "cores": threads},
            "one_thread": {"value": float(np.median(r_one)), "windows": r_one, "steps_per_window": win_one,
                           "cores": 1},
            "startup_steps": 5}


def cpu_dambreak(threads: int, win: int = 5) -> dict:
    """The 128 x 64 x 64 dam break as the reference's driver runs it
    (benchmarks_3d_dambreak.cpp:74-146): UCCD transport, no mass correction, ppe_tol 1e-4,
    ppe_tol2 1e-10, ppe_max_iter 100, and iter never advanced, so ab_solve runs SOR every
    step; reinitialisation (30 TVD-RK3 steps) every 20 steps, timed once on its own."""
    import numpy as np
    O, P = _port(threads)
    g, prm, phi = dambreak_setup(O.Grid)
    prm.update(ppe_tol=1e-4, ppe_tol2=1e-10, ppe_max_iter=100, ppe_initer=1)
    s = P.twophase(g, ["slip"] * 6, ["neumann"] * 6, prm,
                   dict(scheme=0, n_mpls=0, reinit_every=0, ppe_mode=0, reinit_lambda=1))
    s.set("phi", phi)
    s.call("init")

    def step():
        s.set_scalars(iter=0.0)
        s.call("step", 1)

    step()
    r_all = _windows(step, 3, win)
    t0 = time.perf_counter()
    s.call("reinit")
    reinit_s = time.perf_counter() - t0
    P.lib.port_set_threads(1)
    r_one = _windows(step, 3, 1)
    P.lib.port_set_threads(threads)
    med = float(np.median(r_all))
    return {"all_cores": {"value": med, "windows": r_all, "steps_per_window": win, "cores": threads},
            "one_thread": {"value": float(np.median(r_one)), "windows": r_one, "steps_per_window": 1, "cores": 1},
            "reinit_s_all_cores": reinit_s,
            "with_reinit_every_20": 1.0 / (1.0 / med + reinit_s / 20.0),
            "unit": "steps/s",
            "note": "windows exclude the reinitialisation; with_reinit_every_20 adds it at the driver's rate "
                    "(the GPU figure includes it)"}


def spheres_field(n: int):
    """The construction of poisson_problem on the host (same seeded generator, same draws) on an
    n^3 grid: (density, right-hand side = div of the random wall-tight face velocity, mean
    removed) as ghosted float64 arrays."""
    import numpy as np
    import torch
    gen = torch.Generator(device="cpu").manual_seed(20261203)
    h = 1.0 / n
    c = (np.arange(n) + 0.5) * h
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    phi = np.full((n, n, n), -1e9)
    for _ in range(12):
        r = 0.05 + 0.15 * torch.rand(1, generator=gen).item()
        cen = [r + (1 - 2 * r) * torch.rand(1, generator=gen).item() for _ in range(3)]
        phi = np.maximum(phi, r - np.sqrt((X - cen[0]) ** 2 + (Y - cen[1]) ** 2 + (Z - cen[2]) ** 2))
    del X, Y, Z
    w = 1.5 * h
    H = np.where(phi < -w, 0.0, np.where(phi > w, 1.0, 0.5 * (1 + phi / w + np.sin(np.pi * phi / w) / np.pi)))
    rho = np.ones((n + 6,) * 3)
    rho[3:-3, 3:-3, 3:-3] = 1.0 + 999.0 * H
    del H, phi
    div = np.zeros((n, n, n))
    shapes = ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))
    for a in range(3):
        u = torch.rand(shapes[a], generator=gen, dtype=torch.float64).numpy() - 0.5
        sl = [slice(None)] * 3
        for e in (0, -1):
            sl[a] = e
            u[tuple(sl)] = 0.0
        div += np.diff(u, axis=a) / h
    rhs = np.zeros((n + 6,) * 3)
    rhs[3:-3, 3:-3, 3:-3] = div - div.mean()
    return rho, rhs


def cpu_sor(threads: int) -> dict:
    """projection()'s SOR (omega 1.5, in-place sweeps, per-sweep mean removal; the reference's
    pressure solve for this equation, projection_method.cpp:576-627) on the spheres problem:
    ms per sweep at 256^3 (mean of 3 sweeps all cores, 2 sweeps one thread), and the sweeps
    and time to relative residual 1e-10 at 64^3, measured on all cores (residual formed every
    100 sweeps).  The one-thread 64^3 time and the 256^3 time to 1e-10 are extrapolations,
    labelled as such: SOR's sweep count grows as h^-2."""
    O, P = _port(threads)
    out = {}
    g = O.Grid(3, (256,) * 3, (0.0,) * 3, (1.0,) * 3)
    rho, rhs = spheres_field(256)
    _, n3, _, sec = P.sor_solve(g, rho, rhs, max_sweeps=3)
    ms_all = 1e3 * sec / n3
    P.lib.port_set_threads(1)
    _, n1, _, sec = P.sor_solve(g, rho, rhs, max_sweeps=2, parallel=False)
    ms_one = 1e3 * sec / n1
    P.lib.port_set_threads(threads)
    del rho, rhs
    g64 = O.Grid(3, (64,) * 3, (0.0,) * 3, (1.0,) * 3)
    rho, rhs = spheres_field(64)
    _, sweeps, rel, sec64 = P.sor_solve(g64, rho, rhs, rel_tol=1e-10, max_sweeps=200000, check_every=100)
    P.lib.port_set_threads(1)
    _, nn, _, sec1 = P.sor_solve(g64, rho, rhs, max_sweeps=200, parallel=False)
    P.lib.port_set_threads(threads)
    ms64_one = 1e3 * sec1 / nn
    out["sor_ms_per_sweep_256^3"] = {"all_cores": ms_all, "one_thread": ms_one, "cores": threads}
    out["sor_to_1e-10_64^3"] = {"sweeps": sweeps, "final_relres": rel, "all_cores_s": sec64,
                                "one_thread_s_extrapolated": sweeps * ms64_one / 1e3,
                                "one_thread_ms_per_sweep": ms64_one}
    out["sor_to_1e-10_256^3_s_extrapolated"] = {
        "all_cores": sweeps * 16 * ms_all / 1e3, "one_thread": sweeps * 16 * ms_one / 1e3,
        "how": "sweeps at 64^3 x 16 (h^-2) x measured ms per sweep at 256^3"}
    return out


def cpu_baselines_fresh(threads: int) -> dict:
    """The CPU baselines of the bench line, measured in a fresh Python process that imports
    neither torch nor CUDA, as the reference arm (--impl reference) runs: measured in the
    process that had just driven the GPU, the same bubble windows gave ~10 steps/s against
    16.6 in a fresh process on the same box."""
    code = ("import json, bench; t = %d; print(json.dumps({'bubble': bench.cpu_bubble(t), "
            "'dambreak': bench.cpu_dambreak(t), 'sor': bench.cpu_sor(t), 'mg': bench.cpu_multigrid_256(t)}))"
            % threads)
    r = subprocess.run([sys.executable, "-c", code], cwd=os.path.dirname(os.path.abspath(__file__)),
                       capture_output=True, text=True, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_multigrid_256(threads: int) -> dict:
    """The reference multigrid (v_cycle with its steepest-descent relax, restated) on the
    256^2 Dirichlet problem to relative residual 1e-10: median of 3 solves, all cores and
    one thread."""
    import numpy as np
    O, P = _port(threads)
    n = 256
    g = O.Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
    xc = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    rhs = -(2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)).T.ravel()
    out = {}
    for key, th in (("all_cores", threads), ("one_thread", 1)):
        P.lib.port_set_threads(th)
        P.mg_poisson(g, rhs, True, 1e-10, 400)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            _, cyc, hist = P.mg_poisson(g, rhs, True, 1e-10, 400)
            ts.append(time.perf_counter() - t0)
        out[key] = {"ms_to_tol": 1e3 * float(np.median(ts)), "cycles": cyc, "final_relres": float(hist[-1]),
                    "cores": th}
    P.lib.port_set_threads(threads)
    return out


def run_reference(args) -> None:
    ws, rank, local = dist_init()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    b = cpu_bubble(threads)
    rate = b["all_cores"]["value"]
    n = 3 * b["all_cores"]["steps_per_window"]
    line = {"metric": "time steps/s", "value": rate, "unit": "steps/s", "n_gpus": args.gpus, "steps": n,
            "warmup": b["startup_steps"], "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded analytic bubble)",
            "config": config_block({"parallelism": "host OpenMP", "pressure_solver": "reference schedule: SOR "
                                    "for 5 steps, then fast pressure correction on the reference multigrid"}),
            "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": threads, "kind": "port",
                             "model": cpu_model(),
                             "sample": f"median of 3 windows of {b['all_cores']['steps_per_window']} steps after "
                                       "the 5 start-up steps", "one_thread": b["one_thread"]},
            "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU leg
def vcycle_bytes(levels, ndim: int, w: int) -> float:
    """Algorithmic bytes of one V(2,2) cycle by the fixed model: per interior cell of the
    finest level, [4w(nu1 + nu2) + 5w + 2w/2^d] * 2^d / (2^d - 1) -- a full red-black sweep
    reads x, b and the density and writes x (4w); residual + restriction 3w + w/2^d;
    prolongation + correction 2w + w/2^d; the coarser levels add the geometric factor.
    V(2,2) gives 24.29w per cell in 3D and 28.33w in 2D."""
    cells = 1
    for a in range(ndim):
        cells *= levels[0][a]
    c = 2 ** ndim
    return cells * (4 * w * 4 + 5 * w + 2 * w / c) * c / (c - 1)


def poisson_problem(torch, Grid, n=256):
    """The n^3 variable-density pressure equation: density 1 + 999 H(phi), phi from 12 seeded
    spheres, Neumann walls, zero-mean right-hand side from a random divergent velocity.
    Returns (grid, rho, rhs) as ghosted FP64 device fields."""
    g = Grid(3, (n, n, n), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    dev = torch.device("cuda")
    gen = torch.Generator(device="cpu").manual_seed(20261203)
    h = 1.0 / n
    c = (torch.arange(n, dtype=torch.float64, device=dev) + 0.5) * h
    X, Y, Z = torch.meshgrid(c, c, c, indexing="ij")
    phi = torch.full((n, n, n), -1e9, dtype=torch.float64, device=dev)
    for _ in range(12):
        r = 0.05 + 0.15 * torch.rand(1, generator=gen).item()
        cen = [r + (1 - 2 * r) * torch.rand(1, generator=gen).item() for _ in range(3)]
        phi = torch.maximum(phi, r - torch.sqrt((X - cen[0]) ** 2 + (Y - cen[1]) ** 2 + (Z - cen[2]) ** 2))
    del X, Y, Z
    w = 1.5 * h
    H = torch.where(phi < -w, torch.zeros_like(phi), torch.where(phi > w, torch.ones_like(phi),
                    0.5 * (1 + phi / w + torch.sin(torch.pi * phi / w) / torch.pi)))
    rho = torch.ones(g.shape, dtype=torch.float64, device=dev)
    rho[3:-3, 3:-3, 3:-3] = 1.0 + 999.0 * H
    # ghost density: copy the boundary cells (any finite value works: wall faces carry no flux)
    rho[:3], rho[-3:] = rho[3:4].clone(), rho[-4:-3].clone()
    rho[:, :3], rho[:, -3:] = rho[:, 3:4].clone(), rho[:, -4:-3].clone()
    rho[:, :, :3], rho[:, :, -3:] = rho[:, :, 3:4].clone(), rho[:, :, -4:-3].clone()
    del H, phi
    # rhs = div u of a random face velocity with zero normal velocity on the walls
    u = torch.rand((n + 1, n, n), generator=gen, dtype=torch.float64).to(dev) - 0.5
    u[0], u[-1] = 0, 0
    div = (u[1:] - u[:-1]) / h
    del u
    v = torch.rand((n, n + 1, n), generator=gen, dtype=torch.float64).to(dev) - 0.5
    v[:, 0], v[:, -1] = 0, 0
    div += (v[:, 1:] - v[:, :-1]) / h
    del v
    wv = torch.rand((n, n, n + 1), generator=gen, dtype=torch.float64).to(dev) - 0.5
    wv[:, :, 0], wv[:, :, -1] = 0, 0
    div += (wv[:, :, 1:] - wv[:, :, :-1]) / h
    del wv
    rhs = torch.zeros(g.shape, dtype=torch.float64, device=dev)
    rhs[3:-3, 3:-3, 3:-3] = div - div.mean()
    del div
    return g, rho, rhs


def poisson_block(torch, Poisson, Grid, hbm):
    """256^3 variable-density pressure equation solved to relative residual 1e-10 with FP64
    V-cycles (FP64 conjugate gradients) and with FP32 V-cycles inside FP32 conjugate
    gradients inside FP64 iterative refinement."""
    g, rho, rhs = poisson_problem(torch, Grid)
    dev = rho.device
    out = {"grid": "256^3", "density": "1 + 999 H(phi), 12 seeded spheres r in [0.05, 0.2]",
           "rel_tol": 1e-10}
    for name, fp32 in (("fp64", False), ("fp32_refined", True)):
        ps = Poisson(g, bc=0, density=True, fp32=fp32)
        ps.set_density(rho)
        p = torch.zeros(g.shape, dtype=torch.float64, device=dev)
        ps.solve(rhs, p, rel_tol=1e-10, max_iter=100)   # warm
        times, its = [], []
        for _ in range(3):
            p.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            it, rr = ps.solve(rhs, p, rel_tol=1e-10, max_iter=100)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
            its.append(it)
        ncyc = 20
        ms = ps.time_vcycles(rhs, p, ncyc) / ncyc
        by = vcycle_bytes(ps.levels(), 3, 4 if fp32 else 8)
        out[name] = {"ms_to_tol": min(times), "iterations": its[0], "final_relres": rr,
                     "vcycle_ms": ms, "vcycle_alg_bytes": by, "vcycle_gbs": by / ms / 1e6,
                     "vcycle_frac_of_hbm": by / ms / 1e6 / hbm["hbm_gbs"]}
        ps.close()
        del p
    out["fp32_speedup"] = out["fp64"]["ms_to_tol"] / out["fp32_refined"]["ms_to_tol"]
    return out


def stock_block(torch, args, flush, clocks_cls) -> dict:
    """The same bubble step under the reference's own pressure schedule, the one the reference
    arm runs (projection_method.cpp:755-777: the projection equation while iter < 5, then
    pressure_guess_solution + init_ppe_fpc_coefficients + fast_pressure_correction on the
    constant-coefficient multigrid, ppe_tol 1e-8 absolute, at most 100 cycles, ppe_initer 1),
    which is the C++ drop-in's default.  Timed like the headline (graph replay, L2 flushed
    before each step, CUDA events), after the five projection steps and the warm-up, over at
    most 50 steps and e2e over the next 50 through the C ABI with the same four fields up and
    down: windows inside the first ~110 steps, where the reference arm's windows (steps 6-155)
    are."""
    from scihpc_gb300 import Grid, TwoPhase
    g = Grid(2, (NX, NY), DOMAIN[0], DOMAIN[1])
    h = min(g.spacing())
    prm = physics(h)
    prm.update(ppe_tol=1e-8, ppe_max_iter=100, ppe_initer=1)
    tp = TwoPhase(g, ["no_slip"] * 6, ["neumann"] * 6, prm, scheme=1, n_mpls=5, reinit_every=1,
                  fp32=args.ppe == "fp32")
    tp.set_ppe_schedule(1, 1)
    tp.set("phi", initial_phi(g.shape))
    tp.init()
    stream = torch.cuda.ExternalStream(tp.stream())
    tp.step(5 + args.warmup, graph=True, sync=True)
    it0 = tp.graph_stats()["ppe_iters_total"]
    torch.cuda.synchronize()
    nt = max(1, min(args.steps, 50))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nt)]
    clocks = clocks_cls(torch.cuda.current_device())
    with clocks:
        for k in range(nt):
            flush.fill_(float(k))
            torch.cuda.current_stream().synchronize()
            ev[k][0].record(stream)
            tp.step(1, graph=True, sync=False)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    iters = tp.graph_stats()["ppe_iters_total"] - it0
    names = ["phi", "u", "v", "p"]
    hb = {nm: torch.empty(g.shape, dtype=torch.float64).pin_memory() for nm in names}
    for nm in names:
        tp.download_ptr(nm, hb[nm].data_ptr())
    n_e2e = nt
    torch.cuda.synchronize()
    it1 = tp.graph_stats()["ppe_iters_total"]
    t0 = time.perf_counter()
    ptrs = [hb[nm].data_ptr() for nm in names]
    # three windows of n_e2e steps on the host clock, the median reported (a host-side stall
    # in one window does not decide the figure)
    e2e_w = []
    for w in range(3):
        if w:
            t0 = time.perf_counter()
        for _ in range(n_e2e):
            tp.upload_many_ptr(names, ptrs)
            tp.step(1, graph=True, sync=False)
            tp.download_many_ptr(names, ptrs)
        e2e_w.append(n_e2e / (time.perf_counter() - t0))
    e2e = sorted(e2e_w)[1]
    it_e2e = (tp.graph_stats()["ppe_iters_total"] - it1) / (3 * n_e2e)
    diag = tp.diagnostics()
    tp.close()
    return {"schedule": "reference: projection while iter < 5, then fast pressure correction (constant-coefficient "
                        "multigrid, ppe_tol 1e-8 absolute, at most 100 cycles)",
            "steps_timed": nt, "steps_per_s": nt / (ms / 1e3), "ms_per_step": ms / nt,
            "e2e_steps_per_s": e2e, "e2e_windows": e2e_w, "fpc_cycles_per_step": iters / nt,
            "e2e_fpc_cycles_per_step": it_e2e, "clocks": clocks.summary(),
            "diagnostics": diag,
            "note": "same schedule and tolerances as the reference arm (--impl reference); the headline solves the "
                    "variable-density projection equation to a relative residual of 1e-10 every step"}


def run_ours(args) -> None:
    import numpy as np
    import torch
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    from scihpc_gb300 import Grid, Poisson, TwoPhase, lib
    lib()   # raises if the CUDA library is missing: there is no CPU path
    g = Grid(2, (NX, NY), DOMAIN[0], DOMAIN[1])
    h = min(g.spacing())
    tp = TwoPhase(g, ["no_slip"] * 6, ["neumann"] * 6, physics(h), scheme=1, n_mpls=5, reinit_every=1,
                  fp32=args.ppe == "fp32")
    phi0 = initial_phi(g.shape)
    tp.set("phi", phi0)
    tp.init()
    stream = torch.cuda.ExternalStream(tp.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    tp.step(args.warmup, graph=not args.eager, sync=True)
    it0 = tp.graph_stats()["ppe_iters_total"]
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with clocks:
        t_wall = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.current_stream().synchronize()
            ev[k][0].record(stream)
            tp.step(1, graph=not args.eager, sync=False)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    barrier(ws)
    torch.cuda.synchronize()
    ms_local = sum(a.elapsed_time(b) for a, b in ev)
    ms_total = max_over_ranks(ws, ms_local, torch.device("cuda"))
    value = ws * args.steps / (ms_total / 1e3)
    gs = tp.graph_stats()
    ppe_iters = gs["ppe_iters_total"] - it0
    launches = args.steps * (gs["pre"] + gs["post"]) + gs["body"] * ppe_iters
    diag = tp.diagnostics()
    if args.lite:
        if rank == 0:
            print(json.dumps({"metric": "time steps/s", "value": value, "lite": True, "gpu_launches": launches,
                              "ppe_iters_per_step": ppe_iters / args.steps, "graph": gs}), flush=True)
        return

    # end to end through the public API with host buffers: per step, upload the state
    # (phi, u, v, p) from pinned host memory, one step, download it again
    names = ["phi", "u", "v", "p"]
    hb = {nm: torch.empty(g.shape, dtype=torch.float64).pin_memory() for nm in names}
    for nm in names:
        tp.download_ptr(nm, hb[nm].data_ptr())
    nbytes = len(names) * g.size * 8
    e2e_steps = max(1, min(args.steps, 50))
    ptrs = [hb[nm].data_ptr() for nm in names]
    # five windows of e2e_steps steps, each timed on the host clock (max over ranks); the line
    # reports the median window, so that a host-side stall (windows of 239 and 410 against
    # ~570 steps/s were seen) does not decide the figure, and lists all five
    windows = []
    for _ in range(5):
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            tp.upload_many_ptr(names, ptrs)
            tp.step(1, graph=True, sync=False)
            tp.download_many_ptr(names, ptrs)   # on the step's stream: returns once the fields are on the host
        windows.append(ws * e2e_steps / max_over_ranks(ws, time.perf_counter() - t0, torch.device("cuda")))
    e2e = {"value": sorted(windows)[2], "unit": "steps/s", "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes, "steps": e2e_steps, "windows": windows,
           "api": "scihpc_twophase_upload_many (4 fields) + scihpc_twophase_step + "
                  "scihpc_twophase_download_many (4 fields)"}

    # roofline of the step's dominant kernel: the reinitialisation's gradient kernel
    # (k_reinit_a2d, the largest share of the step's launch list), FP64-bound on
    # L2-resident data, against the FP64 roof measured here; the pressure V-cycle (the
    # HBM-bound kernel group at 256^3) beside it
    from scihpc_gb300.native import measure_fp64_peak
    hbm = peaks()
    fp64_peak = measure_fp64_peak()
    ra_ms = tp.time_reinit_gradient(200)
    ra_flops = REINIT_FLOPS_2D * NX * NY
    roof = {"bound": "fp64", "kernel": "k_reinit_a2d (Godunov |grad phi| + redistance source + lambda fields)",
            "achieved": ra_flops / (ra_ms * 1e-3) / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": ra_flops / (ra_ms * 1e-3) / 1e12 / fp64_peak,
            "peak_src": "measured in this run (chains of FP64 fused multiply-adds on every SM, CUDA events)",
            "traffic": REINIT_TRAFFIC_BYTES, "alg_flops_per_launch": ra_flops, "launch_ms": ra_ms,
            "flops_per_cell": REINIT_FLOPS_2D, "share_of_step": REINIT_SHARE,
            "traffic_src": REINIT_TRAFFIC_SRC}
    fp32 = args.ppe == "fp32"
    ps = Poisson(g, bc=0, density=True, fp32=fp32)
    ps.set_density(tp.device_ptr("rho"))
    ptmp = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    ncyc = 200
    vms = ps.time_vcycles(tp.device_ptr("rhs"), ptmp, ncyc) / ncyc
    vb = vcycle_bytes(ps.levels(), 2, 4 if fp32 else 8)
    roof["vcycle_128x256"] = {"bound": "hbm", "kernel": f"pressure V(2,2) cycle, all levels ({'FP32' if fp32 else 'FP64'})",
                              "achieved": vb / vms / 1e6, "peak": hbm["hbm_gbs"], "unit": "GB/s",
                              "frac": vb / vms / 1e6 / hbm["hbm_gbs"], "peak_src": hbm["src"], "traffic": None,
                              "alg_bytes_per_launch": vb, "launch_ms": vms,
                              "note": "L2-resident working set: latency bound, model bytes"}
    ps.close()

    line = {"metric": "time steps/s", "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded analytic bubble)",
            "config": config_block({"parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                                    "pressure_precision": PPE_DESC[args.ppe]}),
            "clocks": clocks.summary(), "e2e": e2e, "gpu_launches": int(launches),
            "ppe_iters_per_step": ppe_iters / args.steps, "wall_s": t_wall, "roofline": roof,
            "diagnostics": diag}
    blocks = set(args.blocks.split(","))
    if rank == 0 and "stock" in blocks:
        line["stock_schedule"] = stock_block(torch, args, flush, Clocks)
    if rank == 0 and not args.no_poisson and "poisson" in blocks:
        line["poisson_256^3"] = poisson_block(torch, Poisson, Grid, hbm)
        v = line["poisson_256^3"]["fp32_refined"]
        roof["vcycle_256^3"] = {"bound": "hbm", "kernel": "pressure V(2,2) cycle, all levels (FP32), 256^3",
                                "achieved": v["vcycle_gbs"], "peak": hbm["hbm_gbs"], "unit": "GB/s",
                                "frac": v["vcycle_frac_of_hbm"], "peak_src": hbm["src"],
                                "alg_bytes_per_launch": v["vcycle_alg_bytes"], "launch_ms": v["vcycle_ms"],
                                "traffic": VCYCLE_256_TRAFFIC_BYTES, "traffic_src": VCYCLE_256_TRAFFIC_SRC}
    if rank == 0 and not args.no_poisson:
        if "dirichlet" in blocks:
            line["poisson_256^2_dirichlet"] = dirichlet_block(torch, Poisson, Grid, cpu=False)
        if "dambreak" in blocks:
            line["dambreak_3d"] = dambreak_block(torch, TwoPhase, Grid)
        if "learned" in blocks:
            line["learned_guess"] = learned_block(torch, ntrain=args.learned_train)
        if "learned3" in blocks:
            line["learned_guess_3d"] = learned3_block(torch)
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cb = cpu_baselines_fresh(threads)
        b = cb["bubble"]
        model = cpu_model()
        line["cpu_baseline"] = {"value": b["all_cores"]["value"], "unit": "steps/s", "cores": threads, "kind": "port",
                                "model": model,
                                "sample": f"median of 3 windows of {b['all_cores']['steps_per_window']} time steps of "
                                          "the same workload after the reference schedule's 5 start-up steps "
                                          "(reference algorithm restated in oracle/port, all host cores)",
                                "one_thread": b["one_thread"]}
        line["cpu_baselines"] = {"model": model, "cores": threads,
                                 "rising_bubble_128x256": b,
                                 "dambreak_3d_128x64x64": cb["dambreak"],
                                 "poisson_spheres_sor": cb["sor"],
                                 "poisson_256^2_dirichlet_reference_mg": cb["mg"],
                                 "process": "a fresh Python process without torch or a CUDA context, as the "
                                            "reference arm runs"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def dirichlet_block(torch, Poisson, Grid, cpu: bool) -> dict:
    """256^2 constant-coefficient Poisson problem with the reference's Dirichlet operator
    (-lap p = 2 pi^2 sin(pi x) sin(pi y) on [0,1]^2, zero guess) to relative residual 1e-10:
    FP64 V-cycles in FP64 CG and FP32 V-cycles in FP64 refinement on the GPU; with `cpu`, the
    reference multigrid (v_cycle, restated in oracle/port) on the host cores beside it."""
    import numpy as np
    n = 256
    g = Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
    h = 1.0 / n
    xc = (np.arange(n) + 0.5) * h
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    f = 2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
    rhs_h = np.zeros((n + 6, n + 6, 1))
    rhs_h[3:-3, 3:-3, 0] = -f   # A p = -f with A the reference's +laplacian
    rhs = torch.from_numpy(rhs_h).cuda()
    out = {"grid": "256^2", "problem": "-lap p = 2 pi^2 sin(pi x) sin(pi y), Dirichlet (reference operator)",
           "rel_tol": 1e-10}
    for name, fp32 in (("fp64", False), ("fp32_refined", True)):
        ps = Poisson(g, bc=1, density=False, fp32=fp32)
        p = torch.zeros(rhs.shape, dtype=torch.float64, device="cuda")
        ps.solve(rhs, p, rel_tol=1e-10, max_iter=100)   # warm
        times = []
        for _ in range(3):
            p.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            it, rr = ps.solve(rhs, p, rel_tol=1e-10, max_iter=100)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        out[name] = {"ms_to_tol": min(times), "iterations": it, "final_relres": rr}
        ps.close()
    out["fp32_speedup"] = out["fp64"]["ms_to_tol"] / out["fp32_refined"]["ms_to_tol"]
    out["note"] = ("timed by CUDA events; repeated solves with the same inputs run as one captured CUDA graph "
                   "(conditional while-node over the iterations, one host synchronisation per solve)")
    if cpu:
        import oracle as O
        gg = O.Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))
        port = O.Checker("port")
        port.mg_poisson(gg, (-f).T.ravel(), True, 1e-10, 400)   # warm
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            _, cyc, hist = port.mg_poisson(gg, (-f).T.ravel(), True, 1e-10, 400)
            ts.append(time.perf_counter() - t0)
        out["cpu_baseline"] = {"value": 1e3 * float(np.median(ts)), "unit": "ms to rel. residual 1e-10",
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": f"reference multigrid v_cycle ({cyc} cycles, final relres "
                                         f"{float(hist[-1]):.1e}), median of 3"}
    return out


def dambreak_setup(Grid):
    """Grid, parameters and initial level set of the 128 x 64 x 64 dam break (dambreak_block)."""
    import numpy as np
    n = (128, 64, 64)
    g = Grid(3, n, (0.0, 0.0, 0.0), (4.0, 2.0, 2.0))
    h = min(4.0 / n[0], 2.0 / n[1], 2.0 / n[2])
    Uc = float(np.sqrt(9.81))
    prm = dict(density_ratio=1.2 / 1000.0, viscosity_ratio=1.8e-5 / 1e-3, Re=1000.0 * Uc / 1e-3, Fr=1.0, We=-1.0,
               ls_width=1.5 * h, rdt=0.1 * h, max_CFL=0.1, min_CFL=1e-4, positive_ref=1.0, ppe_tol=PPE_TOL,
               ppe_tol2=0.0, ppe_max_iter=200, ppe_omega=1.5, ppe_initer=1, dt0=1.0)
    c = [(np.arange(n[a]) + 0.5) * (4.0, 2.0, 2.0)[a] / n[a] for a in range(3)]
    X, Y, Z = np.meshgrid(*c, indexing="ij")
    phi = np.zeros(g.shape)
    phi[3:-3, 3:-3, 3:-3] = np.where((X < 1.0) & (Z < 1.0), np.minimum(1.0 - X, 1.0 - Z),
                                     -np.sqrt(np.maximum(X - 1.0, 0.0) ** 2 + np.maximum(Z - 1.0, 0.0) ** 2))
    return g, prm, phi


def dambreak_block(torch, TwoPhase, Grid, steps: int = 40, warmup: int = 3) -> dict:
    """3D dam break, 128 x 64 x 64 cells on [0,4] x [0,2] x [0,2]: water column [0,1] x [0,2] x
    [0,1] (signed distance to its free surfaces), air/water 1000/1.2 density and 1e-3/1.8e-5
    viscosity, gravity 9.81 along -z, L = 1, no surface tension, slip walls on all faces, UCCD
    transport, reinitialisation every 20 steps (the reference's dam-break driver), pressure to
    relative residual 1e-10 each step with FP64 V-cycles and with FP32 V-cycles in FP64
    refinement.  Graph replay; the working set (~60 fields of 0.6 M cells) exceeds L2."""
    g, prm, phi = dambreak_setup(Grid)
    out = {"grid": "128x64x64 on [0,4]x[0,2]x[0,2]", "steps_timed": steps,
           "physics": "rho 1000/1.2, mu 1e-3/1.8e-5, g 9.81 (-z), L 1, no surface tension, slip walls",
           "step": "find_dt + UCCD/TVD-RK3 transport + ab_solve (pressure to rel. residual 1e-10); "
                   "reinit every 20 steps"}
    for name, fp32 in (("fp64", False), ("fp32_refined", True)):
        tp = TwoPhase(g, ["slip"] * 6, ["neumann"] * 6, prm, scheme=0, n_mpls=0, reinit_every=20, fp32=fp32)
        tp.set("phi", phi)
        tp.init()
        tp.step(warmup, graph=True, sync=True)
        it0 = tp.graph_stats()["ppe_iters_total"]
        stream = torch.cuda.ExternalStream(tp.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        tp.step(steps, graph=True, sync=False)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        d = tp.diagnostics()
        out[name] = {"steps_per_s": steps / (ms / 1e3), "ms_per_step": ms / steps,
                     "ppe_iters_per_step": (tp.graph_stats()["ppe_iters_total"] - it0) / steps,
                     "t": tp.scalars()["t"], "div": d["div"], "volume": d["volume"]}
        tp.close()
    out["fp32_speedup"] = out["fp32_refined"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    return out


def learned_block(torch, n: int = 512, factor: int = 4, ntrain: int = 2048, ntest: int = 16,
                  steps: int = 3000, chunk: int = 2048) -> dict:
    """Learned initial guess, 2D benchmark configuration: 512^2 Rayleigh-Taylor-type fields
    (density ratio 3, interface from 8 seeded sinusoids, right-hand side the divergence of a
    seeded random wall-tight velocity; learned.cfg4_problem), pairs of consecutive steps
    solved by the FP32-refined multigrid to 1e-10 on the GPU (2048 training pairs, 16 held-out
    pairs from seeds >= 10^6; above `chunk` training pairs they are generated chunk by chunk
    and visited once each).  The tensor-core U-Net (4 levels, 16-128 channels) runs on the
    grid coarsened factor x factor and predicts the coarse error of the previous pressure
    (scihpc_unet_create_coarse); Adam training on the GPU.  Time to 1e-10 on the held-out
    pairs from the previous pressure and from the network's guess (inference included), with
    the same solver and buffers (graph replay, one host synchronisation per solve)."""
    import time as _t
    import numpy as np
    from scihpc_gb300 import Grid, Poisson, UNet
    from scihpc_gb300.learned import guess_errors, make_snapshots_cfg4, train, train_cfg4_stream
    dev = torch.device("cuda")
    stream = ntrain > chunk
    t0 = _t.perf_counter()
    tr = None if stream else make_snapshots_cfg4(n, range(ntrain), torch, dev)
    te = make_snapshots_cfg4(n, range(10 ** 6, 10 ** 6 + ntest), torch, dev)
    t_snap = _t.perf_counter() - t0
    net = UNet(n, n, seed=0, factor=factor)
    g = Grid(2, (n, n), (0.0, 0.0), (1.0, 1.0))

    def test_loss():
        return float(np.mean([net.loss_grad(g, *s) for s in te]))

    loss_before = test_loss()
    torch.cuda.synchronize()
    t0 = _t.perf_counter()
    if stream:   # snapshot generation included in the training time
        losses = train_cfg4_stream(net, n, range(ntrain), chunk, 1e-3, torch, dev)
        steps = len(losses)
    else:
        losses = train(net, tr, steps, 1e-3, torch, cosine=True)
    torch.cuda.synchronize()
    t_train = _t.perf_counter() - t0
    loss_after = test_loss()
    err_ratio = guess_errors(te, torch, net)
    del tr
    hc = n // factor
    layers = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (64, 128, 3),
              (128, 128, 3), (192, 64, 2), (64, 64, 2), (96, 32, 1), (32, 32, 1), (48, 16, 0), (16, 16, 0), (16, 16, 0)]
    flops = sum(2.0 * 9 * ci * co * (hc >> lv) ** 2 for ci, co, lv in layers)
    ps = Poisson(g, bc=0, density=True, fp32=True)
    rho_b, rhs_b, pp_b, p_b = (torch.zeros_like(te[0][0]) for _ in range(4))

    def load(snap):
        rho_b.copy_(snap[0])
        rhs_b.copy_(snap[1])
        pp_b.copy_(snap[2])
        ps.set_density(rho_b)
        torch.cuda.synchronize()

    def run(use_net, zero=False):
        torch.cuda.synchronize()
        t1 = _t.perf_counter()
        if zero:
            p_b.zero_()
        else:
            p_b.copy_(pp_b)
        if use_net:
            net.infer(g, rho_b, rhs_b, pp_b, p_b)
        it, rr = ps.solve(rhs_b, p_b, rel_tol=1e-10, max_iter=200, use_guess=True)
        torch.cuda.synchronize()
        return _t.perf_counter() - t1, it, rr

    load(te[0])
    for _ in range(3):   # first calls: capture of the solve graph for these buffers, warm-up
        run(False)
        run(True)
    res = {False: [], True: []}
    it_zero = []
    for snap in te:
        load(snap)
        for use_net in (False, True):
            res[use_net].append(run(use_net))
        it_zero.append(run(False, zero=True)[1])
    t_inf = []
    for _ in range(20):
        torch.cuda.synchronize()
        t1 = _t.perf_counter()
        net.infer(g, rho_b, rhs_b, pp_b, p_b)
        torch.cuda.synchronize()
        t_inf.append(_t.perf_counter() - t1)
    ps.close()
    net.close()
    it0 = [r[1] for r in res[False]]
    it1 = [r[1] for r in res[True]]
    return {"grid": f"{n}x{n}", "network_grid": f"{hc}x{hc}", "train_snapshots": ntrain, "test_snapshots": ntest,
            "train_steps": steps, "snapshot_s": t_snap, "train_ms_per_step": 1e3 * t_train / steps,
            "train_streamed": stream,
            "lr": "1e-3, half-cosine decay to 0", "test_loss_before": loss_before, "test_loss_after": loss_after,
            "train_loss_first150": float(np.mean(losses[:150])), "train_loss_last150": float(np.mean(losses[-150:])),
            "infer_ms": 1e3 * float(np.median(t_inf)), "infer_conv_tflops": flops / float(np.median(t_inf)) / 1e12,
            "guess_error_ratio_mean": float(np.mean(err_ratio)), "guess_error_ratio_max": float(np.max(err_ratio)),
            "vcycles_from_zero": float(np.mean(it_zero)),
            "vcycles_from_pprev": float(np.mean(it0)), "vcycles_from_net": float(np.mean(it1)),
            "pairs_fewer_iterations_with_net": int(sum(b < a for a, b in zip(it0, it1))),
            "pairs_more_iterations_with_net": int(sum(b > a for a, b in zip(it0, it1))),
            "ms_to_tol_from_pprev": 1e3 * float(np.mean([r[0] for r in res[False]])),
            "ms_to_tol_from_net_incl_inference": 1e3 * float(np.mean([r[0] for r in res[True]])),
            "max_relres": float(max(r[2] for r in res[False] + res[True])),
            "note": "host-timed per solve with synchronisations on both sides; FP32-refined multigrid to 1e-10 "
                    "from the previous pressure or from the network's guess (inference included)"}


def learned3_block(torch, n: int = 256, ntrain: int = 16, ntest: int = 3, steps: int = 400) -> dict:
    """Learned initial guess in 3D (tensor-core U-Net, 3 levels, 16-64 channels, at half the
    grid's resolution): pairs of consecutive steps of the n^3 spheres problem (density
    1 + 999 H, smooth random divergent right-hand side) solved to 1e-10, Adam training on the
    GPU, then time to 1e-10 on held-out pairs: FP64 multigrid and FP32-refined multigrid from
    the previous pressure, and FP32-refined from the network's guess (inference included)."""
    import time as _t
    import numpy as np
    from scihpc_gb300 import Grid, Poisson, UNet
    from scihpc_gb300.learned import guess_errors, make_snapshots3, train
    dev = torch.device("cuda")
    t0 = _t.perf_counter()
    tr = make_snapshots3(n, range(ntrain), torch, dev)
    te = make_snapshots3(n, range(10 ** 6, 10 ** 6 + ntest), torch, dev)
    torch.cuda.synchronize()
    t_snap = _t.perf_counter() - t0
    g = Grid(3, (n, n, n), (0.0,) * 3, (1.0,) * 3)
    net = UNet(n, n, n, seed=0)

    def test_loss():
        return float(np.mean([net.loss_grad(g, *s) for s in te]))

    loss_before = test_loss()
    torch.cuda.synchronize()
    t0 = _t.perf_counter()
    losses = train(net, tr, steps, 1e-3, torch, cosine=True)
    torch.cuda.synchronize()
    t_train = _t.perf_counter() - t0
    loss_after = test_loss()
    err_ratio = guess_errors(te, torch, net)
    # convolution work of one inference: 2 * 27 * ci * co per voxel of each layer's level
    layers = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (96, 32, 1), (32, 32, 1),
              (48, 16, 0), (16, 16, 0), (16, 16, 0)]
    vox = (n // 2) ** 3
    flops = sum(2.0 * 27 * ci * co * vox / 8 ** lv for ci, co, lv in layers)
    rho, rhs, pprev, _ = te[0]
    guess = pprev.clone()
    for _ in range(2):
        net.infer(g, rho, rhs, pprev, guess)
    torch.cuda.synchronize()
    t0 = _t.perf_counter()
    for _ in range(5):
        net.infer(g, rho, rhs, pprev, guess)
    torch.cuda.synchronize()
    t_inf = (_t.perf_counter() - t0) / 5
    out = {"grid": f"{n}^3", "network_grid": f"{n // 2}^3", "train_pairs": ntrain, "test_pairs": ntest,
           "train_steps": steps, "snapshot_s": t_snap, "train_ms_per_step": 1e3 * t_train / steps,
           "lr": "1e-3, half-cosine decay to 0", "test_loss_before": loss_before, "test_loss_after": loss_after,
           "train_loss_first20": float(np.mean(losses[:20])), "train_loss_last20": float(np.mean(losses[-20:])),
           "infer_ms": 1e3 * t_inf, "infer_conv_tflops": flops / t_inf / 1e12,
           "guess_error_ratio_mean": float(np.mean(err_ratio)), "guess_error_ratio_max": float(np.max(err_ratio))}
    p = torch.zeros_like(pprev)
    for name, fp32, use_net in (("fp64_from_pprev", False, False), ("fp32_refined_from_pprev", True, False),
                                ("fp32_refined_from_net", True, True), ("fp32_refined_from_zero", True, None)):
        ps = Poisson(g, bc=0, density=True, fp32=fp32)
        times, its, rrs = [], [], []
        for rho, rhs, pprev, _ in te:
            ps.set_density(rho)
            for timed in (False, True):   # the untimed solve warms up and captures the solve graph
                if use_net is None:
                    p.zero_()
                else:
                    p.copy_(pprev)
                torch.cuda.synchronize()
                t0 = _t.perf_counter()
                if use_net:
                    net.infer(g, rho, rhs, pprev, p)
                it, rr = ps.solve(rhs, p, rel_tol=1e-10, max_iter=200, use_guess=True)
                torch.cuda.synchronize()
                if timed:
                    times.append(_t.perf_counter() - t0)
                    its.append(it)
                    rrs.append(rr)
        ps.close()
        out[name] = {"ms_to_tol": 1e3 * float(np.mean(times)), "iterations": float(np.mean(its)),
                     "max_relres": float(max(rrs))}
    net.close()
    out["fp32_learned_speedup_vs_fp64"] = out["fp64_from_pprev"]["ms_to_tol"] / out["fp32_refined_from_net"]["ms_to_tol"]
    out["fp32_speedup_vs_fp64"] = out["fp64_from_pprev"]["ms_to_tol"] / out["fp32_refined_from_pprev"]["ms_to_tol"]
    out["note"] = ("host-timed per solve (inference included for the network's guess); every solve iterates to "
                   "1e-10, so the network can only change the iteration count")
    return out


def profile_poisson(precision: str, n: int = 256) -> None:
    """One density update and three solver iterations of the n^3 pressure equation (the
    spheres problem): the case the profiles of the pressure kernels are captured on."""
    import torch
    from scihpc_gb300 import Grid, Poisson, lib
    lib()
    g, rho, rhs = poisson_problem(torch, Grid, n)
    ps = Poisson(g, bc=0, density=True, fp32=precision == "fp32")
    ps.set_density(rho)
    p = torch.zeros(g.shape, dtype=torch.float64, device=rho.device)
    it, rr = ps.solve(rhs, p, rel_tol=1e-10, max_iter=3)
    torch.cuda.synchronize()
    print(json.dumps({"profile": "poisson 256^3", "precision": precision, "iterations": it, "relres": rr}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-poisson", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--lite", action="store_true", help="timed steps only (for kernel launch lists)")
    ap.add_argument("--eager", action="store_true", help="launch kernels one by one instead of graph replay")
    ap.add_argument("--ppe", default="fp32", choices=["fp32", "fp64"],
                    help="pressure V-cycles in FP32 inside FP64 refinement (default) or all FP64")
    ap.add_argument("--profile-unet", action="store_true",
                    help="only a few training steps of the 256^2 learned guess (profiling case)")
    ap.add_argument("--profile-unet3", action="store_true",
                    help="only a few training steps of the 3D learned guess on a 128^3 grid (profiling case)")
    ap.add_argument("--profile-dambreak", action="store_true",
                    help="init and two steps of the 128x64x64 dam break, kernel by kernel (profiling case)")
    ap.add_argument("--profile-reinit3d", action="store_true",
                    help="the dam break's 3D reinitialisation gradient kernel, 53 launches (profiling case)")
    ap.add_argument("--profile-poisson", choices=["fp32", "fp64"],
                    help="only three iterations of the n^3 pressure solve (profiling case)")
    ap.add_argument("--poisson-n", type=int, default=256, help="grid of --profile-poisson")
    ap.add_argument("--blocks", default="stock,poisson,dirichlet,dambreak,learned,learned3",
                    help="comma-separated extra blocks of the bench line")
    ap.add_argument("--learned-train", type=int, default=2048,
                    help="training pairs of the 512^2 learned-guess block (above 2048 they are "
                         "generated in chunks of 2048 and visited once each)")
    args = ap.parse_args()
    if args.profile_unet:
        import torch
        from scihpc_gb300 import UNet, lib
        from scihpc_gb300.learned import make_snapshots, train
        lib()
        snaps = make_snapshots(256, range(4), torch, torch.device("cuda"))
        net = UNet(256, 256, seed=0)
        losses = train(net, snaps, 4, 1e-3, torch)
        print(json.dumps({"profile": "unet 256^2 training steps", "loss": losses}))
    elif args.profile_unet3:
        import torch
        from scihpc_gb300 import UNet, lib
        from scihpc_gb300.learned import make_snapshots3, train
        lib()
        snaps = make_snapshots3(128, range(2), torch, torch.device("cuda"))
        net = UNet(128, 128, 128, seed=0)
        losses = train(net, snaps, 3, 1e-3, torch)
        print(json.dumps({"profile": "unet3 128^3 training steps", "loss": losses}))
    elif args.profile_dambreak:
        import torch
        from scihpc_gb300 import Grid, TwoPhase, lib
        lib()
        g, prm, phi = dambreak_setup(Grid)
        tp = TwoPhase(g, ["slip"] * 6, ["neumann"] * 6, prm, scheme=0, n_mpls=0, reinit_every=20, fp32=True)
        tp.set("phi", phi)
        tp.init()
        tp.step(2, graph=False, sync=True)
        print(json.dumps({"profile": "dambreak 128x64x64, init + 2 steps", "scalars": tp.scalars()}))
    elif args.profile_reinit3d:
        import torch
        from scihpc_gb300 import Grid, TwoPhase, lib
        lib()
        g, prm, phi = dambreak_setup(Grid)
        tp = TwoPhase(g, ["slip"] * 6, ["neumann"] * 6, prm, scheme=0, n_mpls=0, reinit_every=20, fp32=True)
        tp.set("phi", phi)
        tp.init()
        tp.step(3, graph=True, sync=True)
        ms = tp.time_reinit_gradient(50)
        print(json.dumps({"profile": "dambreak 128x64x64, reinitialisation gradient kernel", "launch_ms": ms}))
    elif args.profile_poisson:
        profile_poisson(args.profile_poisson, args.poisson_n)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
