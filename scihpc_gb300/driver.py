"""Configured two-phase runs: ``python -m scihpc_gb300.driver config.json``.

The part of the reference's benchmarks_2d_*.cpp drivers (benchmarks_2d_bubble_rising.cpp,
benchmarks_2d_dambreak.cpp) with the settings in a JSON file instead of the source: the grid,
the boundary conditions, the fluid (nondimensionalised as set_parameters does, global.cpp:
31-52, or given as ratios and numbers), the initial level set, the numerics and the run --
number of steps, progress lines, checkpoints written and resumed through the session's
checkpoint / restore, and legacy VTK files in the format of the reference's vtkWriter
(vtkWriter.cpp:18-111: STRUCTURED_POINTS, CELL_DATA, big-endian doubles).

Configuration (every key but "grid" and "initial" has a default)::

    {
      "grid":     {"n": [128, 256], "lo": [0, 0], "hi": [1, 2]},
      "boundary": {"velocity": "no_slip", "scalar": "neumann"},
      "fluid":    {"rho": [1000, 100], "mu": [10, 1], "sigma": 24.5, "gravity": 0.98,
                   "length": 1.0, "velocity": null, "positive_ref": false},
                  -- or {"density_ratio": .., "viscosity_ratio": .., "Re": .., "Fr": .., "We": ..}
      "initial":  {"shape": "sphere", "center": [0.5, 0.5], "radius": 0.25}
                  -- or {"shape": "box", "lo": [0, 0], "hi": [1, 2]} (+1 inside, -1 outside, then
                     "reinit_steps" redistance steps, as the dam-break driver does)
      "numerics": {"advection": "weno5", "mass_correction_steps": 5, "reinit_every": 1,
                   "pressure": "fp32", "source": "compact", "max_cfl": 0.2, "min_cfl": 1e-4,
                   "ppe_tol": 1e-10, "ppe_max_iter": 200, "ls_width_cells": 1.5,
                   "rdt_cells": 0.25},
      "run":      {"steps": 100, "graph": true, "log_every": 10, "checkpoint_every": 0,
                   "checkpoint": "run.ckpt", "restart": null, "vtk_every": 0, "vtk_prefix": "run"}
    }

"sphere" gives phi = radius - |x - center| (positive inside); with "positive_ref": false (the
bubble driver's choice) the inside is the light fluid.  "source": "second_order" runs the
projection step of benchmarks_2d_dambreak.cpp (ab_solve_sec).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import struct
import sys

import numpy as np

from .native import Grid, TwoPhase

__all__ = ["load_config", "fluid_parameters", "initial_level_set", "write_vtk", "run"]

DEFAULTS = {
    "boundary": {"velocity": "no_slip", "scalar": "neumann"},
    "fluid": {"rho": [1000.0, 100.0], "mu": [10.0, 1.0], "sigma": 24.5, "gravity": 0.98, "length": 1.0,
              "velocity": None, "positive_ref": False},
    "numerics": {"advection": "weno5", "mass_correction_steps": 5, "reinit_every": 1, "pressure": "fp32",
                 "source": "compact", "max_cfl": 0.2, "min_cfl": 1e-4, "ppe_tol": 1e-10, "ppe_max_iter": 200,
                 "ls_width_cells": 1.5, "rdt_cells": 0.25},
    "run": {"steps": 100, "graph": True, "log_every": 10, "checkpoint_every": 0, "checkpoint": "run.ckpt",
            "restart": None, "vtk_every": 0, "vtk_prefix": "run"},
}


def load_config(path_or_dict) -> dict:
    """The configuration with every missing section key taken from DEFAULTS."""
    cfg = path_or_dict if isinstance(path_or_dict, dict) else json.load(open(path_or_dict))
    for key in ("grid", "initial"):
        if key not in cfg:
            raise ValueError(f"configuration: '{key}' is required")
    out = {k: dict(v) for k, v in DEFAULTS.items()}
    for k, v in cfg.items():
        if k in out and isinstance(v, dict):
            out[k].update(v)
        else:
            out[k] = v
    n = out["grid"]["n"]
    if not 2 <= len(n) <= 3 or any(int(m) < 4 for m in n):
        raise ValueError("configuration: grid.n must list 2 or 3 sizes of at least 4 cells")
    return out


def fluid_parameters(cfg: dict, h: float) -> dict:
    """The session's parameter dictionary: set_parameters' nondimensional numbers
    (global.cpp:31-52: density and viscosity ratios rho2/rho1, mu2/mu1; Uc = sqrt(g L) unless a
    velocity scale is given; Re = rho1 Uc L / mu1, Fr = Uc / sqrt(g L), We = rho1 Uc^2 L / sigma,
    We = -1 without surface tension) or the numbers given directly, and the numerics."""
    f, num = cfg["fluid"], cfg["numerics"]
    if "density_ratio" in f:
        prm = {k: float(f[k]) for k in ("density_ratio", "viscosity_ratio", "Re", "Fr", "We")}
    else:
        (r1, r2), (m1, m2) = f["rho"], f["mu"]
        g, L = float(f["gravity"]), float(f["length"])
        uc = float(f["velocity"]) if f.get("velocity") else math.sqrt(g * L)
        sigma = float(f.get("sigma") or 0.0)
        prm = dict(density_ratio=r2 / r1, viscosity_ratio=m2 / m1, Re=r1 * uc * L / m1,
                   Fr=uc / math.sqrt(g * L) if g > 0 else -1.0,
                   We=r1 * uc * uc * L / sigma if sigma > 0 else -1.0)
    prm.update(ls_width=num["ls_width_cells"] * h, rdt=num["rdt_cells"] * h, max_CFL=num["max_cfl"],
               min_CFL=num["min_cfl"], positive_ref=1.0 if f.get("positive_ref") else 0.0,
               ppe_tol=num["ppe_tol"], ppe_tol2=0.0, ppe_max_iter=num["ppe_max_iter"], ppe_omega=1.5,
               ppe_initer=1, dt0=1.0)
    return prm


def initial_level_set(cfg: dict, grid: Grid) -> np.ndarray:
    """phi on the ghosted grid (interior cells; the session fills the ghosts)."""
    ini, g = cfg["initial"], cfg["grid"]
    n = [int(m) for m in g["n"]]
    lo, hi = [float(v) for v in g["lo"]], [float(v) for v in g["hi"]]
    xs = [lo[a] + (np.arange(n[a]) + 0.5) * (hi[a] - lo[a]) / n[a] for a in range(len(n))]
    X = np.meshgrid(*xs, indexing="ij")
    if ini["shape"] == "sphere":
        c, r = ini["center"], float(ini["radius"])
        val = r - np.sqrt(sum((X[a] - float(c[a])) ** 2 for a in range(len(n))))
    elif ini["shape"] == "box":
        inside = np.ones(X[0].shape, dtype=bool)
        for a in range(len(n)):
            inside &= (X[a] >= float(ini["lo"][a])) & (X[a] <= float(ini["hi"][a]))
        val = np.where(inside, 1.0, -1.0)
    else:
        raise ValueError(f"configuration: unknown initial shape {ini['shape']!r}")
    phi = np.zeros(grid.shape)
    if len(n) == 2:
        phi[3:-3, 3:-3, 0] = val
    else:
        phi[3:-3, 3:-3, 3:-3] = val
    return phi


def write_vtk(path: str, grid: Grid, scalars: dict, vectors: dict) -> None:
    """Legacy VTK as the reference's vtkWriter writes it (vtkWriter.cpp:18-111): structured
    points over the cell corners, cell data in x-fastest order, big-endian doubles."""
    n = list(grid.n) + [1] * (3 - len(grid.n))
    lo = list(grid.lo) + [0.0] * (3 - len(grid.lo))
    d = [(grid.hi[a] - grid.lo[a]) / grid.n[a] if a < len(grid.n) else 0.0 for a in range(3)]
    dims = [m + 1 if a < len(grid.n) else 1 for a, m in enumerate(n)]
    cells = int(np.prod([m - 1 for m in dims if m > 1]))

    def interior(a):
        if len(grid.n) == 2:
            return a[3:-3, 3:-3, 0:1]
        return a[3:-3, 3:-3, 3:-3]

    with open(path, "wb") as fh:
        fh.write(b"# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS\n")
        fh.write(f"DIMENSIONS {dims[0]} {dims[1]} {dims[2]}\n".encode())
        fh.write(f"ORIGIN {lo[0]:g} {lo[1]:g} {lo[2]:g}\n".encode())
        fh.write(f"SPACING {d[0]:g} {d[1]:g} {d[2]:g}\n".encode())
        fh.write(f"CELL_DATA {cells}\n".encode())
        for name, a in scalars.items():
            fh.write(f"SCALARS {name} double 1\nLOOKUP_TABLE default\n".encode())
            fh.write(np.ascontiguousarray(interior(a).transpose(2, 1, 0)).astype(">f8").tobytes())
        for name, (u, v, w) in vectors.items():
            fh.write(f"VECTORS {name} double\n".encode())
            comp = np.stack([interior(u), interior(v), interior(w)], axis=-1)   # [i][j][k][3]
            fh.write(np.ascontiguousarray(comp.transpose(2, 1, 0, 3)).astype(">f8").tobytes())


def run(cfg: dict, out=sys.stdout) -> dict:
    """Runs the configured problem; returns the last diagnostics and scalars."""
    g = cfg["grid"]
    nd = len(g["n"])
    grid = Grid(nd, tuple(int(m) for m in g["n"]), tuple(float(v) for v in g["lo"]), tuple(float(v) for v in g["hi"]))
    h = min((grid.hi[a] - grid.lo[a]) / grid.n[a] for a in range(nd))
    num, rn, bc = cfg["numerics"], cfg["run"], cfg["boundary"]
    vel_bc = bc["velocity"] if isinstance(bc["velocity"], list) else [bc["velocity"]] * 6
    scalar_bc = bc["scalar"] if isinstance(bc["scalar"], list) else [bc["scalar"]] * 6
    tp = TwoPhase(grid, vel_bc, scalar_bc, fluid_parameters(cfg, h),
                  scheme=1 if num["advection"] == "weno5" else 0, n_mpls=int(num["mass_correction_steps"]),
                  reinit_every=int(num["reinit_every"]), fp32=num["pressure"] == "fp32")
    tp.set_source_scheme(1 if num["source"] == "second_order" else 0)
    start = 0
    if rn.get("restart"):
        tp.restore(rn["restart"])
        start = int(round(tp.scalars()["iter"]))
        print(f"restart {rn['restart']} at step {start} t {tp.scalars()['t']:.6g}", file=out)
    else:
        tp.set("phi", initial_level_set(cfg, grid))
        for _ in range(int(cfg["initial"].get("reinit_steps", 0))):
            tp.find_sign()
            tp.reinit_step(1)
        tp.init()
    steps = int(rn["steps"])
    log_every, ck_every, vtk_every = int(rn["log_every"]), int(rn["checkpoint_every"]), int(rn["vtk_every"])

    def vtk(step):
        write_vtk(f"{rn['vtk_prefix']}{step}.vtk", grid, {"phi": tp.get("phi"), "pressure": tp.get("p")},
                  {"nvel": (tp.get("nu"), tp.get("nv"), tp.get("nw") if nd == 3 else np.zeros(grid.shape))})

    if vtk_every > 0 and start == 0:
        vtk(0)
    diag = {}
    step = start
    while step < steps:
        chunk = steps - step
        for every in (log_every, ck_every, vtk_every):
            if every > 0:
                chunk = min(chunk, every - step % every)
        tp.step(chunk, graph=bool(rn["graph"]))
        step += chunk
        if log_every > 0 and step % log_every == 0 or step == steps:
            diag = tp.diagnostics()
            sc = tp.scalars()
            print(f"step {step} t {sc['t']:.6g} dt {sc['dt']:.4g} mass {diag['mass']:.10g} "
                  f"volume {diag['volume']:.10g} div {diag['div']:.3e}", file=out, flush=True)
        if ck_every > 0 and step % ck_every == 0:
            tp.checkpoint(rn["checkpoint"])
        if vtk_every > 0 and step % vtk_every == 0:
            vtk(step)
    result = {"diagnostics": tp.diagnostics(), "scalars": tp.scalars()}
    tp.close()
    return result


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m scihpc_gb300.driver", description=__doc__.split("\n\n")[0])
    ap.add_argument("config", help="JSON configuration file")
    ap.add_argument("--steps", type=int, help="override run.steps")
    ap.add_argument("--restart", help="override run.restart (a checkpoint to resume from)")
    args = ap.parse_args(argv)
    cfg = load_config(args.config)
    if args.steps is not None:
        cfg["run"]["steps"] = args.steps
    if args.restart:
        cfg["run"]["restart"] = args.restart
    for key in ("checkpoint", "vtk_prefix"):
        d = os.path.dirname(str(cfg["run"][key]))
        if d:
            os.makedirs(d, exist_ok=True)
    run(cfg)
    return 0


if __name__ == "__main__":
    sys.exit(main())
