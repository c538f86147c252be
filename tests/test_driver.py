"""The JSON-configured driver (scihpc_gb300/driver.py): configuration defaults, set_parameters'
nondimensionalisation (global.cpp:31-52), initial level sets and the vtkWriter file layout on
the CPU; on the GPU a configured run, and a restart from its checkpoint that continues bit for
bit."""
import io
import math

import numpy as np
import pytest

from scihpc_gb300 import driver as DR
from scihpc_gb300.native import Grid

BUBBLE = {
    "grid": {"n": [16, 32], "lo": [0.0, 0.0], "hi": [1.0, 2.0]},
    "initial": {"shape": "sphere", "center": [0.43, 0.57], "radius": 0.23},
    "numerics": {"ppe_tol": 1e-10},
    "run": {"steps": 6, "graph": True, "log_every": 3},
}


def test_config_defaults_and_validation():
    cfg = DR.load_config(BUBBLE)
    assert cfg["numerics"]["advection"] == "weno5" and cfg["numerics"]["ppe_tol"] == 1e-10
    assert cfg["boundary"] == {"velocity": "no_slip", "scalar": "neumann"}
    with pytest.raises(ValueError):
        DR.load_config({"grid": {"n": [16, 32], "lo": [0, 0], "hi": [1, 2]}})
    with pytest.raises(ValueError):
        DR.load_config({"grid": {"n": [16], "lo": [0], "hi": [1]}, "initial": {"shape": "sphere"}})


def test_fluid_parameters_follow_set_parameters():
    """rho 1000/100, mu 10/1, sigma 24.5, g 0.98, L 1 (Hysing's first case)."""
    h = 1.0 / 16
    prm = DR.fluid_parameters(DR.load_config(BUBBLE), h)
    uc = math.sqrt(0.98)
    assert prm["density_ratio"] == 0.1 and prm["viscosity_ratio"] == 0.1
    assert abs(prm["Re"] - 1000 * uc / 10) <= 1e-12 * prm["Re"]
    assert abs(prm["Fr"] - 1.0) <= 1e-15 and abs(prm["We"] - 1000 * uc * uc / 24.5) <= 1e-12 * prm["We"]
    assert prm["ls_width"] == 1.5 * h and prm["rdt"] == 0.25 * h and prm["positive_ref"] == 0.0
    given = dict(BUBBLE, fluid={"density_ratio": 0.5, "viscosity_ratio": 2.0, "Re": 10.0, "Fr": 1.0, "We": -1.0})
    assert DR.fluid_parameters(DR.load_config(given), h)["density_ratio"] == 0.5


def test_initial_level_sets():
    cfg = DR.load_config(BUBBLE)
    grid = Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
    phi = DR.initial_level_set(cfg, grid)
    x = (np.arange(16) + 0.5) / 16
    y = (np.arange(32) + 0.5) / 16
    X, Y = np.meshgrid(x, y, indexing="ij")
    assert np.array_equal(phi[3:-3, 3:-3, 0], 0.23 - np.sqrt((X - 0.43) ** 2 + (Y - 0.57) ** 2))
    box = DR.load_config(dict(BUBBLE, initial={"shape": "box", "lo": [0, 0], "hi": [0.5, 1.0]}))
    pb = DR.initial_level_set(box, grid)[3:-3, 3:-3, 0]
    assert set(np.unique(pb)) == {-1.0, 1.0} and pb[0, 0] == 1.0 and pb[-1, -1] == -1.0


def test_vtk_layout(tmp_path):
    """Header of vtkWriter::create and x-fastest big-endian cell data (vtkWriter.cpp:18-111)."""
    grid = Grid(2, (4, 3), (0.0, -1.0), (2.0, 0.5))
    f = np.zeros(grid.shape)
    f[3:-3, 3:-3, 0] = np.arange(12.0).reshape(4, 3)
    path = tmp_path / "a.vtk"
    DR.write_vtk(str(path), grid, {"phi": f}, {"v": (f, 2 * f, 0 * f)})
    raw = path.read_bytes()
    head = (b"# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS\n"
            b"DIMENSIONS 5 4 1\nORIGIN 0 -1 0\nSPACING 0.5 0.5 0\nCELL_DATA 12\n"
            b"SCALARS phi double 1\nLOOKUP_TABLE default\n")
    assert raw.startswith(head)
    vals = np.frombuffer(raw[len(head):len(head) + 96], dtype=">f8")
    assert np.array_equal(vals, np.arange(12.0).reshape(4, 3).T.ravel())   # x fastest
    vec = np.frombuffer(raw[len(head) + 96 + len(b"VECTORS v double\n"):], dtype=">f8").reshape(3, 4, 3)
    assert np.array_equal(vec[:, :, 1], 2 * np.arange(12.0).reshape(4, 3).T)


@pytest.mark.gpu
def test_configured_run_and_restart(tmp_path):
    ck = str(tmp_path / "run.ckpt")
    cfg = DR.load_config(dict(BUBBLE, run=dict(BUBBLE["run"], checkpoint_every=3, checkpoint=ck, vtk_every=3,
                                                 vtk_prefix=str(tmp_path / "bubble"))))
    log = io.StringIO()
    full = DR.run(cfg, out=log)
    lines = [ln for ln in log.getvalue().splitlines() if ln.startswith("step ")]
    assert [int(ln.split()[1]) for ln in lines] == [3, 6]
    for k in (0, 3, 6):
        assert (tmp_path / f"bubble{k}.vtk").stat().st_size > 16 * 32 * 8 * 4
    # the checkpoint holds step 6; resume from a copy written at step 3 by a second run
    cfg3 = DR.load_config(dict(BUBBLE, run=dict(BUBBLE["run"], steps=3, checkpoint_every=3, checkpoint=ck)))
    DR.run(cfg3, out=io.StringIO())
    resumed = DR.run(DR.load_config(dict(BUBBLE, run=dict(BUBBLE["run"], restart=ck))), out=io.StringIO())
    assert resumed["scalars"] == full["scalars"]
    assert resumed["diagnostics"] == full["diagnostics"]
    m = full["diagnostics"]["mass"]
    assert np.isfinite(m) and m > 0


def test_shipped_configurations_load():
    import glob
    import os
    here = os.path.join(os.path.dirname(DR.__file__), "configs")
    files = sorted(glob.glob(os.path.join(here, "*.json")))
    assert len(files) >= 2
    for f in files:
        cfg = DR.load_config(f)
        DR.fluid_parameters(cfg, 0.01)
