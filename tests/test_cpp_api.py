"""The reference-style C++ API (scihpc_gb300/cpp/scihpc/*.h over libscihpc_cpp.so): a driver
written the way the reference's benchmark drivers are (structured_grid, wrapper with
bc_info, runge_kutta with identity_flux/convection/mpls/lsf_redistance_lambda,
projection_method::find_source/ab_solve, find_dt, lsf_mass, vtkWriter) compiles against it
and, on a GPU, reproduces the CPU restatement of the reference step by step."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_params, bubble_phi, rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "bubble_driver.cpp")
G = O.Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
CENTER, RADIUS = (0.43, 0.57), 0.23


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from scihpc_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "bubble_driver")
    r = subprocess.run(["g++", "-O2", "-Wall", DRIVER, "-o", exe] + build.cxx_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_compiles_and_links(driver):
    assert os.path.exists(driver)


def run_driver(driver, tmp_path, steps, weno, vtk=False, second_order=False, compose=False, exact=False):
    prm = bubble_params(G, ppe_tol=1e-12)
    vals = dict(nx=G.n[0], ny=G.n[1], x0=G.lo[0], x1=G.hi[0], y0=G.lo[1], y1=G.hi[1], cx=CENTER[0], cy=CENTER[1],
                r=RADIUS, density_ratio=prm["density_ratio"], viscosity_ratio=prm["viscosity_ratio"], Re=prm["Re"],
                Fr=prm["Fr"], We=prm["We"], ls_width=prm["ls_width"], rdt=prm["rdt"], max_CFL=prm["max_CFL"],
                min_CFL=prm["min_CFL"], ppe_tol=prm["ppe_tol"], ppe_max_iter=prm["ppe_max_iter"],
                positive_ref=prm["positive_ref"], steps=steps, weno=int(weno), second_order=int(second_order),
                compose=int(compose), exact=int(exact))
    pf = tmp_path / "params.txt"
    pf.write_text("".join(f"{k} = {float(v)!r}\n" for k, v in vals.items()))
    out = tmp_path / "out.bin"
    args = [driver, str(pf), str(out)] + ([str(tmp_path / "bubble")] if vtk else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.float64)
    n = int(np.prod(G.shape))
    fields = {nm: raw[q * n:(q + 1) * n].reshape(G.shape) for q, nm in enumerate(["phi", "p", "u", "v"])}
    return fields, r.stdout, prm


def port_state(prm, steps, weno, second_order=False, ppe_mode=2):
    port = O.Checker("port").twophase(G, ["no_slip"] * 6, ["neumann"] * 6, prm,
                                      dict(scheme=int(weno), n_mpls=5, reinit_every=1, ppe_mode=ppe_mode,
                                           reinit_lambda=1))
    port.set_exact_tol(1e-14)
    port.set("phi", bubble_phi(G, CENTER, RADIUS))
    port.call("init")
    port.call("set_source_scheme", int(second_order))
    for _ in range(steps):
        port.call("step", 1)
    return port


@pytest.mark.gpu
@pytest.mark.parametrize("weno", [False, True], ids=["uccd", "weno5"])
def test_driver_matches_oracle(driver, tmp_path, weno):
    fields, log, prm = run_driver(driver, tmp_path, 2, weno)
    port = port_state(prm, 2, weno)
    I = G.interior()
    assert rel_l2(fields["phi"][I], port.get("phi")[I]) <= 1e-10, log
    for nm in ("p", "u", "v"):
        assert rel_l2(fields[nm][I], port.get(nm)[I]) <= 1e-9, (nm, log)
    t_line = [ln for ln in log.splitlines() if ln.startswith("t ")][-1].split()
    assert abs(float(t_line[1]) - port.scalars()["t"]) <= 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("compose", [False, True], ids=["ab_solve", "stages"])
def test_driver_stock_schedule_matches_oracle(driver, tmp_path, compose):
    """Seven steps through the drop-in with its default pressure schedule -- the reference's:
    projection() for iter < 5, then pressure_guess_solution, init_ppe_fpc_coefficients and
    fast_pressure_correction -- either inside projection_method::ab_solve or composed stage by
    stage by the driver (store, find_source, find_intermediate_velocity, ..., node_from_face),
    against the restatement of that schedule with both equations solved exactly (ppe_mode 3)."""
    fields, log, prm = run_driver(driver, tmp_path, 7, True, compose=compose)
    port = port_state(prm, 7, True, ppe_mode=3)
    I = G.interior()
    assert rel_l2(fields["phi"][I], port.get("phi")[I]) <= 1e-10, log
    for nm in ("p", "u", "v"):
        assert rel_l2(fields[nm][I], port.get(nm)[I]) <= 1e-9, (nm, log)


@pytest.mark.gpu
def test_driver_exact_schedule_matches_oracle(driver, tmp_path):
    """The projection equation every step (scihpc_cpp_set_pressure_schedule(0, 0)) over seven
    steps against ppe_mode 2."""
    fields, log, prm = run_driver(driver, tmp_path, 7, True, exact=True)
    port = port_state(prm, 7, True, ppe_mode=2)
    I = G.interior()
    assert rel_l2(fields["phi"][I], port.get("phi")[I]) <= 1e-10, log
    for nm in ("p", "u", "v"):
        assert rel_l2(fields[nm][I], port.get(nm)[I]) <= 1e-9, (nm, log)


@pytest.mark.gpu
def test_driver_second_order_matches_oracle(driver, tmp_path):
    """The same loop with projection_method::ab_solve_sec (second_order_solver derivatives in
    find_source_sec, as benchmarks_2d_dambreak.cpp calls it) through the drop-in."""
    fields, log, prm = run_driver(driver, tmp_path, 2, False, second_order=True)
    port = port_state(prm, 2, False, second_order=True)
    I = G.interior()
    assert rel_l2(fields["phi"][I], port.get("phi")[I]) <= 1e-10, log
    for nm in ("p", "u", "v"):
        assert rel_l2(fields[nm][I], port.get(nm)[I]) <= 1e-9, (nm, log)


@pytest.mark.gpu
def test_vtk_output(driver, tmp_path):
    """Legacy VTK written by vtkWriter: header as the reference writes it, big-endian doubles
    of the interior cells, x fastest."""
    fields, log, prm = run_driver(driver, tmp_path, 1, False, vtk=True)
    data = (tmp_path / "bubble0.vtk").read_bytes()
    head = data[:400].split(b"\n")
    assert head[0] == b"# vtk DataFile Version 3.0" and head[2] == b"BINARY"
    assert head[3] == b"DATASET STRUCTURED_POINTS"
    assert head[4] == f"DIMENSIONS {G.n[0] + 1} {G.n[1] + 1} 1".encode()
    assert head[7] == f"CELL_DATA {G.n[0] * G.n[1]}".encode()
    start = data.index(b"LOOKUP_TABLE default\n") + len(b"LOOKUP_TABLE default\n")
    phi = np.frombuffer(data[start:start + 8 * G.n[0] * G.n[1]], dtype=">f8").reshape(G.n[1], G.n[0]).T
    assert np.array_equal(phi, fields["phi"][3:-3, 3:-3, 0])
