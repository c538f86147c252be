"""Transport by runge_kutta::tvd_rk3 outside a two-phase session: the reference's 1D drivers
(benchmarks_1d_wave.cpp: identity_flux + convection; benchmarks_1d_IBE.cpp: burgers_flux +
Hamilton_Jacobi, the velocity copied from phi before every step) and the same pairs in 2D and
3D, through the GPU-backed C++ drop-in (tests/cpp/transport_driver.cpp), against the oracle's
restatement (port_transport_rk3), itself pinned bit for bit to the compiled reference."""
import math
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.helpers import rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "transport_driver.cpp")

# (ndim, n, lo, hi, bc code, flux kind, rhs kind, dt, steps, velocity from phi)
CASES = [
    (1, (32,), -1.0, 1.0, 0, 0, 0, 6e-4, 40, False),     # 1D wave, periodic
    (1, (40,), 0.0, 1.0, 0, 1, 1, 2.5e-4, 40, True),     # 1D inviscid Burgers, periodic
    (2, (16, 12), 0.0, 1.0, 0, 0, 0, 5e-4, 10, False),   # 2D convection, periodic
    (2, (12, 16), 0.0, 1.0, 1, 1, 1, 5e-4, 10, False),   # 2D Hamilton-Jacobi (Burgers flux), Neumann
    (3, (8, 10, 12), 0.0, 1.0, 0, 0, 1, 5e-4, 4, False),  # 3D Hamilton-Jacobi (identity flux), periodic
    (1, (32,), -1.0, 1.0, 0, 0, 2, 6e-4, 40, False),     # 1D convection_sec, periodic
    (2, (16, 12), 0.0, 1.0, 1, 0, 2, 5e-4, 10, False),   # 2D convection_sec, Neumann
]


def case_inputs(case, seed=0):
    ndim, n, lo, hi, bc = case[:5]
    g = O.Grid(ndim, n, (lo,) * ndim, (hi,) * ndim)
    rng = np.random.default_rng(seed)
    I = g.interior()
    phi = np.zeros(g.shape)
    xs = [lo + (np.arange(n[a]) + 0.5) * (hi - lo) / n[a] for a in range(ndim)]
    X = np.meshgrid(*xs, indexing="ij")
    smooth = np.sin(math.pi * X[0])
    for a in range(1, ndim):
        smooth = smooth * np.cos(math.pi * X[a])
    phi[I] = smooth.reshape(phi[I].shape) * 0.5 + 0.05 * rng.standard_normal(phi[I].shape)
    port = O.Checker("port")
    t, v = [bc] * 6, [0.0] * 6
    phi = port.bc_fill(g, 0, t, v, phi)
    vel = []
    for a in range(3):
        u = np.zeros(g.shape)
        if a < ndim:
            u[I] = 0.6 + 0.3 * rng.standard_normal(u[I].shape)
            u = port.bc_fill(g, 0, t, v, u)
        vel.append(u)
    return g, t, v, phi, vel


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    from scihpc_gb300 import build
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "transport_driver")
    r = subprocess.run(["g++", "-O2", "-Wall", DRIVER, "-o", exe] + build.cxx_flags(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_transport_driver_compiles_and_links(driver):
    assert os.path.exists(driver)


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("case", CASES)
def test_oracle_transport_matches_reference_bit_for_bit(case):
    """The restatement of tvd_rk3 with both flux / right-hand-side pairs is the reference's
    runge_kutta, convection, Hamilton_Jacobi and burgers_flux, bit for bit."""
    ndim, n, lo, hi, bc, fk, rk, dt, steps, vfp = case
    g, t, v, phi, vel = case_inputs(case)
    a = O.Checker("port").transport_rk3(g, t, v, fk, rk, dt, steps, phi, *vel, vel_from_phi=vfp)
    b = O.Checker("ref").transport_rk3(g, t, v, fk, rk, dt, steps, phi, *vel, vel_from_phi=vfp)
    assert np.array_equal(a, b), np.abs(a - b).max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_transport_matches_oracle(driver, tmp_path, case):
    ndim, n, lo, hi, bc, fk, rk, dt, steps, vfp = case
    g, t, v, phi, vel = case_inputs(case)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    np.concatenate([phi.ravel()] + [u.ravel() for u in vel]).tofile(inp)
    args = [driver, "field", str(ndim)] + [str(k) for k in n] + [repr(lo), repr(hi), str(bc), str(fk), str(rk),
                                                                 repr(dt), str(steps), str(int(vfp)), str(inp),
                                                                 str(out)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    gpu = np.fromfile(out, dtype=np.float64).reshape(g.shape)
    ref = O.Checker("port").transport_rk3(g, t, v, fk, rk, dt, steps, phi, *vel, vel_from_phi=vfp)
    I = g.interior()
    # the GPU's line solves are a scan formulation: round-off differs, the scheme does not
    assert rel_l2(gpu[I], ref[I]) <= 1e-12, rel_l2(gpu[I], ref[I])


def oracle_table(ibe, levels):
    """The reference drivers' final fields, errors and step counts for n = 16 .. 16 * 2^(levels-1)."""
    port = O.Checker("port")
    rows = []
    for cnt in range(levels):
        n = 16 << cnt
        lo, hi = (0.0, 1.0) if ibe else (-1.0, 1.0)
        g = O.Grid(1, (n,), (lo,), (hi,))
        h = (hi - lo) / n
        xc = lo + (np.arange(n) + 0.5) * h
        phi, u = np.zeros(g.shape), np.zeros(g.shape)
        if ibe:
            phi[3:-3, 0, 0] = np.sin(2 * math.pi * xc) / (2 * math.pi * 2.0)
        else:
            phi[3:-3, 0, 0] = np.sin(math.pi * xc)
            u[3:-3, 0, 0] = 1.0
        phi = port.bc_fill(g, 0, [0] * 6, [0.0] * 6, phi)
        if not ibe:
            u = port.bc_fill(g, 0, [0] * 6, [0.0] * 6, u)
        dt = 0.01 * h
        steps = 0
        while steps * dt < (1.5 if ibe else 2.0):
            steps += 1
        z = np.zeros(g.shape)
        out = port.transport_rk3(g, [0] * 6, [0.0] * 6, int(ibe), int(ibe), dt, steps, phi, u, z, z, ibe)
        rows.append((n, steps, out))
    return rows


@pytest.mark.gpu
@pytest.mark.parametrize("ibe", [False, True])
def test_gpu_reference_1d_driver_tables(driver, tmp_path, ibe):
    """benchmarks_1d_wave.cpp / benchmarks_1d_IBE.cpp through the drop-in at n = 16 .. 128: the
    same step counts, final fields equal to the oracle's, and the reference scheme's orders of
    convergence (5.0 for the wave; 2.7, 4.7, 5.9 for Burgers before the shock)."""
    levels = 4
    out = tmp_path / "tab.bin"
    r = subprocess.run([driver, "ibe" if ibe else "wave", str(levels), str(out)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [ln.split() for ln in r.stdout.splitlines()]
    raw = np.fromfile(out, dtype=np.float64)
    pos = 0
    for (n, steps, ref), row in zip(oracle_table(ibe, levels), rows):
        assert int(row[0]) == n and int(row[3]) == steps, (row, n, steps)
        gpu = raw[pos:pos + ref.size].reshape(ref.shape)
        pos += ref.size
        assert rel_l2(gpu[3:-3], ref[3:-3]) <= 1e-11, (n, rel_l2(gpu[3:-3], ref[3:-3]))
    orders = [float(row[2]) for row in rows[1:]]
    want = [2.69, 4.65, 5.85] if ibe else [5.03, 5.02, 5.01]
    assert all(abs(o - w) <= 0.02 for o, w in zip(orders, want)), orders
