"""Kernel-level parity of the CUDA library (through the C ABI) against the CPU restatement
of the reference (oracle/port), on seeded inputs.  Boundary fills and extrapolations are
integer index work and must match bit for bit; the FP64 stencils and line solves must
agree to round-off (tolerances below)."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_phi, grid2, grid3, smooth_field

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# FP64 round-off tolerance of derivative-type outputs, relative to the field's max |value|
# (different summation order and reciprocal multiplications; the reference uses divisions).
TOL = 1e-12
# The upwind CCD system amplifies round-off more (non-symmetric blocks): measured up to
# 1.2e-10 on 11-point lines with h = 0.2.
TOL_UCCD = 1e-9


@pytest.fixture(scope="module")
def port():
    return O.Checker("port")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def native_grid(g):
    from scihpc_gb300 import Grid
    return Grid(g.ndim, tuple(g.n), tuple(g.lo), tuple(g.hi))


def ws(g):
    from scihpc_gb300 import Workspace
    return Workspace(native_grid(g))


GRIDS = [grid2(), grid2(9, 14, (-1.0, 0.5), (2.0, 3.0)), grid3(), grid3(6, 5, 7)]
# line lengths for every register tier of the warp-cooperative solver (<= 128, 256, 512
# points) and one longer line for the sequential fallback; in 3D the shared-memory sequential
# solves run (one to 32 lines per block, blocks with fewer lines than the others)
LONG = [grid2(120, 9), grid2(7, 250), grid2(500, 5), grid2(5, 600), grid3(40, 6, 260), grid3(70, 33, 37)]


@pytest.mark.parametrize("gi", range(len(GRIDS)))
@pytest.mark.parametrize("bctype", range(5))
def test_bc_fill_bitexact(port, gi, bctype):
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(100 + 7 * gi + bctype)
    vals = list(rng.standard_normal(6))
    for loc in range(g.ndim + 1):
        f = rng.standard_normal(g.shape)
        ref = port.bc_fill(g, loc, [bctype] * 6, vals, f)
        d = dev(f)
        w.bc_fill(loc, [bctype] * 6, vals, d)
        out = host(d)
        assert np.array_equal(out, ref), (loc, np.abs(out - ref).max())


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_bc_fill_mixed_types_bitexact(port, gi):
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(300 + gi)
    for trial in range(6):
        types = []
        for a in range(3):
            if rng.random() < 0.2:
                types += [0, 0]
            else:
                types += list(rng.integers(1, 5, size=2))
        vals = list(rng.standard_normal(6))
        loc = int(rng.integers(0, g.ndim + 1))
        f = rng.standard_normal(g.shape)
        ref = port.bc_fill(g, loc, types, vals, f)
        d = dev(f)
        w.bc_fill(loc, types, vals, d)
        assert np.array_equal(host(d), ref), (types, loc)


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_extrapolations_bitexact(port, gi):
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(400 + gi)
    f = rng.standard_normal(g.shape)
    for loc in range(g.ndim + 1):
        ref = port.flux_extrapolate(g, loc, f)
        out = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        w.flux_extrapolate(loc, dev(f), out)
        assert np.array_equal(host(out), ref), loc
    ref = port.zero_order_extrapolation(g, f)
    d = dev(f)
    w.zero_order_extrapolation(d)
    assert np.array_equal(host(d), ref)


@pytest.mark.parametrize("gi", range(len(GRIDS) + len(LONG)))
def test_uccd(port, gi):
    g = (GRIDS + LONG)[gi]
    w = ws(g)
    rng = np.random.default_rng(500 + gi)
    flux = smooth_field(g, rng)
    vel = [rng.standard_normal(g.shape) for _ in range(3)]
    ref = port.uccd(g, flux, *vel)
    for a in range(g.ndim):
        f1 = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        f2 = torch.zeros_like(f1)
        w.uccd(a, dev(flux), dev(vel[a]), f1, f2)
        o1, o2 = host(f1), host(f2)
        assert np.abs(o1 - ref[a]).max() <= TOL_UCCD * np.abs(ref[a]).max(), a
        assert np.abs(o2 - ref[3 + a]).max() <= TOL_UCCD * np.abs(ref[3 + a]).max(), a


@pytest.mark.parametrize("gi", range(len(GRIDS) + len(LONG)))
def test_ccd_and_mixed(port, gi):
    g = (GRIDS + LONG)[gi]
    w = ws(g)
    rng = np.random.default_rng(600 + gi)
    flux = smooth_field(g, rng)
    ref = port.ccd(g, flux, mixed=True)
    d1 = [torch.zeros(g.shape, dtype=torch.float64, device="cuda") for _ in range(3)]
    d2 = [torch.zeros_like(d1[0]) for _ in range(3)]
    mx = [torch.zeros_like(d1[0]) for _ in range(3)]
    for a in range(g.ndim):
        w.ccd(a, dev(flux), d1[a], d2[a])
    # mixed derivatives extrapolate their source in place, as the reference does
    w.ccd_mixed(1, d1[0], mx[0])
    if g.ndim > 2:
        w.ccd_mixed(2, d1[1], mx[1])
        w.ccd_mixed(0, d1[2], mx[2])
    outs = [host(t) for t in d1 + d2 + mx]
    for q in list(range(g.ndim)) + [3 + a for a in range(g.ndim)] + ([6] if g.ndim == 2 else [6, 7, 8]):
        assert np.abs(outs[q] - ref[q]).max() <= TOL * max(np.abs(ref[q]).max(), 1e-300), q


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_weno5(port, gi):
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(700 + gi)
    flux = smooth_field(g, rng) + 0.3 * np.sign(smooth_field(g, rng))   # with jumps
    vel = [rng.standard_normal(g.shape) for _ in range(3)]
    ref = port.weno5(g, flux, *vel)
    I = g.interior()
    for a in range(g.ndim):
        out = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        w.weno5(a, dev(flux), dev(vel[a]), out)
        o = host(out)
        assert np.abs(o[I] - ref[a][I]).max() <= TOL * np.abs(ref[a][I]).max(), a


@pytest.mark.parametrize("g", [LONG[0], LONG[1], LONG[4], LONG[5]], ids=lambda g: "x".join(map(str, g.n)))
def test_weno5_long(port, g):
    """Grids with several warp segments along the contiguous axis and several tiles (and
    partial ones) along the others: every face is computed once and shared by its two cells."""
    w = ws(g)
    rng = np.random.default_rng(750)
    flux = smooth_field(g, rng) + 0.3 * np.sign(smooth_field(g, rng))
    vel = [rng.standard_normal(g.shape) for _ in range(3)]
    ref = port.weno5(g, flux, *vel)
    I = g.interior()
    for a in range(g.ndim):
        out = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
        w.weno5(a, dev(flux), dev(vel[a]), out)
        o = host(out)
        assert np.abs(o[I] - ref[a][I]).max() <= TOL * np.abs(ref[a][I]).max(), a
        ghosts = np.ones(o.shape, dtype=bool)
        ghosts[I] = False
        assert not np.any(o[ghosts]), a   # only interior cells are written


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_godunov(port, gi):
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(800 + gi)
    phi = 0.2 * smooth_field(g, rng)
    sign = np.sign(rng.standard_normal(g.shape))
    ref = port.godunov(g, phi, sign)
    out = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    w.godunov_gradient(dev(phi), dev(sign), out)
    assert np.abs(host(out) - ref).max() <= TOL * np.abs(ref).max()


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_stabilized_upon_gradient(port, gi):
    """stabilized_upon_gradient (godunov_gradient.cpp:159-181): the Godunov gradient, its
    device-side maximum over every cell and the division of phi by it."""
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(820 + gi)
    phi = 0.2 * smooth_field(g, rng)
    sign = np.sign(rng.standard_normal(g.shape))
    ref_phi, ref_grad = port.stabilize(g, phi, sign)
    d_phi = dev(phi)
    grad = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    w.stabilized_upon_gradient(d_phi, dev(sign), grad)
    assert np.abs(host(grad) - ref_grad).max() <= TOL * np.abs(ref_grad).max()
    assert np.abs(host(d_phi) - ref_phi).max() <= TOL * np.abs(ref_phi).max()


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_guess_from_history_bitexact(port, gi):
    """guess_from_history (flux.cpp:653-662): 2 old - old2 on every cell, bit for bit."""
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(840 + gi)
    old, old2 = rng.standard_normal(g.shape), rng.standard_normal(g.shape)
    out = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    w.guess_from_history(dev(old), dev(old2), out)
    assert np.array_equal(host(out), port.guess_from_history(g, old, old2))


@pytest.mark.parametrize("ndim", [2, 3])
def test_lsf_fields_and_integrals(port, ndim):
    if ndim == 2:
        g = grid2(24, 40)
        phi = bubble_phi(O.Grid(2, g.n, g.lo, g.hi), (0.5, 0.9), 0.3)
        from oracle import Checker
        phi = port.bc_fill(g, 0, [1] * 6, [0.0] * 6, phi)
    else:
        g = grid3(12, 14, 10)
        rng = np.random.default_rng(11)
        phi = 0.1 * smooth_field(g, rng)
    h = min(g.spacing())
    prm = [1.5 * h, 0.001, 0.01, 0.0]
    ref = port.lsf_fields(g, prm, phi)
    w = ws(g)
    outs = [torch.zeros(g.shape, dtype=torch.float64, device="cuda") for _ in range(5)]
    w.lsf_fields(prm, dev(phi), *outs)
    for q in range(5):
        o = host(outs[q])
        assert np.abs(o - ref[q]).max() <= 1e-14 * max(1.0, np.abs(ref[q]).max()), q
    mass, vol = w.lsf_integrals(prm, dev(phi))
    rmass, rvol = port.lsf_integrals(g, prm, phi)
    assert abs(mass - rmass) <= 1e-13 * abs(rmass)
    assert abs(vol - rvol) <= 1e-13 * abs(rvol)


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_second_order_solver(port, gi):
    """second_order_solver's stencils (second_order_solver.cpp:7-241): the same arithmetic in
    the same order, so bit for bit -- central with the mixed derivatives, and upwind-biased
    (which leaves the ghost points of its axis as they were)."""
    g = GRIDS[gi]
    w = ws(g)
    rng = np.random.default_rng(700 + gi)
    flux = smooth_field(g, rng) + 0.01 * rng.standard_normal(g.shape)
    vel = [rng.standard_normal(g.shape) for _ in range(3)]
    central, upwind = port.sec(g, flux), port.sec(g, flux, *vel)
    z = lambda: torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    d1 = []
    for a in range(g.ndim):
        f1, f2 = z(), z()
        w.sec_derivative(a, dev(flux), None, f1, f2)
        assert np.array_equal(host(f1), central[a]) and np.array_equal(host(f2), central[3 + a]), a
        d1.append(f1)
        u1, u2 = z(), z()
        w.sec_derivative(a, dev(flux), dev(vel[a]), u1, u2)
        assert np.array_equal(host(u1), upwind[a]) and np.array_equal(host(u2), upwind[3 + a]), a
    pairs = [(1, 0, 6)] + ([(2, 1, 7), (0, 2, 8)] if g.ndim > 2 else [])
    for b, src, k in pairs:
        out = z()
        w.sec_mixed(b, d1[src], out)
        assert np.array_equal(host(out), central[k]), (b, k)
