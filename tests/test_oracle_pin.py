"""The CPU restatement (oracle/port) pinned to the reference itself (oracle/_ref, compiled
from the reference's own sources) on seeded inputs.  Bit-for-bit wherever the arithmetic
order is the same: every boundary fill, extrapolation, UCCD/CCD line solve, WENO5, Godunov
gradient, level-set field and integral, and whole two-phase time steps.  Skipped where the
reference sources are absent (the committed golden fixtures cover that case)."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_params, bubble_phi, grid2, grid3, smooth_field

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")


@pytest.fixture(scope="module")
def both():
    O.build(ref=True)
    return O.Checker("port"), O.Checker("ref")


GRIDS = [grid2(), grid2(9, 14, (-1.0, 0.5), (2.0, 3.0)), grid3(), grid3(6, 5, 7)]


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_fills_bitexact(both, gi):
    P, R = both
    g = GRIDS[gi]
    rng = np.random.default_rng(gi)
    for loc in range(g.ndim + 1):
        for t in range(5):
            vals = rng.standard_normal(6)
            f = rng.standard_normal(g.shape)
            assert np.array_equal(P.bc_fill(g, loc, [t] * 6, vals, f), R.bc_fill(g, loc, [t] * 6, vals, f))
        f = rng.standard_normal(g.shape)
        assert np.array_equal(P.flux_extrapolate(g, loc, f), R.flux_extrapolate(g, loc, f))
    assert np.array_equal(P.zero_order_extrapolation(g, f), R.zero_order_extrapolation(g, f))


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_stencils_bitexact(both, gi):
    P, R = both
    g = GRIDS[gi]
    rng = np.random.default_rng(50 + gi)
    flux = smooth_field(g, rng)
    vel = [rng.standard_normal(g.shape) for _ in range(3)]
    assert np.array_equal(P.uccd(g, flux, *vel)[:g.ndim], R.uccd(g, flux, *vel)[:g.ndim])
    assert np.array_equal(P.ccd(g, flux), R.ccd(g, flux))
    assert np.array_equal(P.weno5(g, flux, *vel), R.weno5(g, flux, *vel))
    phi = 0.2 * smooth_field(g, rng)
    sign = np.sign(rng.standard_normal(g.shape))
    assert np.array_equal(P.godunov(g, phi, sign), R.godunov(g, phi, sign))
    prm = [0.15, 0.001, 0.01, 0.0]
    assert np.array_equal(P.lsf_fields(g, prm, phi), R.lsf_fields(g, prm, phi))
    assert np.array_equal(P.lsf_integrals(g, prm, phi), R.lsf_integrals(g, prm, phi))


def test_multigrid_levels_and_history(both):
    P, R = both
    for nd, n in [(2, (256, 256)), (2, (128, 256)), (3, (128, 64, 64)), (2, (144, 144)), (3, (256, 256, 256))]:
        assert P.mg_levels(nd, n) == R.mg_levels(nd, n)
    g = O.Grid(2, (64, 64), (0.0, 0.0), (1.0, 1.0))
    xc = (np.arange(64) + 0.5) / 64
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    rhs = (-2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)).T.ravel()
    sa, ca, ha = P.mg_poisson(g, rhs, True, 1e-10, 60)
    sb, cb, hb = R.mg_poisson(g, rhs, True, 1e-10, 60)
    assert ca == cb
    # the coarsest-level direct solve differs (dense LU here, Eigen SparseLU there)
    assert np.allclose(ha, hb, rtol=1e-2, atol=0)
    assert np.abs(sa - sb).max() <= 1e-12 * np.abs(sb).max()


def test_two_phase_steps_bitexact(both):
    P, R = both
    g = O.Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
    prm = bubble_params(g, 1e-12)
    prm.update(ppe_tol=1e-30, ppe_tol2=0.0, ppe_max_iter=500)
    opt = dict(scheme=1, n_mpls=5, reinit_every=1, ppe_mode=1, reinit_lambda=1)
    s = [C.twophase(g, ["no_slip"] * 6, ["neumann"] * 6, prm, opt) for C in (P, R)]
    phi = bubble_phi(g, (0.43, 0.57), 0.23)
    for x in s:
        x.set("phi", phi)
        x.call("init")
    for k in range(2):
        for x in s:
            x.call("step", 1)
        for nm in ("phi", "p", "u", "v", "nu", "nv", "rho", "curvature"):
            assert np.array_equal(s[0].get(nm), s[1].get(nm)), (k, nm)
        assert s[0].scalars() == s[1].scalars()


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_second_order_solver_bitexact(both, gi):
    """second_order_solver (second_order_solver.cpp:7-241): central + mixed and upwind-biased."""
    P, R = both
    g = GRIDS[gi]
    rng = np.random.default_rng(40 + gi)
    f = smooth_field(g, rng) + 0.01 * rng.standard_normal(g.shape)
    u, v, w = (rng.standard_normal(g.shape) for _ in range(3))
    assert np.array_equal(P.sec(g, f), R.sec(g, f))
    assert np.array_equal(P.sec(g, f, u, v, w), R.sec(g, f, u, v, w))


def test_two_phase_steps_second_order_bitexact(both):
    """Time steps with ab_solve_sec (find_source_sec: second_order_solver for the level set's
    derivatives, convection_sec for the momentum, projection_method.cpp:314-382, 779-801)."""
    P, R = both
    g = O.Grid(2, (16, 32), (0.0, 0.0), (1.0, 2.0))
    prm = bubble_params(g, 1e-12)
    prm.update(ppe_tol=1e-30, ppe_tol2=0.0, ppe_max_iter=500)
    opt = dict(scheme=0, n_mpls=5, reinit_every=1, ppe_mode=1, reinit_lambda=1)
    s = [C.twophase(g, ["no_slip"] * 6, ["neumann"] * 6, prm, opt) for C in (P, R)]
    phi = bubble_phi(g, (0.43, 0.57), 0.23)
    for x in s:
        x.set("phi", phi)
        x.call("init")
        x.call("set_source_scheme", 1)
    I = g.interior()
    for k in range(2):
        for x in s:
            x.call("step", 1)
        for nm in ("phi", "p", "u", "v", "nu", "nv", "rho", "curvature"):
            # the upwind-biased derivatives never write the ghost points of their axis, so a
            # few ghost cells of the velocities hold the same non-finite values on both sides
            a, b = s[0].get(nm), s[1].get(nm)
            assert np.array_equal(a, b, equal_nan=True), (k, nm)
            assert np.isfinite(a[I]).all(), (k, nm)
        assert s[0].scalars() == s[1].scalars()
