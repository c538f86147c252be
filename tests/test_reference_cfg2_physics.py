"""Why the rising-bubble benchmark uses Hysing's TC1 fluid instead of the stated one.  The
reference implementation itself (oracle/_ref, compiled from its own sources), run with its
own stock schedule and solver settings (WENO5 transport, five mpls steps, reinitialisation
every step, SOR for five steps then the fast pressure correction, ppe_tol 1e-8, CFL 0.2)
on the benchmark's 128 x 256 grid (bubble r = 0.25 at (0.5, 0.5) in [0,1] x [0,2]):

* with the stated fluid (density 1000 / 1, viscosity 10 / 0.1, surface tension 1.96,
  gravity 0.98) the velocity grows about 2.5x per step from step 6 and passes 10 by step
  20, and the enclosed volume, which the scheme conserves to 1e-5 otherwise, moves by more
  than 10 %: the scheme is unstable for this density ratio at this resolution;
* with TC1 (1000 / 100, 10 / 1, 24.5, 0.98), same grid and settings, the velocity stays
  bounded and the volume holds to 1e-4.

(The restatement with exact pressure solves shows the same: the stated fluid reaches
|u| ~ 35 at step 20 and non-finite values a few steps later.)"""
import numpy as np
import pytest

import oracle as O
from tests.helpers import bubble_params

pytestmark = [pytest.mark.slow, pytest.mark.skipif(not O.ref_available(), reason="reference sources not present")]

G = O.Grid(2, (128, 256), (0.0, 0.0), (1.0, 2.0))


def tc1_params(h):
    Uc = np.sqrt(0.98)
    return dict(density_ratio=0.1, viscosity_ratio=0.1, Re=1000.0 * Uc / 10.0, Fr=Uc / np.sqrt(0.98),
                We=1000.0 * Uc * Uc / 24.5, ls_width=1.5 * h, rdt=0.25 * h, positive_ref=0.0)


def run_reference(prm, steps):
    prm = dict(prm)
    prm.update(ppe_tol=1e-8, ppe_tol2=1e-7, ppe_max_iter=100, ppe_initer=1, ppe_omega=1.5, max_CFL=0.2,
               min_CFL=1e-4, dt0=1.0)
    s = O.Checker("ref").twophase(G, ["no_slip"] * 6, ["neumann"] * 6, prm,
                                  dict(scheme=1, n_mpls=5, reinit_every=1, ppe_mode=0, reinit_lambda=1))
    h = 1.0 / 128
    xc = (np.arange(128) + 0.5) * h
    yc = (np.arange(256) + 0.5) * h
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    phi = np.zeros(G.shape)
    phi[3:-3, 3:-3, 0] = 0.25 - np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
    s.set("phi", phi)
    s.call("init")
    vol0 = s.diagnostics()["volume"]
    I = G.interior()
    umax = []
    for _ in range(steps):
        s.call("step", 1)
        umax.append(max(np.abs(s.get("u")[I]).max(), np.abs(s.get("v")[I]).max()))
    return np.array(umax), s.diagnostics()["volume"] / vol0 - 1.0


def test_stated_fluid_is_unstable_in_the_reference_scheme():
    umax, dvol = run_reference(bubble_params(G), 20)
    assert not np.isfinite(umax[-1]) or umax[-1] > 10.0, umax
    assert umax[14] > 50.0 * umax[6], umax            # exponential growth from step 7 on
    assert not np.isfinite(dvol) or abs(dvol) > 0.1, dvol


def test_tc1_fluid_stays_bounded_in_the_reference_scheme():
    umax, dvol = run_reference(tc1_params(1.0 / 128), 20)
    assert np.isfinite(umax).all() and umax.max() < 10.0, umax
    assert abs(dvol) < 1e-4, dvol
