"""How far the second step of the 16 x 8 x 8 dam break can be reproduced at all: the CPU
restatement against itself, its velocities after the first step perturbed in the last bits
(relative 1e-15 of their maximum, two seeds).  The second step's pressure right-hand side
div(u*)/dt is a small difference of O(1) face velocities at density ratio 833, and the
step's pressure and velocity move by ~2e-9 and ~8e-9 -- the same for perturbations from
1e-15 to 1e-13, so no implementation that rounds differently can agree with the restatement
to the 1e-9 bound after that step.  The GPU parity test of that step
(test_gpu_dambreak3d.py) takes its 5e-8 bound from this spread."""
import numpy as np
import pytest

import oracle as O
from tests.helpers import rel_l2
from tests.test_gpu_dambreak3d import G, column_phi, dambreak_params


def second_step(eps, seed):
    prm = dambreak_params(G, ppe_tol=1e-13)
    port = O.Checker("port").twophase(G, ["slip"] * 6, ["neumann"] * 6, prm,
                                      dict(scheme=0, n_mpls=0, reinit_every=1, ppe_mode=2, reinit_lambda=1))
    port.set_exact_tol(1e-14)
    port.set("phi", column_phi(G))
    port.call("init")
    port.call("step", 1)
    rng = np.random.default_rng(seed)
    if eps:
        for nm in ("u", "v", "w"):
            a = port.get(nm)
            a[3:-3, 3:-3, 3:-3] += eps * np.abs(a).max() * rng.standard_normal(a[3:-3, 3:-3, 3:-3].shape)
            port.set(nm, a)
    port.call("step", 1)
    return {nm: port.get(nm) for nm in ("phi", "p", "u", "v", "w")}


def test_dambreak_second_step_spread_under_last_bit_perturbation():
    I = G.interior()
    base = second_step(0.0, 0)
    for seed in (0, 1):
        pert = second_step(1e-15, seed)
        vnorm = np.sqrt(sum(np.linalg.norm(base[nm][I]) ** 2 for nm in ("u", "v", "w")))
        e_p = rel_l2(pert["p"][I], base["p"][I])
        e_v = max(np.linalg.norm(pert[nm][I] - base[nm][I]) / vnorm for nm in ("u", "v", "w"))
        assert rel_l2(pert["phi"][I], base["phi"][I]) <= 1e-15
        # above the 1e-9 parity bound, within the 5e-8 the GPU test allows
        assert 1e-9 < e_p < 5e-8 and 1e-9 < e_v < 5e-8, (seed, e_p, e_v)
