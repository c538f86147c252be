"""The CPU restatement of the learned guess (oracle/unet_ref.py) pinned by finite
differences: with the BF16/FP32 roundings switched off, its analytic gradient of the loss
matches central differences for weights and biases of every layer."""
import numpy as np

from oracle import unet_ref as R


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(R, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    monkeypatch.setattr(R, "f32", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(0)
    h = w = 16
    x0 = rng.standard_normal((h * w, 16))
    x0[:, 3:] = 0.0
    t = rng.standard_normal(h * w)
    p = R.init_params(1).astype(np.float64)
    p[-16:] = 0.3
    _, grad, _ = R.loss_and_gradient(p, x0, t, h, w)
    lay, _ = R.param_layout()
    eps = 1e-5
    for k, (wo, bo) in enumerate(lay):
        for i in (wo + 3, bo):
            q = p.copy()
            q[i] += eps
            lp, _, _ = R.loss_and_gradient(q, x0, t, h, w)
            q[i] -= 2 * eps
            lm, _, _ = R.loss_and_gradient(q, x0, t, h, w)
            fd = (lp - lm) / (2 * eps)
            # ReLU kinks inside +-eps make a few entries differ by ~0.5 %
            assert abs(fd - grad[i]) <= 1e-2 * abs(fd) + 1e-9, (k, i, fd, grad[i])


def test_oracle3_gradient_matches_finite_differences(monkeypatch):
    """The same for the 3D restatement (oracle/unet3_ref.py) on an 8^3 network grid."""
    from oracle import unet3_ref as R3
    monkeypatch.setattr(R3, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    monkeypatch.setattr(R3, "f32", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(0)
    g = (8, 8, 8)
    P = 512
    x0 = rng.standard_normal((P, 16))
    x0[:, 3:] = 0.0
    t = rng.standard_normal(P)
    p = R3.init_params(1).astype(np.float64)
    p[-16:] = 0.3
    _, grad, _ = R3.loss_and_gradient(p, x0, t, g)
    lay, _ = R3.param_layout()
    eps = 1e-5
    for k, (wo, bo) in enumerate(lay):
        for i in (wo + 5, bo):
            q = p.copy()
            q[i] += eps
            lp, _, _ = R3.loss_and_gradient(q, x0, t, g)
            q[i] -= 2 * eps
            lm, _, _ = R3.loss_and_gradient(q, x0, t, g)
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - grad[i]) <= 1e-2 * abs(fd) + 1e-9, (k, i, fd, grad[i])


def test_oracle3_pack_unpack_are_consistent():
    """Half-resolution packing averages 2 x 2 x 2 cells; unpacking a zero correction gives the
    previous pressure and a unit correction adds s everywhere."""
    from oracle import unet3_ref as R3
    rng = np.random.default_rng(4)
    rho, rhs, pprev = (rng.standard_normal((8, 8, 16)) for _ in range(3))
    x0, target, sp, g = R3.pack(rho, rhs, pprev, pprev)
    assert g == (4, 4, 8) and x0.shape == (128, 16) and np.all(target == 0.0)
    assert np.array_equal(R3.unpack(np.zeros(128), pprev, sp), pprev)
    assert np.allclose(R3.unpack(np.ones(128), pprev, sp), pprev + sp)
