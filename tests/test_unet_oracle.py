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
