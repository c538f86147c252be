"""CPU restatement of the 3D learned pressure guess, for the tests only (test infrastructure,
like the rest of oracle/; nothing in the product imports it).

The reference has no learned component, so this is a restatement from the mathematics of the
network scihpc_gb300/csrc/unet3.cu implements: 3x3x3 convolutions (stride 1, zero padding 1)
on [voxels][channels] arrays, their data and weight gradients, 2x2x2 average pooling, nearest
upsampling with skip concatenation, ReLU, the mean-squared-error loss of the normalised
pressure correction, and the half-resolution packing of the inputs.  Arithmetic is float64;
values are rounded to BF16 where the GPU stores BF16 (unet_ref.bf16), so the comparison
measures the GPU's accumulation order, not a different quantisation.
"""
from __future__ import annotations

import numpy as np

from .unet_ref import bf16, f32

# (input tensor, output tensor, ci, co, relu, level) -- the table of unet3.cu
LAYERS = [("X0", "E1A", 16, 16, 1, 0), ("E1A", "E1", 16, 16, 1, 0), ("P1", "E2A", 16, 32, 1, 1),
          ("E2A", "E2", 32, 32, 1, 1), ("P2", "B1", 32, 64, 1, 2), ("B1", "B2", 64, 64, 1, 2),
          ("C2", "D2A", 96, 32, 1, 1), ("D2A", "D2", 32, 32, 1, 1), ("C1", "D1A", 48, 16, 1, 0),
          ("D1A", "D1", 16, 16, 1, 0), ("D1", "OUT", 16, 16, 0, 0)]
TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]   # t = 9(dz+1)+3(dy+1)+(dx+1)


def param_layout():
    """Offsets of each layer's weights [co][27][ci] and biases [co] in the flat parameter array."""
    off, out = 0, []
    for (_, _, ci, co, _, _) in LAYERS:
        w = off
        off += co * 27 * ci
        out.append((w, off))
        off += co
    return out, off


def _shifted(x, g, dz, dy, dx):
    """x [d*h*w][c] -> rows p of x[p + (dz, dy, dx)] (zero outside the grid)."""
    d, h, w = g
    c = x.shape[1]
    v = np.zeros((d + 2, h + 2, w + 2, c))
    v[1:-1, 1:-1, 1:-1] = x.reshape(d, h, w, c)
    return v[1 + dz:1 + dz + d, 1 + dy:1 + dy + h, 1 + dx:1 + dx + w].reshape(d * h * w, c)


def im2col(x, g):
    return np.concatenate([_shifted(x, g, *s) for s in TAPS], axis=1)


def conv(x, wt, b, g, relu):
    """y[p][co] = b[co] + sum_{t, ci} x[p + off(t)][ci] wt[co][t][ci]"""
    co = wt.shape[0]
    y = im2col(x, g) @ wt.reshape(co, -1).T
    if b is not None:
        y = y + b
    return np.maximum(y, 0.0) if relu else y


def conv_dgrad(dz, wt, g):
    """dx[q][ci] = sum_{t, co} dz[q - off(t)][co] wt[co][t][ci]"""
    co, _, ci = wt.shape
    out = np.zeros((int(np.prod(g)), ci))
    for t, (a, b, c) in enumerate(TAPS):
        out += _shifted(dz @ wt[:, t, :], g, -a, -b, -c)
    return out


def conv_wgrad(x, dz, g):
    """dw[co][t][ci] = sum_p x[p + off(t)][ci] dz[p][co]"""
    co = dz.shape[1]
    return (dz.T @ im2col(x, g)).reshape(co, 27, -1)


def _blocks(x, g):
    d, h, w = g
    return x.reshape(d // 2, 2, h // 2, 2, w // 2, 2, x.shape[1])


def pool(x, g):
    a = _blocks(x, g)
    return (0.125 * a.sum(axis=(1, 3, 5))).reshape(-1, x.shape[1])


def up(u, g):
    """nearest upsampling of u (grid g / 2) to grid g"""
    d, h, w = g
    c = u.shape[1]
    v = u.reshape(d // 2, h // 2, w // 2, c)
    return v.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2).reshape(-1, c)


def up_back(gy, g):
    return _blocks(gy, g).sum(axis=(1, 3, 5)).reshape(-1, gy.shape[1])


def pack(rho, rhs, pprev, pnew=None):
    """Interior 3D fields [n0][n1][n2] -> x0 [voxels][16] (BF16) at half resolution, the
    normalised target and the pressure scale s."""
    n = rho.size
    mean = rho.mean()
    sd = np.sqrt(max((rho * rho).sum() / n - mean * mean, 0.0)) + 1e-12
    rr = np.sqrt((rhs * rhs).sum() / n) + 1e-300
    sp = np.sqrt((pprev * pprev).sum() / n)
    sp = sp if sp > 0 else 1.0
    g = tuple(s // 2 for s in rho.shape)

    def avg(f):
        return _blocks(f.reshape(-1, 1), rho.shape).mean(axis=(1, 3, 5)).ravel()

    x0 = np.zeros((int(np.prod(g)), 16))
    x0[:, 0] = (avg(rho) - mean) / sd
    x0[:, 1] = avg(rhs) / rr
    x0[:, 2] = avg(pprev) / sp
    target = None if pnew is None else f32(avg(pnew - pprev) / sp)
    return bf16(x0), target, sp, g


def unpack(out0, pprev, sp):
    """guess = pprev + s * (out channel 0 prolonged piecewise-constant), interior cells"""
    g = tuple(s // 2 for s in pprev.shape)
    o = out0.reshape(g).repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)
    return pprev + sp * o


def forward(params, x0, g0):
    """All activations (BF16-rounded where the GPU stores BF16; OUT is float32)."""
    lay, _ = param_layout()
    G = [tuple(s >> l for s in g0) for l in range(3)]
    a = {"X0": x0}

    def run(k):
        i, o, ci, co, relu, lv = LAYERS[k]
        wo, bo = lay[k]
        wt = bf16(params[wo:wo + co * 27 * ci].reshape(co, 27, ci))
        b = params[bo:bo + co].astype(np.float64)
        y = conv(a[i], wt, b, G[lv], relu)
        a[o] = f32(y) if o == "OUT" else bf16(y)

    run(0)
    run(1)
    a["P1"] = bf16(pool(a["E1"], G[0]))
    run(2)
    run(3)
    a["P2"] = bf16(pool(a["E2"], G[1]))
    run(4)
    run(5)
    a["C2"] = np.concatenate([up(a["B2"], G[1]), a["E2"]], axis=1)
    run(6)
    run(7)
    a["C1"] = np.concatenate([up(a["D2"], G[0]), a["E1"]], axis=1)
    run(8)
    run(9)
    run(10)
    return a


def loss_and_gradient(params, x0, target, g0):
    """Mean-squared error of OUT[:, 0] against the target and its gradient with respect to
    the flat parameter array (layout of param_layout)."""
    lay, n = param_layout()
    G = [tuple(s >> l for s in g0) for l in range(3)]
    a = forward(params, x0, g0)
    P = int(np.prod(g0))
    d = a["OUT"][:, 0] - target
    loss = float((d * d).sum() / P)
    g = {"OUT": np.zeros((P, 16))}
    g["OUT"][:, 0] = f32(2.0 * d / P)
    grad = np.zeros(n)
    gskip = {}

    def layer(k):
        i, o, ci, co, relu, lv = LAYERS[k]
        wo, bo = lay[k]
        wt = bf16(params[wo:wo + co * 27 * ci].reshape(co, 27, ci))
        dz = bf16(g[o] * (a[o] > 0) if relu else g[o])
        grad[wo:wo + co * 27 * ci] = conv_wgrad(a[i], dz, G[lv]).ravel()
        grad[bo:bo + co] = dz.sum(axis=0)
        if k > 0:
            g[i] = conv_dgrad(dz, wt, G[lv])

    def split(cat, u, s, lv):
        cu = a[u].shape[1]
        g[u] = up_back(g[cat][:, :cu], G[lv])
        gskip[s] = g[cat][:, cu:]

    def poolback(p, e, lv):
        g[e] = gskip[e] + 0.125 * up(g[p], G[lv])

    for k in (10, 9, 8):
        layer(k)
    split("C1", "D2", "E1", 0)
    for k in (7, 6):
        layer(k)
    split("C2", "B2", "E2", 1)
    for k in (5, 4):
        layer(k)
    poolback("P2", "E2", 1)
    for k in (3, 2):
        layer(k)
    poolback("P1", "E1", 0)
    for k in (1, 0):
        layer(k)
    return loss, grad, a


def init_params(seed):
    """He-normal weights (the last layer scaled by 0.01), zero biases."""
    lay, n = param_layout()
    rng = np.random.default_rng(seed)
    p = np.zeros(n, dtype=np.float32)
    for k, (_, _, ci, co, _, _) in enumerate(LAYERS):
        sd = np.sqrt(2.0 / (27 * ci)) * (0.01 if k == len(LAYERS) - 1 else 1.0)
        wo, _ = lay[k]
        p[wo:wo + co * 27 * ci] = rng.normal(0.0, sd, co * 27 * ci)
    return p
