"""CPU restatement of the learned pressure guess, for the tests only (test infrastructure,
like the rest of oracle/; nothing in the product imports it).

The reference has no learned component, so this is a restatement from the mathematics of the
network scihpc_gb300/csrc/unet.cu implements: 3x3 convolutions (stride 1, zero padding 1) on
[pixels][channels] arrays, their data and weight gradients, 2x2 average pooling, nearest
upsampling with skip concatenation, ReLU, and the mean-squared-error loss of the normalised
pressure correction.  Arithmetic is float64; values are rounded to BF16 (round to nearest
even, through float32) at the points where the GPU stores BF16 -- activations and the ReLU-
masked gradients that feed the tensor cores -- so the comparison measures the GPU's
accumulation order, not a different quantisation.
"""
from __future__ import annotations

import numpy as np

# (input tensor, output tensor, ci, co, relu, level) -- the table of unet.cu
TENSORS = ["X0", "E1A", "E1", "P1", "E2A", "E2", "P2", "E3A", "E3", "P3", "B1", "B2", "C3", "D3A", "D3", "C2",
           "D2A", "D2", "C1", "D1A", "D1", "OUT"]
LAYERS = [("X0", "E1A", 16, 16, 1, 0), ("E1A", "E1", 16, 16, 1, 0), ("P1", "E2A", 16, 32, 1, 1),
          ("E2A", "E2", 32, 32, 1, 1), ("P2", "E3A", 32, 64, 1, 2), ("E3A", "E3", 64, 64, 1, 2),
          ("P3", "B1", 64, 128, 1, 3), ("B1", "B2", 128, 128, 1, 3), ("C3", "D3A", 192, 64, 1, 2),
          ("D3A", "D3", 64, 64, 1, 2), ("C2", "D2A", 96, 32, 1, 1), ("D2A", "D2", 32, 32, 1, 1),
          ("C1", "D1A", 48, 16, 1, 0), ("D1A", "D1", 16, 16, 1, 0), ("D1", "OUT", 16, 16, 0, 0)]


def bf16(x):
    """Round to BF16 (nearest even) through float32, returned as float64."""
    f = np.asarray(x, dtype=np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def f32(x):
    """Round to float32, returned as float64 (where the GPU keeps FP32)."""
    return np.asarray(x, dtype=np.float64).astype(np.float32).astype(np.float64)


def param_layout():
    """Offsets of each layer's weights [co][9][ci] and biases [co] in the flat parameter array."""
    off, out = 0, []
    for (_, _, ci, co, _, _) in LAYERS:
        w = off
        off += co * 9 * ci
        out.append((w, off))
        off += co
    return out, off


def _shifted(x, h, w, dy, dx):
    """x [h*w][c] -> rows p of x[p + (dy, dx)] (zero outside the image)."""
    c = x.shape[1]
    img = np.zeros((h + 2, w + 2, c))
    img[1:-1, 1:-1] = x.reshape(h, w, c)
    return img[1 + dy:1 + dy + h, 1 + dx:1 + dx + w].reshape(h * w, c)


def im2col(x, h, w):
    return np.concatenate([_shifted(x, h, w, t // 3 - 1, t % 3 - 1) for t in range(9)], axis=1)


def conv(x, wt, b, h, w, relu):
    """y[p][co] = b[co] + sum_{t, ci} x[p + off(t)][ci] wt[co][t][ci]"""
    co = wt.shape[0]
    y = im2col(x, h, w) @ wt.reshape(co, -1).T
    if b is not None:
        y = y + b
    return np.maximum(y, 0.0) if relu else y


def conv_dgrad(dz, wt, h, w):
    """dx[q][ci] = sum_{t, co} dz[q - off(t)][co] wt[co][t][ci]"""
    co, _, ci = wt.shape
    dx = np.zeros((h * w, ci))
    for t in range(9):
        dy_, dx_ = t // 3 - 1, t % 3 - 1
        dx += _shifted(dz @ wt[:, t, :], h, w, -dy_, -dx_)
    return dx


def conv_wgrad(x, dz, h, w):
    """dw[co][t][ci] = sum_p x[p + off(t)][ci] dz[p][co]"""
    co = dz.shape[1]
    return (dz.T @ im2col(x, h, w)).reshape(co, 9, -1)


def pool(x, h, w):
    c = x.shape[1]
    a = x.reshape(h // 2, 2, w // 2, 2, c)
    return (0.25 * ((a[:, 0, :, 0] + a[:, 0, :, 1]) + a[:, 1, :, 0] + a[:, 1, :, 1])).reshape(-1, c)


def up(u, h, w):
    """nearest upsampling of u [(h/2)*(w/2)][c] to [h*w][c]"""
    c = u.shape[1]
    return np.repeat(np.repeat(u.reshape(h // 2, w // 2, c), 2, axis=0), 2, axis=1).reshape(-1, c)


def up_back(g, h, w):
    c = g.shape[1]
    a = g.reshape(h // 2, 2, w // 2, 2, c)
    return (a[:, 0, :, 0] + a[:, 0, :, 1] + a[:, 1, :, 0] + a[:, 1, :, 1]).reshape(-1, c)


def pack(rho, rhs, pprev, pnew=None):
    """Interior 2D fields [h][w] -> x0 [h*w][16] (BF16) and the normalised target."""
    n = rho.size
    mean = rho.mean()
    sd = np.sqrt(max((rho * rho).sum() / n - mean * mean, 0.0)) + 1e-12
    rr = np.sqrt((rhs * rhs).sum() / n) + 1e-300
    sp = np.sqrt((pprev * pprev).sum() / n)
    sp = sp if sp > 0 else 1.0
    x0 = np.zeros((n, 16))
    x0[:, 0] = ((rho - mean) / sd).ravel()
    x0[:, 1] = (rhs / rr).ravel()
    x0[:, 2] = (pprev / sp).ravel()
    target = None if pnew is None else f32(((pnew - pprev) / sp).ravel())
    return bf16(x0), target, sp


def pack_coarse(rho, rhs, pprev, d, fac, pnew=None):
    """The coarse-correction mode (scihpc_unet_create_coarse): interior 2D fields [n0][n1] and
    the spacing d -> x0 of the (n0/fac) x (n1/fac) network image, the normalised coarse target,
    and the output scale s_e.  Per coarse pixel: mean density, mean residual of pprev in the
    pressure equation (face coefficient 2 / (rho_c + rho_nb) / d^2 on interior faces), mean
    pprev; target = mean of (pnew - pprev) / s_e, s_e = 0.1 rms(r - mean r)."""
    n0, n1 = rho.shape
    lap = np.zeros_like(pprev)
    for a, dd in ((0, d[0]), (1, d[1])):
        w = 2.0 / (dd * dd)
        lo = [slice(None)] * 2
        hi = [slice(None)] * 2
        lo[a], hi[a] = slice(0, -1), slice(1, None)
        lo, hi = tuple(lo), tuple(hi)
        flux = w / (rho[lo] + rho[hi]) * (pprev[hi] - pprev[lo])   # face between lo and hi
        lap[lo] += flux
        lap[hi] -= flux
    r = rhs - lap
    hc, wc = n0 // fac, n1 // fac
    mean = lambda f: f.reshape(hc, fac, wc, fac).mean(axis=(1, 3))
    cin = [f32(mean(rho)), f32(mean(r)), f32(mean(pprev))]
    P = hc * wc
    mr = cin[0].sum() / P
    sd = np.sqrt(max((cin[0] * cin[0]).sum() / P - mr * mr, 0.0)) + 1e-12
    m1 = cin[1].sum() / P
    rr = np.sqrt(max((cin[1] * cin[1]).sum() / P - m1 * m1, 0.0)) + 1e-300
    sp = np.sqrt((cin[2] * cin[2]).sum() / P)
    sp = sp if sp > 0 else 1.0
    se = 0.1 * rr
    x0 = np.zeros((P, 16))
    x0[:, 0] = f32((cin[0] - mr) / sd).ravel()
    x0[:, 1] = f32((cin[1] - m1) / rr).ravel()
    x0[:, 2] = f32(cin[2] / sp).ravel()
    target = None if pnew is None else f32((mean(pnew - pprev) / se).ravel())
    return bf16(x0), target, se


def unpack_coarse(out0, pprev, se, fac):
    """guess = pprev + se * bilinear interpolation of the coarse output (pixel centres,
    clamped at the walls) on the interior cells."""
    n0, n1 = pprev.shape
    hc, wc = n0 // fac, n1 // fac
    o = np.asarray(out0, dtype=np.float64).reshape(hc, wc)

    def axis(n, nc):
        x = np.clip((np.arange(n) + 0.5) / fac - 0.5, 0.0, nc - 1)
        k0 = x.astype(int)
        k1 = np.minimum(k0 + 1, nc - 1)
        return k0, k1, x - k0

    i0, i1, wi = axis(n0, hc)
    j0, j1, wj = axis(n1, wc)
    W_ = wi[:, None]
    V_ = wj[None, :]
    v = (1 - W_) * ((1 - V_) * o[i0][:, j0] + V_ * o[i0][:, j1]) + W_ * ((1 - V_) * o[i1][:, j0] + V_ * o[i1][:, j1])
    return pprev + se * v


def forward(params, x0, h, w):
    """All activations (BF16-rounded where the GPU stores BF16; OUT is float32)."""
    lay, _ = param_layout()
    H = [h >> l for l in range(4)]
    W = [w >> l for l in range(4)]
    a = {"X0": x0}

    def run(k):
        i, o, ci, co, relu, lv = LAYERS[k]
        wo, bo = lay[k]
        wt = bf16(params[wo:wo + co * 9 * ci].reshape(co, 9, ci))
        b = params[bo:bo + co].astype(np.float64)
        y = conv(a[i], wt, b, H[lv], W[lv], relu)
        a[o] = f32(y) if o == "OUT" else bf16(y)

    run(0)
    run(1)
    a["P1"] = bf16(pool(a["E1"], H[0], W[0]))
    run(2)
    run(3)
    a["P2"] = bf16(pool(a["E2"], H[1], W[1]))
    run(4)
    run(5)
    a["P3"] = bf16(pool(a["E3"], H[2], W[2]))
    run(6)
    run(7)
    a["C3"] = np.concatenate([up(a["B2"], H[2], W[2]), a["E3"]], axis=1)
    run(8)
    run(9)
    a["C2"] = np.concatenate([up(a["D3"], H[1], W[1]), a["E2"]], axis=1)
    run(10)
    run(11)
    a["C1"] = np.concatenate([up(a["D2"], H[0], W[0]), a["E1"]], axis=1)
    run(12)
    run(13)
    run(14)
    return a


def loss_and_gradient(params, x0, target, h, w):
    """Mean-squared error of OUT[:, 0] against the target and its gradient with respect to
    the flat parameter array (layout of param_layout)."""
    lay, n = param_layout()
    H = [h >> l for l in range(4)]
    W = [w >> l for l in range(4)]
    a = forward(params, x0, h, w)
    P = h * w
    d = a["OUT"][:, 0] - target
    loss = float((d * d).sum() / P)
    g = {"OUT": np.zeros((P, 16))}
    g["OUT"][:, 0] = f32(2.0 * d / P)
    grad = np.zeros(n)
    gskip = {}

    def layer(k):
        i, o, ci, co, relu, lv = LAYERS[k]
        wo, bo = lay[k]
        wt = bf16(params[wo:wo + co * 9 * ci].reshape(co, 9, ci))
        dz = g[o] * (a[o] > 0) if relu else g[o]
        dz = bf16(dz)
        grad[wo:wo + co * 9 * ci] = conv_wgrad(a[i], dz, H[lv], W[lv]).ravel()
        grad[bo:bo + co] = dz.sum(axis=0)
        if k > 0:
            g[i] = conv_dgrad(dz, wt, H[lv], W[lv])

    def split(cat, u, s, lv):
        cu = a[u].shape[1]
        g[u] = up_back(g[cat][:, :cu], H[lv], W[lv])
        gskip[s] = g[cat][:, cu:]

    def poolback(p, e, lv):
        g[e] = gskip[e] + 0.25 * up(g[p], H[lv], W[lv])

    for k in (14, 13, 12):
        layer(k)
    split("C1", "D2", "E1", 0)
    for k in (11, 10):
        layer(k)
    split("C2", "D3", "E2", 1)
    for k in (9, 8):
        layer(k)
    split("C3", "B2", "E3", 2)
    for k in (7, 6):
        layer(k)
    poolback("P3", "E3", 2)
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
        sd = np.sqrt(2.0 / (9 * ci)) * (0.01 if k == len(LAYERS) - 1 else 1.0)
        wo, _ = lay[k]
        p[wo:wo + co * 9 * ci] = rng.normal(0.0, sd, co * 9 * ci)
    return p
