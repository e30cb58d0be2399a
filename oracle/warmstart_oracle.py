"""CPU oracle of the learned warm start network (test infrastructure only; nothing in the product imports it).

The network has no counterpart in the reference (it is an addition beside the plain IBR_gradient solver), so
this oracle is pinned by itself: in FP64 mode (bf16=False) its analytic gradients are checked against central
finite differences of its own loss (tests/test_warmstart.py). In BF16 mode it rounds to bfloat16 at the points
where the GPU stores BF16 (weights, activations, skip sums, output-layer gradients, data gradients) and
accumulates in FP64, so the GPU (FP32 accumulation in tensor memory) must agree with it to within BF16
rounding of a few intermediate values.

Layouts (as the C ABI): input x[b][y][x][48]; u0, target, prediction [b][3][y][x]; parameters flat FP32, per
layer W[cout][ky][kx][cin] then bias[cout], layers in NET order.
"""
from __future__ import annotations

import numpy as np

# (cin, cout, ks, stride, relu), the order of the flat parameter vector
NET = [
    (48, 32, 3, 1, 1), (32, 64, 3, 2, 1), (64, 128, 3, 2, 1), (128, 256, 3, 2, 1),
    (256, 256, 3, 1, 1), (256, 128, 1, 1, 0), (128, 128, 3, 1, 1), (128, 64, 1, 1, 0),
    (64, 64, 3, 1, 1), (64, 32, 1, 1, 0), (32, 32, 3, 1, 1), (32, 3, 3, 1, 0),
]
CHANNELS = 48


def param_count() -> int:
    return sum(co * (k * k * ci + 1) for ci, co, k, _, _ in NET)


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(a: np.ndarray) -> np.ndarray:
    """bfloat16 bit patterns (uint16) of the rounded values, for building device inputs."""
    f = np.ascontiguousarray(bf16(a), dtype=np.float32)
    return (f.view(np.uint32) >> 16).astype(np.uint16)


def split_params(theta: np.ndarray) -> list[tuple[np.ndarray, np.ndarray]]:
    out, off = [], 0
    for ci, co, k, _, _ in NET:
        n = co * k * k * ci
        out.append((theta[off:off + n].reshape(co, k * k, ci).astype(np.float64),
                    theta[off + n:off + n + co].astype(np.float64)))
        off += n + co
    return out


def _im2col(x: np.ndarray, k: int, s: int) -> np.ndarray:
    """x [B,H,W,C] -> [B, H/s, W/s, k*k, C] with zero padding (k - 1) / 2."""
    B, H, W, C = x.shape
    Ho, Wo = H // s, W // s
    if k == 1:
        return x[:, ::s, ::s, None, :]
    xp = np.zeros((B, H + 2, W + 2, C), x.dtype)
    xp[:, 1:H + 1, 1:W + 1] = x
    cols = np.empty((B, Ho, Wo, 9, C), x.dtype)
    for ky in range(3):
        for kx in range(3):
            cols[:, :, :, ky * 3 + kx] = xp[:, ky:ky + s * Ho:s, kx:kx + s * Wo:s]
    return cols


def _col2im(dcols: np.ndarray, shape: tuple, k: int, s: int) -> np.ndarray:
    """Adjoint of _im2col: dcols [B, Ho, Wo, k*k, C] -> dx [B, H, W, C]."""
    B, H, W, C = shape
    Ho, Wo = H // s, W // s
    if k == 1:
        dx = np.zeros(shape, dcols.dtype)
        dx[:, ::s, ::s] = dcols[:, :, :, 0]
        return dx
    dxp = np.zeros((B, H + 2, W + 2, C), dcols.dtype)
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + s * Ho:s, kx:kx + s * Wo:s] += dcols[:, :, :, ky * 3 + kx]
    return dxp[:, 1:H + 1, 1:W + 1]


def conv(x, w, b, k, s):
    cols = _im2col(x, k, s)
    B, Ho, Wo = cols.shape[:3]
    y = cols.reshape(B * Ho * Wo, -1) @ w.reshape(w.shape[0], -1).T
    if b is not None:
        y = y + b
    return y.reshape(B, Ho, Wo, -1)


def conv_dgrad(dy, w, xshape, k, s):
    B, Ho, Wo, Co = dy.shape
    dcols = dy.reshape(-1, Co) @ w.reshape(Co, -1)
    return _col2im(dcols.reshape(B, Ho, Wo, k * k, -1), xshape, k, s)


def conv_wgrad(x, dy, k, s):
    cols = _im2col(x, k, s)
    Co = dy.shape[-1]
    return (dy.reshape(-1, Co).T @ cols.reshape(dy.shape[0] * dy.shape[1] * dy.shape[2], -1)).reshape(Co, k * k, -1)


def up2(t):
    return t.repeat(2, axis=1).repeat(2, axis=2)


def down_sum(d):
    B, H, W, C = d.shape
    return d.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward_backward(theta: np.ndarray, x: np.ndarray, u0: np.ndarray, target: np.ndarray | None,
                     bf16_mode: bool = True):
    """Prediction, loss and the flat gradient (None without a target). x [B,H,W,48], u0/target [B,3,H,W]."""
    q = bf16 if bf16_mode else (lambda a: np.asarray(a, np.float64))
    P = split_params(theta)
    W = [(q(w), b) for w, b in P]
    x = q(x)
    relu = lambda a: np.maximum(a, 0.0)

    def f(l, inp):
        ci, co, k, s, r = NET[l]
        y = conv(inp, W[l][0], W[l][1], k, s)
        return relu(y) if r else y

    a0 = q(f(0, x)); a1 = q(f(1, a0)); a2 = q(f(2, a1)); a3 = q(f(3, a2)); a4 = q(f(4, a3))
    # the 1 x 1 decoder layers keep t in FP32: the device adds it to the skip in the same epilogue
    t5 = f(5, a4); s5 = q(relu(up2(t5) + a2))
    a6 = q(f(6, s5)); t7 = f(7, a6); s7 = q(relu(up2(t7) + a1))
    a8 = q(f(8, s7)); t9 = f(9, a8); s9 = q(relu(up2(t9) + a0))
    a10 = q(f(10, s9))
    y = f(11, a10)                                          # FP32 on the device
    pred = u0 + y.transpose(0, 3, 1, 2)
    if target is None:
        return pred, None, None
    d = pred - target
    n = d.size
    loss = float(np.mean(d * d))
    dy11 = q(2.0 * d.transpose(0, 2, 3, 1) / n)

    grads = [None] * len(NET)
    mask = lambda g, a: np.where(a > 0, g, 0.0)

    def back(l, inp, dy, add=None, m=None, need_dx=True):
        ci, co, k, s, _ = NET[l]
        grads[l] = (conv_wgrad(inp, dy, k, s), dy.sum(axis=(0, 1, 2)))
        if not need_dx:
            return None
        dx = conv_dgrad(dy, W[l][0], inp.shape, k, s)
        if add is not None:
            dx = dx + add
        if m is not None:
            dx = mask(dx, m)
        return q(dx)

    g10 = back(11, a10, dy11, m=a10)
    gs9 = back(10, s9, g10, m=s9)
    dt9 = q(down_sum(gs9))
    g8 = back(9, a8, dt9, m=a8)
    gs7 = back(8, s7, g8, m=s7)
    dt7 = q(down_sum(gs7))
    g6 = back(7, a6, dt7, m=a6)
    gs5 = back(6, s5, g6, m=s5)
    dt5 = q(down_sum(gs5))
    g4 = back(5, a4, dt5, m=a4)
    g3 = back(4, a3, g4, m=a3)
    g2 = back(3, a2, g3, add=gs5, m=a2)
    g1 = back(2, a1, g2, add=gs7, m=a1)
    g0 = back(1, a0, g1, add=gs9, m=a0)
    back(0, x, g0, need_dx=False)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
    return pred, loss, flat


def layer_slices() -> list[tuple[slice, slice]]:
    """(weights, bias) slices of each layer in the flat parameter vector."""
    out, off = [], 0
    for ci, co, k, _, _ in NET:
        n = co * k * k * ci
        out.append((slice(off, off + n), slice(off + n, off + n + co)))
        off += n + co
    return out


def init_params(seed: int) -> np.ndarray:
    """Seeded random parameters (numpy generator; not the device's initialiser) for the oracle checks."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (ci, co, k, _, r) in enumerate(NET):
        sd = np.sqrt((2.0 if r else 1.0) / (k * k * ci))
        parts.append(rng.normal(0.0, sd, co * k * k * ci))
        parts.append(rng.normal(0.0, 0.05, co))
    return np.concatenate(parts).astype(np.float32)
