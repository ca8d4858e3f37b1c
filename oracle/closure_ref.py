"""TEST INFRASTRUCTURE, NOT PRODUCT CODE.

FP64 numpy restatement of the learned closure's network, conservation projection, loss
and gradients (lbm_closure.cu), used to check the GPU forward and backward kernels.
Optionally rounds the inputs, weights and activations to BF16 the way the GPU stores
them, so that the remaining difference is the FP32 accumulation order.
"""
import numpy as np

EX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.float64)
EY = np.array([0, 0, -1, 0, 1, -1, -1, 1, 1], dtype=np.float64)
W9 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + 9 * 9 * 32].reshape(9, 9, 32); o += 9 * 9 * 32
    b1 = p[o:o + 32]; o += 32
    W2 = p[o:o + 9 * 32 * 32].reshape(9, 32, 32); o += 9 * 32 * 32
    b2 = p[o:o + 32]; o += 32
    W3 = p[o:o + 9 * 32 * 9].reshape(9, 32, 9); o += 9 * 32 * 9
    b3 = p[o:o + 9]; o += 9
    return W1, b1, W2, b2, W3, b3


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def shift(x, dy, dx, periodic):
    """s[:, y, x] = x[:, y + dy, x + dx] (zero outside unless periodic)."""
    if periodic:
        return np.roll(np.roll(x, -dy, axis=1), -dx, axis=2)
    n, H, W, C = x.shape
    s = np.zeros_like(x)
    ys0, ys1 = max(0, -dy), min(H, H - dy)
    xs0, xs1 = max(0, -dx), min(W, W - dx)
    s[:, ys0:ys1, xs0:xs1] = x[:, ys0 + dy:ys1 + dy, xs0 + dx:xs1 + dx]
    return s


def conv(x, W, b, periodic):
    out = np.zeros(x.shape[:3] + (W.shape[2],))
    for t in range(9):
        out += shift(x, t // 3 - 1, t % 3 - 1, periodic) @ W[t]
    return out + b


def forward(x0, params, periodic=False, emulate_bf16=True):
    W1, b1, W2, b2, W3, b3 = unpack(params)
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    x0 = r(x0)
    x1 = r(np.maximum(conv(x0, r(W1), b1, periodic), 0.0))
    x2 = r(np.maximum(conv(x1, r(W2), b2, periodic), 0.0))
    y = conv(x2, r(W3), b3, periodic)
    return x0, x1, x2, y


def project(v):
    s = v.sum(-1, keepdims=True)
    sx = (v * EX).sum(-1, keepdims=True)
    sy = (v * EY).sum(-1, keepdims=True)
    return v - W9 * (s + 3.0 * (EX * sx + EY * sy))


def project_t(g):
    a = (W9 * g).sum(-1, keepdims=True)
    ax = (W9 * EX * g).sum(-1, keepdims=True)
    ay = (W9 * EY * g).sum(-1, keepdims=True)
    return g - a - 3.0 * (EX * ax + EY * ay)


def project_domain(y):
    """Field means of the output's density and momentum removed (y: (..., H, W, 9))."""
    m = y.sum(-1).mean(axis=(-2, -1))[..., None, None, None]
    jx = (y * EX).sum(-1).mean(axis=(-2, -1))[..., None, None, None]
    jy = (y * EY).sum(-1).mean(axis=(-2, -1))[..., None, None, None]
    return y - W9 * (m + 3.0 * (EX * jx + EY * jy))


def loss_and_grad(x0, T, params, emulate_bf16=True, project_cell=True):
    """Mean loss over the interior [3, S-3)^2 and the logical gradient vector; the loss
    compares P(y) (project_cell) or y with T."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    x0, x1, x2, y = forward(x0, params, False, emulate_bf16)
    n, H, W, _ = y.shape
    m = np.zeros((n, H, W, 1))
    m[:, 3:H - 3, 3:W - 3] = 1.0
    T = bf16(T) if emulate_bf16 else T
    e = ((project(y) if project_cell else y) - T) * m
    count = n * (H - 6) * (W - 6) * 9
    loss = float((e * e).sum() / count)
    gy = (project_t(2.0 * e / count) if project_cell else 2.0 * e / count) * m
    return loss, backward(x0, x1, x2, gy, params)


def backward(x0, x1, x2, gy, params):
    """Logical gradient vector from the output gradient gy (zero-padded convolutions)."""
    W1, b1, W2, b2, W3, b3 = unpack(params)

    def dweights(x, g):
        dW = np.stack([shift(x, t // 3 - 1, t % 3 - 1, False).reshape(-1, x.shape[-1]).T @ g.reshape(-1, g.shape[-1])
                       for t in range(9)])
        return dW, g.sum(axis=(0, 1, 2))

    def dinput(g, Wt):
        out = np.zeros(g.shape[:3] + (Wt.shape[1],))
        for t in range(9):
            out += shift(g @ Wt[t].T, -(t // 3 - 1), -(t % 3 - 1), False)
        return out

    dW3, db3 = dweights(x2, gy)
    g2 = dinput(gy, W3) * (x2 > 0)
    dW2, db2 = dweights(x1, g2)
    g1 = dinput(g2, W2) * (x1 > 0)
    dW1, db1 = dweights(x0, g1)
    return pack(dW1, db1, dW2, db2, dW3, db3)


def stress_loss_and_grad(x0, T, params, factor, emulate_bf16=True):
    """The stress target's loss (lbm_closure.cu k_stress_residual / k_stress_grad): over the
    interior [4, S-4)^2, r = -factor sum_i e_i P(y)_i(x - e_i) - sum_i e_i T_i(x); mean of
    |r|^2 over the interior's cells and both components, and the logical gradient vector."""
    x0, x1, x2, y = forward(x0, params, False, emulate_bf16)
    n, H, W, _ = y.shape
    T = bf16(T) if emulate_bf16 else T
    Py = project(y)
    mx = np.zeros((n, H, W))
    my = np.zeros((n, H, W))
    for i in range(1, 9):  # P(y)_i of the cell x - e_i: shift by -e_i
        s = shift(Py[..., i:i + 1], -int(EY[i]), -int(EX[i]), False)[..., 0]
        mx += EX[i] * s
        my += EY[i] * s
    mask = np.zeros((n, H, W))
    mask[:, 4:H - 4, 4:W - 4] = 1.0
    rx = (-factor * mx - (T * EX).sum(-1)) * mask
    ry = (-factor * my - (T * EY).sum(-1)) * mask
    count = n * (H - 8) * (W - 8) * 2
    loss = float(((rx * rx) + (ry * ry)).sum() / count)
    g = np.zeros_like(y)
    for i in range(1, 9):  # r at x + e_i: shift by +e_i
        sx = shift(rx[..., None], int(EY[i]), int(EX[i]), False)[..., 0]
        sy = shift(ry[..., None], int(EY[i]), int(EX[i]), False)[..., 0]
        g[..., i] = -factor * 2.0 / count * (EX[i] * sx + EY[i] * sy)
    return loss, backward(x0, x1, x2, project_t(g), params)
