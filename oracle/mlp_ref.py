"""Test infrastructure only: numpy restatement of the learned warm start's
network (the product's tcgen05 kernels are checked against it; nothing in
the product imports this file).

Network and loss as the product defines them: a0 = bf16(x); z_l = a_{l-1}
W_l^T + b_l; a_l = bf16(relu(z_l)) (l = 1..3); y = a_3 . w4 + b4; loss =
1/(2n) sum (y - t)^2, with the backward pass rounding each layer's delta to
BF16 as the kernels do.  rounding=False gives the same formulas in plain
float64 (for finite-difference checks of the backward formulas).
"""
import numpy as np

F = 128
NP = 3 * F * F + 3 * F + F + 1


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    W = p[: 3 * F * F].reshape(3, F, F)
    b = p[3 * F * F: 3 * F * F + 3 * F].reshape(3, F)
    w4 = p[3 * F * F + 3 * F: 3 * F * F + 4 * F]
    b4 = p[3 * F * F + 4 * F]
    return W, b, w4, b4


def forward(p, x, rounding=True):
    W, b, w4, b4 = unpack(p)
    rd = (lambda a: bf16(a).astype(np.float64)) if rounding else (lambda a: np.asarray(a, np.float64))
    a = [rd(x)]
    for l in range(3):
        z = a[-1] @ rd(W[l]).T + b[l]
        a.append(rd(np.maximum(z, 0.0)))
    y = a[3] @ w4 + b4
    return y, a


def gradients(p, x, t, rounding=True):
    W, b, w4, b4 = unpack(p)
    rd = (lambda a: bf16(a).astype(np.float64)) if rounding else (lambda a: np.asarray(a, np.float64))
    y, a = forward(p, x, rounding)
    n = len(x)
    e = y - np.asarray(t, np.float64)
    loss = 0.5 * np.sum(e * e) / n
    dy = e / n
    gW = np.zeros((3, F, F))
    gb = np.zeros((3, F))
    gw4 = a[3].T @ dy
    gb4 = dy.sum()
    d = rd(np.where(a[3] > 0, dy[:, None] * w4[None, :], 0.0))
    for l in (2, 1, 0):
        gW[l] = d.T @ a[l]
        gb[l] = d.sum(0)
        if l > 0:
            dh = d @ rd(W[l])
            d = rd(np.where(a[l] > 0, dh, 0.0))
    g = np.concatenate([gW.ravel(), gb.ravel(), gw4, [gb4]])
    return g, loss


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(NP, np.float32)
    lim = np.sqrt(6.0 / F)
    p[: 3 * F * F] = rng.uniform(-lim, lim, 3 * F * F)
    p[3 * F * F: 3 * F * F + 3 * F] = rng.uniform(-0.1, 0.1, 3 * F)
    p[3 * F * F + 3 * F: 3 * F * F + 4 * F] = rng.uniform(-np.sqrt(3.0 / F), np.sqrt(3.0 / F), F)
    p[-1] = 0.05
    return p
