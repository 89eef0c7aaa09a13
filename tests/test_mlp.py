"""The learned warm start's network: numpy restatement (oracle/mlp_ref.py)
checked by finite differences on the CPU; the tcgen05 forward, backward and
Adam kernels checked against it on the GPU."""
import numpy as np
import pytest

import lsgb300
import mlp_ref


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (n, 128)).astype(np.float32)
    # a smooth target of a few features (a stand-in for distances)
    t = (0.5 * x[:, 3] + 0.25 * np.tanh(x[:, 7]) - 0.1 * x[:, 0] * x[:, 1]).astype(np.float32)
    return x, t


def test_reference_backward_matches_finite_differences():
    p = mlp_ref.init_params(1).astype(np.float64)
    x, t = _data(16, 2)
    g, loss = mlp_ref.gradients(p, x, t, rounding=False)
    rng = np.random.default_rng(3)
    idx = np.concatenate([rng.choice(3 * 128 * 128, 24, replace=False), np.arange(3 * 128 * 128, mlp_ref.NP)[::37],
                          [mlp_ref.NP - 1]])
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        _, lp = mlp_ref.gradients(q, x, t, rounding=False)
        q[i] -= 2 * eps
        _, lm = mlp_ref.gradients(q, x, t, rounding=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_helper():
    v = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], np.float32)
    r = mlp_ref.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == -2.5
    assert abs(r[4] - 3.0e-3) < 3.0e-3 * 2 ** -8


@pytest.mark.gpu
def test_forward_matches_reference():
    m = lsgb300.MLP(0)
    p = mlp_ref.init_params(4)
    m.set_params(p)
    x, _ = _data(1000, 5)  # not a multiple of the 128-sample tile
    y = m.predict(x)
    yr, _ = mlp_ref.forward(p, x)
    scale = np.abs(yr).max() + 1e-3
    err = np.abs(y - yr) / scale
    assert err.max() < 2e-2 and np.median(err) < 2e-3, (err.max(), np.median(err))


@pytest.mark.gpu
def test_gradients_match_reference():
    m = lsgb300.MLP(0)
    p = mlp_ref.init_params(6)
    m.set_params(p)
    x, t = _data(777, 7)
    g, loss = m.gradients(x, t)
    gr, lr = mlp_ref.gradients(p, x, t)
    assert abs(loss - lr) <= 1e-2 * lr + 1e-6
    for sl in (slice(0, 3 * 128 * 128), slice(3 * 128 * 128, 3 * 128 * 128 + 384), slice(-129, None)):
        a, b = g[sl], gr[sl]
        rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-12)
        assert rel < 3e-2, (sl, rel)


@pytest.mark.gpu
def test_training_reduces_loss():
    m = lsgb300.MLP(3)
    x, t = _data(1 << 15, 9)
    _, l0 = m.gradients(x[:4096], t[:4096])
    last = m.train(x, t, epochs=30, batch=4096, lr=1e-3)
    _, l1 = m.gradients(x[:4096], t[:4096])
    assert np.isfinite(last) and l1 < 0.2 * l0, (l0, l1, last)


@pytest.mark.gpu
def test_gradients_over_many_tiles_per_cta_match_reference_and_repeat():
    # more 128-sample tiles than SMs: each backward CTA accumulates several
    # tiles in tensor memory, the per-CTA rows are summed in a fixed order
    m = lsgb300.MLP(0)
    p = mlp_ref.init_params(8)
    m.set_params(p)
    x, t = _data(40000, 11)
    g, loss = m.gradients(x, t)
    g2, loss2 = m.gradients(x, t)
    assert np.array_equal(g.view(np.uint32), g2.view(np.uint32)) and loss == loss2
    gr, lr = mlp_ref.gradients(p, x, t)
    assert abs(loss - lr) <= 1e-2 * lr + 1e-6
    for sl in (slice(0, 3 * 128 * 128), slice(3 * 128 * 128, 3 * 128 * 128 + 384), slice(-129, None)):
        a, b = g[sl], gr[sl]
        rel = np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-12)
        assert rel < 3e-2, (sl, rel)
