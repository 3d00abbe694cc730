"""The radiance-cache MLP oracle: its backward pass against finite differences.

oracle/nrc.py is the checker of the GPU training kernels, so its own
gradients are checked first, in float64 without bfloat16 rounding, by
central differences of the loss.
"""
import numpy as np

from oracle import nrc


def test_parameter_count():
    assert nrc.N_PARAMS == 26304 + 259
    assert nrc.N_FEAT == 216


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(7)
    p = nrc.init_params(3).astype(np.float64)
    p[-3:] = 0.3                                  # outputs away from zero
    x = np.concatenate([rng.uniform(0, 1, (32, 3)), rng.normal(size=(32, 6))], axis=1)
    t = rng.uniform(0.0, 2.0, (32, 3))

    def loss(q):
        y, _ = nrc.forward(q, x, bf16_ops=False)
        den = y * y + nrc.LOSS_EPS               # the denominator is held constant
        return float(np.sum((y - t) ** 2 / den_fixed) / y.size), den

    y, cache = nrc.forward(p, x, bf16_ops=False)
    den_fixed = y * y + nrc.LOSS_EPS
    _, dy = nrc.loss_and_dy(y, t)
    g = nrc.backward(cache, dy, bf16_ops=False)
    idx = rng.choice(nrc.N_PARAMS, 60, replace=False)
    idx = np.concatenate([idx, np.arange(nrc.N_PARAMS - 200, nrc.N_PARAMS)])
    h = 1e-6
    for i in idx:
        q1 = p.copy(); q1[i] += h
        q2 = p.copy(); q2[i] -= h
        fd = (loss(q1)[0] - loss(q2)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_training_reduces_loss():
    rng = np.random.default_rng(1)
    p = nrc.init_params(5).astype(np.float64)
    x = np.concatenate([rng.uniform(0, 1, (256, 3)), rng.normal(size=(256, 6))], axis=1)
    t = 0.5 + 0.3 * np.sin(3 * x[:, :3])         # a smooth target of position
    m = np.zeros_like(p); v = np.zeros_like(p)
    first = None
    for step in range(1, 61):
        y, cache = nrc.forward(p, x)
        l, dy = nrc.loss_and_dy(y, t)
        first = l if first is None else first
        g = nrc.backward(cache, dy)
        p, m, v = nrc.adam_step(p, g, m, v, step)
    y, _ = nrc.forward(p, x)
    assert nrc.loss_and_dy(y, t)[0] < 0.2 * first
