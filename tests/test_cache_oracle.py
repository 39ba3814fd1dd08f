"""The FP64 radiance-cache oracle checked against central finite
differences, and its emulated-precision mode against the exact one (CPU)."""
import numpy as np
import pytest

from oracle import radiance_cache as rc


def _problem(n=64, seed=3):
    rng = np.random.default_rng(seed)
    params = np.zeros(rc.PARAM_COUNT)
    for l, (o, i) in enumerate(rc.SHAPES):
        w = rng.uniform(-1, 1, size=(o, i)) * np.sqrt(6.0 / i)
        if l == 5:
            w[rc.OUTPUTS:] = 0.0
        params[rc.OFFSETS[l]:rc.OFFSETS[l + 1]] = w.ravel()
    x = rng.uniform(0, 1, size=(n, rc.INPUTS))
    t = rng.uniform(0, 2, size=(n, rc.OUTPUTS))
    t[::7, 0] = -1.0   # samples without a target
    return params, x, t


def test_encoding_layout():
    x = np.linspace(0.05, 0.95, 10)[None, :]
    f = rc.encode(x)
    assert f.shape == (1, 256)
    j, b = 3, 5
    assert f[0, 24 * j + 2 * b] == pytest.approx(np.sin(np.pi * 2 ** b * x[0, j]))
    assert f[0, 24 * j + 2 * b + 1] == pytest.approx(np.cos(np.pi * 2 ** b * x[0, j]))
    assert np.array_equal(f[0, 240:250], x[0])
    assert f[0, 250] == 1.0 and not f[0, 251:].any()


def test_gradients_match_finite_differences():
    params, x, t = _problem()
    _, g = rc.loss_and_grads(params, x, t)
    rng = np.random.default_rng(0)
    # a few parameters from every layer (real rows of the output layer)
    picks = []
    for l, (o, i) in enumerate(rc.SHAPES):
        rows = rc.OUTPUTS if l == 5 else o
        for _ in range(4):
            picks.append(rc.OFFSETS[l] + rng.integers(rows) * i + rng.integers(i))
    h = 1e-6
    for k in picks:
        # the denominator (y^2 + 0.01) is held constant in the loss gradient:
        # differentiate the loss with the denominator frozen at params
        y0, _, _ = rc.forward(params, x)
        valid = t[:, 0] >= 0
        den = y0 * y0 + 0.01

        def frozen(p):
            y, _, _ = rc.forward(p, x)
            d = y - np.where(valid[:, None], t, 0.0)
            return np.sum(np.where(valid[:, None], d * d / den, 0.0))

        pp, pm = params.copy(), params.copy()
        pp[k] += h
        pm[k] -= h
        fd = (frozen(pp) - frozen(pm)) / (2 * h)
        assert g[k] == pytest.approx(fd, rel=1e-5, abs=1e-7), k


def test_padded_rows_have_no_gradient():
    params, x, t = _problem()
    _, g = rc.loss_and_grads(params, x, t)
    assert not g[rc.OFFSETS[5] + rc.OUTPUTS * rc.HIDDEN:].any()


def test_emulated_precision_is_close_to_exact():
    params, x, t = _problem(n=256)
    l0, g0 = rc.loss_and_grads(params, x, t)
    l1, g1 = rc.loss_and_grads(params, x, t, emulate=True)
    assert l1 == pytest.approx(l0, rel=2e-2)
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < 3e-2


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.01171875, -3.0e-3, 65504.0, 0.0])
    r = rc.round_bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0              # tie -> even
    assert r[2] == 1.015625         # tie -> even (odd neighbour below)
    assert abs(r[3] - v[3]) <= 2 ** -8 * abs(v[3])
    assert r[5] == 0.0
