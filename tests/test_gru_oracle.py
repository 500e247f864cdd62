"""The float64 GRU oracle: exact gradient (finite differences) and BF16 rounding."""

import numpy as np

from oracle import gru as G


def _problem(seed=0, B=3, T=6):
    rng = np.random.default_rng(seed)
    theta = G.init_params(seed, scale=2.0)
    x = rng.normal(size=(B, T, G.X))
    y = rng.normal(scale=0.5, size=(B, T))
    h0 = rng.normal(scale=0.3, size=(B, G.H))
    return theta, x, y, h0


def test_oracle_gradient_matches_finite_differences():
    theta, x, y, h0 = _problem()
    _, g = G.loss_and_grad(theta, x, y, h0, quantize=False)
    rng = np.random.default_rng(1)
    # a few entries of every parameter block
    blocks = [(G.OFF_WH, G.OFF_WX), (G.OFF_WX, G.OFF_BX), (G.OFF_BX, G.OFF_BH), (G.OFF_BH, G.OFF_WO),
              (G.OFF_WO, G.OFF_BO), (G.OFF_BO, G.NPARAM)]
    idx = np.concatenate([rng.integers(a, b, size=min(4, b - a)) for a, b in blocks])
    eps = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        fd = (G.loss_and_grad(tp, x, y, h0)[0] - G.loss_and_grad(tm, x, y, h0)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1) wins; 1 + 3*2^-8 rounds up
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 3.1415926])
    q = G.bf16(v)
    np.testing.assert_array_equal(q[:4], [1.0, 1.0, 1.0 + 2.0 ** -6, -2.5])
    assert abs(q[4] - 3.140625) < 1e-12


def test_quantised_oracle_stays_close_to_exact():
    theta, x, y, h0 = _problem(2)
    l0, g0 = G.loss_and_grad(theta, x, y, h0, quantize=False)
    l1, g1 = G.loss_and_grad(theta, x, y, h0, quantize=True)
    assert abs(l1 - l0) < 2e-2 * abs(l0)
    assert np.linalg.norm(g1 - g0) < 5e-2 * np.linalg.norm(g0)


def test_step_matches_forward():
    theta, x, y, h0 = _problem(3, B=2, T=4)
    ys, hT, _ = G.forward(theta, x, h0)
    h = h0
    for t in range(x.shape[1]):
        h, yt = G.step(theta, x[:, t], h)
        np.testing.assert_allclose(yt, ys[:, t], rtol=0, atol=1e-12)
    np.testing.assert_allclose(h, hT, atol=1e-12)
