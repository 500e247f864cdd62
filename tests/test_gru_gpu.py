"""GRU training kernels (tensor-core forward / backward, Adam) against the float64 oracle."""

import numpy as np
import pytest

from oracle import gru as G

pytestmark = pytest.mark.gpu


def _problem(seed, n, T):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, T, G.X)).astype(np.float32)
    y = rng.normal(scale=0.5, size=(n, T)).astype(np.float32)
    theta = G.init_params(seed, scale=2.0).astype(np.float32)
    return theta, x, y


def test_gru_forward_and_gradient_match_oracle(native_lib, cuda_device):
    from braincell_gb300.gru import GRUTrainer

    # 40 sequences: the last M tile is ragged (rows 32..39 of 48)
    theta, x, y = _problem(5, 40, 30)
    rng = np.random.default_rng(9)
    h0 = rng.normal(scale=0.3, size=(40, G.H)).astype(np.float32)
    tr = GRUTrainer(x, y, theta, batch=40, window=30, device=cuda_device)
    loss, g, yout = tr.gradient(np.arange(40), 0, 30, h0)
    ys, _, cache = G.forward(theta.astype(np.float64), x.astype(np.float64), h0.astype(np.float64), quantize=True)
    # forward: FP32 arithmetic around BF16 products against float64 with the same rounding points
    np.testing.assert_allclose(yout, ys, rtol=0, atol=2e-4)
    ref_loss = float(np.mean((ys - y) ** 2))
    assert abs(loss - ref_loss) < 1e-4 * ref_loss
    gref = G.backward(theta.astype(np.float64), x.astype(np.float64), y.astype(np.float64), ys, cache, quantize=True)
    blocks = {"Wh": (G.OFF_WH, G.OFF_WX), "Wx": (G.OFF_WX, G.OFF_BX), "bx": (G.OFF_BX, G.OFF_BH),
              "bh": (G.OFF_BH, G.OFF_WO), "wo": (G.OFF_WO, G.OFF_BO), "bo": (G.OFF_BO, G.NPARAM)}
    for name, (a, b) in blocks.items():
        err = np.linalg.norm(g[a:b] - gref[a:b]) / max(np.linalg.norm(gref[a:b]), 1e-30)
        assert err < 1e-2, (name, err)
    # and the gradient is the gradient: the exact float64 one is close as well
    g_exact = G.loss_and_grad(theta.astype(np.float64), x.astype(np.float64), y.astype(np.float64),
                              h0.astype(np.float64), quantize=False)[1]
    assert np.linalg.norm(g - g_exact) / np.linalg.norm(g_exact) < 5e-2


def test_gru_window_offset_and_subset(native_lib, cuda_device):
    from braincell_gb300.gru import GRUTrainer

    theta, x, y = _problem(6, 20, 50)
    ids = np.array([7, 3, 19, 0, 11])
    tr = GRUTrainer(x, y, theta, batch=16, window=20, device=cuda_device)
    loss, g, yout = tr.gradient(ids, 25, 20)
    ys, _, cache = G.forward(theta.astype(np.float64), x[ids, 25:45].astype(np.float64), np.zeros((5, G.H)))
    np.testing.assert_allclose(yout, ys, atol=2e-4)
    gref = G.backward(theta.astype(np.float64), x[ids, 25:45].astype(np.float64), y[ids, 25:45].astype(np.float64),
                      ys, cache)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) < 1e-2


def test_gru_training_reduces_loss(native_lib, cuda_device):
    from braincell_gb300.gru import GRUTrainer

    # target: a leaky integral of the first input (a task a GRU learns quickly)
    rng = np.random.default_rng(3)
    n, T = 64, 200
    x = np.zeros((n, T, G.X), np.float32)
    x[:, :, 0] = rng.normal(size=(n, T))
    x[:, :, 2] = rng.normal(size=(n, 1))
    y = np.zeros((n, T), np.float32)
    acc = np.zeros(n)
    for t in range(T):
        acc = 0.9 * acc + 0.1 * x[:, t, 0] + 0.05 * x[:, t, 2]
        y[:, t] = acc
    tr = GRUTrainer(x, y, batch=32, window=50, lr=3e-3, device=cuda_device, seed=1)
    before = tr.evaluate(x, y)
    tr.train(epochs=15)
    after = tr.evaluate(x, y)
    assert after < 0.2 * before, (before, after)
    # the trained weights are the ones the predictions used
    th = tr.theta()
    ys, _, _ = G.forward(th.astype(np.float64), x[:4].astype(np.float64), np.zeros((4, G.H)))
    np.testing.assert_allclose(tr.predict(x[:4]), ys, atol=5e-4)


def test_backward_gradients_are_bit_reproducible(native_lib, cuda_device):
    # the per-CTA gradient rows are summed in a fixed order: two runs of the same
    # window give the same gradient bit for bit (a batch of several CTAs)
    from braincell_gb300.gru import GRUTrainer
    from braincell_gb300 import surrogate as S

    m = S.load_model(S.PACKAGED_MODEL)
    rng = np.random.default_rng(1)
    x = rng.normal(size=(96, 30, G.X)).astype(np.float32)
    y = rng.normal(scale=0.5, size=(96, 30)).astype(np.float32)
    tr = GRUTrainer(x, y, m.theta, batch=96, window=30)
    ids = np.arange(96)
    _, g1, _ = tr.gradient(ids, 0, 30)
    _, g2, _ = tr.gradient(ids, 0, 30)
    assert np.array_equal(g1, g2)
    assert np.count_nonzero(g1) > 0.9 * g1.size
