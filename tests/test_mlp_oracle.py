"""The surrogate MLP's CPU oracle (oracle/mlp.py): bf16 rounding, GELU and its derivative, and
the hand-written backward pass against finite differences.  No GPU."""
import numpy as np
import torch

from oracle import mlp as OM


def test_bf16_rounding_matches_torch():
    x = np.random.default_rng(0).normal(size=10000).astype(np.float32) * 10.0 ** np.arange(-4, 6)[
        np.arange(10000) % 10]
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    assert np.array_equal(OM.bf16(x), ref)


def test_gelu_grad_is_the_derivative():
    p = np.linspace(-6, 6, 2001)
    h = 1e-6
    fd = (OM.gelu(p + h) - OM.gelu(p - h)) / (2 * h)
    np.testing.assert_allclose(OM.gelu_grad(p), fd, atol=1e-8)


def test_backward_matches_finite_differences_without_rounding(monkeypatch):
    # with the bf16 rounding switched off the oracle's backward is the exact gradient (the
    # forward still rounds activations to float32, so the difference step is 1e-3)
    monkeypatch.setattr(OM, "bf16", lambda x: np.asarray(x, np.float64))
    rng = np.random.default_rng(1)
    Ws = [rng.normal(0, 0.5, (6, 4)), rng.normal(0, 0.5, (6, 6))]
    bs = [rng.normal(0, 0.1, 6), rng.normal(0, 0.1, 6)]
    wh, bh = rng.normal(0, 0.5, 6), 0.2
    X = rng.normal(size=(5, 4))
    t = rng.normal(size=5)

    def loss(Ws_, bs_, wh_, bh_):
        y, _ = OM.forward(X, Ws_, bs_, wh_, bh_)
        return np.mean((y - t) ** 2)

    y, cache = OM.forward(X, Ws, bs, wh, bh)
    dWs, dbs, dwh, dbh = OM.backward(cache, Ws, wh, y, t)
    eps = 1e-3
    for l in range(2):
        for (i, j) in [(0, 0), (3, 2), (5, 3)]:
            Wp = [W.copy() for W in Ws]
            Wm = [W.copy() for W in Ws]
            Wp[l][i, j] += eps
            Wm[l][i, j] -= eps
            fd = (loss(Wp, bs, wh, bh) - loss(Wm, bs, wh, bh)) / (2 * eps)
            assert abs(fd - dWs[l][i, j]) < 3e-4 + 1e-3 * abs(fd)
        bp = [b.copy() for b in bs]
        bp[l][1] += eps
        bm = [b.copy() for b in bs]
        bm[l][1] -= eps
        fd = (loss(Ws, bp, wh, bh) - loss(Ws, bm, wh, bh)) / (2 * eps)
        assert abs(fd - dbs[l][1]) < 3e-4 + 1e-3 * abs(fd)
    whp, whm = wh.copy(), wh.copy()
    whp[2] += eps
    whm[2] -= eps
    fd = (loss(Ws, bs, whp, bh) - loss(Ws, bs, whm, bh)) / (2 * eps)
    assert abs(fd - dwh[2]) < 3e-4 + 1e-3 * abs(fd)
    fd = (loss(Ws, bs, wh, bh + eps) - loss(Ws, bs, wh, bh - eps)) / (2 * eps)
    assert abs(fd - dbh) < 3e-4 + 1e-3 * abs(fd)
