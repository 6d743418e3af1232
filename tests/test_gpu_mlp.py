"""The surrogate's tensor-core kernels on the GPU: the tcgen05 GEMM and its fused epilogues
against products of the same bf16 operands in float64, and the whole MLP's forward pass and
gradients against the CPU oracle (oracle/mlp.py), plus a short training run."""
import numpy as np
import pytest
import torch

from dmipy_sim_gb300 import _lib
from dmipy_sim_gb300.mlp import MLP
from oracle import mlp as OM

pytestmark = pytest.mark.gpu


def _gemm(A, Bm, M, N, K, epi, splits=1, bias=None, P=None, ldht=0, want_t=False):
    dev = A.device
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    g = _lib.Gemm()
    g.A, g.B, g.M, g.N, g.K = A.data_ptr(), Bm.data_ptr(), M, N, K
    g.lda, g.ldb, g.epilogue, g.splits = A.shape[1], Bm.shape[1], epi, splits
    out = {}
    if epi == _lib.EPI_STORE_F32:
        out["C"] = torch.full((splits, M, N), np.nan, device=dev)
        g.C = out["C"].data_ptr()
    else:
        out["H"] = torch.empty(M, N, dtype=torch.bfloat16, device=dev)
        g.H = out["H"].data_ptr()
        if want_t:
            out["HT"] = torch.zeros(N, ldht, dtype=torch.bfloat16, device=dev)
            g.HT, g.ldht = out["HT"].data_ptr(), ldht
        if epi == _lib.EPI_BIAS_GELU:
            g.bias = bias.data_ptr()
            out["P"] = torch.empty(M, N, device=dev)
            g.P = out["P"].data_ptr()
        else:
            g.P = P.data_ptr()
    g.err = err.data_ptr()
    import ctypes
    _lib.check(_lib.load().dmsim_gemm_bf16(ctypes.byref(g), _lib.stream_handle()), "gemm")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return out


def _rand_bf16(rows, cols, seed, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    return (torch.randn(rows, cols, generator=g) * scale).to(torch.bfloat16)


@pytest.mark.parametrize("M,N,K,splits", [(128, 128, 64, 1), (1000, 256, 256, 1),
                                          (4103, 384, 128, 1), (256, 256, 1024, 4),
                                          (300, 128, 512, 8)])
def test_gemm_store_f32(cuda, M, N, K, splits):
    A, Bm = _rand_bf16(M, K, 1), _rand_bf16(N, K, 2)
    out = _gemm(A.to(cuda), Bm.to(cuda), M, N, K, _lib.EPI_STORE_F32, splits=splits)
    C = out["C"].double().sum(0).cpu().numpy()
    ref = A.double().numpy() @ Bm.double().numpy().T
    assert np.all(np.isfinite(C))
    np.testing.assert_allclose(C, ref, rtol=1e-5, atol=1e-4 * np.sqrt(K))


def test_gemm_bias_gelu_and_transpose(cuda):
    M, N, K = 777, 256, 192
    A, Bm = _rand_bf16(M, K, 3, 0.2), _rand_bf16(N, K, 4, 0.2)
    bias = torch.linspace(-1, 1, N)
    out = _gemm(A.to(cuda), Bm.to(cuda), M, N, K, _lib.EPI_BIAS_GELU, bias=bias.to(cuda),
                ldht=832, want_t=True)
    p_ref = A.double().numpy() @ Bm.double().numpy().T + bias.double().numpy()
    P = out["P"].cpu().numpy()
    np.testing.assert_allclose(P, p_ref, rtol=1e-5, atol=1e-4)
    H = out["H"].float().cpu().numpy()
    h_ref = OM.bf16(OM.gelu(P.astype(np.float64)).astype(np.float32))
    # the kernel's MUFU tanh and the oracle's tanh may round one bf16 step apart
    np.testing.assert_allclose(H, h_ref, rtol=8e-3, atol=1e-6)
    assert np.mean(H == h_ref) > 0.99
    HT = out["HT"].float().cpu().numpy()
    assert np.array_equal(HT[:, :M], H.T)


def test_gemm_gelu_backward(cuda):
    M, N, K = 640, 256, 256
    A, Bm = _rand_bf16(M, K, 5, 0.1), _rand_bf16(N, K, 6, 0.1)
    P = torch.randn(M, N, generator=torch.Generator().manual_seed(7))
    out = _gemm(A.to(cuda), Bm.to(cuda), M, N, K, _lib.EPI_GELU_BWD, P=P.to(cuda), ldht=M,
                want_t=True)
    ref = (A.double().numpy() @ Bm.double().numpy().T) * OM.gelu_grad(P.double().numpy())
    H = out["H"].float().cpu().numpy()
    np.testing.assert_allclose(H, OM.bf16(ref.astype(np.float32)), rtol=8e-3, atol=1e-5)
    assert np.array_equal(out["HT"].float().cpu().numpy(), H.T)


def _net(seed=0, n_in=69):
    net = MLP(n_in, width=256, depth=4, seed=seed)
    rng = np.random.default_rng(seed)
    for b in net.b:
        b.copy_(torch.as_tensor(rng.normal(0, 0.05, b.shape[0]), dtype=torch.float32))
    net.b_head.fill_(0.1)
    return net


def _oracle_params(net):
    return ([W.cpu().numpy() for W in net.W], [b.cpu().numpy() for b in net.b],
            net.w_head.cpu().numpy(), float(net.b_head.item()))


def test_mlp_forward_matches_oracle(cuda):
    net = _net(1)
    x = np.random.default_rng(2).normal(size=(1000, 69)).astype(np.float32)
    y = net.predict(x).cpu().numpy()
    Ws, bs, wh, bh = _oracle_params(net)
    y_ref, _ = OM.forward(OM.pack(x, net.kp), Ws, bs, wh, bh)
    np.testing.assert_allclose(y, y_ref, atol=2e-2 * np.std(y_ref) + 1e-3)
    assert np.corrcoef(y, y_ref)[0, 1] > 0.9999


def _randomise(net, seed):
    g = torch.Generator().manual_seed(seed)
    for b in net.b:
        b.copy_(torch.randn(b.shape, generator=g) * 0.3)
    net.b_head.copy_(torch.randn(1, generator=g))
    net.set_normalisation(np.linspace(-0.5, 0.5, net.n_in), np.linspace(0.5, 2.0, net.n_in))


@pytest.mark.parametrize("rows", [1, 127, 128, 129, 4099, 300_001])
def test_fused_forward_matches_the_layer_by_layer_pass(cuda, rows):
    """The one-launch forward pass (activations on chip) against the four GEMMs + head on the
    same bf16 weights: the two differ only in fp32 summation order, which can flip a bf16
    rounding of an activation now and then."""
    net = _net(5)
    _randomise(net, 6)
    assert net.fused()
    x = torch.as_tensor(np.random.default_rng(7).normal(size=(rows, 69)).astype(np.float32),
                        device=cuda)
    y_f = net.predict_fused(x).cpu().numpy()
    y_l = net.predict_layers(x).cpu().numpy()
    torch.cuda.synchronize()
    net.check_errors()
    assert np.all(np.isfinite(y_f))
    np.testing.assert_allclose(y_f, y_l, atol=2e-3 * np.std(y_l) + 2e-3)
    if rows > 1000:
        assert np.corrcoef(y_f, y_l)[0, 1] > 0.99999


def test_fused_forward_matches_oracle_with_biases(cuda):
    net = _net(8)
    _randomise(net, 9)
    x = np.random.default_rng(10).normal(size=(2000, 69)).astype(np.float32)
    y = net.predict_fused(torch.as_tensor(x, device=cuda)).cpu().numpy()
    net.check_errors()
    Ws, bs, wh, bh = _oracle_params(net)
    xs = OM.pack(x, net.kp, net.shift.cpu().numpy(), net.scale.cpu().numpy())
    y_ref, _ = OM.forward(xs, Ws, bs, wh, bh)
    np.testing.assert_allclose(y, y_ref, atol=2e-2 * np.std(y_ref) + 1e-3)
    assert np.corrcoef(y, y_ref)[0, 1] > 0.9999


def test_mlp_gradients_match_oracle(cuda):
    net = _net(3)
    rng = np.random.default_rng(4)
    B = 512
    x = rng.normal(size=(B, 69)).astype(np.float32)
    t = np.tanh(x[:, 0] - 0.5 * x[:, 1]).astype(np.float32)
    bf = net.gradients(x, t)
    torch.cuda.synchronize()
    net.check_errors()
    Ws, bs, wh, bh = _oracle_params(net)
    y_ref, cache = OM.forward(OM.pack(x, net.kp), Ws, bs, wh, bh)
    dWs, dbs, dwh, dbh = OM.backward(cache, Ws, wh, y_ref, t)

    def close(gpu, ref, what):
        gpu = np.asarray(gpu, np.float64)
        rel = np.linalg.norm(gpu - ref) / max(np.linalg.norm(ref), 1e-30)
        cos = float(np.sum(gpu * ref) / max(np.linalg.norm(gpu) * np.linalg.norm(ref), 1e-30))
        assert rel < 2e-2 and cos > 0.9998, f"{what}: rel {rel:.3e} cos {cos:.6f}"

    np.testing.assert_allclose(bf["y"].cpu().numpy(), y_ref, atol=2e-2 * np.std(y_ref) + 1e-3)
    for l in range(net.depth):
        close(bf["dW"][l].sum(0).cpu().numpy(), dWs[l], f"dW{l}")
        close(bf["db"][l].cpu().numpy(), dbs[l], f"db{l}")
    close(bf["dw_head"].cpu().numpy(), dwh, "dw_head")
    assert abs(float(bf["db_head"].item()) - dbh) < 1e-3 * max(1.0, abs(dbh))
    loss = float(bf["loss"].item()) / B
    assert abs(loss - np.mean((y_ref - t) ** 2)) < 2e-2 * max(loss, 1e-6)


def test_adamw_matches_oracle(cuda):
    net = _net(5)
    x = np.random.default_rng(6).normal(size=(256, 69)).astype(np.float32)
    t = np.sin(x[:, 2]).astype(np.float32)
    p0 = net.w_head.cpu().numpy().astype(np.float64)
    bf = net.gradients(x, t)
    g = bf["dw_head"].cpu().numpy().astype(np.float64)
    net.set_lr(1e-2)
    net.hp[4] = 0.01
    net._update(bf)
    torch.cuda.synchronize()
    ref, _, _ = OM.adamw(p0, 0.0, 0.0, g, 1, 1e-2, wd=0.01)
    np.testing.assert_allclose(net.w_head.cpu().numpy(), ref, rtol=1e-5, atol=1e-7)


def test_mlp_training_graph_reduces_loss(cuda):
    net = MLP(8, width=256, depth=4, seed=7, lr=2e-3)
    rng = np.random.default_rng(8)
    X = rng.uniform(-1, 1, size=(1 << 15, 8)).astype(np.float32)
    T = (np.sin(2 * X[:, 0]) * np.exp(-X[:, 1] ** 2) + 0.3 * X[:, 2] * X[:, 3]).astype(np.float32)
    Xd, Td = torch.as_tensor(X, device=cuda), torch.as_tensor(T, device=cuda)
    B = 1024
    net.capture_step(B)
    first = None
    for step in range(400):
        i = (step * B) % len(X)
        loss = net.train_step(Xd[i:i + B], Td[i:i + B])
        if step == 0:
            first = float(loss.item())
    torch.cuda.synchronize()
    net.check_errors()
    y = net.predict(X[:4096]).cpu().numpy()
    mse = float(np.mean((y - T[:4096]) ** 2))
    assert mse < 0.05 * first, (first, mse)
    assert int(net.hp[5].item()) == 400
