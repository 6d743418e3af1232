"""CPU restatement of the surrogate MLP's forward and backward pass -- TEST INFRASTRUCTURE ONLY.

Imported by tests/ as the checker of the GPU kernels (dmipy_sim_gb300/csrc/mlp.cu); the product
package never imports it.  The network has no counterpart in the reference: this file is the
specification the kernels are held to.  It rounds to bf16 exactly where the GPU path stores bf16
(packed inputs, weights, hidden activations, layer gradients) and accumulates in float64, so the
GPU's fp32 tensor-core accumulation differs from it only by fp32 summation error and by the
occasional bf16 rounding flip that error causes.
"""
import math

import numpy as np

_C0 = math.sqrt(2.0 / math.pi)
_C1 = 0.044715


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(x.shape)


def gelu(p):
    """GELU in its tanh form: 0.5 p (1 + tanh(sqrt(2/pi) (p + 0.044715 p^3)))."""
    return 0.5 * p * (1.0 + np.tanh(_C0 * (p + _C1 * p ** 3)))


def gelu_grad(p):
    t = np.tanh(_C0 * (p + _C1 * p ** 3))
    return 0.5 * (1.0 + t) + 0.5 * p * (1.0 - t * t) * _C0 * (1.0 + 3.0 * _C1 * p * p)


def pack(x, kp, shift=None, scale=None):
    x = np.asarray(x, np.float64)
    if shift is not None:
        x = x - shift
    if scale is not None:
        x = x * scale
    out = np.zeros((x.shape[0], kp), np.float32)
    out[:, :x.shape[1]] = x
    return bf16(out)


def forward(X0, Ws, bs, w_head, b_head):
    """X0 (B, Kp) bf16-valued; Ws[l] (N, K) fp32 master weights (rounded to bf16 here).
    Returns y (B,) and the cache (inputs of each layer, pre-activations)."""
    xs, ps = [X0.astype(np.float64)], []
    for W, b in zip(Ws, bs):
        p = xs[-1] @ bf16(W).astype(np.float64).T + np.asarray(b, np.float64)
        ps.append(p)
        xs.append(bf16(gelu(p).astype(np.float32)).astype(np.float64))
    y = xs[-1] @ np.asarray(w_head, np.float64) + float(b_head)
    return y, (xs, ps)


def backward(cache, Ws, w_head, y, target):
    """Gradients of mean((y - t)^2): dW (list), db (list), dw_head, db_head."""
    xs, ps = cache
    B = len(y)
    dy = 2.0 * (y - np.asarray(target, np.float64)) / B
    dy32 = dy.astype(np.float32).astype(np.float64)
    w = np.asarray(w_head, np.float64)
    dP = bf16((dy32[:, None] * w[None, :] * gelu_grad(ps[-1])).astype(np.float32))
    dP = dP.astype(np.float64)
    dWs, dbs = [None] * len(Ws), [None] * len(Ws)
    dw_head = xs[-1].T @ dy32
    db_head = float(np.sum(dy32))
    for l in range(len(Ws) - 1, -1, -1):
        dWs[l] = dP.T @ xs[l]
        dbs[l] = dP.sum(axis=0)
        if l > 0:
            dh = dP @ bf16(Ws[l]).astype(np.float64)
            dP = bf16((dh * gelu_grad(ps[l - 1])).astype(np.float32)).astype(np.float64)
    return dWs, dbs, dw_head, db_head


def adamw(p, m, v, g, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    upd = (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p * (1 - lr * wd) - lr * upd, m, v
