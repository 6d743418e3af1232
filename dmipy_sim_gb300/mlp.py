"""The surrogate's multilayer perceptron on the GB300 tensor cores.

``depth`` hidden layers of ``width`` units with GELU (tanh form), a linear head to one output,
bf16 weights and activations with fp32 accumulation, trained with AdamW on the mean squared
error.  Inference (:meth:`MLP.predict`) is one launch of ``dmsim_mlp_forward``, the whole network
per 128-row tile on chip.  In training every matrix product is ``dmsim_gemm_bf16`` (tcgen05,
csrc/mlp.cu) with its epilogue fused:

forward   H_l = gelu(X_l W_l^T + b_l)            BIAS_GELU (stores P_l and H_l^T when training)
head      y = H_L w + b; dy = 2 (y - t) / B; dP_L = dy w gelu'(P_L)       dmsim_mlp_head
backward  dP_{l-1} = (dP_l W_l) * gelu'(P_{l-1})  GELU_BWD with B operand W_l^T
          dW_l = dP_l^T X_l                       STORE_F32, K (= batch) split over CTAs
          db_l = row sums of dP_l^T; dw = H_L^T dy  dmsim_rowdot_bf16
update    AdamW on fp32 masters, refreshing the bf16 W_l and W_l^T copies   dmsim_adamw

Activations are kept in both layouts (row-major for the next forward product, transposed for
the weight gradient), written by the producing epilogue, so every product is K-major.  A
training step is a fixed sequence of launches on preallocated buffers; :meth:`MLP.capture_step`
records it as a CUDA graph.
"""
import ctypes

import numpy as np
import torch

from . import _lib

BF16 = torch.bfloat16


def _ceil(x, m):
    return (x + m - 1) // m * m


class MLP:
    def __init__(self, n_in, width=256, depth=4, seed=0, lr=1e-3, weight_decay=0.0,
                 betas=(0.9, 0.999), eps=1e-8, device=None):
        if width % 128:
            raise ValueError("width must be a multiple of 128")
        self.lib = _lib.load()
        self.dev = device or _lib.device()
        self.n_in, self.width, self.depth = int(n_in), int(width), int(depth)
        self.kp = _ceil(self.n_in, 128)  # padded input width (the weight-gradient product's N)
        g = torch.Generator().manual_seed(int(seed))
        self.W, self.b = [], []
        for l in range(depth):
            k = self.kp if l == 0 else width
            fan_in = self.n_in if l == 0 else width
            W = torch.randn(width, k, generator=g) * np.sqrt(2.0 / fan_in)
            if l == 0:
                W[:, self.n_in:] = 0.0
            self.W.append(W.to(self.dev))
            self.b.append(torch.zeros(width, device=self.dev))
        self.w_head = (torch.randn(width, generator=g) * np.sqrt(1.0 / width)).to(self.dev)
        self.b_head = torch.zeros(1, device=self.dev)
        self.Wb = [W.to(BF16).contiguous() for W in self.W]
        self.WTb = [W.t().contiguous().to(BF16) for W in self.W]
        params = self.W + self.b + [self.w_head, self.b_head]
        self.m = [torch.zeros_like(p) for p in params]
        self.v = [torch.zeros_like(p) for p in params]
        self.hp = torch.tensor([lr, betas[0], betas[1], eps, weight_decay, 0.0],
                               dtype=torch.float32, device=self.dev)
        self.shift = torch.zeros(self.n_in, device=self.dev)
        self.scale = torch.ones(self.n_in, device=self.dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._bufs = {}
        self.graph = None

    # ---- parameters ---------------------------------------------------------------------------
    def set_normalisation(self, shift, scale):
        self.shift.copy_(torch.as_tensor(np.asarray(shift, np.float32)))
        self.scale.copy_(torch.as_tensor(np.asarray(scale, np.float32)))

    def set_lr(self, lr):
        self.hp[0] = float(lr)

    def state_dict(self):
        return {"W": [w.cpu() for w in self.W], "b": [b.cpu() for b in self.b],
                "w_head": self.w_head.cpu(), "b_head": self.b_head.cpu(),
                "shift": self.shift.cpu(), "scale": self.scale.cpu(),
                "shape": (self.n_in, self.width, self.depth)}

    def load_state_dict(self, sd):
        for dst, src in zip(self.W, sd["W"]):
            dst.copy_(src)
        for dst, src in zip(self.b, sd["b"]):
            dst.copy_(src)
        self.w_head.copy_(sd["w_head"])
        self.b_head.copy_(sd["b_head"])
        self.shift.copy_(sd["shift"])
        self.scale.copy_(sd["scale"])
        self.refresh_bf16()

    def refresh_bf16(self):
        for l, W in enumerate(self.W):
            self.Wb[l].copy_(W.to(BF16))
            self.WTb[l].copy_(W.t().to(BF16))

    # ---- buffers ------------------------------------------------------------------------------
    def _buffers(self, B, train):
        key = (int(B), bool(train))
        if key in self._bufs:
            return self._bufs[key]
        dev, w = self.dev, self.width
        ldt = _ceil(B, 64)
        bf = dict(B=B, ldt=ldt)
        bf["x"] = torch.empty(B, self.n_in, device=dev)
        bf["X0"] = torch.empty(B, self.kp, dtype=BF16, device=dev)
        bf["H"] = [torch.empty(B, w, dtype=BF16, device=dev) for _ in range(self.depth)]
        bf["y"] = torch.empty(B, device=dev)
        if train:
            if B % 64:
                raise ValueError("the training batch must be a multiple of 64 rows")
            bf["X0T"] = torch.zeros(self.kp, ldt, dtype=BF16, device=dev)
            bf["P"] = [torch.empty(B, w, device=dev) for _ in range(self.depth)]
            bf["HT"] = [torch.zeros(w, ldt, dtype=BF16, device=dev) for _ in range(self.depth)]
            bf["dP"] = [torch.empty(B, w, dtype=BF16, device=dev) for _ in range(self.depth)]
            bf["dPT"] = [torch.zeros(w, ldt, dtype=BF16, device=dev) for _ in range(self.depth)]
            bf["t"] = torch.empty(B, device=dev)
            bf["dy"] = torch.empty(B, device=dev)
            bf["sqerr"] = torch.empty(B, device=dev)
            bf["loss"] = torch.zeros(1, device=dev)
            kch = B // 64
            splits = 1
            while splits * 2 <= 64 and kch % (splits * 2) == 0 and kch // (splits * 2) >= 2:
                splits *= 2
            bf["splits"] = splits
            bf["dW"] = [torch.empty(splits, w, self.W[l].shape[1], device=dev)
                        for l in range(self.depth)]
            bf["db"] = [torch.empty(w, device=dev) for _ in range(self.depth)]
            bf["dw_head"] = torch.empty(w, device=dev)
            bf["db_head"] = torch.empty(1, device=dev)
        self._bufs[key] = bf
        return bf

    # ---- launches -----------------------------------------------------------------------------
    def _gemm(self, A, lda, Bm, ldb, M, N, K, epi, splits=1, C=None, bias=None, P=None, H=None,
              HT=None, ldht=0):
        g = _lib.Gemm()
        g.A, g.B, g.M, g.N, g.K = A.data_ptr(), Bm.data_ptr(), M, N, K
        g.lda, g.ldb, g.epilogue, g.splits = lda, ldb, epi, splits
        g.C = None if C is None else C.data_ptr()
        g.bias = None if bias is None else bias.data_ptr()
        g.P = None if P is None else P.data_ptr()
        g.H = None if H is None else H.data_ptr()
        g.HT = None if HT is None else HT.data_ptr()
        g.ldht = ldht
        g.err = self.err.data_ptr()
        _lib.check(self.lib.dmsim_gemm_bf16(ctypes.byref(g), _lib.stream_handle()),
                   "dmsim_gemm_bf16")

    def _forward_into(self, bf, train):
        s = _lib.stream_handle()
        B, w, ldt = bf["B"], self.width, bf["ldt"]
        _lib.check(self.lib.dmsim_mlp_pack(
            bf["x"].data_ptr(), B, self.n_in, self.kp, self.shift.data_ptr(),
            self.scale.data_ptr(), bf["X0"].data_ptr(),
            bf["X0T"].data_ptr() if train else None, ldt, s), "dmsim_mlp_pack")
        x, kx = bf["X0"], self.kp
        for l in range(self.depth):
            self._gemm(x, kx, self.Wb[l], self.Wb[l].shape[1], B, w, kx, _lib.EPI_BIAS_GELU,
                       bias=self.b[l], P=bf["P"][l] if train else None, H=bf["H"][l],
                       HT=bf["HT"][l] if train else None, ldht=ldt)
            x, kx = bf["H"][l], w
        _lib.check(self.lib.dmsim_mlp_head(
            x.data_ptr(), B, w, self.w_head.data_ptr(), self.b_head.data_ptr(),
            bf["y"].data_ptr(), bf["t"].data_ptr() if train else None,
            bf["dy"].data_ptr() if train else None, bf["sqerr"].data_ptr() if train else None,
            bf["P"][-1].data_ptr() if train else None,
            bf["dP"][-1].data_ptr() if train else None,
            bf["dPT"][-1].data_ptr() if train else None, ldt, s), "dmsim_mlp_head")

    def _backward_into(self, bf):
        s = _lib.stream_handle()
        B, w, ldt, splits = bf["B"], self.width, bf["ldt"], bf["splits"]
        for l in range(self.depth - 1, -1, -1):
            Kl = self.W[l].shape[1]
            xT = bf["X0T"] if l == 0 else bf["HT"][l - 1]
            self._gemm(bf["dPT"][l], ldt, xT, ldt, w, Kl, B, _lib.EPI_STORE_F32, splits=splits,
                       C=bf["dW"][l])
            _lib.check(self.lib.dmsim_rowdot_bf16(bf["dPT"][l].data_ptr(), w, B, ldt, None,
                                                  bf["db"][l].data_ptr(), s), "rowdot")
            if l > 0:
                self._gemm(bf["dP"][l], w, self.WTb[l], w, B, Kl, w, _lib.EPI_GELU_BWD,
                           P=bf["P"][l - 1], H=bf["dP"][l - 1], HT=bf["dPT"][l - 1], ldht=ldt)
        _lib.check(self.lib.dmsim_rowdot_bf16(bf["HT"][-1].data_ptr(), w, B, ldt,
                                              bf["dy"].data_ptr(), bf["dw_head"].data_ptr(), s),
                   "rowdot")
        _lib.check(self.lib.dmsim_sum_f32(bf["dy"].data_ptr(), B, bf["db_head"].data_ptr(), s),
                   "sum")
        _lib.check(self.lib.dmsim_sum_f32(bf["sqerr"].data_ptr(), B, bf["loss"].data_ptr(), s),
                   "sum")

    def _update(self, bf):
        s = _lib.stream_handle()
        lib, hp = self.lib, self.hp.data_ptr()
        _lib.check(lib.dmsim_adam_advance(hp, s), "adam_advance")
        nl = self.depth
        for l in range(nl):
            W = self.W[l]
            _lib.check(lib.dmsim_adamw(
                W.data_ptr(), self.m[l].data_ptr(), self.v[l].data_ptr(), bf["dW"][l].data_ptr(),
                bf["splits"], W.numel(), W.shape[1], hp, self.Wb[l].data_ptr(),
                self.WTb[l].data_ptr(), W.shape[0], s), "adamw")
            b = self.b[l]
            _lib.check(lib.dmsim_adamw(
                b.data_ptr(), self.m[nl + l].data_ptr(), self.v[nl + l].data_ptr(),
                bf["db"][l].data_ptr(), 1, b.numel(), b.numel(), hp, None, None, 1, s), "adamw")
        for p, m, v, g in ((self.w_head, self.m[2 * nl], self.v[2 * nl], bf["dw_head"]),
                           (self.b_head, self.m[2 * nl + 1], self.v[2 * nl + 1], bf["db_head"])):
            _lib.check(lib.dmsim_adamw(p.data_ptr(), m.data_ptr(), v.data_ptr(), g.data_ptr(), 1,
                                       p.numel(), p.numel(), hp, None, None, 1, s), "adamw")

    # ---- public -------------------------------------------------------------------------------
    def fused(self):
        """Whether :meth:`predict` runs the one-launch forward pass (width 256, up to 128
        inputs, up to 8 layers)."""
        return self.width == 256 and self.kp == 128 and self.depth <= 8

    def predict(self, x, chunk=1 << 20):
        """y (B,) for inputs x (B, n_in) (numpy or tensor, fp32): the fused forward pass
        (``dmsim_mlp_forward``: one launch, activations on chip) when the shape allows, else the
        layer-by-layer GEMMs."""
        x = torch.as_tensor(np.asarray(x, np.float32) if not torch.is_tensor(x) else x)
        x = x.to(self.dev, torch.float32)
        if self.fused():
            return self.predict_fused(x)
        return self.predict_layers(x, chunk)

    def predict_fused(self, x, out=None):
        """The one-launch forward pass on a contiguous fp32 device tensor x (B, n_in)."""
        x = x.contiguous()
        y = torch.empty(len(x), device=self.dev) if out is None else out
        f = _lib.MlpFwd()
        f.x, f.rows, f.n_in, f.depth = x.data_ptr(), len(x), self.n_in, self.depth
        f.shift, f.scale = self.shift.data_ptr(), self.scale.data_ptr()
        for l in range(self.depth):
            f.W[l] = self.Wb[l].data_ptr()
            f.bias[l] = self.b[l].data_ptr()
        f.w_head, f.b_head = self.w_head.data_ptr(), self.b_head.data_ptr()
        f.y, f.err = y.data_ptr(), self.err.data_ptr()
        _lib.check(self.lib.dmsim_mlp_forward(ctypes.byref(f), _lib.stream_handle()),
                   "dmsim_mlp_forward")
        return y

    def predict_layers(self, x, chunk=1 << 20):
        """The forward pass as layer-by-layer tensor-core GEMMs (the training path)."""
        x = torch.as_tensor(np.asarray(x, np.float32) if not torch.is_tensor(x) else x)
        x = x.to(self.dev, torch.float32)
        out = torch.empty(len(x), device=self.dev)
        for s0 in range(0, len(x), chunk):
            xs = x[s0:s0 + chunk]
            bf = self._buffers(len(xs), False)
            bf["x"].copy_(xs)
            self._forward_into(bf, False)
            out[s0:s0 + len(xs)] = bf["y"]
        return out

    def forward_cached(self, x):
        """Forward with the training cache kept (for gradient checks): returns the buffers."""
        bf = self._buffers(len(x), True)
        bf["x"].copy_(torch.as_tensor(x, dtype=torch.float32, device=self.dev))
        self._forward_into(bf, True)
        return bf

    def gradients(self, x, t):
        """Forward + backward on one batch without an update; returns the buffers (dW partials
        per split, db, dw_head, db_head, loss)."""
        bf = self._buffers(len(x), True)
        bf["x"].copy_(torch.as_tensor(x, dtype=torch.float32, device=self.dev))
        bf["t"].copy_(torch.as_tensor(t, dtype=torch.float32, device=self.dev))
        self._forward_into(bf, True)
        self._backward_into(bf)
        return bf

    def step_launch(self, bf):
        """One training step on the batch already in bf['x'], bf['t'] (capturable)."""
        self._forward_into(bf, True)
        self._backward_into(bf)
        self._update(bf)

    def capture_step(self, B):
        """Record a training step on a B-row batch as a CUDA graph; returns the buffers whose
        'x' and 't' the caller fills before each replay."""
        bf = self._buffers(B, True)
        bf["x"].zero_()
        bf["t"].zero_()
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        hp0 = self.hp.clone()
        state = [p.clone() for p in self.W + self.b + [self.w_head, self.b_head]]
        with torch.cuda.stream(side):   # warm-up outside capture (attribute setup, tensor maps)
            self.step_launch(bf)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        torch.cuda.synchronize(self.dev)
        # undo the warm-up step
        for p, s0 in zip(self.W + self.b + [self.w_head, self.b_head], state):
            p.copy_(s0)
        for t in self.m + self.v:
            t.zero_()
        self.hp.copy_(hp0)
        self.refresh_bf16()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.step_launch(bf)
        self._graph_bufs = bf
        return bf

    def train_step(self, x, t):
        """One AdamW step on (x, t); returns the batch loss as a device tensor (sum of squared
        errors / B)."""
        B = len(x)
        if self.graph is not None and self._graph_bufs["B"] == B:
            bf = self._graph_bufs
            bf["x"].copy_(x, non_blocking=True)
            bf["t"].copy_(t, non_blocking=True)
            self.graph.replay()
        else:
            bf = self._buffers(B, True)
            bf["x"].copy_(x)
            bf["t"].copy_(t)
            self.step_launch(bf)
        return bf["loss"] / B

    def launches_per_step(self):
        d = self.depth
        return 1 + d + 1 + (2 * d - 1) + d + 1 + 2 + 1 + (2 * d + 2)

    def check_errors(self):
        n = int(self.err.item())
        if n:
            raise RuntimeError(f"{n} GEMM tile(s) gave up waiting (tensor-core pipeline stalled)")
