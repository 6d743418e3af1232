"""Compressed walk representations: the replay representation of a walk, compressed
(compression.py of dmipy-sim).

A walk's replay observables are linear functionals of its trajectories, which compress along two
redundancies:

* temporal -- a deliverable gradient waveform is band-limited, so ``temporal_dct`` keeps the
  lowest ``K`` orthonormal DCT-II bands of every path (walker-preserving; lossless for any
  acquisition inside the band);
* ensemble -- walkers are exchangeable: ``lowrank`` keeps ``K`` Karhunen-Loeve modes with exact
  per-walker coefficients (walker-preserving); ``gaussian`` / ``marginal`` keep only the
  coefficient distribution and resample it at replay (gradient replay only).

The per-walker physics channels have their own codecs: run-length rows for compartment labels and
bound fractions, sparse/dense quantisation or the detrended cumulative DCT for the boundary local
time.  ``mode_space_phi`` / ``mode_space_signal`` replay straight from the compressed basis.

On the GPU: the temporal projections (``encode_temporal_dct``, ``encode_boundary_dct``, the
compressed trajectory export) run ``dmsim_project_modes`` and the mode-space and fidelity replays
run ``dmsim_replay``; the Karhunen-Loeve factorisations, run-length codecs and inverse DCTs are
host numpy, as in the reference.
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.fft import dct as _dct
from scipy.fft import idct as _idct

from . import _lib
from .constants import GAMMA

WALKER_PRESERVING = ("temporal_dct", "lowrank")
DISTRIBUTIONAL = ("gaussian", "marginal")
ALL_METHODS = WALKER_PRESERVING + DISTRIBUTIONAL
POSITION_AXES = ("pos_x", "pos_y", "pos_z")
_F16, _F32 = 2, 4


# ------------------------------------------------------------------ the device projection
def dct_basis(n_t, K):
    """The first ``K`` orthonormal DCT-II basis rows (K, n_t), float64: ``basis @ x`` equals
    ``scipy.fft.dct(x, type=2, norm="ortho")[:K]`` (core.py:1383-1387)."""
    K = min(int(K), int(n_t))
    return _dct(np.eye(int(n_t)), type=2, norm="ortho", axis=0)[:K]


def _device_series(x, n_ch):
    dev = _lib.device()
    t = x if torch.is_tensor(x) else torch.from_numpy(np.ascontiguousarray(x))
    if t.dtype not in (torch.float16, torch.float32):
        t = t.to(torch.float32)
    t = t.to(dev).contiguous()
    if t.dim() == 2:
        t = t.unsqueeze(-1)
    if t.dim() != 3 or t.shape[2] != n_ch:
        raise ValueError(f"expected a (n_walkers, n_t, {n_ch}) series, got {tuple(x.shape)}")
    return t


def project_modes(x, K, *, cumulative=False):
    """DCT-II bands of per-walker series on the GPU (``dmsim_project_modes``).

    ``x`` (n_walkers, n_t, 3) or (n_walkers, n_t) -- numpy or a CUDA tensor, float16/float32.
    Returns a CUDA float32 tensor (n_walkers, K, n_ch).  ``cumulative`` (one channel): the
    detrended running sum B_t - B_T t/T is projected instead and ``(endpoint B_T, modes)`` is
    returned (the boundary-local-time codec, compression.py:224-249)."""
    lib = _lib.load()
    n_ch = 1 if (x.ndim == 2 or cumulative) else int(x.shape[2])
    xt = _device_series(x, n_ch)
    n_w, n_t, _ = xt.shape
    basis = torch.from_numpy(dct_basis(n_t, K).astype(np.float32)).to(xt.device)
    Kc = int(basis.shape[0])
    out = torch.empty((n_w, Kc, n_ch), dtype=torch.float32, device=xt.device)
    ramp = end = None
    if cumulative:
        ramp = torch.linspace(0.0, 1.0, n_t, dtype=torch.float32, device=xt.device)
        end = torch.empty(n_w, dtype=torch.float32, device=xt.device)
    if n_w:
        rc = lib.dmsim_project_modes(_lib.ptr(xt), 1 if xt.dtype == torch.float16 else 0, n_w,
                                     n_t, n_ch, _lib.ptr(basis), Kc, _lib.ptr(ramp),
                                     _lib.ptr(end), _lib.ptr(out), _lib.stream_handle())
        _lib.check(rc, "dmsim_project_modes")
    if cumulative:
        return end, out[:, :, 0]
    return out


def _replay_sums(series, G, gamma_dt, log_w=None, want_phi=False):
    """``dmsim_replay`` of a (n, n_t, 3) series against G (n_meas, n_t, 3): the per-walker phase
    phi = gamma_dt sum_t G . r and the sums (sum e^lw cos phi, sum e^lw sin phi, ...)."""
    lib = _lib.load()
    dev = _lib.device()
    tr = _device_series(series, 3)
    n_w, n_t, _ = tr.shape
    G = np.asarray(G, np.float64)
    n_meas = G.shape[0]
    Gd = torch.from_numpy(np.ascontiguousarray(G.transpose(1, 0, 2)).astype(np.float32)).to(dev)
    lw = None if log_w is None else torch.from_numpy(
        np.ascontiguousarray(log_w, np.float32)).to(dev)
    sums = torch.zeros((n_meas, 3), dtype=torch.float64, device=dev)
    phi = torch.empty((n_w, n_meas), dtype=torch.float32, device=dev) if want_phi else None
    nbytes = lib.dmsim_replay_workspace_bytes(n_w, n_t, n_meas)
    ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
    rc = lib.dmsim_replay(_lib.ptr(tr), 1 if tr.dtype == torch.float16 else 0, n_w, n_t,
                          _lib.ptr(Gd), n_meas, np.float32(gamma_dt), _lib.ptr(lw),
                          _lib.ptr(sums), _lib.ptr(phi), _lib.ptr(ws), nbytes,
                          _lib.stream_handle())
    _lib.check(rc, "dmsim_replay")
    return sums.cpu().numpy(), (None if phi is None else phi.cpu().numpy().astype(np.float64))


# --------------------------------------------------------------------------------- encoders
def encode_temporal_dct(X, K):
    """Lowest ``K`` orthonormal DCT-II bands of each path, per axis (compression.py:54-62):
    ``(arrays, meta, nbytes)`` with the axis-per-tensor position layout."""
    n_w, n_t, _ = X.shape
    C = project_modes(X, K).cpu().numpy()
    arrays = pack_position_arrays(C, np.float32)
    meta = {"method": "temporal_dct", "K": int(C.shape[1]), "n_t": int(n_t)}
    return arrays, meta, n_w * 3 * int(C.shape[1]) * _F16


def _kl(X):
    """Karhunen-Loeve factorisation of the flattened paths (compression.py:65-70)."""
    n_w, n_t, _ = X.shape
    Xf = np.asarray(X, np.float64).reshape(n_w, 3 * n_t)
    mean = Xf.mean(0, keepdims=True)
    U, s, Vt = np.linalg.svd(Xf - mean, full_matrices=False)
    return Xf, mean, U, s, Vt, n_t


def encode_lowrank(X, K, _cache=None):
    """``K`` KL modes + exact per-walker coefficients (compression.py:73-82)."""
    Xf, mean, U, s, Vt, n_t = _cache or _kl(X)
    K = min(int(K), s.shape[0])
    A = U[:, :K] * s[:K]
    arrays = {"modes": Vt[:K].astype(np.float32), "mean": mean[0].astype(np.float32),
              "coeffs": A.astype(np.float16)}
    meta = {"method": "lowrank", "K": int(K), "n_t": int(n_t)}
    return arrays, meta, X.shape[0] * K * _F16 + K * 3 * n_t * _F16 + 3 * n_t * _F16


def encode_gaussian(X, K, _cache=None):
    """``K`` KL modes + the Gaussian (mean, covariance) of the coefficients (compression.py:85-96)."""
    Xf, mean, U, s, Vt, n_t = _cache or _kl(X)
    K = min(int(K), s.shape[0])
    A = U[:, :K] * s[:K]
    cov = np.cov(A, rowvar=False) if K > 1 else np.array([[A.var()]])
    arrays = {"modes": Vt[:K].astype(np.float32), "mean": mean[0].astype(np.float32),
              "coeff_mean": A.mean(0).astype(np.float32), "coeff_cov": cov.astype(np.float32)}
    meta = {"method": "gaussian", "K": int(K), "n_t": int(n_t), "n_walkers": int(X.shape[0])}
    return arrays, meta, (K * 3 * n_t + K * K + 3 * n_t) * _F32


def encode_marginal(X, K, Q=256, _cache=None):
    """``K`` KL modes + ``Q`` quantiles of every coefficient's marginal (compression.py:99-110)."""
    Xf, mean, U, s, Vt, n_t = _cache or _kl(X)
    K = min(int(K), s.shape[0])
    A = U[:, :K] * s[:K]
    arrays = {"modes": Vt[:K].astype(np.float32), "mean": mean[0].astype(np.float32),
              "coeff_quantiles": np.quantile(A, np.linspace(0, 1, Q), axis=0).astype(np.float32)}
    meta = {"method": "marginal", "K": int(K), "n_t": int(n_t), "Q": int(Q),
            "n_walkers": int(X.shape[0])}
    return arrays, meta, (K * 3 * n_t + K * Q + 3 * n_t) * _F32


ENCODERS = {"temporal_dct": encode_temporal_dct, "lowrank": encode_lowrank,
            "gaussian": encode_gaussian, "marginal": encode_marginal}


def encode(X, method="temporal_dct", K=32, **kw):
    if method not in ENCODERS:
        raise ValueError(f"unknown method {method!r}; choose from {list(ENCODERS)}")
    return ENCODERS[method](X, K, **kw)


# ------------------------------------------------------------------ run-length row coding
def rle_encode_rows(A):
    """Row-wise run-length code of a piecewise-constant integer matrix (n_w, n_t) as flat
    (values int16, lengths int32, runs per row int32, n_t) (compression.py:117-128)."""
    A = np.asarray(A)
    n_w, n_t = A.shape
    if n_w == 0:
        return (np.zeros(0, np.int16), np.zeros(0, np.int32), np.zeros(0, np.int32), int(n_t))
    change = np.ones((n_w, n_t), bool)
    change[:, 1:] = A[:, 1:] != A[:, :-1]
    rows, starts = np.nonzero(change)                     # row-major: runs in order
    counts = np.bincount(rows, minlength=n_w).astype(np.int32)
    nxt = np.empty_like(starts)
    nxt[:-1] = starts[1:]
    last = np.ones(len(starts), bool)
    last[:-1] = rows[1:] != rows[:-1]
    nxt[last] = n_t
    return (A[rows, starts].astype(np.int16), (nxt - starts).astype(np.int32), counts, int(n_t))


def rle_decode_rows(vals, lens, counts, n_t):
    """Inverse of :func:`rle_encode_rows` (compression.py:131-135): (n_w, n_t) int16."""
    vals = np.asarray(vals)
    lens = np.asarray(lens, np.int64)
    counts = np.asarray(counts, np.int64)
    flat = np.repeat(vals, lens)
    return flat.reshape(counts.size, int(n_t)).astype(np.int16)


# ------------------------------------------------------------ per-walker channel codecs
def encode_bound_fraction(bfrac, Q=256):
    """Bound fraction in [0, 1] quantised to Q levels, run-length coded (compression.py:139-148)."""
    q = np.rint(np.clip(np.asarray(bfrac, np.float64), 0.0, 1.0) * (Q - 1)).astype(np.int32)
    vals, lens, counts, n_t = rle_encode_rows(q)
    arrays = {"bfrac_rle_vals": vals.astype(np.uint8 if Q <= 256 else np.int32),
              "bfrac_rle_lens": lens.astype(np.uint16 if n_t < 65535 else np.int32),
              "bfrac_rle_counts": np.asarray(counts, np.int32)}
    return arrays, {"channel": "bound_fraction", "Q": int(Q), "n_t": int(n_t)}


def decode_bound_fraction(arrays, meta):
    q = rle_decode_rows(arrays["bfrac_rle_vals"], arrays["bfrac_rle_lens"],
                        arrays["bfrac_rle_counts"], int(meta["n_t"]))
    return q.astype(np.float32) / float(meta["Q"] - 1)


def encode_boundary_local_time(dlog, nlevels=4096):
    """Per-step boundary local time, sparse CSR when that is smaller than dense int8, each
    quantised against the largest |value| (compression.py:158-187)."""
    A = np.asarray(dlog, np.float64)
    n_w, n_t = A.shape
    scale = float(np.abs(A).max()) + 1e-30
    nz_r, nz_c = np.nonzero(A)
    if len(nz_r) * 4 + n_w * 4 <= n_w * n_t:
        arrays = {"blt_counts": np.bincount(nz_r, minlength=n_w).astype(np.int32),
                  "blt_cols": nz_c.astype(np.int16 if n_t <= 32000 else np.int32),
                  "blt_qvals": np.rint(A[nz_r, nz_c] / scale * (nlevels - 1)).astype(
                      np.int16 if nlevels <= 32000 else np.int32)}
        return arrays, {"channel": "boundary_local_time", "mode": "sparse", "n_t": int(n_t),
                        "scale": scale, "nlevels": int(nlevels)}
    q = np.rint(np.clip(A / scale, -1.0, 1.0) * 127.0).astype(np.int8)
    return {"blt_dense_q": q}, {"channel": "boundary_local_time", "mode": "dense",
                                "n_t": int(n_t), "scale": scale, "nlevels": 127}


def decode_boundary_local_time(arrays, meta):
    n_t, scale, nl = int(meta["n_t"]), float(meta["scale"]), int(meta["nlevels"])
    if meta.get("mode") == "dense" or "blt_dense_q" in arrays:
        return (np.asarray(arrays["blt_dense_q"], np.float64) * scale / nl).astype(np.float32)
    counts = np.asarray(arrays["blt_counts"], np.int64)
    cols = np.asarray(arrays["blt_cols"], np.int64)
    q = np.asarray(arrays["blt_qvals"], np.float64)
    out = np.zeros((counts.size, n_t), np.float32)
    rows = np.repeat(np.arange(counts.size), counts)
    out[rows, cols] = (q * scale / (nl - 1)).astype(np.float32)
    return out


def encode_boundary_dct(dlog, K=16, dtype=np.float32):
    """Cumulative boundary local time B(t), detrended by its exact endpoint, in ``K`` DCT-II bands
    (compression.py:210-238); the projection runs on the GPU."""
    n_w, n_t = np.shape(dlog)[:2]
    end, C = project_modes(dlog, K, cumulative=True)
    arrays = {"blt_dct_coeffs": C.cpu().numpy().astype(dtype),
              "blt_endpoint": end.cpu().numpy().astype(np.float32)}
    meta = {"channel": "boundary_local_time", "mode": "dct", "n_t": int(n_t),
            "K": int(C.shape[1]), "dtype": np.dtype(dtype).name}
    return arrays, meta


def decode_boundary_dct(arrays, meta):
    """Per-save increments ell(t) = diff(B) of the reconstructed cumulative local time
    (compression.py:241-249)."""
    n_t = int(meta["n_t"])
    C = np.asarray(arrays["blt_dct_coeffs"], np.float64)
    end = np.asarray(arrays["blt_endpoint"], np.float64)
    B = _idct(C, axis=1, type=2, norm="ortho", n=n_t) + end[:, None] * np.linspace(0.0, 1.0, n_t)
    return np.diff(B, axis=1, prepend=np.zeros((B.shape[0], 1))).astype(np.float32)


def encode_compartment(comp, Q=256):
    """Integer labels: lossless run-length rows; fractional occupancy: quantised to Q levels
    over [0, max] then run-length rows (compression.py:252-271)."""
    A = np.asarray(comp)
    if np.array_equal(A, np.round(A)):
        vals, lens, counts, n_t = rle_encode_rows(A.astype(np.int32))
        return ({"comp_rle_vals": vals.astype(np.int16), "comp_rle_lens": lens.astype(np.int32),
                 "comp_rle_counts": np.asarray(counts, np.int32)},
                {"channel": "compartment", "fractional": False, "n_t": int(n_t)})
    scale = float(np.nanmax(np.abs(A))) or 1.0
    q = np.rint(np.clip(A, 0.0, scale) / scale * (Q - 1)).astype(np.int32)
    vals, lens, counts, n_t = rle_encode_rows(q)
    return ({"comp_rle_vals": vals.astype(np.uint8 if Q <= 256 else np.int32),
             "comp_rle_lens": lens.astype(np.uint16 if n_t < 65535 else np.int32),
             "comp_rle_counts": np.asarray(counts, np.int32)},
            {"channel": "compartment", "fractional": True, "Q": int(Q), "scale": scale,
             "n_t": int(n_t)})


def decode_compartment(arrays, meta):
    q = rle_decode_rows(arrays["comp_rle_vals"], arrays["comp_rle_lens"],
                        arrays["comp_rle_counts"], int(meta["n_t"]))
    if meta.get("fractional"):
        return q.astype(np.float32) / float(meta["Q"] - 1) * float(meta.get("scale", 1.0))
    return q.astype(np.int16)


# Codec of each per-walker channel, by the channel name the pack metadata records.
_CHANNELS = (
    ("bound_fraction", encode_bound_fraction, decode_bound_fraction),
    ("boundary_local_time", encode_boundary_local_time, decode_boundary_local_time),
    ("boundary_dct", encode_boundary_dct, decode_boundary_dct),
    ("compartment", encode_compartment, decode_compartment),
)
CHANNEL_ENCODERS = {name: enc for name, enc, _ in _CHANNELS}
CHANNEL_DECODERS = {name: dec for name, _, dec in _CHANNELS}


# ------------------------------------------------------------------ position layout
def pack_position_arrays(C, dtype=np.float32):
    """(n_w, K, 3) coefficients -> one (n_w, K) tensor per axis, ``pos_x/pos_y/pos_z``: an axis
    subset and a walker prefix are then contiguous reads (compression.py:372-377)."""
    C = np.asarray(C)
    return {POSITION_AXES[i]: np.ascontiguousarray(C[:, :, i]).astype(dtype)
            for i in range(C.shape[2])}


def has_axis_layout(arrays):
    return POSITION_AXES[0] in arrays


def read_position_coeffs(arrays, axes=None, dtype=np.float64):
    """Coefficients (n_w, K, n_axes) from the axis-per-tensor layout; ``axes`` selects axes by
    index.  A pack without that layout is an error, not a guess (compression.py:384-410)."""
    if not has_axis_layout(arrays):
        raise KeyError(f"pack has no position axes {POSITION_AXES}; found {sorted(arrays)}. "
                       "Re-encode (n_walkers, K, 3) coefficients with pack_position_arrays(); "
                       "mixed position layouts are not read.")
    present = [i for i, k in enumerate(POSITION_AXES) if k in arrays]
    want = list(present if axes is None else axes)
    missing = [i for i in want if i not in present]
    if missing:
        raise KeyError(f"pack does not carry position axes {missing} "
                       f"(has {[POSITION_AXES[i] for i in present]})")
    return np.stack([np.asarray(arrays[POSITION_AXES[i]], dtype) for i in want], axis=2)


def is_walker_preserving(method):
    return method in WALKER_PRESERVING


def _stored_coeffs(arrays, meta, n, rng):
    A = np.asarray(arrays["coeffs"], np.float64)
    if n is not None and n != A.shape[0]:
        raise ValueError("lowrank preserves its stored walker count only")
    return A


def _gaussian_coeffs(arrays, meta, n, rng):
    """n draws of the stored coefficient Gaussian: mean + Z L^T, L the Cholesky factor of the
    covariance (a 1e-30 ridge keeps it positive definite), Z standard normal (n, K)."""
    cov = np.asarray(arrays["coeff_cov"], np.float64)
    chol = np.linalg.cholesky(cov + 1e-30 * np.eye(cov.shape[0]))
    z = rng.standard_normal((n, cov.shape[0]))
    return z @ chol.T + np.asarray(arrays["coeff_mean"], np.float64)


def _marginal_coeffs(arrays, meta, n, rng):
    """n draws of independent coefficients, each through its stored quantile table (inverse-CDF
    sampling with linear interpolation between equally spaced probabilities)."""
    table = np.asarray(arrays["coeff_quantiles"], np.float64)
    probs = np.linspace(0.0, 1.0, table.shape[0])
    u = rng.random((n, table.shape[1]))
    out = np.empty_like(u)
    for k in range(table.shape[1]):
        out[:, k] = np.interp(u[:, k], probs, table[:, k])
    return out


_COEFF_SOURCES = {"lowrank": _stored_coeffs, "gaussian": _gaussian_coeffs,
                  "marginal": _marginal_coeffs}


def _sample_coeffs(arrays, meta, n_walkers=None, seed=0):
    """Per-walker Karhunen-Loeve coefficients (n, K): the stored ones of a walker-preserving pack,
    or n draws (default: the recorded walker count, else 100,000) from the coefficient
    distribution of a distributional one, from numpy's generator seeded with ``seed`` (the
    decode contract of compression.py:290-306)."""
    method = meta["method"]
    if method not in _COEFF_SOURCES:
        raise ValueError(f"unknown method {method!r}")
    n = n_walkers
    if method != "lowrank":
        n = n_walkers or int(meta.get("n_walkers", 100_000))
    return _COEFF_SOURCES[method](arrays, meta, n, np.random.default_rng(seed))


def decode(arrays, meta, n_walkers=None, seed=0):
    """Positions (n_walkers, n_t, 3) float64 from stored arrays (compression.py:413-423)."""
    n_t = int(meta["n_t"])
    if meta["method"] == "temporal_dct":
        return _idct(read_position_coeffs(arrays), axis=1, type=2, norm="ortho",
                     n=n_t).astype(np.float64)
    modes = np.asarray(arrays["modes"], np.float64)
    mean = np.asarray(arrays.get("mean", np.zeros(modes.shape[1])), np.float64)
    X = _sample_coeffs(arrays, meta, n_walkers, seed) @ modes + mean
    return X.reshape(X.shape[0], n_t, 3)


# ---------------------------------------------------------------------- mode-space replay
def mode_space_phi(arrays, meta, G, dt, n_walkers=None, seed=0):
    """Phase phi (n_w, n_meas) straight from the compressed basis (compression.py:431-453).

    ``temporal_dct``: phi = gamma dt sum_{k,d} C_kd DCT(G)_kd over the stored bands, one
    ``dmsim_replay`` pass over the (n_w, K, 3) coefficients on the GPU.  KL methods:
    phi = A c(G) + phi0 with c(G) = gamma dt V vec(G) (host)."""
    G = np.asarray(G, np.float64)
    n_meas = G.shape[0]
    if meta.get("method", "temporal_dct") == "temporal_dct":
        C = read_position_coeffs(arrays, dtype=np.float32)
        Ghat = _dct(G, axis=1, type=2, norm="ortho")[:, :C.shape[1], :]
        _, phi = _replay_sums(C, Ghat, GAMMA * dt, want_phi=True)
        return phi
    Gf = G.reshape(n_meas, -1)
    modes = np.asarray(arrays["modes"], np.float64)
    mean = np.asarray(arrays.get("mean", np.zeros(modes.shape[1])), np.float64)
    A = _sample_coeffs(arrays, meta, n_walkers, seed)
    return A @ ((GAMMA * dt) * (modes @ Gf.T)) + ((GAMMA * dt) * (Gf @ mean))[None, :]


def mode_space_signal(arrays, meta, G, dt, logw=None, weights=None, n_walkers=None, seed=0):
    """Complex signal <w e^(logw + i phi)> / <w> (n_meas,) from the compressed basis
    (compression.py:456-465)."""
    if meta.get("method", "temporal_dct") == "temporal_dct":
        C = read_position_coeffs(arrays, dtype=np.float32)
        n_w = C.shape[0]
        w = np.ones(n_w) if weights is None else np.asarray(weights, np.float64)
        lw = (np.zeros(n_w) if logw is None else np.asarray(logw, np.float64))
        Ghat = _dct(np.asarray(G, np.float64), axis=1, type=2, norm="ortho")[:, :C.shape[1], :]
        with np.errstate(divide="ignore"):
            sums, _ = _replay_sums(C, Ghat, GAMMA * dt, log_w=lw + np.log(w))
        return (sums[:, 0] + 1j * sums[:, 1]) / w.sum()
    phi = mode_space_phi(arrays, meta, G, dt, n_walkers=n_walkers, seed=seed)
    n_w = phi.shape[0]
    lw = np.zeros(n_w) if logw is None else np.asarray(logw, float)
    w = np.ones(n_w) if weights is None else np.asarray(weights, float)
    return (np.exp(lw[:, None] + 1j * phi) * (w / w.sum())[:, None]).sum(0)


def _rates(times):
    """1 / T per compartment, 0 where T <= 0 (no relaxation)."""
    T = np.asarray(times, float)
    return np.where(T > 0, 1.0 / np.maximum(T, 1e-30), 0.0)


def relaxation_logweight(comp, T2_per_comp, T1_per_comp, dt, chi=None):
    """Bulk-relaxation log-weight per walker, -dt sum_t [chi_t R2(c_t) + (1 - chi_t) R1(c_t)]
    (chi = 1 throughout without a coherence mask), from the compartment channel (the contract of
    compression.py:468-485): integer labels index the per-compartment rates; a fractional
    channel is the occupancy f of compartment 1 and mixes the rates of compartments 0 and 1 as
    (1 - f) R(0) + f R(1)."""
    comp = np.asarray(comp)
    r2, r1 = _rates(T2_per_comp), _rates(T1_per_comp)
    fractional = np.issubdtype(comp.dtype, np.floating) and not np.array_equal(comp,
                                                                                np.round(comp))
    if fractional:
        f = np.clip(comp, 0.0, 1.0)
        rate2 = r2[0] + f * (r2[1] - r2[0])
        rate1 = r1[0] + f * (r1[1] - r1[0])
    else:
        idx = comp.astype(np.int64)
        rate2, rate1 = r2[idx], r1[idx]
    if chi is None:
        return -dt * np.sum(rate2, axis=1)
    c = np.asarray(chi, float)
    return -dt * (rate2 @ c + rate1 @ (1.0 - c))


def surface_logweight(blt, rho_over_D, chi=None):
    """Surface-relaxation log-weight per walker, (rho / D) sum_t chi_t ell_t, from the boundary
    channel ell stored at rho / D = 1 (compression.py:488-493)."""
    ell = np.asarray(blt, np.float64)
    total = ell.sum(axis=1) if chi is None else ell @ np.asarray(chi, float)
    return float(rho_over_D) * total


# ------------------------------------------------------------------ envelope and fidelity
# The acquisition envelope a pack is certified over (b in s/m^2): PGSE at these b-values and
# directions, cosine OGSE of these period counts, short-delta PGSE at shortd_b; lobe timings as
# fractions of the walk's duration.  These values are part of the pack format (they fix what a
# pack's fidelity record means) and equal the reference's defaults.
_DEFAULT_ENVELOPE = dict(bvals=(0.0, 0.5e9, 1e9, 2e9, 3e9),
                         dirs=((0, 0, 1), (1, 0, 0), (1, 0, 1)),
                         ogse_periods=(1, 2, 3, 5), shortd_b=1e9,
                         shortd_deltas_frac=(0.2, 0.1, 0.05, 0.025),
                         delta_frac=0.2, Delta_frac=0.5)


def default_envelope():
    """A fresh copy of the default certification envelope (compression.py:497-503)."""
    return {k: ([list(x) if isinstance(x, tuple) else x for x in v] if isinstance(v, tuple)
                else v) for k, v in _DEFAULT_ENVELOPE.items()}


def _bipolar(t, delta, Delta):
    return (t < delta).astype(float) - ((t >= Delta) & (t < Delta + delta)).astype(float)


def acquisition_battery(n_t, dt, env):
    """Refocused test waveforms G (M, n_t, 3) float32 and per-measurement metadata: PGSE over
    the envelope's b-values and directions, cosine OGSE of each period count, short-delta PGSE
    (compression.py:510-536).  Each profile is scaled to its b-value by the left-point q."""
    t = np.arange(n_t) * dt
    T = n_t * dt
    G, meta = [], []

    def add(prof, fam, d, b, **extra):
        q = GAMMA * dt * np.cumsum(prof)
        b_unit = dt * np.sum(q ** 2)
        amp = 0.0 if b <= 0 else np.sqrt(b / b_unit)
        dv = np.asarray(d, float)
        dv = dv / np.linalg.norm(dv)
        G.append(amp * prof[:, None] * dv[None, :])
        meta.append(dict(fam=fam, b=float(b), Gpeak=abs(amp), **extra))

    pgse = _bipolar(t, env["delta_frac"] * T, env["Delta_frac"] * T)
    for d in env["dirs"]:
        for b in env["bvals"]:
            add(pgse, "PGSE", d, b, f_hz=1.0 / (2 * env["delta_frac"] * T))
    for nper in env["ogse_periods"]:
        prof = np.cos(2 * np.pi * nper * t / T)
        for d in env["dirs"]:
            for b in env["bvals"]:
                add(prof, f"OGSE{nper}", d, b, f_hz=nper / T)
    for fr in env["shortd_deltas_frac"]:
        delta = fr * T
        Delta = min(0.55 * T, T - delta - dt)
        prof = _bipolar(t, delta, Delta)
        for d in env["dirs"]:
            add(prof, "SHORTD", d, env["shortd_b"], f_hz=1.0 / (2 * delta))
    return np.asarray(G, np.float32), meta


class _DeviceReplay:
    """One upload of a (n_w, n_t, 3) series, replayed against a waveform set as often as needed:
    complex <w e^lw e^(i phi)> over all walkers or over a subset (the rest weighted out)."""

    def __init__(self, series, dt, G):
        self.tr = _device_series(series, 3)
        self.gdt = GAMMA * float(dt)
        self.G = np.asarray(G, np.float64)

    def signal(self, w=None, logw=None, subset=None):
        n_w = self.tr.shape[0]
        ww = np.ones(n_w) if w is None else np.asarray(w, np.float64)
        lw = np.zeros(n_w) if logw is None else np.asarray(logw, np.float64)
        if subset is not None:
            keep = np.zeros(n_w, bool)
            keep[subset] = True
            ww = np.where(keep, ww, 0.0)
        with np.errstate(divide="ignore"):
            sums, _ = _replay_sums(self.tr, self.G, self.gdt, log_w=lw + np.log(ww))
        return (sums[:, 0] + 1j * sums[:, 1]) / ww.sum()


def measure_fidelity(traj, dt_traj, decoded_pos, env=None, w=None, logw=None):
    """Largest complex replay error of the decoded positions against the raw ones per acquisition
    family, with the split-half Monte-Carlo floor of the raw walk (compression.py:551-579)."""
    env = env or default_envelope()
    n_w, n_t = traj.shape[0], traj.shape[1]
    G, meta = acquisition_battery(n_t, float(dt_traj), env)
    raw = _DeviceReplay(traj, dt_traj, G)
    S_raw = raw.signal(w, logw)
    S_dec = _DeviceReplay(decoded_pos, dt_traj, G).signal(w, logw)
    return _fidelity_report(raw, S_raw, S_dec, meta, n_w, w, logw)


def _fidelity_report(raw, S_raw, S_dec, meta, n_w, w, logw):
    idx = np.random.default_rng(0).permutation(n_w)
    h = n_w // 2
    Sa = raw.signal(w, logw, subset=idx[:h])
    Sb = raw.signal(w, logw, subset=idx[h:])
    floor = np.abs(Sa - Sb) / 2.0
    per_fam = {}
    for f in sorted({m["fam"] for m in meta}):
        j = np.array([i for i, m in enumerate(meta) if m["fam"] == f])
        per_fam[f] = dict(err_max=float(np.abs(S_dec[j] - S_raw[j]).max()),
                          floor_max=float(floor[j].max()))
    err_all = float(np.abs(S_dec - S_raw).max())
    floor_all = float(floor.max())
    return dict(metric="max_abs_complex_signal_error", err_max=err_all, floor_max=floor_all,
                noise_floor=float(1 / np.sqrt(n_w)), within_2x_floor=bool(err_all <= 2 * floor_all),
                per_family=per_fam)


def _candidate_signals(X, traj, dt_traj, method, G, K_grid, w, logw):
    """(K, decoded-walk signal over G) for every K of the grid, in order.  Temporal-DCT
    candidates replay straight from the K lowest bands (the transform is orthonormal, so this
    equals replaying the decoded positions); the Karhunen-Loeve ones replay their decoded walk."""
    n_t = traj.shape[1]
    if method == "temporal_dct":
        bands = project_modes(X, max(K_grid)).cpu().numpy()
        for K in K_grid:
            k = min(K, bands.shape[1])
            arrays = pack_position_arrays(bands[:, :k], np.float32)
            yield K, mode_space_signal(arrays, {"method": method, "K": int(k), "n_t": int(n_t)},
                                       G, dt_traj, logw=logw, weights=w)
        return
    factors = _kl(X)
    keep_n = X.shape[0] if is_walker_preserving(method) else None
    for K in K_grid:
        arrays, mm, _ = ENCODERS[method](X, K, _cache=factors)
        yield K, _DeviceReplay(decode(arrays, mm, n_walkers=keep_n), dt_traj, G).signal(w, logw)


def auto_select_modes(X, traj, dt_traj, method="temporal_dct", env=None, tol=2.0,
                      err_target=None, K_grid=(8, 16, 32, 48, 64, 96, 128), w=None, logw=None,
                      verbose=False):
    """The smallest mode count of ``K_grid`` whose replay error over the envelope meets
    ``err_target`` (else ``tol`` x the walk's split-half floor), with its fidelity report; the
    largest count's when none does (the rule of compression.py:582-603).  The raw walk is
    uploaded to the GPU once and replayed against every candidate."""
    env = env or default_envelope()
    G, meta = acquisition_battery(traj.shape[1], float(dt_traj), env)
    raw = _DeviceReplay(traj, dt_traj, G)
    S_raw = raw.signal(w, logw)
    chosen = None
    for K, S_dec in _candidate_signals(X, traj, dt_traj, method, G, K_grid, w, logw):
        report = _fidelity_report(raw, S_raw, S_dec, meta, traj.shape[0], w, logw)
        limit = err_target if err_target is not None else tol * report["floor_max"]
        if verbose:
            print(f"{method} with {K} modes: replay error {report['err_max']:.4f}, "
                  f"limit {limit:.4f}", flush=True)
        chosen = (K, report)
        if report["err_max"] <= limit:
            break
    return chosen


__all__ = ["WALKER_PRESERVING", "DISTRIBUTIONAL", "ALL_METHODS", "POSITION_AXES", "dct_basis",
           "project_modes", "encode_temporal_dct", "encode_lowrank", "encode_gaussian",
           "encode_marginal", "ENCODERS", "encode", "rle_encode_rows", "rle_decode_rows",
           "encode_bound_fraction", "decode_bound_fraction", "encode_boundary_local_time",
           "decode_boundary_local_time", "encode_boundary_dct", "decode_boundary_dct",
           "encode_compartment", "decode_compartment", "CHANNEL_ENCODERS", "CHANNEL_DECODERS",
           "pack_position_arrays", "has_axis_layout", "read_position_coeffs",
           "is_walker_preserving", "decode", "mode_space_phi", "mode_space_signal",
           "relaxation_logweight", "surface_logweight", "default_envelope",
           "acquisition_battery", "measure_fidelity", "auto_select_modes"]
