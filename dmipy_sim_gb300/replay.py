"""Replay packs (``.rpk``) and the compiled-scheme forward (replay.py of dmipy-sim).

A replay pack holds one converged walk in compressed form -- temporal DCT-II bands of every
walker's trajectory (one tensor per axis), optional spin weights and boundary-local-time bands --
so the signal of any gradient waveform is reconstructed without walking again:

    phi_i(m) = sum_{k,c} C_{i,k,c} W_{(k,c),m},   W = gamma dt DCT(G_m)[:K]   (Parseval)
    E(m)     = | sum_i w_i e^{(rho/D) s_i} e^{i phi_i(m)} | / sum_i w_i

``compile_scheme`` builds W on the host (an FFT per measurement); ``replay_signal`` runs the
contraction and the weighted complex mean on the GPU (``dmsim_replay`` over the (n_w, K, 3)
coefficients).  The container is the safetensors layout -- an 8-byte little-endian header length,
a JSON header naming each tensor's dtype, shape and byte range plus a ``__metadata__`` map of
strings, then the raw little-endian tensor bytes -- with the pack's JSON metadata under the
``"rpk"`` key; it is read and written here without the safetensors package.
"""
import json
import struct

import numpy as np
from scipy.fft import dct as _dct

from . import compression as _cx
from .constants import GAMMA

__all__ = ["ReplayPack", "read_rpk", "write_rpk", "compile_scheme", "replay_signal",
           "surface_logweight"]

_DTYPES = {"F64": np.float64, "F32": np.float32, "F16": np.float16, "I64": np.int64,
           "I32": np.int32, "I16": np.int16, "I8": np.int8, "U64": np.uint64, "U32": np.uint32,
           "U16": np.uint16, "U8": np.uint8, "BOOL": np.bool_}
_CODES = {np.dtype(v).str.lstrip("<>|="): k for k, v in _DTYPES.items()}


def _code(a):
    key = a.dtype.str.lstrip("<>|=")
    if key not in _CODES:
        raise TypeError(f"dtype {a.dtype} cannot be stored in a replay pack")
    return _CODES[key]


# --------------------------------------------------------------------- container I/O
def write_rpk(path, arrays, metadata):
    """Write ``arrays`` (name -> ndarray) as tensors and ``metadata`` (a dict) as JSON under the
    header's ``"rpk"`` key (replay.py:40-46)."""
    names = sorted(arrays)
    header, blobs, off = {}, [], 0
    for k in names:
        a = np.ascontiguousarray(arrays[k])
        if a.dtype.byteorder == ">":
            a = a.astype(a.dtype.newbyteorder("<"))
        b = a.tobytes()
        header[k] = {"dtype": _code(a), "shape": [int(s) for s in a.shape],
                     "data_offsets": [off, off + len(b)]}
        blobs.append(b)
        off += len(b)
    header["__metadata__"] = {"rpk": json.dumps(dict(metadata))}
    h = json.dumps(header, separators=(",", ":")).encode("utf-8")
    h += b" " * ((8 - len(h) % 8) % 8)
    with open(path, "wb") as f:
        f.write(struct.pack("<Q", len(h)))
        f.write(h)
        for b in blobs:
            f.write(b)


def _read_container(path):
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 8:
        raise ValueError(f"{path}: not a replay pack (shorter than its header length)")
    (n,) = struct.unpack("<Q", raw[:8])
    if 8 + n > len(raw):
        raise ValueError(f"{path}: header length {n} runs past the end of the file")
    header = json.loads(raw[8:8 + n].decode("utf-8"))
    meta = header.pop("__metadata__", None) or {}
    data = memoryview(raw)[8 + n:]
    arrays = {}
    for k, spec in header.items():
        dt = np.dtype(_DTYPES[spec["dtype"]]).newbyteorder("<")
        b, e = (int(x) for x in spec["data_offsets"])
        if not (0 <= b <= e <= len(data)):
            raise ValueError(f"{path}: tensor {k!r} byte range [{b}, {e}) is outside the data")
        shape = tuple(int(s) for s in spec["shape"])
        if (e - b) != int(np.prod(shape, dtype=np.int64)) * dt.itemsize:
            raise ValueError(f"{path}: tensor {k!r} has {e - b} bytes for shape {shape}")
        arrays[k] = np.frombuffer(data[b:e], dtype=dt).reshape(shape).astype(dt.newbyteorder("="))
    return arrays, meta


def read_rpk(path):
    """Read a replay pack (replay.py:49-58)."""
    arrays, hdr = _read_container(path)
    meta = json.loads(hdr.get("rpk") or hdr.get("json") or "{}")
    return ReplayPack(arrays, meta, source=str(path))


class ReplayPack:
    """A loaded replay pack: the channel ``arrays`` plus ``meta`` (replay.py:61-121)."""

    def __init__(self, arrays, meta, source=None):
        self.arrays = dict(arrays)
        self.meta = dict(meta)
        self.source = source

    @property
    def dct_coeffs(self):
        """(n_walkers, K, n_axes) position coefficients from the axis-per-tensor layout."""
        return _cx.read_position_coeffs(self.arrays, dtype=np.float32)

    @property
    def spin_weights(self):
        w = self.arrays.get("spin_weights")
        return np.ones(self.dct_coeffs.shape[0]) if w is None else w

    @property
    def blt_dct(self):
        return self.arrays.get("blt_dct")

    @property
    def K(self):
        return int(self.dct_coeffs.shape[1])

    @property
    def n_walkers(self):
        return int(self.dct_coeffs.shape[0])

    @property
    def n_t(self):
        wp = self.meta.get("walk_params", {})
        return int(self.meta.get("n_t") or wp.get("n_t"))

    @property
    def dt(self):
        wp = self.meta.get("walk_params", {})
        return float(self.meta.get("dt") or wp.get("dt_traj") or wp.get("dt"))

    @property
    def id(self):
        return self.meta.get("id")

    @property
    def method(self):
        return self.meta.get("compression", {}).get("method")

    license = property(lambda self: self.meta.get("license"))
    citation = property(lambda self: self.meta.get("citation"))
    fidelity = property(lambda self: self.meta.get("fidelity"))
    replay_envelope = property(lambda self: self.meta.get("replay_envelope"))
    provenance = property(lambda self: self.meta.get("provenance"))


# ------------------------------------------------------------------ compiled-scheme forward
def compile_scheme(G, dt, K, gyromagnetic_ratio=GAMMA):
    """The acquisition's projection W (3K, n_meas) onto the pack's first K DCT-II bands:
    W[(k, c), m] = gamma dt DCT(G_m)[k, c] (replay.py:125-136).  ``G`` (n_meas, n_t, 3) T/m on
    the pack's save grid, ``dt`` its interval."""
    G = np.asarray(G, np.float64)
    Ghat = _dct(G, type=2, norm="ortho", axis=1)[:, :K, :]
    return (gyromagnetic_ratio * dt * Ghat).reshape(G.shape[0], Ghat.shape[1] * 3).T


def surface_logweight(blt_dct, rho_over_D, n_t, chi_hat=None):
    """(rho/D) sum_t chi(t) ell_i(t) per walker from boundary-local-time DCT bands: the DC band
    times sqrt(n_t) without a gate, the contraction with the gate's DCT ``chi_hat`` with one
    (replay.py:139-150)."""
    blt = np.asarray(blt_dct, np.float64)
    if chi_hat is None:
        s = np.sqrt(n_t) * blt[:, 0]
    else:
        chi_hat = np.asarray(chi_hat, np.float64)[: blt.shape[1]]
        s = blt[:, : chi_hat.shape[0]] @ chi_hat
    return rho_over_D * s


def replay_signal(pack, W, *, rho_over_D=0.0, chi_hat=None, complex_signal=False):
    """Signal of a compiled scheme ``W`` replayed against ``pack`` (a ReplayPack or an arrays
    dict): magnitude per measurement, or the complex value (replay.py:153-174).  The contraction
    C W and the weighted complex mean run on the GPU."""
    a = pack.arrays if isinstance(pack, ReplayPack) else pack
    C = _cx.read_position_coeffs(a, dtype=np.float32)
    n_w, K, n_ax = C.shape
    W = np.asarray(W, np.float64)
    if W.shape[0] != K * n_ax:
        raise ValueError(f"scheme has {W.shape[0]} rows, the pack {K} bands x {n_ax} axes")
    w0 = np.asarray(a.get("spin_weights", np.ones(n_w)), np.float64)
    lw = np.zeros(n_w)
    blt = a.get("blt_dct")
    if blt is not None and rho_over_D:
        n_t = pack.n_t if isinstance(pack, ReplayPack) else None
        lw = surface_logweight(blt, rho_over_D, n_t, chi_hat)
    Gk = W.T.reshape(W.shape[1], K, n_ax)
    if n_ax != 3:   # a pack with an axis subset: the missing axes carry no phase
        C = np.concatenate([C, np.zeros((n_w, K, 3 - n_ax), np.float32)], axis=2)
        Gk = np.concatenate([Gk, np.zeros((Gk.shape[0], K, 3 - n_ax))], axis=2)
    with np.errstate(divide="ignore"):
        sums, _ = _cx._replay_sums(C, Gk, 1.0, log_w=lw + np.log(w0))
    S = (sums[:, 0] + 1j * sums[:, 1]) / w0.sum()
    return S if complex_signal else np.abs(S)
