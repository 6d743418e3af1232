"""A batching numpy stand-in for ``jax``: ``vmap`` runs the per-walker function ONCE on all
walkers at the same time.

``jaxstub.py`` runs the reference's per-walker functions one walker at a time (``vmap`` is a
Python loop), which costs ~0.3 ms per walker-sub-step on a packed substrate: far too slow for
fixtures of tens of thousands of walkers over thousands of sub-steps.  This module keeps the same
idea (the reference's modules run unmodified, ``jax.numpy`` is numpy, ``lax.scan`` is a loop,
``jit`` the identity) but gives ``vmap`` real batching semantics:

* a value that depends on the mapped axis is a :class:`BArr`, an ndarray ``v`` of shape
  ``(B, *logical_shape)``; the reference's code sees only the logical shape.  Ufuncs align a
  ``BArr`` with unbatched arrays by padding its logical shape on the left (numpy broadcasting
  then does the rest), reductions / ``argmin`` / ``stack`` / ``concatenate`` shift their axis by
  one, indexing keeps the batch axis, and an index that is itself batched gathers per walker;
* ``jax.random`` keys are 64-bit counters (a scalar, or one per walker when batched); ``split``
  and the draws hash a key with an index through the SplitMix64 finaliser, so a batched walk
  and the same walk run walker by walker draw identical numbers (that is how the batching is
  checked: ``check_batching`` below).

Anything the reference does that this module does not implement raises ``NotImplementedError``
rather than computing something else.  Test infrastructure only (fixture generation).
"""
import importlib
import sys
import types

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _fmix(z):
    """SplitMix64 output finaliser on uint64 arrays (bijective 64-bit mixer)."""
    z = np.asarray(z, np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def _child(s, i):
    """Key number i derived from key(s) s (uint64 arrays, broadcasting)."""
    with np.errstate(over="ignore"):
        t = _fmix(np.asarray(i, np.uint64) * np.uint64(0x9E3779B97F4A7C15) + np.uint64(0x632BE59BD9B4E019))
        return _fmix(np.asarray(s, np.uint64) ^ t)


# ------------------------------------------------------------------------------------------------
# batched values
# ------------------------------------------------------------------------------------------------
class BArr:
    """A per-walker value: ``v`` has shape (B, *logical_shape)."""

    __array_priority__ = 1000

    def __init__(self, v):
        self.v = np.asarray(v)

    # logical array attributes
    @property
    def shape(self):
        return self.v.shape[1:]

    @property
    def ndim(self):
        return self.v.ndim - 1

    @property
    def dtype(self):
        return self.v.dtype

    @property
    def size(self):
        return int(np.prod(self.shape))

    @property
    def T(self):
        return BArr(np.swapaxes(self.v, -1, -2)) if self.ndim == 2 else self

    def astype(self, dtype, *a, **k):
        return BArr(self.v.astype(np.dtype(dtype)))

    def __len__(self):
        if self.ndim == 0:
            raise TypeError("len() of a batched scalar")
        return self.shape[0]

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]

    def __array__(self, *a, **k):
        raise NotImplementedError("a batched value was used where a concrete array is needed")

    def __bool__(self):
        raise NotImplementedError("Python control flow on a batched value")

    def __float__(self):
        raise NotImplementedError("float() of a batched value")

    # indexing
    def __getitem__(self, idx):
        idx = idx if isinstance(idx, tuple) else (idx,)
        if not any(isinstance(e, BArr) for e in idx):
            if any(isinstance(e, np.ndarray) and e.dtype == bool for e in idx):
                raise NotImplementedError("boolean mask indexing of a batched value")
            return BArr(self.v[(slice(None),) + idx])
        return BArr(_gather(self.v, idx))

    @property
    def at(self):
        base = self

        class _Index:
            def __getitem__(self, idx):
                class _Set:
                    def set(self, val):
                        if isinstance(idx, BArr) or (isinstance(idx, tuple) and
                                                     any(isinstance(e, BArr) for e in idx)):
                            raise NotImplementedError("batched index in .at[]")
                        out = base.v.copy()
                        tgt = out[(slice(None),) + (idx if isinstance(idx, tuple) else (idx,))]
                        val_v = _align([val], len(base.v), tgt.ndim - 1)[0]
                        out[(slice(None),) + (idx if isinstance(idx, tuple) else (idx,))] = val_v
                        return BArr(out)
                return _Set()
        return _Index()

    def sum(self, axis=None, **k):
        return np.sum(self, axis=axis, **k)

    def dot(self, other):
        return np.dot(self, other)

    def reshape(self, *shape):
        shape = shape[0] if len(shape) == 1 and isinstance(shape[0], (tuple, list)) else shape
        return BArr(self.v.reshape((len(self.v),) + tuple(shape)))

    # arithmetic: every operator is its ufunc (dispatched to __array_ufunc__)
    def __add__(s, o): return np.add(s, o)
    def __radd__(s, o): return np.add(o, s)
    def __sub__(s, o): return np.subtract(s, o)
    def __rsub__(s, o): return np.subtract(o, s)
    def __mul__(s, o): return np.multiply(s, o)
    def __rmul__(s, o): return np.multiply(o, s)
    def __truediv__(s, o): return np.true_divide(s, o)
    def __rtruediv__(s, o): return np.true_divide(o, s)
    def __floordiv__(s, o): return np.floor_divide(s, o)
    def __mod__(s, o): return np.remainder(s, o)
    def __pow__(s, o): return np.power(s, o)
    def __rpow__(s, o): return np.power(o, s)
    def __neg__(s): return np.negative(s)
    def __abs__(s): return np.absolute(s)
    def __lt__(s, o): return np.less(s, o)
    def __le__(s, o): return np.less_equal(s, o)
    def __gt__(s, o): return np.greater(s, o)
    def __ge__(s, o): return np.greater_equal(s, o)
    def __eq__(s, o): return np.equal(s, o)
    def __ne__(s, o): return np.not_equal(s, o)
    def __and__(s, o): return np.logical_and(s, o) if s.dtype == bool else np.bitwise_and(s, o)
    def __rand__(s, o): return s.__and__(o)
    def __or__(s, o): return np.logical_or(s, o) if s.dtype == bool else np.bitwise_or(s, o)
    def __ror__(s, o): return s.__or__(o)
    def __invert__(s): return np.logical_not(s) if s.dtype == bool else np.invert(s)
    def __matmul__(s, o): return _dot(s, o)
    def __rmatmul__(s, o): return _dot(o, s)
    __hash__ = None

    def __array_ufunc__(self, ufunc, method, *inputs, **kw):
        if method != "__call__" or "out" in kw:
            raise NotImplementedError(f"{ufunc.__name__}.{method} on a batched value")
        if ufunc is np.matmul:
            return _dot(*inputs)
        B = _batch(inputs)
        vals = _align(inputs, B)
        res = ufunc(*vals, **kw)
        if isinstance(res, tuple):
            return tuple(BArr(r) for r in res)
        return BArr(res)

    def __array_function__(self, func, types_, args, kwargs):
        h = _HANDLERS.get(func)
        if h is None:
            raise NotImplementedError(f"numpy.{func.__name__} on a batched value")
        return h(*args, **kwargs)


def _batch(items):
    for x in items:
        if isinstance(x, BArr):
            return len(x.v)
        if isinstance(x, (list, tuple)):
            b = _batch(x)
            if b is not None:
                return b
    return None


def _lrank(x):
    if isinstance(x, BArr):
        return x.ndim
    if isinstance(x, (int, float, bool, complex)):
        return 0
    return np.ndim(x)


def _align(items, B, rank=None):
    """Physical operands for an elementwise op: BArr values padded to (B, 1.., *shape)."""
    r = max(_lrank(x) for x in items) if rank is None else rank
    out = []
    for x in items:
        if isinstance(x, BArr):
            v = x.v
            if len(v) != B:
                raise ValueError("batch sizes differ")
            out.append(v.reshape((B,) + (1,) * (r - x.ndim) + x.shape))
        else:
            out.append(x)
    return out


def _lift(x, B):
    """x as a BArr (unbatched values broadcast over the batch)."""
    if isinstance(x, BArr):
        return x
    a = np.asarray(x)
    return BArr(np.broadcast_to(a, (B,) + a.shape))


def _gather(v, idx):
    """v[(batch,) + idx] where some index entries are batched integer arrays."""
    B = len(v)
    ents = list(idx)
    # contiguous advanced indices from position 0 only (numpy then keeps them first)
    n_adv = 0
    for e in ents:
        if isinstance(e, (BArr, np.ndarray, int, np.integer)):
            n_adv += 1
        else:
            break
    if any(isinstance(e, BArr) for e in ents[n_adv:]):
        raise NotImplementedError("batched index after a slice")
    ranks = [e.ndim if isinstance(e, BArr) else np.ndim(e) for e in ents[:n_adv]]
    r = max(ranks) if ranks else 0
    ar = np.arange(B).reshape((B,) + (1,) * r)
    adv = [e.v.reshape((B,) + (1,) * (r - e.ndim) + e.shape) if isinstance(e, BArr) else e
           for e in ents[:n_adv]]
    return v[tuple([ar] + adv + ents[n_adv:])]


def _ax(axis, nd):
    if axis is None:
        return tuple(range(1, nd + 1))
    if isinstance(axis, (tuple, list)):
        return tuple(_ax(a, nd)[0] if not isinstance(a, tuple) else a for a in axis)
    return (axis + 1,) if axis >= 0 else (axis,)


def _reduce(fn):
    def h(a, axis=None, *args, **kw):
        if not isinstance(a, BArr):
            return fn(a, axis, *args, **kw)
        ax = _ax(axis, a.ndim)
        ax = ax if len(ax) != 1 else ax[0]
        return BArr(fn(a.v, ax, *args, **kw))
    return h


def _argred(fn):
    def h(a, axis=None, **kw):
        if axis is None:
            return BArr(fn(a.v.reshape(len(a.v), -1), axis=1))
        return BArr(fn(a.v, axis=_ax(axis, a.ndim)[0]))
    return h


def _where(c, x=None, y=None):
    if x is None or y is None:
        raise NotImplementedError("one-argument where on a batched value")
    B = _batch((c, x, y))
    return BArr(np.where(*_align((c, x, y), B)))


def _einsum_dot(a, b):
    """np.dot / matmul for operands of logical rank <= 2, either or both batched."""
    la, lb = _lrank(a), _lrank(b)
    if la == 0 or lb == 0:
        return np.multiply(a, b)
    sa = {1: "k", 2: "mk"}[la]
    sb = {1: "k", 2: "kn"}[lb]
    so = (sa[:-1] + sb[1:])
    ops, ia, ib, zo = [], sa, sb, ""
    if isinstance(a, BArr):
        ia, zo = "z" + sa, "z"
    if isinstance(b, BArr):
        ib, zo = "z" + sb, "z"
    va = a.v if isinstance(a, BArr) else np.asarray(a)
    vb = b.v if isinstance(b, BArr) else np.asarray(b)
    return BArr(np.einsum(f"{ia},{ib}->{zo}{so}", va, vb))


def _dot(a, b):
    if not isinstance(a, BArr) and not isinstance(b, BArr):
        return np.dot(a, b)
    return _einsum_dot(a, b)


def _stack(arrays, axis=0, **kw):
    B = _batch(arrays)
    vs = [_lift(x, B).v for x in arrays]
    return BArr(np.stack(vs, axis=axis + 1 if axis >= 0 else axis))


def _concatenate(arrays, axis=0, **kw):
    B = _batch(arrays)
    vs = [_lift(x, B).v for x in arrays]
    return BArr(np.concatenate(vs, axis=axis + 1 if axis >= 0 else axis))


def _clip(a, a_min=None, a_max=None, **kw):
    B = _batch((a, a_min, a_max))
    x, lo, hi = _align((a, a_min, a_max), B) if a_min is not None and a_max is not None else (
        None, None, None)
    if x is None:
        raise NotImplementedError("one-sided clip on a batched value")
    return BArr(np.clip(x, lo, hi))


def _like(fn):
    def h(a, *args, **kw):
        return BArr(fn(a.v, *args, **kw))
    return h


def _norm(x, ord=None, axis=None, keepdims=False):
    if ord is not None:
        raise NotImplementedError("norm with ord")
    v = x.v
    ax = _ax(axis, x.ndim)
    return BArr(np.sqrt(np.sum(v * v, axis=ax, keepdims=keepdims)))


def _cross(a, b, **kw):
    B = _batch((a, b))
    va, vb = _align((a, b), B)
    return BArr(np.cross(va, vb, **kw))


def _transpose(a, axes=None):
    if axes is None:
        axes = tuple(reversed(range(a.ndim)))
    return BArr(np.transpose(a.v, (0,) + tuple(i + 1 for i in axes)))


def _broadcast_to(a, shape, **kw):
    B = len(a.v)
    return BArr(np.broadcast_to(_align([a], B, len(shape))[0], (B,) + tuple(shape)))


def _round(a, decimals=0, **kw):
    return BArr(np.round(a.v, decimals))


def _einsum(sub, *ops, **kw):
    if "->" not in sub or "..." in sub:
        raise NotImplementedError("einsum form")
    ins, out = sub.split("->")
    ins = ins.split(",")
    B = _batch(ops)
    nins, vs = [], []
    for s, o in zip(ins, ops):
        if isinstance(o, BArr):
            nins.append("Z" + s)
            vs.append(o.v)
        else:
            nins.append(s)
            vs.append(o)
    return BArr(np.einsum(",".join(nins) + "->Z" + out, *vs, **kw))


_HANDLERS = {
    np.where: _where,
    np.sum: _reduce(np.sum), np.mean: _reduce(np.mean), np.max: _reduce(np.max),
    np.min: _reduce(np.min), np.amax: _reduce(np.max), np.amin: _reduce(np.min),
    np.prod: _reduce(np.prod), np.any: _reduce(np.any), np.all: _reduce(np.all),
    np.argmin: _argred(np.argmin), np.argmax: _argred(np.argmax),
    np.dot: _dot, np.stack: _stack, np.concatenate: _concatenate, np.clip: _clip,
    np.zeros_like: _like(np.zeros_like), np.ones_like: _like(np.ones_like),
    np.full_like: _like(np.full_like), np.linalg.norm: _norm, np.cross: _cross,
    np.transpose: _transpose, np.broadcast_to: _broadcast_to, np.round: _round,
    np.einsum: _einsum,
}


# ------------------------------------------------------------------------------------------------
# random keys
# ------------------------------------------------------------------------------------------------
class Key:
    """A PRNG key: uint64 ``s`` (shape () unbatched, (B,) batched)."""

    def __init__(self, s, batched=False):
        self.s = np.asarray(s, np.uint64)
        self.batched = batched


class KeyArray:
    """Keys from ``split``: ``s`` has a leading key axis (then the batch axis, if batched)."""

    def __init__(self, s, batched=False):
        self.s = np.asarray(s, np.uint64)
        self.batched = batched

    def __len__(self):
        return len(self.s)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return KeyArray(self.s[i], self.batched)
        return Key(self.s[i], self.batched)

    def __iter__(self):
        for i in range(len(self.s)):
            yield self[i]


def PRNGKey(seed):
    return Key(_child(np.uint64(int(seed) & 0xFFFFFFFFFFFFFFFF), 0x51ED))


def split(key, num=2):
    n = int(num)
    idx = np.arange(n, dtype=np.uint64).reshape((n,) + (1,) * key.s.ndim)
    return KeyArray(_child(key.s[None, ...], idx), key.batched)


def fold_in(key, data):
    return Key(_child(key.s, np.uint64(int(data) + (1 << 40))), key.batched)


def _bits(key, shape):
    """uint64 draws of the given logical shape, (B, *shape) when batched."""
    n = int(np.prod(shape))
    s = key.s.reshape(key.s.shape + (1,))
    b = _child(s, np.arange(n, dtype=np.uint64) + np.uint64(1 << 20))
    return b.reshape(key.s.shape + tuple(shape))


def _wrap(key, a):
    return BArr(a) if key.batched else a


def normal(key, shape=(), dtype=np.float32):
    shape = tuple(shape)
    b = _bits(key, shape + (2,))
    u1 = ((b[..., 0] >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53   # (0, 1]
    u2 = (b[..., 1] >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return _wrap(key, z.astype(np.float32))


def uniform(key, shape=(), dtype=np.float32, minval=0.0, maxval=1.0):
    shape = tuple(shape)
    b = _bits(key, shape)
    u = (b >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)          # [0, 1)
    out = np.float32(minval) + (np.float32(maxval) - np.float32(minval)) * u
    return _wrap(key, out.astype(np.float32))


def randint(key, shape=(), minval=0, maxval=1):
    shape = tuple(shape)
    b = _bits(key, shape)
    out = int(minval) + (b % np.uint64(int(maxval) - int(minval))).astype(np.int64)
    return _wrap(key, out.astype(np.int32))


# ------------------------------------------------------------------------------------------------
# lax / vmap / jit
# ------------------------------------------------------------------------------------------------
def _index(tree, i):
    if tree is None:
        return None
    if isinstance(tree, tuple):
        return tuple(_index(t, i) for t in tree)
    return tree[i]


def _stack_tree(items):
    if not items or items[0] is None:
        return None
    if isinstance(items[0], tuple):
        return tuple(_stack_tree([it[k] for it in items]) for k in range(len(items[0])))
    if any(isinstance(x, BArr) for x in items):
        return _stack(items)
    return np.stack([np.asarray(x) for x in items])


def _length(tree):
    if isinstance(tree, tuple):
        return _length(tree[0])
    return len(tree)


def scan(f, init, xs=None, length=None):
    n = length if xs is None else _length(xs)
    carry = init
    ys = []
    for i in range(n):
        carry, y = f(carry, _index(xs, i))
        ys.append(y)
    return carry, _stack_tree(ys)


LOOP_VMAP = False     # True: vmap runs walker by walker (the check of the batching)


def _unbatch_tree(x, B):
    if isinstance(x, tuple):
        return tuple(_unbatch_tree(e, B) for e in x)
    if isinstance(x, BArr):
        return x.v
    if x is None:
        return None
    a = np.asarray(x)
    return np.broadcast_to(a, (B,) + a.shape).copy()


def vmap(f, in_axes=0):
    def g(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        if any(ax not in (0, None) for ax in axes):
            raise NotImplementedError("vmap in_axes other than 0/None")
        B = next(len(a) for a, ax in zip(args, axes) if ax == 0)
        if LOOP_VMAP:
            outs = []
            for i in range(B):
                sub = []
                for a, ax in zip(args, axes):
                    if ax is None:
                        sub.append(a)
                    elif isinstance(a, KeyArray):
                        sub.append(a[i])
                    else:
                        sub.append(np.asarray(a)[i].view(_AtArray))
                outs.append(f(*sub))
            return _stack_tree(outs)
        bargs = []
        for a, ax in zip(args, axes):
            if ax is None:
                bargs.append(a)
            elif isinstance(a, KeyArray):
                if a.batched:
                    raise NotImplementedError("nested vmap over keys")
                bargs.append(Key(a.s, batched=True))
            elif isinstance(a, BArr):
                raise NotImplementedError("nested vmap")
            else:
                bargs.append(BArr(np.asarray(a)))
        return _unbatch_tree(f(*bargs), B)
    return g


def jit(f=None, **kw):
    if f is None:
        return lambda g: g
    return f


# ------------------------------------------------------------------------------------------------
# jax.numpy
# ------------------------------------------------------------------------------------------------
class _AtArray(np.ndarray):
    """An ndarray with JAX's ``x.at[idx].set(v)``; indexing it with a batched index gathers."""

    def __getitem__(self, idx):
        t = idx if isinstance(idx, tuple) else (idx,)
        if any(isinstance(e, BArr) for e in t):
            B = _batch(t)
            base = np.asarray(self)
            return BArr(_gather(np.broadcast_to(base, (B,) + base.shape), t))
        return super().__getitem__(idx)

    @property
    def at(self):
        base = self

        class _Index:
            def __getitem__(self, idx):
                class _Set:
                    def set(self, v):
                        if isinstance(v, BArr):
                            B = len(v.v)
                            out = np.broadcast_to(np.asarray(base), (B,) + base.shape).copy()
                            t = idx if isinstance(idx, tuple) else (idx,)
                            tgt_nd = out[(slice(None),) + t].ndim - 1
                            out[(slice(None),) + t] = _align([v], B, tgt_nd)[0]
                            return BArr(out)
                        out = np.array(base, copy=True).view(_AtArray)
                        out[idx] = v
                        return out
                return _Set()
        return _Index()


class _DT:
    """A numpy scalar type that also converts batched values (``jnp.float32(x)``)."""

    def __init__(self, t):
        self.t = t
        self.dtype = np.dtype(t)

    def __call__(self, x=0, *a):
        if isinstance(x, BArr):
            return x.astype(self.t)
        return self.t(x, *a)

    def __eq__(self, other):
        try:
            return self.dtype == np.dtype(other)
        except TypeError:
            return False

    def __hash__(self):
        return hash(self.dtype)


def _array(x, dtype=None, *a, **k):
    if isinstance(x, BArr):
        return x.astype(dtype) if dtype is not None else x
    if isinstance(x, (list, tuple)) and _batch(x) is not None:
        s = _stack(list(x))
        return s.astype(dtype) if dtype is not None else s
    return np.array(x, dtype=None if dtype is None else np.dtype(dtype), *a, **k).view(_AtArray)


def _zeros(*a, **k):
    if "dtype" in k and k["dtype"] is not None:
        k["dtype"] = np.dtype(k["dtype"])
    return np.zeros(*a, **k).view(_AtArray)


_DTYPES = {n: _DT(getattr(np, n)) for n in
           ("float16", "float32", "float64", "int8", "int16", "int32", "int64", "uint8",
            "uint32", "uint64", "bool_", "complex64", "complex128")}


class _NumpyModule(types.ModuleType):
    def __getattr__(self, name):
        if name in ("array", "asarray"):
            return _array
        if name == "zeros":
            return _zeros
        if name in _DTYPES:
            return _DTYPES[name]
        return getattr(np, name)


def install():
    """Register the stand-in as ``jax`` in sys.modules."""
    jax = types.ModuleType("jax")
    jnp = _NumpyModule("jax.numpy")
    jnp.linalg = np.linalg
    rnd = types.ModuleType("jax.random")
    for f in (PRNGKey, split, fold_in, normal, uniform, randint):
        setattr(rnd, f.__name__, f)
    lax = types.ModuleType("jax.lax")
    lax.scan = scan
    jax.numpy = jnp
    jax.random = rnd
    jax.lax = lax
    jax.vmap = vmap
    jax.jit = jit
    jax.Array = object
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.devices = lambda *a, **k: ["cpu"]
    jax.default_backend = lambda: "cpu"
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.random"] = rnd
    sys.modules["jax.lax"] = lax


def load_reference(src_root):
    """Import the dmipy_sim hot-path modules from ``src_root`` under this stand-in, without its
    package __init__ (which pulls in optional subsystems)."""
    install()
    pkg = types.ModuleType("dmipy_sim")
    pkg.__path__ = [str(src_root) + "/dmipy_sim"]
    sys.modules["dmipy_sim"] = pkg
    mods = {}
    for m in ("constants", "waveforms", "geometries", "physics", "trajectories", "gpu", "core"):
        mods[m] = importlib.import_module("dmipy_sim." + m)
    return mods
