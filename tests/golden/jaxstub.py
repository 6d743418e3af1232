"""A numpy stand-in for the parts of ``jax`` the dmipy-sim hot path imports.

Used only by ``make_golden.py`` (in a container that has the dmipy-sim sources but no JAX) to run
the reference's own modules unmodified: ``jax.numpy`` maps to numpy, ``lax.scan`` / ``vmap`` are
Python loops, ``jit`` is the identity, and ``jax.random`` draws from numpy generators seeded from
a SeedSequence tree.  A key built with :class:`Injected` makes ``jax.random.uniform`` return a
chosen value, which is how the plug-in known-answer tests pin the Powles draw.
"""
import importlib
import sys
import types

import numpy as np


class Key:
    def __init__(self, ss):
        self.ss = ss


class KeyArray:
    def __init__(self, keys):
        self.keys = list(keys)

    def __len__(self):
        return len(self.keys)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return KeyArray(self.keys[i])
        return self.keys[i]

    def __iter__(self):
        return iter(self.keys)


class Injected:
    """A key whose uniform draw is the given value."""

    def __init__(self, u):
        self.u = np.float32(u)


def _rng(key):
    return np.random.default_rng(key.ss)


def PRNGKey(seed):
    return Key(np.random.SeedSequence(int(seed)))


def split(key, num=2):
    return KeyArray(Key(s) for s in key.ss.spawn(int(num)))


def fold_in(key, data):
    """A key derived from ``key`` and an integer, distinct from its split children."""
    return Key(np.random.SeedSequence(key.ss.entropy,
                                      spawn_key=tuple(key.ss.spawn_key) + (int(data) + (1 << 40),)))


def normal(key, shape=(), dtype=np.float32):
    return _rng(key).standard_normal(shape).astype(np.float32)


def uniform(key, shape=(), dtype=np.float32, minval=0.0, maxval=1.0):
    if isinstance(key, Injected):
        return key.u
    return _rng(key).uniform(minval, maxval, shape).astype(np.float32)


def randint(key, shape=(), minval=0, maxval=1):
    v = _rng(key).integers(minval, maxval, size=shape)
    return np.asarray(v)


def _index(tree, i):
    if tree is None:
        return None
    if isinstance(tree, tuple):
        return tuple(_index(t, i) for t in tree)
    return tree[i]


def _stack(items):
    if not items or items[0] is None:
        return None
    if isinstance(items[0], tuple):
        return tuple(_stack([it[k] for it in items]) for k in range(len(items[0])))
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
    return carry, _stack(ys)


def vmap(f, in_axes=0):
    def g(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = next(len(a) for a, ax in zip(args, axes) if ax == 0)
        outs = [f(*[a[i] if ax == 0 else a for a, ax in zip(args, axes)]) for i in range(n)]
        return _stack(outs)
    return g


def jit(f=None, **kw):
    if f is None:
        return lambda g: g
    return f


class _AtArray(np.ndarray):
    """An ndarray with JAX's functional update ``x.at[idx].set(v)`` (returns a modified copy)."""

    @property
    def at(self):
        base = self

        class _Index:
            def __getitem__(self, idx):
                class _Set:
                    def set(self, v):
                        out = np.array(base, copy=True).view(_AtArray)
                        out[idx] = v
                        return out
                return _Set()
        return _Index()


def _array(*a, **k):
    return np.array(*a, **k).view(_AtArray)


def _zeros(*a, **k):
    return np.zeros(*a, **k).view(_AtArray)


class _NumpyModule(types.ModuleType):
    def __getattr__(self, name):
        if name == "array":
            return _array
        if name == "zeros":
            return _zeros
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
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)   # numpy is FP64-capable
    jax.devices = lambda *a, **k: ["cpu"]
    jax.default_backend = lambda: "cpu"
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.random"] = rnd
    sys.modules["jax.lax"] = lax


def load_reference(src_root):
    """Import the dmipy_sim hot-path modules from ``src_root`` without running its package
    __init__ (which pulls in optional subsystems)."""
    install()
    pkg = types.ModuleType("dmipy_sim")
    pkg.__path__ = [str(src_root) + "/dmipy_sim"]
    sys.modules["dmipy_sim"] = pkg
    mods = {}
    for m in ("constants", "waveforms", "geometries", "physics", "trajectories", "gpu", "core"):
        mods[m] = importlib.import_module("dmipy_sim." + m)
    return mods
