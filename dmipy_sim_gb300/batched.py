"""Batched Monte-Carlo walks: many independent ``simulate()`` instances in one enqueue.

Each :class:`Instance` is what one ``simulate(n_walkers, diffusivity, waveform, geometry, seed,
T2, T1)`` call of dmipy-sim computes (core.py:193-762): its own geometry, waveform, relaxivity,
permeability, walker count, n_t and seed, with the same engine routing and sub-step rules as
:func:`dmipy_sim_gb300.simulate` (signals only).  :class:`PreparedBatch` plans the whole set once
(``dmsim_batch_create`` / ``dmsim_batch_bind``) and enqueues it with one ``dmsim_batch_launch``:
persistent kernels, one per geometry/wall/basis-width group, pull walker tiles of every instance
from a device work queue, and the whole enqueue is capturable in a CUDA graph.  An instance
gives exactly the signal that ``simulate`` gives for it (same Philox stream, same fixed-order
reduction), whatever the schedule.
"""
from dataclasses import dataclass, field
from typing import Any, Optional

import ctypes
import numpy as np
import torch

from . import _lib
from .core import (PreparedWalk, WalkResult, _replay_auto_allowed, _replay_gap, _to_frame,
                   _waveform_arrays, fused_sub_steps, replay_sub_steps)


@dataclass
class Instance:
    """One simulate() call of a batch.  ``want_positions`` / ``want_walker_signals`` keep the
    walk-frame final positions / per-walker (log_w, phi) in :meth:`PreparedBatch.results`;
    ``sub_steps`` overrides the engine's sub-step rule; ``r0`` (n_walkers, 3), lab frame, gives
    the start positions (simulate()'s ``r0``) instead of the geometry's seeding."""
    n_walkers: int
    diffusivity: float
    waveform: Any
    geometry: Any
    seed: int = 123
    T2: Optional[float] = None
    T1: Optional[float] = None
    engine: str = "auto"
    want_positions: bool = False
    want_walker_signals: bool = False
    sub_steps: Optional[int] = None
    r0: Optional[Any] = None


@dataclass
class Tuning:
    """Launch shape of a batch (the knobs :func:`autotune` searches).

    blocks_per_sm   resident blocks per SM of each persistent grid (0 = occupancy limit)
    tiles_per_item  320-walker tiles per work item (walkers a block takes per queue pull)
    order           0 = instances in the given order, 1 = costliest first
    concurrent      1 = kernel groups on forked streams (their tails overlap)
    table_bytes     cell-list budget of packed geometries: the grid is as fine as this allows,
                    and lists within it are staged in shared memory
    """
    blocks_per_sm: int = 0
    tiles_per_item: int = 2
    order: int = 1
    concurrent: int = 1
    table_bytes: int = 96 * 1024

    def to_c(self):
        t = _lib.BatchTuning()
        t.blocks_per_sm = int(self.blocks_per_sm)
        t.tiles_per_item = int(self.tiles_per_item)
        t.order = int(self.order)
        t.concurrent_groups = int(self.concurrent)
        t.tab_smem_bytes = int(self.table_bytes)
        return t

    def key(self):
        return (self.blocks_per_sm, self.tiles_per_item, self.order, self.concurrent,
                self.table_bytes)


def _resolve(inst: Instance):
    """PreparedWalk arguments of one instance, routed as simulate() routes it."""
    if inst.engine not in ("auto", "replay", "fused"):
        raise ValueError(f"engine must be 'auto', 'replay', or 'fused'; got {inst.engine!r}")
    wf = inst.waveform.waveform if hasattr(inst.waveform, 'waveform') else inst.waveform
    geom = inst.geometry
    gap = _replay_gap(geom, return_positions=False, return_compartments=False,
                      return_walker_signals=False, diffusivity=inst.diffusivity)
    if inst.engine == "replay" and gap is not None:
        raise NotImplementedError(f"engine='replay' cannot serve this instance: {gap}")
    use_replay = inst.engine == "replay" or (inst.engine == "auto" and gap is None
                                             and _replay_auto_allowed(geom))
    G, chi = _waveform_arrays(wf, geom)
    dt = float(wf.dt)
    S = (replay_sub_steps if use_replay else fused_sub_steps)(geom, inst.diffusivity, dt)
    if inst.sub_steps is not None:
        S = int(inst.sub_steps)
    kw = dict(n_walkers=int(inst.n_walkers), diffusivity=inst.diffusivity, G=G, dt=dt,
              sub_steps=S, phase_per_substep=not use_replay, seed=inst.seed, chi=chi,
              T2=inst.T2, T1=inst.T1, want_positions=bool(inst.want_positions),
              want_walker_signals=bool(inst.want_walker_signals),
              r0=None if inst.r0 is None else _to_frame(geom, inst.r0))
    return kw, bool(getattr(wf, 'stimulated_echo', False))


class PreparedBatch:
    """A planned, bound batch: ``launch()`` enqueues every instance on the current stream (no
    host synchronisation, capturable), ``capture()`` records it into a CUDA graph that
    ``replay()`` relaunches, ``signals()`` synchronises and returns one (M,) array per
    instance."""

    def __init__(self, instances, tuning: Optional[Tuning] = None):
        self.lib = _lib.load()
        self.dev = _lib.device()
        self.tuning = tuning or Tuning()
        self.instances = list(instances)
        self.walks, self.stim = [], []
        for inst in self.instances:
            g = inst.geometry
            if hasattr(g, "cell_list_bytes"):
                g.cell_list_bytes = int(self.tuning.table_bytes)
            kw, stim = _resolve(inst)
            self.walks.append(PreparedWalk(g, allocate_workspace=False, **kw))
            self.stim.append(stim)
        n = len(self.walks)
        P = (_lib.WalkParams * max(n, 1))()
        Gd = (_lib.Geometry * max(n, 1))()
        O = (_lib.WalkOutputs * max(n, 1))()
        for i, w in enumerate(self.walks):
            P[i], Gd[i], O[i] = w.p, w.gdesc, w.o
        self._arrays = (P, Gd, O)
        self._tune_c = self.tuning.to_c()
        h = ctypes.c_void_p()
        nbytes = ctypes.c_size_t()
        rc = self.lib.dmsim_batch_create(n, P, Gd, O, ctypes.byref(self._tune_c),
                                         ctypes.byref(h), ctypes.byref(nbytes))
        _lib.check(rc, "dmsim_batch_create")
        self._h = h
        self.ws_bytes = int(nbytes.value)
        self.ws = torch.empty(max(self.ws_bytes, 256), dtype=torch.uint8, device=self.dev)
        rc = self.lib.dmsim_batch_bind(h, _lib.ptr(self.ws), self.ws_bytes, _lib.stream_handle())
        _lib.check(rc, "dmsim_batch_bind")
        self.graph = None

    def info(self):
        """(kernel groups, instances on the plain path, work items, kernels per launch)."""
        g, s, it, k = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
        _lib.check(self.lib.dmsim_batch_info(self._h, ctypes.byref(g), ctypes.byref(s),
                                             ctypes.byref(it), ctypes.byref(k)),
                   "dmsim_batch_info")
        return dict(groups=g.value, plain=s.value, items=it.value, kernels=k.value)

    @property
    def launches_per_call(self):
        return self.info()["kernels"]

    def walker_steps(self):
        return sum(w.n_walkers * w.n_t * w.sub_steps for w in self.walks)

    def n_signals(self):
        return sum(w.n_meas for w in self.walks)

    def launch(self):
        _lib.check(self.lib.dmsim_batch_launch(self._h, _lib.stream_handle()),
                   "dmsim_batch_launch")

    def capture(self):
        """Record one launch into a CUDA graph (warm the plan up with launch() first)."""
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.launch()
        return self.graph

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def results(self):
        """Synchronise and return one :class:`WalkResult` per instance."""
        torch.cuda.synchronize(self.dev)
        return [w.result() for w in self.walks]

    def signals(self):
        out = []
        for r, stim in zip(self.results(), self.stim):
            s = r.signal[0].astype(np.float32)
            out.append(s * np.float32(0.5) if stim else s)
        return out

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.dmsim_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate_batch(instances, *, tuning: Optional[Tuning] = None, autotune: bool = False,
                   use_graph: bool = False):
    """Signals of many simulate() instances from one batched enqueue: a list of (M_i,) float32
    arrays in instance order.  ``autotune`` picks the launch shape first (see
    :func:`dmipy_sim_gb300.autotune.autotune`); ``use_graph`` runs it as a captured CUDA graph."""
    if autotune:
        from .autotune import autotune as _autotune
        tuning = _autotune(instances)
    b = PreparedBatch(instances, tuning)
    if use_graph:
        b.launch()          # first launch outside capture (module load, attribute setup)
        torch.cuda.synchronize(b.dev)
        for w in b.walks:   # status words accumulate: start the captured run from zero
            w.status.zero_()
        b.replay()
    else:
        b.launch()
    return b.signals()
