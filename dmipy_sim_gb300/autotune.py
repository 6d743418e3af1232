"""Autotuner of the batched walk's launch shape.

The knobs (:class:`dmipy_sim_gb300.batched.Tuning`): resident blocks per SM of the persistent
grids (occupancy against registers and shared memory), walker tiles per work item (queue
traffic against load balance at the tail), the work order (costliest instances first or as
given), concurrent kernel groups, and the cell-list byte budget of packed geometries (a finer
grid means fewer candidates per step; a list within the budget is staged in shared memory).

The search is coordinate descent from the defaults over a reduced copy of the batch: every
instance keeps its geometry, waveform and sub-step count but walks only
``walker_fraction`` of its walkers (at least one work item), so each trial costs a few
milliseconds of GPU time.  Trials are timed with CUDA events on the launching stream
(median of ``repeats`` after a warm-up launch).  Results are cached per batch signature for the
life of the process (and in ``cache_path`` when given).
"""
import dataclasses
import json
import os
import statistics

import torch

from .batched import Instance, PreparedBatch, Tuning

SEARCH = {
    "blocks_per_sm": (0, 1),
    "tiles_per_item": (1, 2, 4, 8),
    "order": (1, 0),
    "concurrent": (1, 0),
    "table_bytes": (96 * 1024, 48 * 1024, 160 * 1024),
}

_CACHE = {}


def signature(instances):
    """A key that identifies the batch's shape classes: per instance the geometry type, wall
    mode class, measurement count bucket, n_t bucket and walker-count decade."""
    sig = []
    for inst in instances:
        g = inst.geometry
        wall = "k" if getattr(g, "permeability", None) else (
            "r" if getattr(g, "surface_relaxivity_t2", None) else "-")
        wf = inst.waveform.waveform if hasattr(inst.waveform, "waveform") else inst.waveform
        M, n_t = wf.G.shape[0], wf.G.shape[1]
        sig.append(f"{type(g).__name__}:{wall}:{(M + 15) // 16}:{(n_t + 499) // 500}:"
                   f"{len(str(int(inst.n_walkers)))}")
    sig.sort()
    try:
        dev = torch.cuda.get_device_name()
    except Exception:
        dev = "?"
    return dev + "|" + ",".join(sig)


def _reduced(instances, walker_fraction, min_walkers):
    return [dataclasses.replace(i, n_walkers=max(min_walkers, int(i.n_walkers * walker_fraction)))
            for i in instances]


def time_batch(instances, tuning, repeats=3):
    """Median seconds of one launch of ``instances`` under ``tuning`` (CUDA events)."""
    b = PreparedBatch(instances, tuning)
    b.launch()                       # warm-up
    torch.cuda.synchronize(b.dev)
    times = []
    for _ in range(repeats):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        b.launch()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    b.close()
    return statistics.median(times)


def autotune(instances, *, walker_fraction=0.05, min_walkers=640, repeats=3, cache_path=None,
             search=None, log=None):
    """Coordinate-descent search of :class:`Tuning` on a reduced copy of ``instances``; returns
    the fastest tuning found (cached per batch signature)."""
    instances = list(instances)
    key = signature(instances)
    if key in _CACHE:
        return _CACHE[key]
    if cache_path and os.path.exists(cache_path):
        with open(cache_path) as f:
            disk = json.load(f)
        if key in disk:
            _CACHE[key] = Tuning(**disk[key])
            return _CACHE[key]
    trial = _reduced(instances, walker_fraction, min_walkers)
    search = search or SEARCH
    best = Tuning()
    best_t = time_batch(trial, best, repeats)
    seen = {best.key(): best_t}
    if log is not None:
        log.append((dataclasses.asdict(best), best_t))
    for knob, values in search.items():
        for v in values:
            cand = dataclasses.replace(best, **{knob: v})
            if cand.key() in seen:
                continue
            t = time_batch(trial, cand, repeats)
            seen[cand.key()] = t
            if log is not None:
                log.append((dataclasses.asdict(cand), t))
            if t < best_t:
                best, best_t = cand, t
    _CACHE[key] = best
    if cache_path:
        disk = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                disk = json.load(f)
        disk[key] = dataclasses.asdict(best)
        with open(cache_path, "w") as f:
            json.dump(disk, f, indent=1)
    return best


__all__ = ["autotune", "time_batch", "signature", "SEARCH", "Instance", "Tuning"]
