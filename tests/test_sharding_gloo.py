"""Sharded walks on two CPU processes (gloo): each rank walks its contiguous walker range (the
walk is keyed by the global walker index), the FP64 partial sums are all-reduced, and the result
equals the single-process walk.  Uses the CPU oracle as the walk, so it runs without a GPU."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from dmipy_sim_gb300.sharding import shard_range

N = 600


def _case():
    from parity_cases import packed_cylinders, waveform
    from dmipy_sim_gb300 import core
    geom = packed_cylinders()
    wf = waveform(n_dirs=3, n_t=40)
    G, _ = core._waveform_arrays(wf, geom)
    S = core.replay_sub_steps(geom, 2e-9, wf.dt)
    return geom, G, wf.dt, S


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import torch.distributed as dist
    from parity_cases import oracle_walk
    from dmipy_sim_gb300.sharding import allreduce_sums
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    geom, G, dt, S = _case()
    off, cnt = shard_range(N, world, rank)
    r = oracle_walk(geom, G, dt, S, False, cnt, seed=3, walker_offset=off, want_walkers=False)
    total = allreduce_sums(r["sums"])
    if rank == 0:
        np.save(out, total)
    dist.destroy_process_group()


def test_shard_range_covers_exactly():
    for n, w in [(10, 3), (1, 4), (1000, 8), (7, 7)]:
        spans = [shard_range(n, w, r) for r in range(w)]
        assert sum(c for _, c in spans) == n
        assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(w - 1))
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_two_rank_gloo_walk_equals_single_process(tmp_path):
    from parity_cases import oracle_walk
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "sums.npy")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    geom, G, dt, S = _case()
    whole = oracle_walk(geom, G, dt, S, False, N, seed=3, want_walkers=False)["sums"]
    np.testing.assert_allclose(np.load(out), whole, rtol=1e-12, atol=1e-12)


def test_instance_shards_cover_every_instance_once_and_balance():
    from dmipy_sim_gb300.sharding import shard_instances
    rng = np.random.default_rng(0)
    costs = rng.lognormal(0, 1.5, 257)
    for w in (1, 2, 3, 8):
        parts = [shard_instances(costs, w, r) for r in range(w)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)


def _batch_worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import torch.distributed as dist
    from parity_cases import oracle_walk
    from dmipy_sim_gb300.sharding import gather_signals, shard_instances
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    geom, G, dt, S = _case()
    sizes = [40, 200, 90, 10, 150, 60]
    mine = shard_instances(sizes, world, rank)
    local = [oracle_walk(geom, G, dt, S, False, sizes[i], seed=100 + i,
                         want_walkers=False)["sums"] for i in mine]
    allsig = gather_signals(local, mine, len(sizes))
    if rank == 0:
        np.save(out, np.stack(allsig))
    dist.destroy_process_group()


def test_two_rank_gloo_instance_shards_equal_single_process(tmp_path):
    from parity_cases import oracle_walk
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "sig.npy")
    mp.start_processes(_batch_worker, args=(2, port, out), nprocs=2, join=True,
                       start_method="spawn")
    geom, G, dt, S = _case()
    sizes = [40, 200, 90, 10, 150, 60]
    ref = np.stack([oracle_walk(geom, G, dt, S, False, n, seed=100 + i,
                                want_walkers=False)["sums"] for i, n in enumerate(sizes)])
    np.testing.assert_array_equal(np.load(out), ref)
