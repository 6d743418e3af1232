"""dmsim_walk_noalloc, the walk for callers that cannot allocate device memory (for example an
XLA custom call, which only gets the buffers XLA hands it): called through the C ABI, two calls in
a row, it must give the same ensemble sums as dmsim_walk with a caller-allocated workspace, and it
must refuse a walk whose scratch exceeds its fixed-size device array.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest
import torch

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import _lib, core

pytestmark = pytest.mark.gpu
D = 2e-9


def _walk(geom, wf, n, **kw):
    G, chi = core._waveform_arrays(wf, geom)
    S = core.replay_sub_steps(geom, D, wf.dt)
    return core.PreparedWalk(geom, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                             phase_per_substep=False, seed=77, chi=chi, **kw)


def _noalloc_sums(w):
    lib = _lib.load()
    sums = torch.full_like(w.sums, float("nan"))
    status = torch.zeros_like(w.status)
    o = _lib.WalkOutputs()
    o.sums = sums.data_ptr()
    o.status = status.data_ptr()
    rc = lib.dmsim_walk_noalloc(w.p, w.gdesc, o, _lib.stream_handle())
    _lib.check(rc, "dmsim_walk_noalloc")
    torch.cuda.synchronize()
    return sums.cpu().numpy(), status.cpu().numpy()


@pytest.mark.parametrize("case", ["packed", "cpmg"])
def test_noalloc_matches_workspace_walk_twice(cuda, case):
    if case == "packed":
        radii, centers, L = d.lattice_cylinders(6, 0.5, 2e-6, 0.4e-6, seed=1)
        geom = d.PackedCylinders(radii, centers, L)
        rng = np.random.default_rng(2)
        bv = rng.normal(size=(20, 3))
        bv /= np.linalg.norm(bv, axis=1, keepdims=True)
        wf = d.set_b(d.pgse(0.01, 0.03, 0.05, bv, 200), 1e9)
        w = _walk(geom, wf, 40_000)
    else:
        geom = d.Sphere(4e-6)
        wf = d.cpmg(8, 6e-3, 0.03, [[1, 0, 0], [0, 1, 0], [0, 0, 1]], n_t_per_echo=30)
        G, chi = core._waveform_arrays(wf, geom)
        w = core.PreparedWalk(geom, n_walkers=30_000, diffusivity=D, G=G, dt=wf.dt,
                              sub_steps=1, phase_per_substep=True, seed=5, T2=0.05,
                              echo_idx=wf.echo_indices)
    w.launch()
    ref = w.result().sums
    for _ in range(2):                     # the second call starts from the first call's scratch
        got, status = _noalloc_sums(w)
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-9)
        assert status[_lib.STATUS_NAMES.index("wait_timeout")] == 0


def test_noalloc_rejects_walks_larger_than_its_scratch(cuda):
    geom = d.Sphere(4e-6)
    wf = d.cpmg(400, 2e-3, 0.03, np.tile([[1.0, 0, 0]], (64, 1)), n_t_per_echo=2)
    G, chi = core._waveform_arrays(wf, geom)
    w = core.PreparedWalk(geom, n_walkers=1_000_000, diffusivity=D, G=G, dt=wf.dt, sub_steps=1,
                          phase_per_substep=True, seed=5, echo_idx=wf.echo_indices)
    assert w.ws_bytes > (16 << 20)
    lib = _lib.load()
    sums = torch.zeros_like(w.sums)
    o = _lib.WalkOutputs()
    o.sums = sums.data_ptr()
    o.status = w.status.data_ptr()
    rc = lib.dmsim_walk_noalloc(w.p, w.gdesc, o, _lib.stream_handle())
    assert rc == -4
    assert b"DMSIM_NOALLOC_SCRATCH_BYTES" in lib.dmsim_last_error()
