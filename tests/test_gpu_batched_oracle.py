"""Batched walks against the CPU oracle (not only against the plain walk).

Each instance of one batched launch -- packed cylinders (reflecting and permeable), packed
spheres with surface relaxivity, a closed triangle mesh -- is walked again by the oracle, the
statement-by-statement CPU restatement of the reference's walk, on the same Philox stream (the
oracle reproduces the kernels' seeding of packed substrates; the mesh walkers start from given
positions).  Over a short walk every walker but a rounding-order few must land where the oracle's
does; over a long walk the ensembles must agree within 4 combined standard errors.
"""
import warnings

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300.batched import Instance, PreparedBatch, _resolve
from parity_cases import oracle_walk

pytestmark = pytest.mark.gpu
D = 2e-9


def _wf(n_dirs, n_t, seed):
    rng = np.random.default_rng(seed)
    bv = rng.normal(size=(n_dirs, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    return d.set_b(d.pgse(0.004, 0.012, 0.05, bv, n_t), np.linspace(3e8, 2e9, n_dirs))


def _pcyl(**kw):
    radii = np.clip(np.random.default_rng(1).lognormal(np.log(1.5e-6), 0.25, 16), 0.8e-6, 3e-6)
    c, L, _ = d.pack_cylinders(radii, target_vf=0.5, seed=2)
    return d.PackedCylinders(radii, c, L, **kw)


def _psph(**kw):
    sr = np.clip(np.random.default_rng(3).normal(1.5e-6, 0.2e-6, 10), 1e-6, 2e-6)
    c, L, _ = d.pack_spheres(sr, target_vf=0.25, seed=3)
    return d.PackedSpheres(sr, c, L, **kw)


def _mesh_and_starts(n, seed):
    V, F = d.icosphere(4e-6, 2)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        g = d.Mesh(V, F)
    rng = np.random.default_rng(seed)
    pts = np.zeros((0, 3))
    while len(pts) < n:
        p = rng.uniform(V.min(0), V.max(0), size=(4 * n, 3))
        pts = np.concatenate([pts, p[d.mesh_contains(V, F, p)]])
    return g, pts[:n].astype(np.float32)


def _head(wf, n):
    """The first n samples of a waveform (a short walk at the waveform's own time step)."""
    if n is None:
        return wf
    return d.Waveform(G=np.ascontiguousarray(wf.G[:, :n]), dt=wf.dt, echo_idx=n - 1)


def _instances(n_t, walkers, keep=None):
    mesh, r0 = _mesh_and_starts(walkers, 4)
    return [
        Instance(walkers, D, _head(_wf(4, n_t, 0), keep), _pcyl(), seed=11),
        Instance(walkers, D, _head(_wf(3, n_t, 1), keep), _pcyl(permeability=2e-5), seed=12),
        Instance(walkers, D, _head(_wf(4, n_t, 2), keep), _psph(surface_relaxivity_t2=1e-5),
                 seed=13, T2=0.06),
        Instance(walkers, D, _head(_wf(3, n_t, 3), keep), mesh, seed=14, r0=r0),
    ]


def _oracle(inst):
    kw, _ = _resolve(inst)
    return oracle_walk(inst.geometry, kw["G"], kw["dt"], kw["sub_steps"],
                       kw["phase_per_substep"], inst.n_walkers, seed=inst.seed, T2=inst.T2,
                       r0=kw.get("r0"), want_walkers=True)


def test_batched_instances_walk_the_oracles_walkers(cuda):
    # a few dozen sub-steps: 2 samples of a 400-sample waveform (40 us each)
    insts = [Instance(**{**i.__dict__, "want_positions": True, "want_walker_signals": True})
             for i in _instances(400, 2048, keep=2)]
    b = PreparedBatch(insts)
    b.launch()
    res = b.results()
    for inst, r in zip(insts, res):
        ora = _oracle(inst)
        pg = r.extras["pos"].cpu().numpy()
        scale = 4e-6
        same = np.max(np.abs(pg - ora["pos"]), axis=1) < 1e-4 * scale
        name = type(inst.geometry).__name__
        assert same.mean() >= 0.97, f"{name}: {same.mean():.3f} of walkers follow the oracle"
        np.testing.assert_allclose(r.extras["phi"].cpu().numpy()[same], ora["phi"][same],
                                   atol=1e-3, rtol=1e-4, err_msg=name)
    b.close()


def test_batched_ensembles_match_the_oracle(cuda):
    insts = _instances(60, 6000)
    b = PreparedBatch(insts)
    b.launch()
    res = b.results()
    for inst, r in zip(insts, res):
        ora = _oracle(inst)
        se = np.sqrt(2.0) * np.maximum(r.stderr[0], 1e-6)
        z = (r.signal[0] - ora["signal"][0]) / se
        assert np.max(np.abs(z)) < 4.0, (type(inst.geometry).__name__, z)
    b.close()
