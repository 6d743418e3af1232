"""Batched walks on the GPU.

Every instance of a mixed batch walks the walkers a plain dmsim_walk of the same parameters walks
(same Philox streams, same step functions).  The batched kernel is a separate compilation of the
same source, and the compiler may fuse a multiply-add in one and not in the other, so the two
agree bit for bit only where the walk does not amplify last-bit differences (free diffusion, a
single cylinder or sphere); in packed substrates and meshes a walker whose last bit differs can
later take another reflection, so there the test asks for the same walkers over a short walk and
the same ensemble over a long one.  Within the batched kernel the result is schedule-independent
(bit-identical under every tuning and as a replayed CUDA graph).  Instances without a shape basis
take the plain path inside the batch."""
import warnings

import numpy as np
import pytest
import torch

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core
from dmipy_sim_gb300.batched import Instance, PreparedBatch, Tuning, _resolve

pytestmark = pytest.mark.gpu
D = 2e-9


def _wf(n_dirs, n_t, seed, ogse=False):
    rng = np.random.default_rng(seed)
    bv = rng.normal(size=(n_dirs, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    w = d.set_b(d.pgse(0.006, 0.02, 0.05, bv, n_t), np.linspace(2e8, 2e9, n_dirs))
    if ogse:
        o = d.ogse(60.0, 0.03, 0.05, bv, n_t)
        return d.Waveform(np.concatenate([w.G, o.G], axis=0), w.dt, n_t - 1)
    return w


def _packed_cyl(**kw):
    rng = np.random.default_rng(1)
    radii = np.clip(rng.lognormal(np.log(1.5e-6), 0.25, 16), 0.8e-6, 3e-6)
    c, L, _ = d.pack_cylinders(radii, target_vf=0.5, seed=2)
    return d.PackedCylinders(radii, c, L, **kw)


def _packed_sph(**kw):
    sr = np.clip(np.random.default_rng(3).normal(1.5e-6, 0.2e-6, 10), 1e-6, 2e-6)
    c, L, _ = d.pack_spheres(sr, target_vf=0.25, seed=3)
    return d.PackedSpheres(sr, c, L, **kw)


def _mesh():
    V, F = d.icosphere(4e-6, 2)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return d.Mesh(V, F)


def _instances():
    R = 4e-6
    return [
        Instance(3000, D, _wf(6, 120, 0), d.FreeDiffusion(), seed=1),
        Instance(2500, D, _wf(5, 90, 1, ogse=True), d.Cylinder(R, (0, 0, 1),
                                                               surface_relaxivity_t2=2e-5), seed=2),
        Instance(1200, 1.5e-9, _wf(4, 60, 2), d.Sphere(R, permeability=1e-5), seed=3),
        Instance(4000, D, _wf(8, 150, 3, ogse=True), _packed_cyl(), seed=4),
        Instance(900, 2.5e-9, _wf(3, 70, 4), _packed_cyl(permeability=2e-5), seed=5),
        Instance(2000, D, _wf(6, 110, 5), _packed_sph(surface_relaxivity_t2=1e-5), seed=6),
        Instance(1500, D, _wf(4, 80, 6), _mesh(), seed=7),
        Instance(0, D, _wf(4, 50, 7), d.FreeDiffusion(), seed=8),
        Instance(700, D, _wf(5, 100, 8), d.Sphere(R), seed=9, T2=0.05),
    ]


def _with_extras(insts):
    return [Instance(**{**i.__dict__, "want_positions": True, "want_walker_signals": True})
            for i in insts]


def _single(inst):
    kw, _ = _resolve(inst)
    return core.run_walk(inst.geometry, **kw)


CHAOTIC = (d.PackedCylinders, d.PackedSpheres, d.Mesh)


def _check_same(rb, rs, n):
    np.testing.assert_allclose(rb.sums, rs.sums, rtol=1e-12, atol=1e-9 * max(n, 1))
    for k in ("pos", "log_w", "phi"):
        if k in rs.extras:
            a, b = rb.extras[k].cpu().numpy(), rs.extras[k].cpu().numpy()
            assert np.array_equal(a, b), f"{k} differs"
    assert rb.status == rs.status


def _check_close(rb, rs, n):
    """Same walkers up to the walks that diverged after a last-bit difference: the ensemble
    agrees within what those few walkers can move it."""
    pa, pb = rb.extras["pos"].cpu().numpy(), rs.extras["pos"].cpu().numpy()
    scale = float(np.max(np.abs(pb))) + 1e-12
    same = np.all(np.abs(pa - pb) <= 1e-4 * scale, axis=1)
    n_div = int((~same).sum())
    diff = np.max(np.abs(rb.signal - rs.signal))
    if same.mean() >= 0.9:
        # a diverged walker moves a signal by at most 2/n (and a close one by a rounding error)
        assert diff <= 2.0 * n_div / max(n, 1) + 1e-4
    else:
        # most walks diverged over the long walk: the two ensembles are alike in distribution
        assert np.all(np.abs(rb.signal - rs.signal) <=
                      4.0 * np.hypot(rb.stderr, rs.stderr) + 1e-4)


def test_batch_matches_plain_walks(cuda):
    insts = _with_extras(_instances())
    b = PreparedBatch(insts, Tuning())
    info = b.info()
    assert info["plain"] == 0 and info["groups"] >= 5
    b.launch()
    res = b.results()
    for inst, rb in zip(insts, res):
        rs = _single(inst)
        if isinstance(inst.geometry, CHAOTIC):
            _check_close(rb, rs, inst.n_walkers)
        else:
            _check_same(rb, rs, inst.n_walkers)
    assert np.all(res[7].sums == 0)


@pytest.mark.parametrize("geom", ["pcyl", "pcyl_kappa", "psph_rho", "mesh"])
def test_batch_short_walks_match_plain_walks(cuda, geom):
    """Over 40 sub-steps of 0.35 um no walk has had room to diverge: every walker agrees
    closely."""
    g = {"pcyl": _packed_cyl, "pcyl_kappa": lambda: _packed_cyl(permeability=2e-5),
         "psph_rho": lambda: _packed_sph(surface_relaxivity_t2=1e-5), "mesh": _mesh}[geom]()
    engine = "fused" if geom == "pcyl_kappa" else "replay"
    shape = np.sin(np.linspace(0.0, 2.0 * np.pi, 20))
    dirs = np.eye(3)[[0, 1, 2, 0]] * np.array([1.0, 1.0, 1.0, 0.5])[:, None]
    wf = d.Waveform((0.2 * shape[None, :, None] * dirs[:, None, :]).astype(np.float32), 1e-5, 19)
    inst = Instance(3000, D, wf, g, seed=11, engine=engine, want_positions=True,
                    want_walker_signals=True, sub_steps=2)
    b = PreparedBatch([Instance(500, D, _wf(3, 20, 1), d.FreeDiffusion()), inst])
    b.launch()
    rb = b.results()[1]
    rs = _single(inst)
    pa, pb = rb.extras["pos"].cpu().numpy(), rs.extras["pos"].cpu().numpy()
    close = np.all(np.abs(pa - pb) <= 1e-3 * max(float(np.max(np.abs(pb))), 1e-6), axis=1)
    assert close.mean() >= 0.995, f"{(~close).sum()} walkers differ"
    np.testing.assert_allclose(rb.signal, rs.signal, atol=4.0 * (~close).sum() / 3000 + 1e-4)


@pytest.mark.parametrize("tuning", [
    Tuning(tiles_per_item=1, order=0, concurrent=0),
    Tuning(tiles_per_item=4, order=1, concurrent=1, blocks_per_sm=1),
    Tuning(tiles_per_item=8, table_bytes=32 * 1024),
])
def test_batch_is_schedule_independent(cuda, tuning):
    insts = _with_extras(_instances()[:7])
    base = PreparedBatch(insts, Tuning())
    base.launch()
    r0 = base.results()
    b = PreparedBatch(insts, tuning)
    b.launch()
    for inst, ra, rb in zip(insts, r0, b.results()):
        if tuning.table_bytes != Tuning().table_bytes and isinstance(
                inst.geometry, (d.PackedCylinders, d.PackedSpheres)):
            # another cell-list grid: the same candidate images, visited in another order, so a
            # walker can differ only where two wall roots tie; those few walkers then diverge
            same = np.all(rb.extras["pos"].cpu().numpy() == ra.extras["pos"].cpu().numpy(), 1)
            assert same.mean() >= 0.98
            np.testing.assert_allclose(rb.signal, ra.signal, atol=0.02)
            continue
        _check_same(rb, ra, inst.n_walkers)


def test_batch_graph_replay_is_exact(cuda):
    insts = _instances()[:7]
    b = PreparedBatch(insts, Tuning(tiles_per_item=2))
    b.launch()
    eager = [r.sums.copy() for r in b.results()]
    b.capture()
    for _ in range(2):
        b.replay()
        torch.cuda.synchronize()
        for e, r in zip(eager, b.results()):
            assert np.array_equal(e, r.sums)


def test_full_rank_waveform_takes_plain_path(cuda):
    rng = np.random.default_rng(11)
    G = rng.normal(size=(12, 64, 3)).astype(np.float32) * 0.02   # 12 unrelated shapes
    wf = d.Waveform(G, 1e-4, 63)
    insts = [Instance(1000, D, wf, d.Sphere(4e-6), seed=3),
             Instance(1000, D, _wf(4, 64, 1), d.Sphere(4e-6), seed=4)]
    b = PreparedBatch(insts)
    assert b.info()["plain"] == 1
    b.launch()
    for inst, rb in zip(insts, b.results()):
        _check_same(rb, _single(inst), inst.n_walkers)


def test_simulate_batch_equals_simulate(cuda):
    insts = _instances()[:3]
    got = d.simulate_batch(insts, use_graph=True)
    for inst, s in zip(insts, got):
        ref = d.simulate(inst.n_walkers, inst.diffusivity, inst.waveform, inst.geometry,
                         seed=inst.seed, T2=inst.T2)
        np.testing.assert_allclose(s, ref, rtol=1e-6, atol=1e-7)


def test_autotune_returns_a_valid_tuning(cuda):
    from dmipy_sim_gb300.autotune import autotune
    log = []
    t = autotune(_instances()[:5], walker_fraction=0.2, repeats=1, log=log,
                 search={"tiles_per_item": (1, 4), "blocks_per_sm": (0, 1)})
    assert isinstance(t, Tuning) and len(log) >= 3
    assert all(np.isfinite(x[1]) and x[1] > 0 for x in log)
