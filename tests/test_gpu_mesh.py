"""Mesh substrate on the GPU: the device step (dmsim_step_kat, the walk kernel's code) against the
reference's own Mesh.reflect / reflect_with_log_weight / permeate calls (kat.npz, closed icosphere
and a periodic box with ghost triangles), whole walks against the CPU oracle's restatement of the
mesh walk (walker by walker on short walks, and as ensembles), seeding and containment, and a mesh
sphere against the analytic sphere (the reference's tests/test_mesh_mc.py check)."""
import warnings

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core

from parity_cases import oracle_walk

pytestmark = pytest.mark.gpu
D = 2e-9


def _mesh(kat, tag, mode):
    kw = {}
    if mode == "relax":
        kw["intra"] = {"surface_relaxivity_t2": 1e-6}
    if mode == "perm":
        kw["permeability"] = 1e-5
        if tag == "msh":
            kw["intra"] = {"surface_relaxivity_t2": 1e-6}
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        if tag == "msh":
            return d.Mesh(kat["mesh_V"], kat["mesh_F"], **kw)
        return d.Mesh(kat["mesh_Vp"], kat["mesh_F"], periodic=True, voxel_min=[-5e-6] * 3,
                      voxel_max=[5e-6] * 3, feature_radius=3e-6, **kw)


@pytest.mark.parametrize("tag", ["msh", "mshp"])
@pytest.mark.parametrize("mode", ["reflect", "relax", "perm"])
def test_mesh_step_matches_reference(cuda, kat, tag, mode):
    key = f"pl_{tag}_{mode}"
    g = _mesh(kat, tag, mode)
    wall = {"reflect": 0, "relax": 1, "perm": 2}[mode]
    out, dl = core.step_kat(g, kat[key + "_r"], kat[key + "_step"], kat[key + "_u"], wall=wall)
    ref = kat[key + "_out"]
    scale = 5e-6
    err = np.max(np.abs(out - ref), axis=1)
    bad = err > 1e-5 * np.maximum(np.max(np.abs(ref), axis=1), scale)
    assert bad.mean() <= 0.02, f"{bad.sum()} of {len(ref)} steps differ (worst {err.max():.3e})"
    dref = kat[key + "_dlog"]
    ok = np.abs(dl * 500.0 - dref) <= 1e-3 * np.abs(dref) + 1e-8
    assert ok.mean() >= 0.97


def test_mesh_walkers_seeded_inside_and_contained(cuda):
    V, F = d.icosphere(5e-6, 3)
    g = d.Mesh(V, F)
    wf = d.set_b(d.pgse(0.01, 0.03, 0.05, [[1, 0, 0], [0, 0, 1]], 200), 1e9)
    G, _ = core._waveform_arrays(wf, g)
    S = core.replay_sub_steps(g, D, wf.dt)
    res = core.run_walk(g, n_walkers=8192, diffusivity=D, G=G[:, :2], dt=wf.dt, sub_steps=S,
                        phase_per_substep=False, seed=3, want_positions=True)
    p0 = core.run_walk(g, n_walkers=8192, diffusivity=D, G=G[:, :1], dt=wf.dt, sub_steps=1,
                       phase_per_substep=False, seed=3, want_positions=True)
    assert res.status["init_fail"] == 0
    assert d.mesh_contains(V, F, p0.extras["pos"].cpu().numpy()).mean() > 0.995
    res = core.run_walk(g, n_walkers=8192, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                        phase_per_substep=False, seed=3, want_positions=True)
    inside = d.mesh_contains(V, F, res.extras["pos"].cpu().numpy())
    assert inside.mean() > 0.995, inside.mean()


def test_mesh_sphere_matches_analytic_sphere(cuda):
    V, F = d.icosphere(5e-6, 4)
    rng = np.random.default_rng(1)
    bv = rng.normal(size=(4, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    wf = d.set_b(d.pgse(0.005, 0.015, 0.05, bv, 120), 1.5e9)
    s_mesh = d.simulate(40_000, D, wf, d.Mesh(V, F), seed=2)
    s_ana = d.simulate(200_000, D, wf, d.Sphere(5e-6), seed=2)
    np.testing.assert_allclose(s_mesh, s_ana, atol=0.02)


@pytest.mark.parametrize("mode", ["reflect", "relax", "perm"])
def test_neighbourhood_lists_give_the_27_cell_walk(cuda, mode):
    """The per-cell hit lists (candidates within the step's reach of the cell, with their bounding
    spheres in list order or read by triangle index), the neighbourhood lists (each candidate of
    the 27-cell gather once, with the centroids the classification reads in list order or by
    triangle index) and the bounding-sphere pruning walk exactly like the 27-cell gather that
    tests a triangle once per grid cell it overlaps."""
    from dmipy_sim_gb300 import substrates as S
    mesh, _ = S.ellipsoid_cell_mesh(n_cells=8, faces_per_cell=600, box=24e-6,
                                    radius_range=(2e-6, 4e-6), permeable=mode == "perm")
    g = mesh.with_walls(2e-6 if mode == "relax" else None, 1e-5 if mode == "perm" else None)
    rng = np.random.default_rng(3)
    wf, _, _, _ = S.free_waveform_set(4, 40, 0.02, rng, n_shapes=1)
    G, _ = core._waveform_arrays(wf, g)
    S_ = core.fused_sub_steps(g, D, wf.dt)
    if mode != "perm":
        S_ *= 16    # steps of about a quarter of the grid cell, as permeable walls give
    res = []
    for lists in ("hit", "hit, spheres by index", "neighbourhood", "centroids by index", "none"):
        w = core.PreparedWalk(g, n_walkers=4096, diffusivity=D, G=G, dt=wf.dt, sub_steps=S_,
                              phase_per_substep=True, seed=9, want_positions=True,
                              want_walker_signals=True)
        if lists.startswith("hit"):
            assert w.gdesc.mesh_hit_start and w.gdesc.mesh_hit_bs
            assert w.gdesc.mesh_hit_reach >= w.p.step_length
        if lists == "hit, spheres by index":
            w.gdesc.mesh_hit_bs = None
        if lists == "centroids by index":
            w.gdesc.mesh_nb_cent = None
        if not lists.startswith("hit"):
            w.gdesc.mesh_hit_start = None
            w.gdesc.mesh_hit_tri = None
        if lists == "none":
            w.gdesc.mesh_nb_start = None
            w.gdesc.mesh_nb_tri = None
            w.gdesc.tri_bs = None
        w.launch()
        res.append(w.result())
    assert g.n_neighbourhood_entries < len(mesh._cell_tri) * 27
    assert g.n_hit_entries < 0.7 * g.n_neighbourhood_entries
    for r in res[1:]:
        for k in ("pos", "phi", "log_w"):
            assert np.array_equal(res[0].extras[k].cpu().numpy(), r.extras[k].cpu().numpy()), k
        assert res[0].status == r.status


def _inside_points(V, F, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = V.min(0), V.max(0)
    pts = np.zeros((0, 3))
    while len(pts) < n:
        p = rng.uniform(lo, hi, size=(4 * n, 3))
        pts = np.concatenate([pts, p[d.mesh_contains(V, F, p)]])
    return pts[:n].astype(np.float32)


def _oracle_mesh(mode):
    V, F = d.icosphere(4e-6, 2)
    kw = {}
    if mode == "relax":
        kw["intra"] = {"surface_relaxivity_t2": 2e-6}
    if mode == "perm":
        kw["permeability"] = {"intra_to_extra": 2e-5, "extra_to_intra": 1e-5}
        kw["surface_relaxivity_t2"] = 1e-6
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return V, F, d.Mesh(V, F, **kw)


def _mesh_walks(mode, n, n_t, seed, want):
    V, F, g = _oracle_mesh(mode)
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(4, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    wf = d.set_b(d.pgse(0.004, 0.012, 0.02, bv, 80), 1e9)
    G, _ = core._waveform_arrays(wf, g)
    S = core.fused_sub_steps(g, D, wf.dt)
    G = G[:, :(n_t or max(1, 60 // S))]       # default: about 60 sub-steps
    r0 = _inside_points(V, F, n, seed)
    gpu = core.run_walk(g, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                        phase_per_substep=True, seed=seed, T2=0.07, r0=r0, want_positions=want,
                        want_walker_signals=want)
    ora = oracle_walk(g, G, wf.dt, S, True, n, seed=seed, T2=0.07, r0=r0, want_walkers=want)
    return g, S, gpu, ora


@pytest.mark.parametrize("mode", ["reflect", "relax", "perm"])
def test_mesh_short_walk_matches_oracle_walker_by_walker(cuda, mode):
    """Both walks read the same Philox stream from the same start positions; over a few dozen
    sub-steps (a few hundred triangle tests each) every walker but a rounding-order few lands on
    the same position with the same phase and log-weight.  Longer mesh walks are chaotic
    billiards: FP32 contraction differences grow with every bounce off the smooth normals."""
    g, S, gpu, ora = _mesh_walks(mode, 2048, None, 11, True)
    pg = gpu.extras["pos"].cpu().numpy()
    same = np.max(np.abs(pg - ora["pos"]), axis=1) < 1e-4 * 4e-6
    assert same.mean() >= 0.97, f"only {same.mean():.3f} of walkers follow the oracle's walk"
    np.testing.assert_allclose(gpu.extras["phi"].cpu().numpy()[same], ora["phi"][same],
                               atol=1e-3, rtol=1e-4)
    np.testing.assert_allclose(gpu.extras["log_w"].cpu().numpy()[same], ora["log_w"][same],
                               rtol=1e-4, atol=1e-6)
    assert gpu.status["nonfinite"] == 0


@pytest.mark.parametrize("mode", ["reflect", "relax", "perm"])
def test_mesh_ensemble_matches_oracle(cuda, mode):
    """The whole echo on the same stream and start positions: signals within 4 combined SE."""
    g, S, gpu, ora = _mesh_walks(mode, 4096, 80, 21, False)
    se = np.sqrt(2.0) * gpu.stderr[0]
    z = (gpu.signal[0] - ora["signal"][0]) / np.maximum(se, 1e-9)
    assert np.max(np.abs(z)) < 4.0, z
