"""Host-side logic against the reference's own outputs (tests/golden/kat.npz): waveform
constructors, b-values, sub-step rules, RSA packing; plus the cell list and the engine routing."""
import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core, geometries

D = 2e-9


def test_pgse_set_b_calc_b(kat):
    w = d.set_b(d.pgse(0.01, 0.04, 0.05, [[1, 0, 0]] * 3, 300), [0, 1e9, 2e9])
    np.testing.assert_array_equal(w.G, kat["wf_pgse_G"])
    assert w.dt == float(kat["wf_pgse_dt"])
    np.testing.assert_allclose(d.calc_b(w), kat["wf_pgse_b"], rtol=2e-6)
    w = d.set_b(d.pgse(0.01, 0.04, 0.05, kat["wf_pgse30_bvecs"], 300), 1e9)
    np.testing.assert_array_equal(w.G, kat["wf_pgse30_G"])


def test_square_pgse_btensor(kat):
    w = d.pgse(0.008, 0.03, 0.1, [[0, 1, 0], [0, 0, 1]], 101, slew_rate=np.inf)
    np.testing.assert_array_equal(w.G, kat["wf_square_G"])
    np.testing.assert_allclose(d.calc_btensor(w), kat["wf_square_btensor"], rtol=2e-6)  # float32 sums
    np.testing.assert_allclose(np.trace(d.calc_btensor(w), axis1=1, axis2=2), d.calc_b(w),
                               rtol=2e-6)


def test_pgste(kat):
    w = d.pgste(0.005, 0.02, 0.08, [[1, 0, 0]], 121)
    np.testing.assert_array_equal(w.G, kat["wf_pgste_G"])
    np.testing.assert_array_equal(np.asarray(w.chi_perp, np.float32), kat["wf_pgste_chi"])
    assert w.stimulated_echo and w.dt == float(kat["wf_pgste_dt"])


@pytest.mark.parametrize("f", [10, 50, 100])
def test_ogse_snapping(kat, f):
    with _nowarn():
        w = d.ogse(float(f), 0.05, 0.06, [[1, 0, 0], [0.6, 0.8, 0]], 1000)
    np.testing.assert_allclose(w.G, kat[f"wf_ogse{f}_G"], rtol=1e-6, atol=1e-9)


class _nowarn:
    def __enter__(self):
        import warnings
        self.c = warnings.catch_warnings()
        self.c.__enter__()
        warnings.simplefilter("ignore")

    def __exit__(self, *a):
        self.c.__exit__(*a)


def test_cpmg(kat):
    w = d.cpmg(16, 5e-3, 0.02, [[1, 0, 0], [0, 0, 1]], n_t_per_echo=100)
    np.testing.assert_array_equal(w.G, kat["wf_cpmg_G"])
    np.testing.assert_array_equal(w.echo_indices, kat["wf_cpmg_echo"])
    assert w.dt == float(kat["wf_cpmg_dt"])


def test_permeable_and_surface_sub_steps(kat):
    for R, dt, n_perm, n_surf in kat["sub_perm_surf"]:
        assert core.permeable_sub_steps(d.Sphere(R, permeability=1e-5), D, dt) == n_perm
        assert core.surface_sub_steps(d.Cylinder(R, (0, 0, 1), surface_relaxivity_t2=1e-6),
                                      D, dt) == n_surf


def test_collision_sub_steps(kat):
    class G:
        pass
    for cs, dt, n in kat["sub_collision"]:
        g = G()
        g.cell_size = cs
        assert core.collision_sub_steps(g, D, dt) == n


def test_replay_sub_steps(kat):
    geoms = {"cyl": d.Cylinder(5e-6, (0, 0, 1)), "sphk": d.Sphere(3e-6, permeability=1e-5),
             "pcyl": d.PackedCylinders([1.1e-6, 2e-6], [[-2e-6, -2e-6], [2.5e-6, 2.5e-6]], 9e-6)}
    for name, g in geoms.items():
        for dt, n in kat[f"sub_replay_{name}"]:
            assert core.replay_sub_steps(g, D, dt) == n


def test_rsa_packing_reproduces_reference(kat):
    c, L, vf = d.pack_cylinders(kat["pack_cyl_radii"], target_vf=0.5, seed=3)
    np.testing.assert_array_equal(c, kat["pack_cyl_centers"])
    assert L == float(kat["pack_cyl_L"])
    c, L, vf = d.pack_spheres(kat["pack_sph_radii"], target_vf=0.3, seed=4)
    np.testing.assert_array_equal(c, kat["pack_sph_centers"])
    assert L == float(kat["pack_sph_L"])


def test_pack_errors():
    with pytest.raises(ValueError, match="exactly one"):
        d.pack_cylinders([1e-6], target_vf=0.2, L=100e-6)
    with pytest.raises(ValueError, match="positive"):
        d.pack_cylinders([-1e-6], target_vf=0.1)
    with pytest.raises(ValueError, match="target_vf"):
        d.pack_spheres([1e-6], target_vf=1.5)


@pytest.mark.parametrize("dim", [2, 3])
def test_cell_list_lists_every_object_within_reach(dim):
    rng = np.random.default_rng(dim)
    if dim == 2:
        radii = np.clip(rng.lognormal(np.log(2e-6), 0.3, 40), 0.7e-6, 4e-6)
        c, L, _ = d.pack_cylinders(radii, target_vf=0.5, seed=1)
    else:
        radii = rng.uniform(1e-6, 2e-6, 30)
        c, L, _ = d.pack_spheres(radii, target_vf=0.25, seed=1)
    reach = 0.6e-6
    n, start, cand, obj = geometries.build_cell_list(c, radii, L, reach)
    h = L / n
    pts = rng.uniform(-L / 2, L / 2, (3000, dim)).astype(np.float32)
    for p in pts:
        idx = np.minimum((np.floor((p + L / 2) / h)).astype(int), n - 1)
        cid = 0
        for a in reversed(range(dim)):
            cid = cid * n + idx[a]
        lst = cand[start[cid]:start[cid + 1]]
        lo = obj[start[cid]:start[cid + 1]]
        # every object whose min image is within R + reach must be listed at that image
        q = p - c
        q -= L * np.floor(q / L + 0.5)
        near = np.nonzero(np.linalg.norm(q, axis=1) < radii + reach)[0]
        for k in near:
            img = p - q[k]
            hit = (lo == k) & np.all(np.abs(lst[:, :dim] - img) < 1e-9 * L + 1e-12, axis=1)
            assert hit.any(), f"object {k} missing from cell {cid}"


def test_routing_and_errors():
    wf = d.pgse(0.01, 0.04, 0.05, [[1, 0, 0]], 50)
    with pytest.raises(ValueError, match="engine"):
        d.simulate(10, D, wf, d.FreeDiffusion(), engine="bogus")
    with pytest.raises(ValueError, match="return_compartments"):
        d.simulate(10, D, wf, d.FreeDiffusion(), return_compartments="x")
    with pytest.raises(NotImplementedError, match="permeab"):
        d.simulate(10, D, wf, d.Sphere(5e-6, permeability=1e-5), engine="replay")
    with pytest.raises(NotImplementedError, match="return_compartments"):
        d.simulate(10, D, wf, d.Sphere(5e-6), engine="replay", return_compartments="final")
    assert core._replay_gap(d.Sphere(5e-6), return_positions=False, return_compartments=False,
                            return_walker_signals=False, diffusivity=D) is None
    assert core._replay_auto_allowed(d.PackedCylinders([1e-6], [[0, 0]], 5e-6))
    with pytest.raises(ValueError, match="echo_indices"):
        d.simulate_cpmg(10, D, wf, d.FreeDiffusion(), require_gpu=False)


def test_no_cpu_fallback_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    wf = d.pgse(0.01, 0.04, 0.05, [[1, 0, 0]], 50)
    with pytest.raises(RuntimeError, match="GPU"):
        d.simulate(10, D, wf, d.FreeDiffusion())


def test_trapezoidal_ogse_and_its_b_formula(kat):
    w = d.trapezoidal_ogse(3, 0.02, 0.03, 0.05, [[1, 0, 0], [0, 0.6, 0.8]], 500)
    np.testing.assert_array_equal(w.G, kat["wf_trap_G"])
    assert w.dt == float(kat["wf_trap_dt"])
    w1 = d.trapezoidal_ogse(1, 0.01, 0.03, 0.08, [[0, 1, 0]], 301, rise_time=5e-4)
    np.testing.assert_array_equal(w1.G, kat["wf_trap1_G"])
    got = [d.b_trapezoidal_ogse(n, 0.02, 0.03, 0.05, 2.5e-4) for n in (1, 2, 3, 4)]
    np.testing.assert_allclose(got, kat["wf_trap_bformula"], rtol=1e-12)


def test_tensor_encodings_and_invariants(kat):
    np.testing.assert_array_equal(d.ste(0.01, 0.03, 0.05, 300).G, kat["wf_ste_G"])
    np.testing.assert_array_equal(d.pte(0.01, 0.03, 0.05, [0.3, 0.4, 0.866], 301).G,
                                  kat["wf_pte_G"])
    np.testing.assert_array_equal(
        d.pte(0.01, 0.03, 0.05, [1.0, 0.1, 0.0], 200, slew_rate=np.inf).G, kat["wf_pte2_G"])
    b, bd, be = d.btensor_invariants(kat["wf_inv_B"])
    np.testing.assert_allclose(b, kat["wf_inv_b"], rtol=1e-12)
    np.testing.assert_allclose(bd, kat["wf_inv_bdelta"], atol=1e-9)
    np.testing.assert_allclose(be, kat["wf_inv_beta"], atol=1e-9)
    assert abs(bd[0]) < 1e-6 and abs(bd[1] + 0.5) < 1e-6 and abs(bd[2] - 1.0) < 1e-6


def test_mesh_hit_list_reach():
    """The hit lists' reach covers the float32 step with the relative margin, lies on the
    1/16-octave ladder of the grid cell (so that walks of similar steps share one set), and is
    not used at or above the cell size (the neighbourhood lists then serve)."""
    from dmipy_sim_gb300.mesh import hit_reach
    cs = 3.2e-7
    rng = np.random.default_rng(0)
    for step in np.concatenate([rng.uniform(1e-9, 0.99 * cs / 1.001, 2000),
                                [cs / 4, 0.2412 * cs, 0.25 * cs, cs / 1.001 * 0.999]]):
        r = hit_reach(float(np.float32(step)), cs)
        if r is None:
            assert float(np.float32(step)) * 1.001 > cs * 2 ** (-1 / 16) * (1 - 1e-6)
            continue
        assert r == float(np.float32(r))
        assert r >= float(np.float32(step)) * 1.001
        assert r < cs
        assert r <= max(float(np.float32(step)) * 1.001 * 2 ** (1 / 16) * (1 + 1e-6),
                        float(np.nextafter(np.float32(step * 1.001), np.float32(np.inf))))
    # the study's steps (a quarter of the grid cell, within 4 %) share at most two sets
    steps = np.linspace(0.241, 0.2503, 100) * cs
    assert len({hit_reach(float(s), cs) for s in steps}) <= 2
    for bad in (0.0, -1.0, float("nan"), float("inf"), cs, 2 * cs):
        assert hit_reach(bad, cs) is None
