"""Host side of the batched study and the surrogate: the seeded instance mix, the free-waveform
sets (refocused, shape basis of low rank), the waveform encoding (its squares integrate to b D),
the hull test and the feature layout.  No GPU."""
import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import substrates as S
from dmipy_sim_gb300 import surrogate as SG
from dmipy_sim_gb300.core import waveform_basis


def test_free_waveforms_are_refocused_low_rank_and_hit_their_b():
    rng = np.random.default_rng(0)
    wf, idx, dirs, b = S.free_waveform_set(40, 300, 0.05, rng, n_shapes=3)
    q_end = np.sum(wf.G, axis=1) * wf.dt                  # net gradient moment at the echo
    assert np.max(np.abs(q_end)) < 1e-5 * np.max(np.abs(wf.G)) * 0.05
    np.testing.assert_allclose(d.calc_b(wf), b, rtol=1e-4, atol=1e3)
    V, C = waveform_basis(wf.G)
    assert V.shape[1] <= 3


def test_q_encoding_squares_integrate_to_b():
    wf = d.set_b(d.pgse(0.01, 0.03, 0.05, [[0, 0, 1], [1, 0, 0], [0.6, 0, 0.8]], 400), 1e9)
    e = S.q_encoding(wf, 400, t_max=(wf.G.shape[1]) * wf.dt)     # fine grid over the waveform
    n = e.shape[1] // 2
    dt = (wf.G.shape[1]) * wf.dt / n
    b = np.sum(e[:, :n] ** 2 + e[:, n:] ** 2, axis=1) * dt * 1e12
    np.testing.assert_allclose(b, 1e9, rtol=0.02)
    assert np.allclose(e[1, :n], 0.0) and np.allclose(e[0, n:], 0.0)   # z is the axis


def test_dimensionless_features_scale_q_by_the_diffusion_length():
    wf = d.set_b(d.pgse(0.01, 0.03, 0.05, [[1, 0, 0]], 200), 2e9)
    p = dict(kind="PackedCylinders", radius=2e-6, f=0.5, kappa=1e-5, rho=1e-6, D=2e-9, TE=0.05)
    X = SG.features(p, wf)
    assert X.shape == (1, 69)
    bD = float(np.sum(X[0, 5:] ** 2))          # sum of squares of the scaled samples ~ b D
    assert 0.5 * 4.0 < bD < 1.5 * 4.0
    np.testing.assert_allclose(X[0, :5], [np.log(2.0), 0.5, 1e-5 * 2e-6 / 2e-9,
                                          1e-6 * 2e-6 / 2e-9, np.log(2.0)], rtol=1e-6)


def test_hull_routing_rules():
    p = dict(kind="PackedCylinders", radius=2e-6, f=0.5, kappa=1e-5, rho=1e-6, D=2e-9)
    assert SG.in_hull(p)
    assert not SG.in_hull({**p, "kind": "PackedSpheres"})
    assert not SG.in_hull({**p, "radius": 8e-6})
    assert not SG.in_hull({**p, "kappa": 5e-4})
    long_wf = d.Waveform(np.zeros((1, 2000, 3), np.float32), 1e-4, 1999)
    assert not SG.in_hull(p, long_wf)


def test_each_surrogate_routes_only_its_own_kind():
    ps = dict(kind="PackedSpheres", radius=2e-6, f=0.3, kappa=1e-5, rho=1e-6, D=2e-9)
    assert SG.in_hull(ps, kind="PackedSpheres")
    assert not SG.in_hull(ps)                                   # the cylinder surrogate's hull
    assert not SG.in_hull({**ps, "f": 0.5}, kind="PackedSpheres")   # beyond what RSA packs
    assert not SG.in_hull(ps, kind="Mesh")
    with pytest.raises(ValueError):
        SG.Surrogate.__init__(object.__new__(SG.Surrogate), kind="Mesh")


def test_sphere_training_instances_are_drawn_in_their_hull():
    insts, params = SG.draw_instances(4, 5, n_meas=8, n_walkers=64, kind="PackedSpheres")
    for inst, p in zip(insts, params):
        assert type(inst.geometry).__name__ == "PackedSpheres"
        assert len(inst.geometry._radii_np) == SG.N_OBJECTS["PackedSpheres"]
        assert p["kind"] == "PackedSpheres"
        assert SG.in_hull(p, inst.waveform, kind="PackedSpheres") or p["f"] < 0.2


def test_instance_mix_is_seeded_and_in_range():
    a, pa = S.instance_mix(12, seed=3, kinds=("PackedCylinders", "PackedSpheres"))
    b, pb = S.instance_mix(12, seed=3, kinds=("PackedCylinders", "PackedSpheres"))
    for x, y in zip(pa, pb):
        assert x == y
    for inst, p in zip(a, pa):
        assert 1e4 <= p["n_walkers"] <= 1e6 and 300 <= p["n_t"] <= 3000
        assert 8 <= p["n_meas"] <= 96 and inst.waveform.G.shape == (p["n_meas"], p["n_t"], 3)
        assert 0.5e-6 <= p["radius"] <= 5e-6 and p["f"] <= S.F_MAX[p["kind"]] + 1e-9
        assert 0 <= p["kappa"] <= 1e-4 and 0 <= p["rho"] <= 5e-6 and 1e-9 <= p["D"] <= 3e-9


def test_uv_sphere_cells_are_closed_and_outward():
    from dmipy_sim_gb300.mesh import _closed_surface, uv_sphere
    V, F = uv_sphere(1.0, 20, 30)
    assert _closed_surface(F) and len(F) == 2 * 30 * 19
    tri = V[F]
    vol = np.einsum("ij,ij->i", tri[:, 0], np.cross(tri[:, 1], tri[:, 2])).sum() / 6.0
    assert 0.97 * 4 / 3 * np.pi < vol <= 4 / 3 * np.pi
