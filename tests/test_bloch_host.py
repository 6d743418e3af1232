"""Vector-Bloch walk, host side: the RF rasterisation, crusher schedule and sequence builders
against dmipy-sim's own (tests/golden/bloch_kat.npz, made by running bloch.py and
pulse_sequence.py unmodified), the echo read-out bookkeeping, the refused options, and the CPU
oracle's Bloch walk against closed forms and against its own scalar walk on the same walk."""
import json
from pathlib import Path

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import bloch as B
from dmipy_sim_gb300 import pulse_sequence as ps
from oracle import oracle as O


@pytest.fixture(scope="module")
def z():
    return np.load(Path(__file__).parent / "golden" / "bloch_kat.npz")


RF_EVENTS = [
    [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}],
    [{'t_s': 0.0, 'flip_deg': 90.0}, {'t_s': 2.05e-3, 'flip_deg': 180.0, 'axis_deg': 0.0,
                                       'duration_s': 1e-3, 'offset_hz': 120.0}],
    [{'t_s': 1e-3, 'flip_deg': 45.0, 'axis_deg': 30.0, 'duration_s': 2.4e-3,
      'offset_hz': -80.0}, {'t_s': 9.99e-3, 'flip_deg': 33.0, 'duration_s': 5e-4}],
]
CRUSHERS = [None, {'windows_s': [(1e-3, 3e-3)], 'n_cycles': 8.0},
            {'windows_s': [(-1e-3, 2e-3), (8e-3, 20e-3)]}]


def test_rf_schedule_matches_reference(z):
    for i, ev in enumerate(RF_EVENTS):
        fl, ax, ca = B._build_rf_schedule(ev, 1e-4, 100)
        np.testing.assert_allclose(fl, z[f"rf{i}_flip"], rtol=1e-15, atol=0)
        np.testing.assert_array_equal(ax, z[f"rf{i}_axis"])
        np.testing.assert_allclose(ca, z[f"rf{i}_carrier"], rtol=1e-15, atol=0)


def test_crusher_schedule_matches_reference(z):
    for i, cr in enumerate(CRUSHERS):
        rate, has = B._build_crusher(cr, 1e-4, 100)
        np.testing.assert_array_equal(rate, z[f"crush{i}_rate"])
        assert has == bool(z[f"crush{i}_has"])


def _seqs():
    return {
        "gre": ps.gradient_echo(5e-3, 1e-4, n_meas=2),
        "se": ps.spin_echo(6e-3, 1e-4, exc_axis_deg=45.0),
        "fexi": ps.fexi(2e-3, 5e-3, 1e-4, g_filter=0.2, g_detect=[0.0, 0.1, 0.2], Delta=4e-3,
                        direction=(1.0, 1.0, 0.0), crush_cycles=16.0),
        "fexi2": ps.fexi(2e-3, 3e-3, 2e-4, g_filter=0.1, g_detect=0.05),
        "mt": ps.prepend_mt_prep(ps.spin_echo(6e-3, 1e-4),
                                 {'offset_hz': 2000.0, 'duration_s': 3e-3, 'b1_hz': 100.0}),
        "mt2": ps.prepend_mt_prep(
            ps.BlochSequence(G=np.zeros((1, 30, 3)), dt=1e-4, rf_events=[
                {'t_s': 0.0, 'flip_deg': 90.0}], echo_steps=[10, 29]),
            {'offset_hz': -500.0, 'duration_s': 1e-3, 'flip_deg': 400.0, 'spoiler_s': 0.0}),
    }


@pytest.mark.parametrize("name", ["gre", "se", "fexi", "fexi2", "mt", "mt2"])
def test_sequence_builders_match_reference(z, name):
    q = _seqs()[name]
    np.testing.assert_array_equal(q.G, z[f"seq_{name}_G"])
    assert q.dt == float(z[f"seq_{name}_dt"])
    ref_rf = json.loads(str(z[f"seq_{name}_rf"]))
    assert len(q.rf_events) == len(ref_rf)
    for a, b in zip(q.rf_events, ref_rf):
        assert set(a) == set(b)
        for k in a:
            assert a[k] == pytest.approx(b[k], rel=1e-15, abs=0), k
    assert q.echo_steps == json.loads(str(z[f"seq_{name}_echo"]))
    cr = json.loads(str(z[f"seq_{name}_crusher"]))
    if cr is None:
        assert q.crusher is None
    else:
        assert q.crusher["n_cycles"] == cr["n_cycles"]
        np.testing.assert_allclose(np.asarray(q.crusher["windows_s"]), np.asarray(cr["windows_s"]),
                                   rtol=1e-15)
    assert [q.complex_signal, q.family] == json.loads(str(z[f"seq_{name}_meta"]))
    if f"seq_{name}_b_detect" in z:
        np.testing.assert_allclose(q.b_detect, z[f"seq_{name}_b_detect"], rtol=1e-13)


def test_echo_read_out_order_duplicates_and_mz():
    """The kernel reads each distinct echo sample once; the host maps them back in the caller's
    order (repeats and negative indices included) and reads Mz at the last sample."""
    uniq = np.array([3, 7, 9], np.int32)
    sums = np.arange(3 * 2 * 3, dtype=np.float64).reshape(3, 2, 3)
    sig, mz = B._finish(sums, 2, uniq, np.array([7, 3, 7]), True)
    assert sig.shape == (2, 3) and sig.dtype == np.complex64
    np.testing.assert_allclose(sig[:, 0], (sums[1, :, 0] + 1j * sums[1, :, 1]) / 2)
    np.testing.assert_allclose(sig[:, 1], (sums[0, :, 0] + 1j * sums[0, :, 1]) / 2)
    np.testing.assert_allclose(sig[:, 2], sig[:, 0])
    np.testing.assert_allclose(mz, sums[2, :, 2] / 2)
    s1 = B._finish(sums, 2, uniq, None, False)
    np.testing.assert_allclose(s1, (sums[2, :, 0] + 1j * sums[2, :, 1]) / 2)


def test_refused_options_fail_before_any_walk():
    """The reference's argument errors, raised before the device is touched."""
    wf = ps.gradient_echo(1e-3, 1e-4)
    with pytest.raises(NotImplementedError):
        d.simulate_bloch(10, 2e-9, wf, d.Sphere(4e-6), wf.rf_events, kappa_MT=1e-5,
                         dwell_time=1e-3, susceptibility=object())
    with pytest.raises(ValueError):
        d.simulate_bloch(10, 2e-9, wf, d.Sphere(4e-6), wf.rf_events, kappa_MT=1e-5,
                         dwell_time=0.0)
    with pytest.raises(TypeError):
        d.simulate_bloch(10, 2e-9, wf, d.FreeDiffusion(), wf.rf_events, kappa_MT=1e-5,
                         dwell_time=1e-3)
    with pytest.raises(ValueError):
        d.simulate_bloch(10, 2e-9, wf, d.Sphere(4e-6), wf.rf_events, kappa_MT=1e-5,
                         dwell_time=1e-3, equilibrate_binding="later")


def test_mt_fast_mode_falls_back_when_unsafe():
    from dmipy_sim_gb300.bloch import _mt_mode
    G = np.zeros((1, 5, 3))
    assert _mt_mode("fast", G, 0.08, 1e-5, d.Sphere(2e-6)) == "fast"
    assert _mt_mode("auto", G, 0.08, 1e-5, d.Sphere(2e-6)) == "burnin"
    assert _mt_mode("off", G, 0.08, 1e-5, d.Sphere(2e-6)) == "off"
    with pytest.warns(UserWarning):
        assert _mt_mode("fast", G, 0.08, 1e-5, d.Box1D(4e-6)) == "burnin"
    G[0, 2, 0] = 0.1
    with pytest.warns(UserWarning):
        assert _mt_mode("fast", G, 0.08, 0.05, d.Sphere(2e-6)) == "burnin"
    assert _mt_mode("fast", G, 0.08, 1e-5, d.Sphere(2e-6)) == "fast"


def test_mt_rotation_tables_are_rodrigues_rotations():
    """The per-sub-step rotations the MT kernel applies: orthogonal, determinant 1, axis
    (f cos ax, f sin ax, dphi) fixed, angle |k|; the bound pool's adds its offset."""
    from dmipy_sim_gb300.bloch import _mt_rotations
    fl, ax, ca = B._build_rf_schedule(RF_EVENTS[2], 1e-4, 100)
    R = _mt_rotations(fl, ax, ca, 7, 1e-4, 120.0, -900.0)
    for t in (0, 12, 99):
        for p in range(2):
            Q = R[t, p]
            np.testing.assert_allclose(Q @ Q.T, np.eye(3), atol=1e-14)
            assert np.linalg.det(Q) == pytest.approx(1.0, abs=1e-14)
            f = np.float64(np.float32(fl[t])) / 7.0
            a = np.float32(ax[t])
            kz = (2 * np.pi * 120.0 * 1e-4 + np.float64(np.float32(ca[t]))) / 7.0
            kz += 2 * np.pi * (-900.0) * 1e-4 / 7.0 if p else 0.0
            k = np.array([f * np.float64(np.cos(a)), f * np.float64(np.sin(a)), kz])
            np.testing.assert_allclose(Q @ k, k, rtol=0, atol=1e-14 * np.linalg.norm(k))
            th = np.linalg.norm(k)
            assert np.arccos(np.clip((np.trace(Q) - 1) / 2, -1, 1)) == pytest.approx(th, abs=1e-7)


def test_two_pool_model_matches_reference():
    from dmipy_sim_gb300 import mt
    z = np.load(Path(__file__).parent / "golden" / "mt_kat.npz")
    np.testing.assert_array_equal(
        mt.two_pool_generator(R1a=1.1, R2a=12.5, R1b=0.9, R2b=1e5, k_f=40.0, k_r=80.0,
                              dw_a=300.0, dw_b=-50.0, w1=700.0, rf_phase=0.4), z["gen"])
    np.testing.assert_array_equal(
        mt.two_pool_generator(R1a=1.0, R2a=10.0, R1b=1.0, R2b=1e4, k_f=30.0, k_r=100.0,
                              M0a=0.8, M0b=0.1), z["gen_m0b"])
    t = np.array([0.0, 1e-3, 5e-3, 0.02, 0.08])
    np.testing.assert_allclose(mt.bloch_mcconnell_transverse(t, T2a=80e-3, T2b=1e-5, k_f=30.0,
                                                             k_r=100.0), z["bmt"], rtol=1e-12)
    np.testing.assert_allclose(
        mt.bloch_mcconnell_transverse(t, T2a=60e-3, T2b=2e-3, k_f=20.0, k_r=50.0, dw_a=100.0,
                                      dw_b=400.0, T1a=0.9, T1b=0.5), z["bmt_dw"], rtol=1e-12)
    np.testing.assert_allclose(mt.bloch_mcconnell_longitudinal(t * 10, T1a=1.0, T1b=0.7,
                                                               k_f=30.0, k_r=90.0), z["bml"],
                               rtol=1e-12)
    np.testing.assert_allclose(
        mt.bloch_mcconnell_longitudinal(t * 10, T1a=1.2, T1b=1.0, k_f=30.0, k_r=90.0, Mza0=1.0,
                                        Mzb0=0.0), z["bml_sat"], rtol=1e-12)
    off = np.array([-5000.0, -500.0, 0.0, 200.0, 2000.0, 20000.0])
    kw = dict(w1_hz=200.0, t_sat=0.025, T1a=1.0, T2a=80e-3, T1b=1.0, T2b=1e-5, k_f=40.0,
              k_r=80.0)
    np.testing.assert_allclose(mt.mt_z_spectrum(off, **kw), z["z_a"], rtol=1e-12)
    np.testing.assert_allclose(mt.mt_z_spectrum(off, read_pool="b", **kw), z["z_b"], rtol=1e-12)
    np.testing.assert_allclose([mt.forward_rate(2e-6, 3e5), mt.backward_rate(0.0125),
                                mt.bound_fraction(2e-6, 0.0125, 3e5),
                                mt.kappa_MT_from_forward_rate(40.0, 1.5e6),
                                mt.dwell_time_from_fraction(0.3, 40.0)], z["misc"], rtol=1e-15)
    np.testing.assert_array_equal(mt.stick_probability(np.array([0.0, 1e-9, 1e-8, 1e-6]), 2e-5,
                                                       2e-9), z["stick"])


def test_mt_sub_step_rule_matches_reference():
    z = np.load(Path(__file__).parent / "golden" / "mt_kat.npz")
    got = [d.mt_sub_steps(d.Sphere(2e-6), 2e-9, 2e-5, 1.0 / 80.0),
           d.mt_sub_steps(d.Sphere(5e-6), 1e-9, 1e-3, 0.01),
           d.mt_sub_steps(d.Cylinder(3e-6, (0, 0, 1)), 2e-9, 1e-4, 1e-5),
           d.mt_sub_steps(d.Box1D(4e-6), 2e-9, 1e-4, 0.02),
           d.mt_sub_steps(d.Box1D(4e-6), 2e-9, 1e-4, 0.0)]
    np.testing.assert_array_equal(got, z["mt_sub"])


def test_oracle_mt_exchange_reaches_equilibrium_fraction():
    """The restated MT walk on a sphere: the bound occupancy relaxes to k_f/(k_f + k_r)."""
    R, D, k_f, k_r = 5e-6, 1e-9, 50.0, 100.0
    dt, n_t = 1e-3, 61
    n_sub = int(np.ceil(dt / (R ** 2 / (3750 * D))))
    g = d.Sphere(R)
    r0 = g.init_positions(2000, 3).astype(np.float32)
    fl, ax, _ = B._build_rf_schedule([{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}], dt, n_t)
    o1 = O.bloch_mt(O.geom_from(g), n_walkers=2000, G=np.zeros((1, 40, 3)), dt=dt, n_sub=n_sub,
                    seed=3, r0=r0, rf_flip=fl[:40], rf_axis=ax[:40], kappa_MT=k_f * R / 3,
                    dwell_time=1 / k_r, D=D)
    o2 = O.bloch_mt(O.geom_from(g), n_walkers=2000, G=np.zeros((1, 21, 3)), dt=dt, n_sub=n_sub,
                    seed=3, r0=o1["r_end"], brem0=o1["brem"], s0=40 * n_sub, rf_flip=fl[:21],
                    rf_axis=ax[:21], kappa_MT=k_f * R / 3, dwell_time=1 / k_r, D=D)
    assert o2["occ_total"].mean() / 21 == pytest.approx(k_f / (k_f + k_r), rel=0.08)


# ---- the oracle's Bloch walk ----------------------------------------------------------------
D = 2e-9


def _rf(events, dt, n_t):
    fl, ax, ca = B._build_rf_schedule(events, dt, n_t)
    return dict(rf_flip=fl, rf_axis=ax, carrier=ca if np.any(ca) else None)


def test_oracle_free_relaxation_and_precession_closed_forms():
    n_t, dt = 200, 2e-4
    G = np.zeros((1, n_t, 3))
    g = O.geom(O.FREE)
    T = n_t * dt
    s = O.bloch(g, n_walkers=64, G=G, dt=dt, sub_steps=1, seed=0, T2=0.05,
                **_rf([{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}], dt, n_t))[0, 0] / 64
    assert s[0] == pytest.approx(np.exp(-T / 0.05), rel=1e-4) and abs(s[1]) < 1e-6
    s = O.bloch(g, n_walkers=64, G=G, dt=dt, sub_steps=1, seed=0, T1=0.8,
                **_rf([{'t_s': 0.0, 'flip_deg': 180.0}], dt, n_t))[0, 0] / 64
    assert s[2] == pytest.approx(1.0 - 2.0 * np.exp(-T / 0.8), abs=1e-4)
    f = 200.0
    car = np.full(n_t, 2 * np.pi * f * 1e-5)
    s = O.bloch(g, n_walkers=8, G=G, dt=1e-5, sub_steps=1, seed=0, carrier=car,
                rf_flip=np.r_[np.pi / 2, np.zeros(n_t - 1)], rf_axis=np.full(n_t, np.pi / 2))[0, 0]
    assert np.angle(s[0] + 1j * s[1]) == pytest.approx(2 * np.pi * f * n_t * 1e-5, rel=1e-4)


def test_oracle_bloch_walk_is_the_scalar_walk():
    """90_y then free precession: Mx + i My = exp(i phi) walker by walker, the scalar engine's
    phasor on the same walk (same draws, steps and phase)."""
    wf = d.set_b(d.pgse(0.01, 0.03, 0.05, [[1, 0, 0], [0, 1, 0]], 300), [1e9, 2e9])
    G = np.asarray(wf.G, np.float32)
    n_t = G.shape[1]
    for g, wall, kw in ((O.geom(O.CYLINDER, radius=5e-6), O.REFLECT, {}),
                        (O.geom(O.SPHERE, radius=4e-6), O.PERMEATE, dict(kappa_over_D=5e3))):
        S = 1 if wall == O.REFLECT else 4
        sb = O.bloch(g, n_walkers=1500, G=G, dt=wf.dt, sub_steps=S, seed=3, wall=wall,
                     **kw, **_rf([{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0}], wf.dt, n_t))
        sw = O.walk(g, n_walkers=1500, G=G, dt=wf.dt, sub_steps=S, phase_per_substep=True,
                    seed=3, wall=wall, **kw)
        np.testing.assert_allclose(sb[0, :, 0], sw["sums"][0, :, 0], atol=2e-3)
        np.testing.assert_allclose(sb[0, :, 1], sw["sums"][0, :, 1], atol=2e-3)


def test_oracle_spin_echo_refocuses_free_diffusion():
    """90_x, 180_y at TE/2 and physical same-sign lobes: |S(TE)| = exp(-bD - TE/T2)."""
    from dmipy_sim_gb300.constants import GAMMA
    TE, dt, nd, g = 40e-3, 1e-4, 100, 0.05
    n_t = int(round(TE / dt)) + 1
    G = np.zeros((1, n_t, 3))
    G[0, 20:20 + nd, 0] = g
    G[0, 220:220 + nd, 0] = g
    rf = _rf([{'t_s': 0.0, 'flip_deg': 90.0}, {'t_s': TE / 2, 'flip_deg': 180.0,
                                                'axis_deg': 90.0}], dt, n_t)
    s = O.bloch(O.geom(O.FREE), n_walkers=20000, G=G, dt=dt, sub_steps=1, seed=1, T2=0.08,
                n_threads=0, **rf)[0, 0] / 20000
    q = GAMMA * g * nd * dt
    b = q * q * (0.02 - nd * dt / 3.0)
    assert abs(s[0] + 1j * s[1]) == pytest.approx(np.exp(-b * D - n_t * dt / 0.08), abs=0.02)


def test_simulate_mixture_weights_compartments_with_their_own_seeds(monkeypatch):
    from dmipy_sim_gb300 import core
    calls = []

    def fake(n_walkers, diffusivity, waveform, geometry, seed):
        calls.append((n_walkers, diffusivity, geometry, seed))
        return np.full(3, float(seed), np.float32)

    monkeypatch.setattr(core, "simulate", fake)
    wf = d.set_b(d.pgse(0.01, 0.03, 0.05, [[1, 0, 0]] * 3, 50), [0, 1e9, 2e9])
    comps = [dict(fraction=0.3, n_walkers=10, diffusivity=1e-9, geometry="a"),
             dict(fraction=0.7, n_walkers=20, diffusivity=2e-9, geometry="b")]
    s = core.simulate_mixture(comps, wf, seed=5)
    assert [c[3] for c in calls] == [5, 6] and [c[2] for c in calls] == ["a", "b"]
    np.testing.assert_allclose(s, 0.3 * 5 + 0.7 * 6, rtol=1e-6)
    with pytest.raises(ValueError):
        core.simulate_mixture([dict(comps[0], fraction=0.5)], wf)
