"""The magnetisation-transfer Bloch walk on the GPU (dmsim_bloch_mt through simulate_bloch with
kappa_MT > 0).

  * walker by walker against the CPU oracle's eager restatement on the same walk (positions,
    residual dwell, bound occupancy) and the ensemble sums, across a sphere, a packed lattice and
    a slab, with RF, offsets, a gradient, a crusher and surface relaxivity;
  * the checks dmipy-sim pins its own MT engine with (tests/test_mt_binding.py,
    test_mt_storage.py, test_mt_zspectrum.py, test_mt_prep_sequence.py there): the emergent
    bound fraction k_f / (k_f + k_r), its sub-step independence, transverse exchange, stored
    longitudinal recovery and the CW Z-spectrum against the two-pool Bloch-McConnell model, the
    equilibration modes, the MT-prepared gradient echo.
"""
from types import SimpleNamespace

import numpy as np
import pytest
import torch

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import bloch as B
from dmipy_sim_gb300 import mt
from oracle import oracle as O
import bloch_cases as bc

pytestmark = pytest.mark.gpu
EXC = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0, 'duration_s': 0.0, 'offset_hz': 0.0}]


def _zero_wf(n_t, dt, n_meas=1):
    return SimpleNamespace(G=np.zeros((n_meas, n_t, 3)), dt=dt)


# ---- the oracle's restatement on the same walk ------------------------------------------------
def _parity_case(name):
    dt, n_t = 1e-4, 60
    G = np.zeros((2, n_t, 3))
    G[0, 5:20, 0] = G[0, 35:50, 0] = 0.08
    G[1, 5:20, 2] = G[1, 35:50, 2] = 0.08
    rf = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0},
          {'t_s': 2.5e-3, 'flip_deg': 180.0, 'axis_deg': 0.0, 'duration_s': 4e-4,
           'offset_hz': 300.0}]
    kw = dict(T2=0.06, T1=0.9, M0=1.0, off_resonance_hz=40.0, off_resonance_bound=-700.0,
              T2_bound=2e-4, T1_bound=0.5, echo_steps=[29, 59], return_mz=True,
              crusher={'windows_s': [(2.8e-3, 3.2e-3)], 'n_cycles': 4.0},
              return_bound_frac=False)
    if name == "sph":
        return d.Sphere(2e-6), G, dt, rf, kw, dict(kappa=3e-5, dwell=4e-3, rho=1e-5, n_sub=6)
    if name == "pcyl":
        # the packed lattice is a chaotic billiard: FP32 rounding of the oracle's unfolded
        # positions and the kernel's in-cell + image-counter positions part walks after a few
        # hundred sub-steps even without binding, so its walker check stays at 48 sub-steps
        Gs = np.zeros((1, 12, 3))
        Gs[0, 2:5, 0] = Gs[0, 7:10, 0] = 0.08
        rfs = [rf[0], dict(rf[1], t_s=6e-4, duration_s=2e-4)]
        return (bc.geometry(d, ("lattice", 0.6)), Gs, dt, rfs,
                dict(kw, echo_steps=[5, 11], crusher={'windows_s': [(6e-4, 8e-4)],
                                                      'n_cycles': 4.0}),
                dict(kappa=2e-4, dwell=3e-4, rho=0.0, n_sub=4))
    return (d.Box1D(3e-6), G[:1], dt, rf, dict(kw, crusher=None),
            dict(kappa=5e-5, dwell=2e-3, rho=2e-5, n_sub=5))


@pytest.mark.parametrize("name", ["sph", "pcyl", "box"])
def test_matches_oracle_on_the_same_walk(cuda, name):
    g, G, dt, rf, kw, mp = _parity_case(name)
    D, n = 2e-9, 2048
    w = B.MTWalk(g, n, D, dt, mp["n_sub"], 9, kappa_MT=mp["kappa"], dwell_time=mp["dwell"],
                 surface_relaxivity=mp["rho"])
    r0 = B._to_frame(g, np.asarray(g.init_positions(n, 9), np.float32)).astype(np.float32)
    w.r.copy_(torch.from_numpy(r0))
    sums, uniq, _, _ = B._mt_run(w, G, dt, rf, **kw)
    fl, ax, ca = B._build_rf_schedule(rf, dt, G.shape[1])
    rate, has = B._build_crusher(kw["crusher"], dt, G.shape[1])
    ora = O.bloch_mt(O.geom_from(g), n_walkers=n, G=G, dt=dt, n_sub=mp["n_sub"], seed=9, r0=r0,
                     rf_flip=fl, rf_axis=ax, carrier=ca, crush=rate if has else None,
                     kappa_MT=mp["kappa"], dwell_time=mp["dwell"], D=D, T2=kw["T2"],
                     T1=kw["T1"], T2_bound=kw["T2_bound"], T1_bound=kw["T1_bound"],
                     off_resonance_hz=kw["off_resonance_hz"],
                     off_resonance_bound=kw["off_resonance_bound"], rho=mp["rho"], M0=kw["M0"],
                     echo_idx=uniq)
    r_end = w.r.cpu().numpy()
    same = np.max(np.abs(r_end - ora["r_end"]), axis=1) < 1e-4 * 2e-6
    assert same.mean() >= 0.97, same.mean()
    np.testing.assert_array_equal(w.brem.cpu().numpy()[same] > 0, ora["brem"][same] > 0)
    np.testing.assert_allclose(w.occ_total.cpu().numpy()[same], ora["occ_total"][same],
                               atol=1e-5)
    assert ora["occ_total"].mean() > 0.01 * G.shape[1]     # binding is active
    assert (ora["brem"] > 0).mean() > 0.02
    diff = np.abs(sums - ora["sums"]) / n
    assert diff.max() < 0.02 and np.median(diff) < 2e-3, diff


# ---- binding (dmipy-sim tests/test_mt_binding.py) ----------------------------------------------
@pytest.mark.parametrize("k_f,k_r", [(50.0, 100.0), (30.0, 150.0), (80.0, 80.0)])
def test_emergent_bound_fraction(cuda, k_f, k_r):
    R, D = 5e-6, 1e-9
    dt, n_t = 1e-3, 61
    _, bfrac = d.simulate_bloch(8000, D, _zero_wf(n_t, dt), d.Sphere(R), EXC,
                                kappa_MT=k_f * R / 3.0, dwell_time=1.0 / k_r, seed=3,
                                return_bound_frac=True)
    assert float(np.mean(bfrac[-20:])) == pytest.approx(k_f / (k_f + k_r), rel=0.08)


def test_binding_timestep_independence(cuda):
    R, D, k_f, k_r = 5e-6, 1e-9, 50.0, 100.0
    dt, n_t = 1e-3, 61

    def run(nsub):
        _, bf = d.simulate_bloch(6000, D, _zero_wf(n_t, dt), d.Sphere(R), EXC,
                                 kappa_MT=k_f * R / 3.0, dwell_time=1.0 / k_r, seed=3,
                                 sub_steps=nsub, return_bound_frac=True)
        return float(np.mean(bf[-20:]))

    assert run(150) == pytest.approx(run(400), rel=0.06)


def test_transverse_exchange_matches_two_pool_model(cuda):
    R, D = 2e-6, 2e-9
    T2a, T2b, k_f, k_r = 80e-3, 1e-5, 30.0, 100.0
    dt, n_t = 1e-3, 31
    echo = list(range(1, n_t))
    g = d.Sphere(R)
    S_mt = np.abs(d.simulate_bloch(12000, D, _zero_wf(n_t, dt), g, EXC, T2=T2a,
                                   kappa_MT=k_f * R / 3.0, dwell_time=1.0 / k_r, T2_bound=T2b,
                                   T1_bound=1.0, seed=5, echo_steps=echo,
                                   equilibrate_binding='off')[0])
    S0 = np.abs(d.simulate_bloch(12000, D, _zero_wf(n_t, dt), g, EXC, T2=T2a, seed=5,
                                 echo_steps=echo)[0])
    A = mt.two_pool_generator(R1a=0.1, R2a=1 / T2a, R1b=1.0, R2b=1 / T2b, k_f=k_f, k_r=k_r)
    t = np.array(echo) * dt
    s0 = np.array([1., 0, 0, 0, 0, 0, 1.])
    S_or = np.array([abs(complex(*mt.evolve_two_pool(s0, tt, A)[[0, 1]])) for tt in t])
    m = t > 0.006
    rel = np.abs(S_mt / S0 - S_or / np.exp(-t / T2a))[m] / (S_or / np.exp(-t / T2a))[m]
    assert np.max(rel) < 0.07, rel


def test_mt_attenuates_more_for_higher_kf(cuda):
    R, D, dt, n_t = 2e-6, 2e-9, 1e-3, 31

    def last_echo(k_f):
        S = np.abs(d.simulate_bloch(8000, D, _zero_wf(n_t, dt), d.Sphere(R), EXC, T2=80e-3,
                                    kappa_MT=k_f * R / 3.0, dwell_time=0.01, T2_bound=1e-5,
                                    seed=7, echo_steps=[n_t - 1])[0])
        return float(S[0])

    assert last_echo(60.0) < last_echo(15.0)


# ---- longitudinal storage (dmipy-sim tests/test_mt_storage.py) ---------------------------------
R_ST, D_ST, KF_ST, KR_ST, T1A, T1B = 5e-6, 1e-9, 30.0, 100.0, 1.0, 0.4
INVERT = [{'t_s': 0.0, 'flip_deg': 180.0, 'axis_deg': 0.0, 'duration_s': 0.0, 'offset_hz': 0.0}]


def _stored_mz(TM, *, with_mt):
    dt = 1e-3
    n_t = int(round(TM / dt)) + 1
    kw = dict(T2=80e-3, T1=T1A, M0=1.0, return_mz=True, seed=4)
    if with_mt:
        kw.update(kappa_MT=KF_ST * R_ST / 3.0, dwell_time=1.0 / KR_ST, T2_bound=1e-5,
                  T1_bound=T1B, equilibrate_binding='off')
    _, mz = d.simulate_bloch(4000, D_ST, _zero_wf(n_t, dt), d.Sphere(R_ST), INVERT, **kw)
    return float(mz[0])


def test_mt_changes_stored_magnetization(cuda):
    d_short = abs(_stored_mz(0.05, with_mt=True) - _stored_mz(0.05, with_mt=False))
    d_long = abs(_stored_mz(0.30, with_mt=True) - _stored_mz(0.30, with_mt=False))
    assert d_long > d_short > 1e-3


def test_storage_recovery_matches_two_pool_model(cuda):
    f_b = KF_ST / (KF_ST + KR_ST)
    A = mt.two_pool_generator(R1a=1 / T1A, R2a=1e3, R1b=1 / T1B, R2b=1e3, k_f=KF_ST, k_r=KR_ST,
                              M0a=1.0 - f_b, M0b=f_b)
    for TM in (0.05, 0.15, 0.4):
        s = mt.evolve_two_pool(np.array([0, 0, -(1 - f_b), 0, 0, -f_b, 1.0]), TM, A)
        assert abs(_stored_mz(TM, with_mt=True) - (s[2] + s[5])) < 0.05


# ---- the CW Z-spectrum (dmipy-sim tests/test_mt_zspectrum.py) -----------------------------------
RZ, DZ, KFZ, KRZ = 2e-6, 2e-9, 40.0, 80.0
T2a, T1a, T2b, T1b = 80e-3, 1.0, 1e-5, 1.0
W1_HZ, T_SAT, DT = 200.0, 0.025, 2e-5


def _mz(offset_hz, *, with_mt, equilibrate='auto', n=32000):
    # on resonance the walker-to-walker spread of Mz (binding histories) makes the 4 % relative
    # tolerance ~3 SE at 8000 walkers; 32000 keep it at ~6 SE
    n_t = int(round(T_SAT / DT)) + 1
    rf = [{'t_s': T_SAT / 2, 'flip_deg': 360.0 * W1_HZ * T_SAT, 'axis_deg': 0.0,
           'duration_s': T_SAT, 'offset_hz': offset_hz}]
    kw = dict(T2=T2a, T1=T1a, return_mz=True, seed=3)
    if with_mt:
        kw.update(kappa_MT=KFZ * RZ / 3.0, dwell_time=1.0 / KRZ, T2_bound=T2b, T1_bound=T1b,
                  equilibrate_binding=equilibrate)
    _, m = d.simulate_bloch(n, DZ, _zero_wf(n_t, DT), d.Sphere(RZ), rf, **kw)
    return float(m[0])


def _model_total(offsets):
    kw = dict(w1_hz=W1_HZ, t_sat=T_SAT, T1a=T1a, T2a=T2a, T1b=T1b, T2b=T2b, k_f=KFZ, k_r=KRZ)
    za = np.atleast_1d(mt.mt_z_spectrum(offsets, read_pool='a', **kw))
    zb = np.atleast_1d(mt.mt_z_spectrum(offsets, read_pool='b', **kw))
    M0b = KFZ / KRZ
    return (za + M0b * zb) / (1.0 + M0b)


def test_emergent_zspectrum_matches_two_pool_model(cuda):
    offsets = np.array([0.0, 500.0, 1000.0, 3000.0, 8000.0])
    m = np.array([_mz(o, with_mt=True) for o in offsets])
    Z = _model_total(offsets)
    rel = np.abs(m - Z) / np.maximum(np.abs(Z), 0.05)
    assert np.max(rel) < 0.04, (m, Z)


def test_equilibrate_binding_modes(cuda):
    Z_tot = float(_model_total(3000.0)[0])
    m_burn = _mz(3000.0, with_mt=True, equilibrate='burnin')
    m_fast = _mz(3000.0, with_mt=True, equilibrate='fast')
    m_off = _mz(3000.0, with_mt=True, equilibrate='off')
    assert abs(m_burn - Z_tot) < 0.02 and abs(m_fast - Z_tot) < 0.02
    assert abs(m_burn - m_fast) < 0.02
    assert m_off - Z_tot > 0.02


def test_mt_dip_shape_and_specificity(cuda):
    mz0, mz500, mz2k = (_mz(o, with_mt=True) for o in (0.0, 500.0, 2000.0))
    assert mz0 < mz500 < mz2k
    free2k = _mz(2000.0, with_mt=False)
    assert 1.0 - mz2k / free2k > 0.03 and free2k > 0.9


def test_mt_prep_gradient_echo_offresonance_mtr(cuda):
    gre = d.gradient_echo(TE=2e-3, dt=DT)
    seq = d.prepend_mt_prep(gre, dict(offset_hz=1500.0, duration_s=20e-3, b1_hz=W1_HZ,
                                      spoiler_s=1e-3, n_cycles=32.0))
    base = dict(T2=T2a, T1=T1a, seed=3)
    mt_kw = dict(kappa_MT=KFZ * RZ / 3.0, dwell_time=1.0 / KRZ, T2_bound=T2b, T1_bound=T1b)
    s_sat = abs(d.run_bloch_sequence(seq, 4000, DZ, d.Sphere(RZ), **base, **mt_kw)[0])
    s_ref = abs(d.run_bloch_sequence(gre, 4000, DZ, d.Sphere(RZ), **base, **mt_kw)[0])
    assert 1.0 - s_sat / s_ref > 0.03


def test_emergent_z_spectrum_helper(cuda):
    z = d.emergent_z_spectrum([0.0, 3000.0], d.Sphere(RZ), n_walkers=8000, diffusivity=DZ,
                              w1_hz=W1_HZ, t_sat=T_SAT, dt=DT, T2=T2a, kappa_MT=KFZ * RZ / 3.0,
                              dwell_time=1.0 / KRZ, T1=T1a, T2_bound=T2b, T1_bound=T1b, seed=3)
    np.testing.assert_allclose(z, _model_total(np.array([0.0, 3000.0])), atol=0.03)


# ---- MT-prep sequences without a bound pool (dmipy-sim tests/test_mt_prep_sequence.py) ---------
def test_mt_prep_free_water_specificity(cuda):
    gre = d.gradient_echo(TE=2e-3, dt=1e-4)

    def sig(offset_hz, flip_deg):
        prep = dict(offset_hz=offset_hz, duration_s=5e-3, flip_deg=flip_deg, spoiler_s=1e-3,
                    n_cycles=32.0)
        return abs(d.run_bloch_sequence(d.prepend_mt_prep(gre, prep), 4000, 2e-9,
                                        d.FreeDiffusion(), T2=0.05, T1=1.0, seed=0)[0])

    base = sig(0.0, 0.0)
    on, off = 1.0 - sig(0.0, 90.0) / base, 1.0 - sig(5000.0, 90.0) / base
    assert on > 0.7 and off < 0.15 and on > off


def test_crusher_dephases_transverse(cuda):
    dt, n_t = 1e-4, 21
    wf = _zero_wf(n_t, dt)
    free = d.simulate_bloch(4000, 2e-9, wf, d.FreeDiffusion(), EXC, seed=0)
    crushed = d.simulate_bloch(4000, 2e-9, wf, d.FreeDiffusion(), EXC, seed=0,
                               crusher={'windows_s': [(0.0, n_t * dt)], 'n_cycles': 32.0})
    assert abs(free[0]) == pytest.approx(1.0, rel=1e-2)
    assert abs(crushed[0]) < 0.1


# ---- the saved MT walk (dmipy-sim mt_walk.py) and its replay -----------------------------------
def test_mt_trajectories_follow_the_oracle_walk(cuda):
    """All-free start: the saved walk is the oracle's MT walk from the same start and draws
    (end positions to float16 precision, occupancy summed over the samples)."""
    R, D, n = 2e-6, 2e-9, 2048
    g = d.Sphere(R)
    traj, dt, nsub, dt_sim, bf, dlog = d.simulate_mt_trajectories(
        n, D, g, 0.004, 1e-4, 3e-5, 2e-3, seed=11, sub_steps=4, equilibrate_binding='off')
    assert traj.dtype == np.float16 and traj.shape == (n, 41, 3) and nsub == 4
    assert bf.shape == dlog.shape == (n, 41)
    r0 = np.asarray(g.init_positions(n, 11), np.float32)
    ora = O.bloch_mt(O.geom_from(g), n_walkers=n, G=np.zeros((1, 41, 3)), dt=dt, n_sub=4,
                     seed=11, r0=r0, rf_flip=np.zeros(41), rf_axis=np.zeros(41), kappa_MT=3e-5,
                     dwell_time=2e-3, D=D)
    # saved in float16 metres, as the reference saves them: micrometre positions are float16
    # subnormals, spaced 2^-24 m (6e-8 m) apart
    err = np.max(np.abs(traj[:, -1].astype(np.float64) - ora["r_end"]), axis=1)
    assert np.mean(err <= 2.0 ** -25 * 1.01) > 0.97
    np.testing.assert_allclose(bf.astype(np.float64).sum(1), ora["occ_total"], atol=41 * 1e-3)
    assert np.all(dlog <= 0) and np.any(dlog < 0) and np.any(bf > 0)


def test_mt_trajectories_bound_fraction_and_replayed_exchange(cuda):
    R, D, k_f, k_r = 2e-6, 2e-9, 30.0, 100.0
    g = d.Sphere(R)
    traj, dt, nsub, _, bf, dlog = d.simulate_mt_trajectories(
        12000, D, g, 0.03, 1e-3, k_f * R / 3.0, 1.0 / k_r, seed=3)
    assert nsub == d.mt_sub_steps(g, D, dt, 1.0 / k_r)
    assert np.all(np.linalg.norm(traj.astype(np.float64), axis=-1) < R + 2.0 ** -24)
    assert float(bf.astype(np.float64).mean()) == pytest.approx(k_f / (k_f + k_r), rel=0.08)
    # replay with the bound-pool blend from an all-free start: transverse exchange against the
    # two-pool model, as for the forward MT walk
    traj0, dt0, _, _, bf0, _ = d.simulate_mt_trajectories(
        12000, D, g, 0.03, 1e-3, k_f * R / 3.0, 1.0 / k_r, seed=4, equilibrate_binding='off')
    echo = list(range(1, 31))
    G0 = np.zeros((1, 31, 3))
    S_mt = np.abs(d.replay_bloch(traj0, dt0, G0, dt0, EXC, T2=80e-3, bound_frac=bf0,
                                 T2_bound=1e-5, T1_bound=1.0, echo_steps=echo))[0]
    S0 = np.abs(d.replay_bloch(traj0, dt0, G0, dt0, EXC, T2=80e-3, echo_steps=echo))[0]
    A = mt.two_pool_generator(R1a=0.1, R2a=1 / 80e-3, R1b=1.0, R2b=1e5, k_f=k_f, k_r=k_r)
    t = np.array(echo) * dt0
    S_or = np.array([abs(complex(*mt.evolve_two_pool(np.array([1., 0, 0, 0, 0, 0, 1.]), tt,
                                                     A)[[0, 1]])) for tt in t])
    m = t > 0.006
    rel = np.abs(S_mt / S0 - S_or / np.exp(-t / 80e-3))[m] / (S_or / np.exp(-t / 80e-3))[m]
    assert np.max(rel) < 0.1, rel
