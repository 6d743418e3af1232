"""The free-flight packed-cylinder kernel (csrc/walk_ff.cuh).

A packed-cylinder walk in the basis phase form runs on the free-flight kernel when asked for
(schedule "free_flight"): each lane walks its own walker and skips the wall scan while the walker
stays inside the wall-free disc of its last scan.  Skipping must not change a single bit: the same
kernel scanning on every sub-step (schedule "scan_every") walks every walker to the same position,
weight and phase, and the two ensembles are equal.  Against the lock-step kernel (a separate compilation of the same step
functions) walkers agree over short walks and ensembles within 4 standard errors over long ones.
"""
import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import core

pytestmark = pytest.mark.gpu
D = 2e-9


def _lattice(**kw):
    radii, centers, L = d.lattice_cylinders(16, 0.6, 2e-6, 0.5e-6, seed=0)
    return d.PackedCylinders(radii, centers, L, **kw)


def _waveform(n_t):
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(6, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    pg = d.set_b(d.pgse(0.004, 0.012, 0.05, bv, n_t), np.linspace(0.5e9, 3e9, 6))
    og = d.set_b(d.ogse(100.0, 0.016, 0.05, bv[:2], n_t), 1e9)
    return d.Waveform(G=np.concatenate([pg.G, og.G]).astype(np.float32), dt=pg.dt,
                      echo_idx=n_t - 1)


# name -> (geometry keywords, fused sub-steps, T2)
CASES = {
    "reflect_replay": (dict(), False, None),
    "reflect_fused_t2": (dict(), True, 0.06),
    "relax_replay": (dict(surface_relaxivity_t2=5e-6), False, None),
    "relax_fused": (dict(surface_relaxivity_t2=5e-6), True, None),
    "permeate_fused": (dict(permeability=2e-5), True, None),
}


def _walk(case, schedule, n_t, n, seed, keep=None, echoes=None):
    kw, fused, T2 = CASES[case]
    geom = _lattice(**kw)
    wf = _waveform(n_t)
    if keep is not None:   # the first samples only, at the waveform's own time step
        wf = d.Waveform(G=np.ascontiguousarray(wf.G[:, :keep]), dt=wf.dt, echo_idx=keep - 1)
    G, chi = core._waveform_arrays(wf, geom)
    S = core.fused_sub_steps(geom, D, wf.dt) if fused else core.replay_sub_steps(geom, D, wf.dt)
    return core.run_walk(geom, n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                         phase_per_substep=fused, seed=seed, chi=chi, T2=T2,
                         want_positions=True, want_walker_signals=True, echo_idx=echoes,
                         schedule=schedule), S


@pytest.mark.parametrize("case", sorted(CASES))
def test_free_flight_is_bit_identical_to_scanning_every_sub_step(cuda, case):
    n_t = 60 if case.startswith("permeate") else 200
    ff, S = _walk(case, "free_flight", n_t, 12000, 5)
    ev, _ = _walk(case, "scan_every", n_t, 12000, 5)
    for key in ("pos", "log_w", "phi"):
        a, b = ff.extras[key].cpu().numpy(), ev.extras[key].cpu().numpy()
        assert np.array_equal(a, b), (key, int(np.sum(a != b)))
    assert np.array_equal(ff.signal, ev.signal)
    assert ff.status == ev.status


def test_free_flight_emits_every_echo(cuda):
    """A CPMG-like echo list: every echo of every walker reaches the sums, in either schedule."""
    n_t = 120
    echoes = np.arange(9, n_t, 10)
    ff, _ = _walk("reflect_fused_t2", "free_flight", n_t, 6000, 3, echoes=echoes)
    ev, _ = _walk("reflect_fused_t2", "scan_every", n_t, 6000, 3, echoes=echoes)
    assert ff.signal.shape[0] == len(echoes)
    assert np.array_equal(ff.signal, ev.signal)
    lk, _ = _walk("reflect_fused_t2", "lockstep", n_t, 6000, 3, echoes=echoes)
    np.testing.assert_allclose(ff.signal, lk.signal, atol=2e-2)


@pytest.mark.parametrize("case", sorted(CASES))
def test_free_flight_walks_the_lockstep_kernels_walkers(cuda, case):
    """Over a short walk the free-flight and lock-step kernels move every walker alike (the two
    compilations may contract a multiply-add differently in rare spots, and a packed substrate is
    a chaotic billiard that amplifies a last-bit difference)."""
    ff, _ = _walk(case, "free_flight", 400, 8000, 9, keep=3)
    lk, _ = _walk(case, "lockstep", 400, 8000, 9, keep=3)
    pf, pl = ff.extras["pos"].cpu().numpy(), lk.extras["pos"].cpu().numpy()
    pos_tol = 1e-4 * 0.9e-6
    same = np.all(np.abs(pf - pl) <= pos_tol, axis=1)
    assert same.mean() >= 0.99, same.mean()
    np.testing.assert_allclose(ff.extras["phi"].cpu().numpy()[same],
                               lk.extras["phi"].cpu().numpy()[same], rtol=1e-5, atol=1e-5)
    rho = CASES[case][0].get("surface_relaxivity_t2", 0.0)
    np.testing.assert_allclose(ff.extras["log_w"].cpu().numpy()[same],
                               lk.extras["log_w"].cpu().numpy()[same], rtol=1e-5,
                               atol=1e-7 + 4 * 2 * rho / D * pos_tol)


@pytest.mark.parametrize("case", sorted(CASES))
def test_free_flight_ensemble_matches_the_lockstep_kernel(cuda, case):
    """Over a long walk the two ensembles agree within 4 combined standard errors."""
    n_t = 60 if case.startswith("permeate") else 120
    ff, _ = _walk(case, "free_flight", n_t, 20000, 10)
    lk, _ = _walk(case, "lockstep", n_t, 20000, 10)
    se = np.hypot(ff.stderr[0], lk.stderr[0])
    z = (ff.signal[0] - lk.signal[0]) / np.maximum(se, 1e-9)
    assert np.max(np.abs(z)) < 4.0, z


def test_schedule_is_validated(cuda):
    geom = _lattice()
    wf = _waveform(20)
    G, chi = core._waveform_arrays(wf, geom)
    with pytest.raises(ValueError):
        core.run_walk(geom, n_walkers=64, diffusivity=D, G=G, dt=wf.dt, sub_steps=2,
                      phase_per_substep=False, seed=0, chi=chi, schedule="sometimes")
