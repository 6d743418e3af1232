"""The vector-Bloch replay of a stored walk (trajectories.replay_bloch): the device replay
against dmipy-sim's own numpy replay_bloch (FP64) on a seeded walk with every option group
(tests/golden/replay_bloch_kat.npz), the hard-pulse twin, and the host helpers of the replay
module against the reference's outputs."""
from pathlib import Path

import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300 import trajectories as T
from golden.make_golden import replay_bloch_cases, replay_bloch_inputs


@pytest.fixture(scope="module")
def z():
    return np.load(Path(__file__).parent / "golden" / "replay_bloch_kat.npz")


def test_replay_helpers_match_reference(z):
    np.testing.assert_array_equal(T.pathway_sign_se(37, 1e-4, 2.2e-3, te_frac=0.45), z["sign_se"])
    np.testing.assert_array_equal(T.unwrap_periodic(z["wrapped"], 6e-6), z["unwrapped"])
    np.testing.assert_array_equal(T.unwrap_periodic(z["wrapped"], 6e-6, periodic_axes=(0, 1, 2)),
                                  z["unwrapped_xyz"])
    np.testing.assert_allclose(T.finite_180_longitudinal_dwell(np.linspace(-3, 3, 11), 2e-3, 0.3),
                               z["dwell180"], rtol=1e-15)
    x = replay_bloch_inputs()
    np.testing.assert_allclose(T.pre_pulse_gradient_phase(x["traj"], x["dt_traj"], x["G"],
                                                          x["dt_wf"], 150), z["phi_pre"],
                               rtol=1e-12, atol=1e-12)


def test_rf_increments_spread_centre_and_shape():
    start, flip, axis, off, act = T._rf_increments(
        [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0},
         {'t_s': 1e-3, 'flip_deg': 180.0, 'duration_s': 4e-4, 'offset_hz': 100.0},
         {'t_s': 2e-3, 'flip_deg': 60.0, 'duration_s': 3e-4, 'b1_envelope': [0.0, 1.0, 0.0]}],
        1e-4, 30)
    assert list(np.diff(start)[:1]) == [1] and act[0] == 1
    assert list(np.nonzero(np.diff(start) > 0)[0]) == [0, 8, 9, 10, 11, 19, 20, 21]
    np.testing.assert_allclose(flip[1:5], np.full(4, np.pi / 4))
    np.testing.assert_allclose(flip[5:].sum(), np.deg2rad(60.0))
    assert flip[6] > flip[5] and flip[6] > flip[7]
    np.testing.assert_allclose(off[8:12], 2 * np.pi * 100.0 * 1e-4)
    assert axis[0] == pytest.approx(np.pi / 2)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["plain", "relax", "comp", "mt", "susc"])
def test_device_replay_matches_reference(cuda, z, name):
    x = replay_bloch_inputs()
    kw = replay_bloch_cases(x)[name]
    got = d.replay_bloch(x["traj"], x["dt_traj"], x["G"], x["dt_wf"], x["rf"], **kw)
    if isinstance(got, tuple):
        np.testing.assert_allclose(got[0], z[f"{name}_mlast"], rtol=1e-9, atol=1e-12)
        got = got[1]
    ref = z[name]
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_device_replay_float16_walk_and_torch_input(cuda):
    import torch
    x = replay_bloch_inputs()
    t16 = x["traj"].astype(np.float16)
    a = d.replay_bloch(t16, x["dt_traj"], x["G"], x["dt_wf"], x["rf"], T2=0.07)
    b = d.replay_bloch(torch.from_numpy(t16).cuda(), x["dt_traj"], x["G"], x["dt_wf"], x["rf"],
                       T2=0.07)
    c = d.replay_bloch(t16.astype(np.float32), x["dt_traj"], x["G"], x["dt_wf"], x["rf"], T2=0.07)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(a, c, rtol=1e-12)


@pytest.mark.gpu
def test_hard_pulse_twin(cuda):
    """replay_bloch_jax: every event hard at its sample, the last one on a shared sample acting,
    echoes in sorted order with repeats."""
    x = replay_bloch_inputs()
    rf = [{'t_s': 0.0, 'flip_deg': 90.0, 'axis_deg': 90.0},
          {'t_s': 7.5e-3, 'flip_deg': 180.0, 'duration_s': 8e-4, 'offset_hz': 250.0},
          {'t_s': 7.5e-3, 'flip_deg': 170.0, 'axis_deg': 10.0}]
    hard = [rf[0], {'t_s': 7.5e-3, 'flip_deg': 170.0, 'axis_deg': 10.0}]
    a = d.replay_bloch_jax(x["traj"], x["dt_traj"], x["G"], x["dt_wf"], rf, T2=0.07,
                           echo_steps=[149, 40, 149])
    b = d.replay_bloch(x["traj"], x["dt_traj"], x["G"], x["dt_wf"], hard, T2=0.07,
                       echo_steps=[40, 149])
    np.testing.assert_allclose(a, b[:, [0, 1, 1]], rtol=1e-12)
