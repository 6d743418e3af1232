"""GPU replay operator against the reference's replay on the same trajectories (kat.npz), and
the walk-once + replay path against the fused single-pass replay semantics."""
import numpy as np
import pytest

import dmipy_sim_gb300 as d
from dmipy_sim_gb300.trajectories import replay as tr_replay

pytestmark = pytest.mark.gpu
D = 2e-9


def test_replay_matches_reference(cuda, kat):
    sig = tr_replay(kat["rep_traj"], float(kat["rep_dt"]), kat["rep_G"], float(kat["rep_dt"]),
                   chi_perp=kat["rep_chi"], dlog_boundary_unit=kat["rep_dlog"], T2=0.08, T1=0.9,
                   surface_relaxivity=1e-5, D=D, stimulated_echo=True)
    np.testing.assert_allclose(sig, kat["rep_signal"], rtol=1e-4, atol=1e-6)
    sig = tr_replay(kat["rep_traj"], float(kat["rep_dt"]), kat["rep_G"], float(kat["rep_dt"]))
    np.testing.assert_allclose(sig, kat["rep_signal_plain"], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("geom", [d.Cylinder(5e-6, (0, 0, 1), surface_relaxivity_t2=1e-6),
                                  d.Sphere(4e-6), d.FreeDiffusion()])
def test_walk_once_replay_equals_single_pass(cuda, geom):
    rng = np.random.default_rng(0)
    bv = rng.normal(size=(6, 3))
    bv /= np.linalg.norm(bv, axis=1, keepdims=True)
    wf = d.set_b(d.pgse(0.01, 0.04, 0.05, bv, 300), 1e9)
    n = 20_000
    T_max = wf.dt * (wf.G.shape[1] - 1)
    out = d.simulate_trajectories(n, D, geom, T_max, wf.dt, seed=7, save_relaxation_data=True)
    traj, dt_traj, S, dt_sim, dlog, comp = out
    assert traj.dtype == np.float16 and traj.shape == (n, wf.G.shape[1], 3)
    rho = geom.surface_relaxivity_t2
    s_rep = tr_replay(traj, dt_traj, wf.G, wf.dt, dlog_boundary_unit=dlog,
                     surface_relaxivity=rho, D=D if rho else None)
    s_one = d.simulate(n, D, wf, geom, seed=7, engine="replay")
    # same walk (same seed and stream); they differ only by the float16 storage of positions
    np.testing.assert_allclose(s_rep, s_one, atol=2e-3)
