"""The wide-block packed-cylinder kernel against the general walk kernel.

A packed-cylinder walk in the basis phase form that exports no trajectories, boundary weights or
occupancies runs on the wide-block kernel (csrc/walk_wide.cuh); asking for per-sub-step
occupancies keeps the general kernel (which computes them alongside the same walk).  Both draw
the same Philox stream and call the same step function, in every wall mode and phase semantics
(replay / fused); the wide kernel only changes the occupancy plan.
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


CASES = {
    "reflect_replay": (dict(), False, True, None),
    "reflect_fused_t2": (dict(), True, True, 0.06),
    "relax_replay": (dict(surface_relaxivity_t2=5e-6), False, True, None),
    "relax_fused": (dict(surface_relaxivity_t2=5e-6), True, True, None),
    "permeate_fused": (dict(permeability=2e-5), True, True, None),
}


def _walks(case, n_t, n, S_max, seed, keep=None):
    kw, fused, basis, T2 = CASES[case]
    geom = _lattice(**kw)
    wf = _waveform(n_t)
    if keep is not None:   # the first samples only: a short walk at the waveform's own time step
        wf = d.Waveform(G=np.ascontiguousarray(wf.G[:, :keep]), dt=wf.dt, echo_idx=keep - 1)
    G, chi = core._waveform_arrays(wf, geom)
    S = core.fused_sub_steps(geom, D, wf.dt) if fused else core.replay_sub_steps(geom, D, wf.dt)
    S = min(S, S_max)
    common = dict(n_walkers=n, diffusivity=D, G=G, dt=wf.dt, sub_steps=S,
                  phase_per_substep=fused, seed=seed, chi=chi, T2=T2, want_positions=True,
                  want_walker_signals=True, use_basis=basis)
    return core.run_walk(geom, **common), core.run_walk(geom, want_comp_occ=True, **common)


@pytest.mark.parametrize("case", sorted(CASES))
def test_wide_kernel_walks_the_general_kernels_walkers(cuda, case):
    """Over a short walk (a couple of dozen sub-steps) the two kernels move every walker alike:
    the compilations may contract a multiply-add differently in rare spots, and a packed
    substrate is a chaotic billiard that amplifies such a last-bit difference, so walker
    identity is asked for over short walks only."""
    wide, gen = _walks(case, 400, 8000, 12, 9, keep=3)     # 40 us samples, <= 36 sub-steps
    pl, pg = wide.extras["pos"].cpu().numpy(), gen.extras["pos"].cpu().numpy()
    pos_tol = 1e-4 * 0.9e-6
    same = np.all(np.abs(pl - pg) <= pos_tol, axis=1)
    assert same.mean() >= 0.99, same.mean()
    np.testing.assert_allclose(wide.extras["phi"].cpu().numpy()[same],
                               gen.extras["phi"].cpu().numpy()[same], rtol=1e-5, atol=1e-5)
    # a wall hit costs 2 rho/D x (penetration depth) of log-weight, and the depth is a
    # difference of two near-equal radii: walkers that agree to pos_tol may differ by
    # 2 rho/D pos_tol per hit (a few hits in this short walk)
    rho = CASES[case][0].get("surface_relaxivity_t2", 0.0)
    np.testing.assert_allclose(wide.extras["log_w"].cpu().numpy()[same],
                               gen.extras["log_w"].cpu().numpy()[same], rtol=1e-5,
                               atol=1e-7 + 4 * 2 * rho / D * pos_tol)


@pytest.mark.parametrize("case", sorted(CASES))
def test_wide_kernel_ensemble_matches_the_general_kernel(cuda, case):
    """Over a long walk the two ensembles agree within 4 combined standard errors."""
    wide, gen = _walks(case, 120, 20000, 12, 10)
    se = np.hypot(wide.stderr[0], gen.stderr[0])
    z = (wide.signal[0] - gen.signal[0]) / np.maximum(se, 1e-9)
    assert np.max(np.abs(z)) < 4.0, z
