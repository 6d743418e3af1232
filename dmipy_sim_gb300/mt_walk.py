"""The magnetisation-transfer random walk saved for replay: ``simulate_mt_trajectories``
(mt_walk.py:43-239 of dmipy-sim).

The walk binds at the walls exactly as the forward MT walk does (``dmsim_bloch_mt`` with the
magnetisation off): a free walker sticks with p = min(1, kappa_MT/D * 2 sum d_perp) and stays put
for an exponential dwell.  Saved per sample: the position, the fraction of the sample's
sub-steps spent bound, and the free pool's boundary log-weight (the wall contacts of free
sub-steps that did not bind).  ``trajectories.replay_bloch`` turns them into signals
(``bound_frac``, ``T2_bound`` / ``T1_bound``).
"""
import numpy as np
import torch

from . import mt as _mt
from .bloch import MTWalk, _MT_GEOMETRIES
from .core import _check_gpu, _to_frame, _to_lab, mt_sub_steps

__all__ = ["simulate_mt_trajectories"]


def simulate_mt_trajectories(n_walkers, diffusivity, geometry, T_max, dt_save, kappa_MT,
                             dwell_time, seed=42, walker_batch_size=50_000, sub_steps=None,
                             equilibrate_binding="auto", require_gpu=None):
    """Random walk with MT surface binding.  Returns ``(trajectories (n, n_t, 3) float16,
    dt_actual, sub_steps, dt_sim, bound_frac (n, n_t) float16, dlog_boundary_unit (n, n_t)
    float16)``; n_t = round(T_max/dt_save) + 1 samples, the bound pool brought to its
    equilibrium occupancy first (``equilibrate_binding``: 'auto'/'burnin', 'fast', 'off')."""
    if kappa_MT > 0.0 and dwell_time <= 0.0:
        raise ValueError("dwell_time must be > 0 when kappa_MT > 0.")
    name = type(geometry).__name__
    if name not in _MT_GEOMETRIES:
        raise TypeError(f"{name} has no reflect_with_log_weight; MT binding needs the "
                        "boundary-local-time channel (Sphere / Cylinder / Box1D / Ellipsoid / "
                        "packed cylinders or spheres).")
    mode = (_mt.resolve_equilibrate_mode(equilibrate_binding, geometry) if kappa_MT > 0.0
            else "off")
    _check_gpu(require_gpu)
    n_walkers = int(n_walkers)
    n_t = int(round(T_max / dt_save)) + 1
    dt_actual = T_max / (n_t - 1)
    if sub_steps is None:
        sub_steps = mt_sub_steps(geometry, diffusivity, dt_actual, dwell_time)
    sub_steps = int(sub_steps)
    dt_sim = dt_actual / sub_steps
    w = MTWalk(geometry, n_walkers, float(diffusivity), dt_actual, sub_steps, seed,
               kappa_MT=float(kappa_MT), dwell_time=float(dwell_time) if dwell_time > 0 else 1.0,
               surface_relaxivity=0.0)
    if not kappa_MT > 0.0:
        w.p.kappa_mt_over_D = 0.0
    r0 = np.asarray(geometry.init_positions(n_walkers, int(seed)), np.float32)
    w.r.copy_(torch.from_numpy(np.ascontiguousarray(_to_frame(geometry, r0), np.float32)))
    if mode == "fast":
        S_V = _mt.surface_to_volume(geometry)
        P_eq = _mt.bound_fraction(kappa_MT, dwell_time, S_V)
        rng = np.random.default_rng([int(seed) & 0xFFFFFFFF, 0xB0117E])
        u_state, u_dwell = rng.random((2, n_walkers), dtype=np.float32)
        b0 = np.where(u_state < np.float32(P_eq),
                      -np.log(np.maximum(u_dwell, np.float32(1e-20)))
                      * np.float32(w.p.dwell_substeps), np.float32(0.0)).astype(np.float32)
        w.brem.copy_(torch.from_numpy(b0))
    elif mode == "burnin":
        # chunks of about one dwell in sub-steps until the occupancy plateaus (mt.py:168-189)
        n_chunk = max(4, int(round(float(dwell_time) / dt_sim)))
        state = {"w": w}

        def chunk(r, keys, brem):
            return r, keys, brem, state["w"].burn_chunk(n_chunk, sub=1)

        _, _, _, _, converged = _mt.equilibrate_burnin_plateau(chunk, None, None, None)
        if not converged:
            import warnings
            warnings.warn("equilibrate_binding: bound occupancy did not plateau within the "
                          "burn-in cap (long-dwell / heterogeneous substrate?); the saved walk "
                          "may be under-equilibrated.", stacklevel=2)
    dev = w.dev
    traj = torch.empty((n_walkers, n_t, 3), dtype=torch.float16, device=dev)
    occ = torch.empty((n_walkers, n_t), dtype=torch.float32, device=dev)
    dlog = torch.empty((n_walkers, n_t), dtype=torch.float32, device=dev)
    w.p.n_meas = 1
    w._run(n_t, 0, {"occ": occ.data_ptr(), "sums": None, "G": None, "rot": None,
                    "crush": None, "n_echo": 0, "echo_idx": None, "traj": traj.data_ptr(),
                    "traj_f16": 1, "dlog_free": dlog.data_ptr()})
    t = traj.cpu().numpy()
    if geometry._frame() is not None:
        t = _to_lab(geometry, t.reshape(-1, 3).astype(np.float32)).reshape(t.shape)
        t = t.astype(np.float16)
    return (t, dt_actual, sub_steps, dt_sim, occ.cpu().numpy().astype(np.float16),
            dlog.cpu().numpy().astype(np.float16))
