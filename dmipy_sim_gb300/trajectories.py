"""Replay operator on saved walks (trajectories.py:360-641 of dmipy-sim).

The gradient phase phi[m, w] = gamma * dt * sum_t G(t) . r_w(t) runs on the GPU
(``dmsim_replay``: FP32 with Kahan compensation, FP64 ensemble sums); the walker-independent
T2/T1 factors and the resampling of G and chi onto the trajectory grid follow the reference's host
code.
"""
import numpy as np
import torch

from . import _lib
from .constants import GAMMA


def _resample(G, chi_perp, n_t_traj, dt_traj, dt_wf):
    """G linearly and chi by nearest neighbour onto the trajectory grid (trajectories.py:470-536)."""
    n_meas, n_t_wf, _ = G.shape
    if abs(dt_wf - dt_traj) / max(abs(dt_traj), 1e-30) > 1e-9:
        t_wf = np.arange(n_t_wf, dtype=np.float64) * dt_wf
        t_tr = np.arange(n_t_traj, dtype=np.float64) * dt_traj
        Gt = np.zeros((n_meas, n_t_traj, 3), dtype=G.dtype)
        for m in range(n_meas):
            for a in range(3):
                Gt[m, :, a] = np.interp(t_tr, t_wf, G[m, :, a], left=0.0, right=0.0)
    elif n_t_wf == n_t_traj:
        Gt = G
    elif n_t_wf > n_t_traj:
        Gt = G[:, :n_t_traj, :]
    else:
        Gt = np.zeros((n_meas, n_t_traj, 3), dtype=G.dtype)
        Gt[:, :n_t_wf, :] = G
    t_wf = np.arange(n_t_wf, dtype=np.float64) * dt_wf
    t_tr = np.arange(n_t_traj, dtype=np.float64) * dt_traj

    def rs(c1):
        step = t_wf[-1] / max(n_t_wf - 1, 1) if n_t_wf > 1 else dt_traj
        idx = np.round(t_tr / step).astype(int)
        ok = (idx >= 0) & (idx < n_t_wf)
        return np.where(ok, c1[np.clip(idx, 0, n_t_wf - 1)], 0.0)

    if chi_perp.ndim == 2:
        chi_r = np.stack([rs(chi_perp[m]) for m in range(n_meas)])
    else:
        chi_r = rs(chi_perp)[None, :]
    return Gt, chi_r


def replay(trajectory, dt_traj, G, dt_wf, *, chi_perp=None, dlog_boundary_unit=None, T2=None,
           T1=None, surface_relaxivity=None, D=None, stimulated_echo=False, comp_traj=None,
           T2_per_comp=None, T1_per_comp=None, return_walker_signals=False, susceptibility=None,
           eps_P=None):
    """Signal of a waveform + relaxation applied to saved trajectories (trajectories.py:360-641).

    ``trajectory`` is (n, n_t, 3) float16/float32 (numpy or a CUDA tensor).  Returns ``signals``
    (n_meas,) float64, or ``(phi (n_meas, n), log_w_total, signals)`` with
    ``return_walker_signals``.
    """
    if isinstance(trajectory, dict) and trajectory.get("compressed"):
        return _replay_compressed(trajectory, G, dt_wf, chi_perp=chi_perp, T2=T2, T1=T1,
                                  surface_relaxivity=surface_relaxivity, D=D,
                                  stimulated_echo=stimulated_echo, comp_traj=comp_traj,
                                  T2_per_comp=T2_per_comp, T1_per_comp=T1_per_comp,
                                  return_walker_signals=return_walker_signals,
                                  susceptibility=susceptibility)
    if isinstance(trajectory, dict):
        raise ValueError("a trajectory dict must be a compressed master (compressed=True)")
    if susceptibility is not None:
        raise NotImplementedError("susceptibility off-resonance replay is not supported")
    lib = _lib.load()
    dev = _lib.device()
    G = np.asarray(G, dtype=np.float32)
    n_meas, n_t_wf, _ = G.shape
    if torch.is_tensor(trajectory):
        tr = trajectory.to(dev)
    else:
        tr = torch.from_numpy(np.ascontiguousarray(trajectory)).to(dev)
    if tr.dtype not in (torch.float16, torch.float32):
        tr = tr.float()
    tr = tr.contiguous()
    n_w, n_t_traj, _ = tr.shape
    chi = np.ones(n_t_wf) if chi_perp is None else np.asarray(chi_perp, dtype=np.float64)
    Gt, chi_r = _resample(G, chi, n_t_traj, float(dt_traj), float(dt_wf))

    # walker-independent and walker-dependent log-weights (trajectories.py:577-613)
    lw_scalar = np.zeros(n_meas)
    lw_walker = None
    if T2_per_comp is not None or T1_per_comp is not None:
        if comp_traj is None:
            raise ValueError("comp_traj required when T2_per_comp/T1_per_comp is provided.")
        comp = np.asarray(comp_traj)

        def inv_at(inv):
            if np.issubdtype(comp.dtype, np.floating):
                if inv.shape[0] != 2:
                    raise ValueError("Fractional (float) comp_traj requires exactly 2 entries")
                return inv[0] + comp.astype(np.float64) * (inv[1] - inv[0])
            return inv[comp]
        if T2_per_comp is not None:
            lw_walker = -dt_traj * (chi_r @ inv_at(1.0 / np.asarray(T2_per_comp, float)).T)
        if T1_per_comp is not None:
            t1 = -dt_traj * ((1.0 - chi_r) @ inv_at(1.0 / np.asarray(T1_per_comp, float)).T)
            lw_walker = t1 if lw_walker is None else lw_walker + t1
    if T2_per_comp is None and T2 is not None:
        lw_scalar -= (dt_traj / T2) * chi_r.sum(axis=1)
    if T1_per_comp is None and T1 is not None:
        lw_scalar -= (dt_traj / T1) * (n_t_traj - chi_r.sum(axis=1))
    if surface_relaxivity is not None:
        if D is None:
            raise ValueError("D (diffusivity) must be provided when surface_relaxivity is not None.")
        if dlog_boundary_unit is None:
            raise ValueError("dlog_boundary_unit must be provided when surface_relaxivity is "
                             "not None.  Re-run simulate_trajectories with save_relaxation_data=True.")
        dl = np.asarray(dlog_boundary_unit, dtype=np.float64)
        ls = (surface_relaxivity / D) * (chi_r @ dl.T)
        lw_walker = ls if lw_walker is None else lw_walker + ls
    if lw_walker is not None and lw_walker.shape[0] != 1:
        raise NotImplementedError("per-measurement chi with walker-dependent relaxation weights "
                                  "is not supported by the GPU replay")

    G_dev = torch.from_numpy(np.ascontiguousarray(Gt.transpose(1, 0, 2))).to(dev)
    lw_dev = None if lw_walker is None else torch.from_numpy(
        lw_walker[0].astype(np.float32)).to(dev)
    sums = torch.zeros((n_meas, 3), dtype=torch.float64, device=dev)
    phi = torch.empty((n_w, n_meas), dtype=torch.float32, device=dev) \
        if return_walker_signals else None
    nbytes = lib.dmsim_replay_workspace_bytes(n_w, n_t_traj, n_meas)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    rc = lib.dmsim_replay(_lib.ptr(tr), 1 if tr.dtype == torch.float16 else 0, n_w, n_t_traj,
                          _lib.ptr(G_dev), n_meas, np.float32(GAMMA * dt_traj), _lib.ptr(lw_dev),
                          _lib.ptr(sums), _lib.ptr(phi), _lib.ptr(ws), nbytes, _lib.stream_handle())
    _lib.check(rc, "dmsim_replay")
    s = sums.cpu().numpy()
    signals = np.exp(lw_scalar) * s[:, 0] / n_w
    if stimulated_echo:
        signals = signals * 0.5
    if return_walker_signals:
        lw_tot = lw_scalar[:, None] + (np.zeros((1, 1)) if lw_walker is None else lw_walker)
        return phi.cpu().numpy().T.astype(np.float64), lw_tot, signals
    return signals


def _replay_compressed(master, G, dt_wf, *, chi_perp, T2, T1, surface_relaxivity, D,
                       stimulated_echo, comp_traj, T2_per_comp, T1_per_comp,
                       return_walker_signals, susceptibility):
    """Replay of a compressed master (simulate_trajectories(compress=K); trajectories.py:258-357).

    The phase is taken in mode space -- the stored (n, K, 3) DCT-II bands contracted with the
    first K bands of DCT(G) on the trajectory grid, one ``dmsim_replay`` pass on the GPU -- and the
    trajectory is never reconstructed.  Surface relaxivity reads the stored cumulative endpoint
    (no gate) or the decoded per-save channel (gated); per-compartment T2/T1 read ``comp_traj``."""
    from scipy.fft import dct
    from . import compression as _cx
    if susceptibility is not None:
        raise NotImplementedError(
            "susceptibility replay needs the raw trajectory: the off-resonance phase is not "
            "linear in position and does not commute with the DCT")
    K, n_t, dt_traj = int(master["K"]), int(master["n_t"]), float(master["dt_traj"])
    C = np.ascontiguousarray(master["pos_modes"], np.float32)
    n_w = C.shape[0]
    G = np.asarray(G, np.float64)
    n_meas, n_t_wf, _ = G.shape
    chi = np.ones(n_t_wf) if chi_perp is None else np.asarray(chi_perp, np.float64)
    Gt, chi_r = _resample(G, chi, n_t, dt_traj, float(dt_wf))
    if chi_perp is None:
        chi_r = np.ones((1, n_t))
    Ghat = dct(Gt, type=2, norm="ortho", axis=1)[:, :K, :]

    lw_scalar = np.zeros(n_meas)
    lw_walker = None

    def add(x):
        nonlocal lw_walker
        lw_walker = x if lw_walker is None else lw_walker + x

    def inv_at(inv, comp):
        comp = np.asarray(comp)
        if np.issubdtype(comp.dtype, np.floating):
            return inv[0] + comp.astype(np.float64) * (inv[1] - inv[0])
        return inv[comp]
    if T2_per_comp is not None:
        comp = comp_traj if comp_traj is not None else master.get("comp_traj")
        if comp is None:
            raise ValueError("comp_traj required when T2_per_comp is provided.")
        add(-dt_traj * (chi_r @ inv_at(1.0 / np.asarray(T2_per_comp, np.float64), comp).T))
    elif T2 is not None:
        lw_scalar -= (dt_traj / T2) * chi_r.sum(1)
    if T1_per_comp is not None:
        comp = comp_traj if comp_traj is not None else master.get("comp_traj")
        if comp is None:
            raise ValueError("comp_traj required when T1_per_comp is provided.")
        add(-dt_traj * ((1.0 - chi_r) @ inv_at(1.0 / np.asarray(T1_per_comp, np.float64),
                                                 comp).T))
    elif T1 is not None:
        lw_scalar -= (dt_traj / T1) * (n_t - chi_r.sum(1))
    if surface_relaxivity is not None:
        if D is None:
            raise ValueError("D must be provided when surface_relaxivity is not None.")
        if "blt_endpoint" not in master:
            raise ValueError("compressed master lacks the boundary channel "
                             "(re-run simulate_trajectories with save_relaxation_data=True).")
        if chi_perp is None:
            add((surface_relaxivity / D) * np.asarray(master["blt_endpoint"], np.float64)[None, :])
        else:
            blt = _cx.decode_boundary_dct(
                {"blt_dct_coeffs": master["blt_modes"], "blt_endpoint": master["blt_endpoint"]},
                {"n_t": n_t, "K": K}).astype(np.float64)
            add((surface_relaxivity / D) * (chi_r @ blt.T))
    if lw_walker is not None and lw_walker.shape[0] != 1:
        raise NotImplementedError("per-measurement chi with walker-dependent relaxation weights "
                                  "is not supported by the GPU replay")
    sums, phi = _cx._replay_sums(C, Ghat, GAMMA * dt_traj,
                                 log_w=None if lw_walker is None else lw_walker[0],
                                 want_phi=return_walker_signals)
    signals = np.exp(lw_scalar) * sums[:, 0] / n_w
    if stimulated_echo:
        signals = signals * 0.5
    if return_walker_signals:
        lw_tot = lw_scalar[:, None] + (np.zeros((1, 1)) if lw_walker is None else lw_walker)
        return phi.T, lw_tot, signals
    return signals


# ---- vector-Bloch replay ------------------------------------------------------------------------
def _per_comp_rates(comp_traj, T2_per_comp, T1_per_comp, inv2, inv1):
    """Per-compartment relaxation rates of the Bloch replay: ``(comp (n_w, n_t) int32, 1/T2 per
    compartment, 1/T1 per compartment)``, or None without per-compartment times.

    The device reads the rates at every walker's compartment id, so the ids must be >= 0 and each
    list must hold an entry for the largest id.  The reference indexes the same lists with the ids
    (trajectories.py:798-803) and raises IndexError on a short list; so does this check, and on a
    negative id too (which the device cannot index)."""
    if T2_per_comp is None and T1_per_comp is None:
        return None
    if comp_traj is None:
        raise ValueError("T2_per_comp / T1_per_comp need comp_traj")
    comp = np.asarray(comp_traj)
    if comp.size and int(np.min(comp)) < 0:
        raise IndexError("comp_traj holds a negative compartment id")
    n_c = int(np.max(comp)) + 1 if comp.size else 1
    t2c = (1.0 / np.asarray(T2_per_comp, np.float64).ravel() if T2_per_comp is not None
           else np.full(n_c, inv2))
    t1c = (1.0 / np.asarray(T1_per_comp, np.float64).ravel() if T1_per_comp is not None
           else np.full(n_c, inv1))
    for name, arr in (("T2_per_comp", t2c), ("T1_per_comp", t1c)):
        if len(arr) < n_c:
            raise IndexError(f"{name} has {len(arr)} entries but comp_traj holds compartment "
                             f"ids up to {n_c - 1}")
    return comp.astype(np.int32), t2c, t1c


def _takes_position_arrays(field):
    """Whether a field callable maps positions (..., 3) to values (...) in one call.

    The providers of this package do; a user callable may instead take one position at a time.
    The probe is one call on two positions: a callable of one position fails it with the shape or
    type error such a callable raises on a (2, 3) array, or returns something other than two
    values.  Any other exception is a fault of the callable and propagates."""
    probe = np.zeros((2, 3), np.float32)
    try:
        out = np.asarray(field(probe), np.float64)
    except (TypeError, ValueError, IndexError):
        return False
    return out.shape == (2,)


def _rf_increments(rf_events, dt_traj, n_t):
    """The RF events as per-sample partial rotations (trajectories.py:888-917): a pulse of
    duration_s > 0 covers round(duration/dt) samples centred on round(t_s/dt) (clipped at 0, the
    last sample absorbing overflow) with equal flips, or flips in proportion to its
    ``b1_envelope`` resampled onto the samples; its carrier adds 2 pi offset dt per sample.
    Returns the CSR offsets (n_t + 1), flips and axes (in event order within a sample), the
    carrier per sample and the pulse-on flags."""
    per = [[] for _ in range(n_t)]
    active = np.zeros(n_t, dtype=np.uint8)
    offset = np.zeros(n_t)
    for ev in rf_events:
        centre = int(round(float(ev['t_s']) / dt_traj))
        dur = float(ev.get('duration_s', 0.0) or 0.0)
        n = max(1, int(round(dur / dt_traj))) if dur > 0.0 else 1
        first = max(0, centre - n // 2)
        total = np.deg2rad(float(ev.get('flip_deg', 180.0)))
        ax = np.deg2rad(float(ev.get('axis_deg', 0.0)))
        dphi = 2.0 * np.pi * float(ev.get('offset_hz', 0.0) or 0.0) * dt_traj
        env = ev.get('b1_envelope', None)
        if env is not None and n > 1:
            env = np.asarray(env, dtype=np.float64)
            env = np.interp(np.linspace(0.0, 1.0, n), np.linspace(0.0, 1.0, len(env)), env)
            flips = total * env / (env.sum() + 1e-30)
        else:
            flips = np.full(n, total / n)
        for j in range(n):
            i = min(first + j, n_t - 1)
            per[i].append((float(flips[j]), ax))
            active[i] = 1
            offset[i] += dphi
    start = np.zeros(n_t + 1, dtype=np.int32)
    start[1:] = np.cumsum([len(p) for p in per])
    flat = [x for p in per for x in p]
    flip = np.array([f for f, _ in flat], dtype=np.float64)
    axis = np.array([a for _, a in flat], dtype=np.float64)
    return start, flip, axis, offset, active


def replay_bloch(trajectory, dt_traj, G, dt_wf, rf_events, *, T2=None, T1=None, comp_traj=None,
                 T2_per_comp=None, T1_per_comp=None, susceptibility=None,
                 extra_phase_per_step=None, dlog_boundary_unit=None, surface_relaxivity=None,
                 D=None, echo_steps=None, echo_per_walker=False, weights=None,
                 return_walker_signals=False, b1_scale=None, slice_offsets=None,
                 slice_gradient=0.0, bound_frac=None, T2_bound=None, T1_bound=None,
                 off_resonance_bound=0.0):
    """Vector-Bloch replay of a stored walk (trajectories.py:734-949): each walker's
    magnetisation through the actual RF events, the physical gradient's precession, per-
    compartment T2/T1, surface relaxivity, an extra per-step phase or a susceptibility field
    (a callable r -> dBz sampled on the host), slice select, B1+ scaling and the MT
    bound-pool blend, in FP64 on the GPU (``dmsim_replay_bloch``).

    Returns the walker-mean Mx + i My (n_meas,) complex at the last sample, or (n_meas,
    n_echo) at the distinct ``echo_steps`` in time order ((n_meas, n_echo, n_walkers) per
    walker with ``echo_per_walker``), or ``(M_last (3, n_walkers), signals)`` with
    ``return_walker_signals``."""
    inv2 = 0.0 if T2 is None else 1.0 / T2
    inv1 = 0.0 if T1 is None else 1.0 / T1
    per_comp = _per_comp_rates(comp_traj, T2_per_comp, T1_per_comp, inv2, inv1)
    dev = _lib.device()
    lib = _lib.load()
    if isinstance(trajectory, torch.Tensor):
        traj_t = trajectory.to(dev).contiguous()
    else:
        traj_t = torch.from_numpy(np.ascontiguousarray(trajectory)).to(dev)
    if traj_t.dtype not in (torch.float16, torch.float32):
        traj_t = traj_t.float()
    n_w, n_t, _ = traj_t.shape
    G = np.asarray(G, dtype=np.float64)
    n_meas, n_t_wf, _ = G.shape
    t_wf = np.arange(n_t_wf, dtype=np.float64) * dt_wf
    t_tr = np.arange(n_t, dtype=np.float64) * dt_traj
    G_tr = np.zeros((n_t, n_meas, 3))
    for m in range(n_meas):
        for a in range(3):
            G_tr[:, m, a] = np.interp(t_tr, t_wf, G[m, :, a], left=0.0, right=0.0)
    keep = []

    def dv(a, dtype):
        if a is None:
            return None
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dtype))).to(dev)
        keep.append(t)
        return t.data_ptr()

    p = _lib.ReplayBlochParams()
    p.n_walkers, p.n_t, p.n_meas = n_w, n_t, n_meas
    p.traj_f16 = 1 if traj_t.dtype == torch.float16 else 0
    p.traj = traj_t.data_ptr()
    p.G = dv(G_tr, np.float64)
    p.gamma_dt = GAMMA * dt_traj
    p.dt_traj = float(dt_traj)
    p.inv_t2, p.inv_t1 = inv2, inv1
    p.e2, p.e1 = float(np.exp(-dt_traj * inv2)), float(np.exp(-dt_traj * inv1))
    if per_comp is not None:
        comp_np, t2c, t1c = per_comp
        p.comp = dv(comp_np, np.int32)
        p.inv_t2_comp, p.inv_t1_comp = dv(t2c, np.float64), dv(t1c, np.float64)
    if bound_frac is not None:
        if T2_bound is None or T1_bound is None:
            raise ValueError("T2_bound and T1_bound are required when bound_frac is set.")
        p.bound_frac = dv(bound_frac, np.float32)
        p.inv_t2_bound, p.inv_t1_bound = 1.0 / float(T2_bound), 1.0 / float(T1_bound)
        p.dphi_bound = 2.0 * np.pi * float(off_resonance_bound) * dt_traj
    if susceptibility is not None and extra_phase_per_step is None:
        field = (susceptibility.delta_bz_fn() if hasattr(susceptibility, "delta_bz_fn")
                 else susceptibility)
        r = (traj_t.float().cpu().numpy() if isinstance(trajectory, torch.Tensor)
             else np.asarray(trajectory, np.float32))
        if _takes_position_arrays(field):         # providers of this package take (..., 3)
            dbz = np.asarray(field(r), np.float64).reshape(n_w, n_t)
        else:                                     # a callable of one position
            dbz = np.array([[float(field(r[w, t])) for t in range(n_t)] for w in range(n_w)])
        extra_phase_per_step = GAMMA * dt_traj * dbz
    p.extra_phase = dv(extra_phase_per_step, np.float64)
    if (surface_relaxivity is not None and dlog_boundary_unit is not None
            and float(surface_relaxivity) != 0.0):
        if D is None:
            raise ValueError("D required when surface_relaxivity is not None.")
        p.dlog = dv(dlog_boundary_unit, np.float32)
        p.rho_over_D = float(surface_relaxivity) / float(D)
    start, flip, axis, offset, active = _rf_increments(rf_events, dt_traj, n_t)
    p.rf_start = dv(start, np.int32)
    p.rf_flip = dv(flip if len(flip) else np.zeros(1), np.float64)
    p.rf_axis = dv(axis if len(axis) else np.zeros(1), np.float64)
    p.rf_offset = dv(offset, np.float64) if np.any(offset != 0.0) else None
    p.rf_active = dv(active, np.uint8)
    p.b1_scale = dv(b1_scale, np.float64)
    if slice_offsets is not None and float(slice_gradient) != 0.0:
        p.slice_dphi = dv(GAMMA * float(slice_gradient) * np.asarray(slice_offsets, np.float64)
                          * dt_traj, np.float64)
    p.weights = dv(weights, np.float64)
    echo = (np.array(sorted(set(int(e) for e in echo_steps)), dtype=np.int32)
            if echo_steps is not None else np.array([n_t - 1], dtype=np.int32))
    echo = echo[(echo >= 0) & (echo < n_t)]
    if len(echo) == 0:
        return np.zeros((n_meas, 0), np.complex128)
    p.n_echo = len(echo)
    p.echo_idx = dv(echo, np.int32)
    sums = torch.zeros((n_meas, len(echo), 2), dtype=torch.float64, device=dev)
    p.sums = sums.data_ptr()
    ew = None
    if echo_steps is not None and echo_per_walker:
        ew = torch.zeros((n_meas, len(echo), n_w, 2), dtype=torch.float64, device=dev)
        p.echo_walker = ew.data_ptr()
    ml = None
    if echo_steps is None and return_walker_signals:
        ml = torch.zeros((3, n_w), dtype=torch.float64, device=dev)
        p.m_last = ml.data_ptr()
    nbytes = lib.dmsim_replay_bloch_workspace_bytes(p)
    if nbytes == 0:
        _lib.check(-1, "dmsim_replay_bloch_workspace_bytes")
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    _lib.check(lib.dmsim_replay_bloch(p, _lib.ptr(ws), nbytes, _lib.stream_handle()),
               "dmsim_replay_bloch")
    torch.cuda.synchronize(dev)
    norm = float(np.sum(weights)) if weights is not None else float(n_w)
    s = sums.cpu().numpy()
    sig = (s[..., 0] + 1j * s[..., 1]) / norm                     # (n_meas, n_echo)
    if echo_steps is not None:
        if echo_per_walker:
            e = ew.cpu().numpy()
            return e[..., 0] + 1j * e[..., 1]
        return sig
    if return_walker_signals:
        return ml.cpu().numpy(), sig[:, 0]
    return sig[:, 0]


def replay_bloch_jax(trajectory, dt_traj, G, dt_wf, rf_events, *, T2=None, T1=None,
                     comp_traj=None, T2_per_comp=None, T1_per_comp=None, susceptibility=None,
                     extra_phase_per_step=None, dlog_boundary_unit=None, surface_relaxivity=None,
                     D=None, echo_steps=None):
    """The hard-pulse form of :func:`replay_bloch` (trajectories.py:952-1030): every event is
    an instantaneous rotation at sample round(t_s/dt) (clipped to the walk; of several events on
    one sample the last one acts), without its duration or carrier; ``echo_steps`` are read in
    sorted order, repeats kept.  Same device replay."""
    n_t = (trajectory.shape[1])
    hard = {}
    for ev in rf_events:
        idx = max(0, min(int(round(float(ev['t_s']) / dt_traj)), n_t - 1))
        hard[idx] = {'t_s': idx * dt_traj, 'flip_deg': float(ev.get('flip_deg', 180.0)),
                     'axis_deg': float(ev.get('axis_deg', 0.0)), 'duration_s': 0.0,
                     'offset_hz': 0.0}
    events = [hard[i] for i in sorted(hard)]
    kw = dict(T2=T2, T1=T1, comp_traj=comp_traj, T2_per_comp=T2_per_comp,
              T1_per_comp=T1_per_comp, susceptibility=susceptibility,
              extra_phase_per_step=extra_phase_per_step, dlog_boundary_unit=dlog_boundary_unit,
              surface_relaxivity=surface_relaxivity, D=D)
    if echo_steps is None:
        return replay_bloch(trajectory, dt_traj, G, dt_wf, events, **kw)
    idx = np.sort(np.asarray([int(e) for e in echo_steps], dtype=np.int64))
    uniq = np.unique(idx)
    sig = replay_bloch(trajectory, dt_traj, G, dt_wf, events, echo_steps=uniq.tolist(), **kw)
    return sig[:, np.searchsorted(uniq, idx)]


# ---- replay helpers (trajectories.py:60-132, 674-731) ------------------------------------------
def pathway_sign_se(n_t, dt, TE, te_frac=0.5):
    """+1 before the refocusing pulse at te_frac * TE, -1 from it on: the sign a static phase
    takes in the scalar replay of a spin echo."""
    t = np.arange(int(n_t), dtype=np.float64) * float(dt)
    return np.where(t < float(te_frac) * float(TE), 1.0, -1.0)


def unwrap_periodic(traj, cell_size, periodic_axes=(0, 1)):
    """Continuous positions from positions folded into a periodic cell of side ``cell_size``:
    along each periodic axis the per-sample displacement is taken as its minimum image and
    summed from the first sample (time is axis -2).  Warns when a displacement approaches
    L/2 (the save step is then too coarse to unwrap unambiguously)."""
    out = np.asarray(traj, dtype=np.float32).copy()
    L = np.float32(cell_size)
    for a in periodic_axes:
        x = out[..., a]
        step = np.diff(x, axis=-1)
        step -= L * np.round(step / L)
        if np.any(np.abs(step) > 0.45 * float(L)):
            import warnings
            warnings.warn("unwrap_periodic: per-save displacement approaches L/2 on a periodic "
                          "axis; the trajectory save step may be too coarse for unambiguous "
                          "unwrapping. Use a finer dt_save.", RuntimeWarning)
        cont = np.empty_like(x)
        cont[..., 0] = x[..., 0]
        cont[..., 1:] = x[..., :1] + np.cumsum(step, axis=-1)
        out[..., a] = cont
    return out


def finite_180_longitudinal_dwell(phi_pre, tau_180, phi_B1=0.0):
    """Time each walker's magnetisation spends along z during a finite 180 pulse of length
    ``tau_180``: sin^2(phi_pre - phi_B1) * tau_180 / 2 for a transverse azimuth phi_pre."""
    return np.sin(np.asarray(phi_pre, dtype=np.float64) - phi_B1) ** 2 * (0.5 * tau_180)


def pre_pulse_gradient_phase(trajectories, dt_traj, G, dt_wf, cutoff_wf_idx):
    """gamma dt_traj sum over samples before the pulse of G(t) . r(t), per measurement and
    walker (n_meas, n_walkers): G linearly resampled onto the walk (zero outside), cut at
    the walk sample of waveform index ``cutoff_wf_idx``."""
    G = np.asarray(G, dtype=np.float32)
    n_meas, n_t_wf, _ = G.shape
    n_w, n_t, _ = trajectories.shape
    cut = max(0, min(int(round(cutoff_wf_idx * dt_wf / dt_traj)), n_t))
    t_wf = np.arange(n_t_wf, dtype=np.float64) * dt_wf
    t_tr = np.arange(n_t, dtype=np.float64) * dt_traj
    Gp = np.zeros((n_meas, n_t, 3))
    for m in range(n_meas):
        for a in range(3):
            Gp[m, :, a] = np.interp(t_tr, t_wf, G[m, :, a], left=0.0, right=0.0)
    Gp[:, cut:, :] = 0.0
    return GAMMA * dt_traj * (Gp.reshape(n_meas, n_t * 3)
                              @ np.asarray(trajectories, np.float64).reshape(n_w, n_t * 3).T)
