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
