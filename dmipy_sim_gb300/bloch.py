"""Forward vector-Bloch walk: ``simulate_bloch`` (bloch.py:212-340 of dmipy-sim).

Every walker carries the magnetisation M = (Mx, My, Mz) of each measurement through the actual
sequence: the diffusive move of the walk, RF rotations about an in-plane B1 axis (finite pulses
spread over their duration), free precession by the physical gradient phase plus off-resonance,
pulse carrier and an optional voxel-scale crusher, and T2 / T1 relaxation with recovery toward
M0.  Echoes and refocusing are emergent.  The walk is the one ``simulate`` runs for the same seed
(same Philox stream, same step rule), executed by the walk kernel's vector-Bloch form
(``dmsim_bloch``): one launch, no per-walker trace.

Not built: the magnetisation-transfer binding walk (``kappa_MT > 0``, bloch.py:343-671) and
susceptibility fields; both raise ``NotImplementedError``.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .constants import GAMMA
from .core import _check_gpu, _to_lab, _waveform_arrays, permeable_sub_steps

__all__ = ["simulate_bloch"]

# geometries whose reference class has no reflect_with_log_weight (the wall weight is off) or no
# permeate (the membrane walk is off), geometries.py
_NO_LOG_WEIGHT = frozenset({"FreeDiffusion", "PermeableShell"})
_NO_PERMEATE = frozenset({"FreeDiffusion", "Box1D"})


def _build_rf_schedule(rf_events, dt, n_t):
    """Per-sample (flip, axis, carrier) in rad from the RF event list (bloch.py:60-89).

    A pulse of ``duration_s`` > 0 covers ``round(duration/dt)`` samples centred on
    ``round(t_s/dt)`` (clipped at 0, the last sample absorbing any overflow) with equal flips;
    ``duration_s`` 0 is a hard pulse on one sample.  Flips and carriers of pulses sharing a
    sample add; the axis is the last pulse's."""
    flip = np.zeros(n_t)
    axis = np.zeros(n_t)
    carrier = np.zeros(n_t)
    for ev in rf_events:
        centre = int(round(float(ev['t_s']) / dt))
        dur = float(ev.get('duration_s', 0.0) or 0.0)
        n = max(1, int(round(dur / dt))) if dur > 0.0 else 1
        first = max(0, centre - n // 2)
        each = np.deg2rad(float(ev.get('flip_deg', 180.0))) / n
        ax = np.deg2rad(float(ev.get('axis_deg', 0.0)))
        dphi = 2.0 * np.pi * float(ev.get('offset_hz', 0.0) or 0.0) * dt
        idx = np.minimum(first + np.arange(n), n_t - 1)
        np.add.at(flip, idx, each)
        axis[idx] = ax
        np.add.at(carrier, idx, dphi)
    return flip, axis, carrier


def _build_crusher(crusher, dt, n_t):
    """Per-sample crusher rate (rad per unit walker coordinate) and whether one is set
    (bloch.py:208-225): over a window of n samples the rate is 2 pi n_cycles / n."""
    rate = np.zeros(n_t)
    if crusher is None:
        return rate, False
    cycles = float(crusher.get('n_cycles', 16.0))
    for t0, t1 in crusher.get('windows_s', []):
        i0 = max(0, int(round(t0 / dt)))
        i1 = min(n_t, int(round(t1 / dt)))
        if i1 > i0:
            rate[i0:i1] = 2.0 * np.pi * cycles / (i1 - i0)
    return rate, True


class BlochWalk:
    """One vector-Bloch walk with its device buffers: ``launch()`` enqueues it on the current
    stream, ``result()`` synchronises and returns the sums (n_echo, M, 3) of Mx, My, Mz."""

    def __init__(self, geometry, *, n_walkers, diffusivity, G, dt, flip, axis, carrier, crush,
                 T2, T1, M0, seed, echo_idx, surface_relaxivity=0.0, r0=None,
                 want_positions=False):
        if getattr(geometry, '_is_myelinated', False) or getattr(geometry, '_is_packed_myelinated',
                                                                False):
            raise NotImplementedError("the vector-Bloch walk does not take myelinated cylinders")
        self.lib = _lib.load()
        dev = self.dev = _lib.device()
        name = type(geometry).__name__
        D = float(diffusivity)
        dt = float(dt)
        kappa = float(getattr(geometry, 'permeability', None) or 0.0)
        has_perm = kappa > 0.0 and name not in _NO_PERMEATE
        rho = float(surface_relaxivity or 0.0)
        has_surf = rho > 0.0 and name not in _NO_LOG_WEIGHT
        # bloch.py:141-144: the permeable walk sub-steps to R/25 and sums the phase per sub-step;
        # the reflecting walk takes one step per sample
        S = permeable_sub_steps(geometry, D, dt) if has_perm else 1
        wall = (_lib.WALL_PERMEATE if has_perm else
                _lib.WALL_RELAX if has_surf else _lib.WALL_REFLECT)
        step_l = np.float32(np.sqrt(6.0 * D * dt / S))
        rho_over_D = np.float32(rho / D) if (has_surf or (has_perm and rho > 0.0)) else 0.0
        self.gdesc, self._keep = geometry._desc(float(step_l), wall, rho_over_D,
                                                np.float32(kappa / D) if has_perm else 0.0, dev)
        G = np.asarray(G, np.float32)
        n_meas, n_t, _ = G.shape
        f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)  # noqa: E731
        self.G_dev = f32(G.transpose(1, 0, 2))
        self.flip_dev, self.axis_dev = f32(flip), f32(axis)
        self.carrier_dev = None if carrier is None else f32(carrier)
        self.crush_dev = None if crush is None else f32(crush)
        self.r0_dev = None if r0 is None else f32(np.asarray(r0).reshape(n_walkers, 3))
        echo = np.asarray(echo_idx, np.int32).ravel()
        self._echo_c = (ctypes.c_int32 * len(echo))(*echo.tolist())
        p = self.p = _lib.WalkParams()
        p.n_walkers = int(n_walkers)
        p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        p.n_t, p.n_meas, p.sub_steps = n_t, n_meas, S
        p.phase_per_substep = 1
        p.step_length = step_l
        p.gamma_dt = np.float32(GAMMA * dt / S)
        p.t2_decay = np.float32(dt / S / T2) if T2 is not None else 0.0
        p.has_weight = 1 if (T2 is not None or rho_over_D != 0.0) else 0
        p.n_echo = len(echo)
        p.echo_idx = self._echo_c
        p.G = self.G_dev.data_ptr()
        p.r0 = None if self.r0_dev is None else self.r0_dev.data_ptr()
        b = self.b = _lib.BlochParams()
        b.rf_flip = self.flip_dev.data_ptr()
        b.rf_axis = self.axis_dev.data_ptr()
        b.carrier = None if self.carrier_dev is None else self.carrier_dev.data_ptr()
        b.crush = None if self.crush_dev is None else self.crush_dev.data_ptr()
        b.m0 = float(M0)
        b.t1_sample = float(np.float32(dt / T1)) if T1 is not None else 0.0
        self.sums = torch.zeros((len(echo), n_meas, 3), dtype=torch.float64, device=dev)
        self.status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        o = self.o = _lib.WalkOutputs()
        o.sums = self.sums.data_ptr()
        o.status = self.status.data_ptr()
        self.pos = None
        if want_positions:
            self.pos = torch.empty((n_walkers, 3), dtype=torch.float32, device=dev)
            o.final_pos = self.pos.data_ptr()
        self.ws_bytes = self.lib.dmsim_bloch_workspace_bytes(p, self.gdesc)
        if self.ws_bytes == 0:
            _lib.check(-1, "dmsim_bloch_workspace_bytes")
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.n_walkers, self.sub_steps = int(n_walkers), S

    def launch(self):
        rc = self.lib.dmsim_bloch(self.p, self.gdesc, self.b, self.o, _lib.ptr(self.ws),
                                  self.ws_bytes, _lib.stream_handle())
        _lib.check(rc, "dmsim_bloch")

    def result(self):
        torch.cuda.synchronize(self.dev)
        return self.sums.cpu().numpy()


def _prepare(n_walkers, diffusivity, waveform, geometry, rf_events, *, T2, T1, M0,
             off_resonance_hz, seed, echo_steps, return_mz, crusher, surface_relaxivity, r0=None,
             want_positions=False):
    if hasattr(waveform, 'waveform'):
        waveform = waveform.waveform
    G, _ = _waveform_arrays(waveform, geometry)      # walk frame, Mesh placement applied
    n_meas, n_t, _ = G.shape
    dt = float(waveform.dt)
    flip, axis, carrier_rf = _build_rf_schedule(rf_events, dt, n_t)
    rate, has_crush = _build_crusher(crusher, dt, n_t)
    carrier = carrier_rf + 2.0 * np.pi * float(off_resonance_hz) * dt
    idx = None
    if echo_steps is not None:
        idx = np.asarray(echo_steps, dtype=np.int64).ravel()
        if np.any(idx >= n_t) or np.any(idx < -n_t):
            raise IndexError(f"echo step out of range for {n_t} samples")
        idx = np.where(idx < 0, idx + n_t, idx)
    want = set() if idx is None else set(idx.tolist())
    if idx is None or return_mz:
        want.add(n_t - 1)
    uniq = np.array(sorted(want), dtype=np.int32)
    w = BlochWalk(geometry, n_walkers=n_walkers, diffusivity=diffusivity, G=G, dt=dt, flip=flip,
                  axis=axis, carrier=carrier if np.any(carrier) else None,
                  crush=rate if has_crush else None, T2=T2, T1=T1, M0=M0, seed=seed,
                  echo_idx=uniq, surface_relaxivity=surface_relaxivity, r0=r0,
                  want_positions=want_positions)
    return w, uniq, idx


def _finish(sums, n_walkers, uniq, idx, return_mz):
    n = max(int(n_walkers), 1)
    xy = (sums[..., 0] + 1j * sums[..., 1]) / n            # (n_unique, M)
    last = len(uniq) - 1                                   # the final sample, when requested
    if idx is None:
        signals = xy[last].astype(np.complex64)            # (M,)
    else:
        signals = xy[np.searchsorted(uniq, idx)].T.astype(np.complex64)   # (M, n_echo)
    if return_mz:
        return signals, (sums[last, :, 2] / n).astype(np.float32)
    return signals


def simulate_bloch(n_walkers, diffusivity, waveform, geometry, rf_events, *,
                   T2=None, T1=None, M0=1.0, off_resonance_hz=0.0, seed=0,
                   echo_steps=None, return_mz=False, crusher=None,
                   surface_relaxivity=0.0,
                   kappa_MT=0.0, dwell_time=0.0, T2_bound=1e-5, T1_bound=1.0,
                   off_resonance_bound=0.0, sub_steps=None, return_bound_frac=False,
                   equilibrate_binding="auto", susceptibility=None, require_gpu=None):
    """Forward vector-Bloch signal of ``rf_events`` on ``waveform.G`` (bloch.py:212-340).

    ``waveform.G`` is the PHYSICAL gradient (n_meas, n_t, 3) on the ``waveform.dt`` grid; RF
    events are dicts ``{t_s, flip_deg, axis_deg, duration_s, offset_hz}``; ``surface_relaxivity``
    (m/s) attenuates Mxy at wall contacts; a permeable geometry walks its membranes with
    sub-steps of R/25.  Returns the walker-mean ``Mx + i My`` (complex64) at the last sample
    (n_meas,) or at ``echo_steps`` (n_meas, n_echo), followed by the final walker-mean ``Mz``
    (n_meas,) with ``return_mz``.
    """
    if kappa_MT and float(kappa_MT) > 0.0:
        raise NotImplementedError("magnetisation-transfer binding walks (kappa_MT > 0) are not "
                                  "built in this engine")
    if susceptibility is not None:
        raise NotImplementedError("susceptibility fields are not built in this engine")
    _check_gpu(require_gpu)
    w, uniq, idx = _prepare(n_walkers, diffusivity, waveform, geometry, rf_events, T2=T2, T1=T1,
                            M0=M0, off_resonance_hz=off_resonance_hz, seed=seed,
                            echo_steps=echo_steps, return_mz=return_mz, crusher=crusher,
                            surface_relaxivity=surface_relaxivity)
    w.launch()
    return _finish(w.result(), n_walkers, uniq, idx, return_mz)


def _bloch_walk(n_walkers, diffusivity, waveform, geometry, rf_events, *, r0=None, **kw):
    """simulate_bloch with explicit walk-frame start positions and the final positions
    (lab frame) appended: the parity tests' entry."""
    return_mz = kw.get("return_mz", False)
    kw.setdefault("T2", None)
    kw.setdefault("T1", None)
    kw.setdefault("M0", 1.0)
    kw.setdefault("off_resonance_hz", 0.0)
    kw.setdefault("seed", 0)
    kw.setdefault("echo_steps", None)
    kw.setdefault("return_mz", False)
    kw.setdefault("crusher", None)
    kw.setdefault("surface_relaxivity", 0.0)
    w, uniq, idx = _prepare(n_walkers, diffusivity, waveform, geometry, rf_events, r0=r0,
                            want_positions=True, **kw)
    w.launch()
    sums = w.result()
    out = _finish(sums, n_walkers, uniq, idx, return_mz)
    pos = _to_lab(geometry, w.pos.cpu().numpy())
    return (out if isinstance(out, tuple) else (out,)) + (pos, sums)
