"""Forward vector-Bloch walk: ``simulate_bloch`` (bloch.py:212-340 of dmipy-sim).

Every walker carries the magnetisation M = (Mx, My, Mz) of each measurement through the actual
sequence: the diffusive move of the walk, RF rotations about an in-plane B1 axis (finite pulses
spread over their duration), free precession by the physical gradient phase plus off-resonance,
pulse carrier and an optional voxel-scale crusher, and T2 / T1 relaxation with recovery toward
M0.  Echoes and refocusing are emergent.  The walk is the one ``simulate`` runs for the same seed
(same Philox stream, same step rule), executed by the walk kernel's vector-Bloch form
(``dmsim_bloch``): one launch, no per-walker trace.

With ``kappa_MT > 0`` the walk binds at the walls (bloch.py:343-671): a free walker sticks with
p = min(1, 2 kappa_MT d_perp / D) per hit and stays put for an exponential dwell, the FP64
magnetisation takes a Strang split per sub-step with the walker's pool (free or bound: its own
T2, T1 and offset), and a burn-in brings the bound occupancy to equilibrium before the sequence
(``dmsim_bloch_mt``).  A susceptibility field provider (``susceptibility.py``: magnetised spheres,
myelin cylinders, a solved grid) is evaluated on the device at every sample; the MT walk takes
none.
"""
import ctypes
import warnings

import numpy as np
import torch

from . import _lib
from .constants import GAMMA
from .core import _check_gpu, _to_frame, _to_lab, _waveform_arrays, permeable_sub_steps

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


def _field_params(susceptibility, geometry, dt, b, dev, keep):
    """Fill the susceptibility fields of ``b`` (dmsim_bloch_params) from a provider."""
    from . import susceptibility as su
    frame = geometry._frame()
    rot = np.eye(3) if frame is None else np.asarray(frame, np.float64).T   # walk -> lab
    if isinstance(susceptibility, su.SusceptibilitySources):
        tab, kind = susceptibility._table(), 1
    elif isinstance(susceptibility, su.MyelinSusceptibility):
        tab, (L, scale, c2a, s2a) = susceptibility._table()
        kind = 2
        if susceptibility.R is not None:
            rot = np.asarray(susceptibility.R, np.float64) @ rot
        b.field_par[:6] = [L, scale, c2a, s2a, float(susceptibility.n_images),
                           1.0 if susceptibility.periodic else 0.0]
    elif isinstance(susceptibility, su.GridSusceptibility):
        tab = np.ascontiguousarray(np.asarray(susceptibility.dB, np.float32))
        kind = 3
        vs = su._voxel(susceptibility.voxel_size, 3)
        b.field_par[:7] = list(np.asarray(susceptibility.origin, float).ravel()) + list(vs) + [
            1.0 if susceptibility.periodic else 0.0]
        b.field_dims[:] = list(tab.shape)
    else:
        raise NotImplementedError(
            "the device walk evaluates SusceptibilitySources, MyelinSusceptibility and "
            "GridSusceptibility; a bare r -> dBz callable is sampled on the host by "
            "trajectories.replay_bloch")
    t = torch.from_numpy(np.ascontiguousarray(tab, np.float32).ravel()).to(dev)
    keep.append(t)
    b.field_kind = kind
    b.field_n = int(tab.shape[0]) if kind != 3 else 0
    b.field_tab = t.data_ptr()
    b.field_rot[:] = [float(v) for v in rot.ravel()]
    b.field_gamma_dt = float(np.float32(GAMMA * dt))


class BlochWalk:
    """One vector-Bloch walk with its device buffers: ``launch()`` enqueues it on the current
    stream, ``result()`` synchronises and returns the sums (n_echo, M, 3) of Mx, My, Mz."""

    def __init__(self, geometry, *, n_walkers, diffusivity, G, dt, flip, axis, carrier, crush,
                 T2, T1, M0, seed, echo_idx, surface_relaxivity=0.0, r0=None,
                 want_positions=False, susceptibility=None):
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
        self._field_keep = []
        if susceptibility is not None:
            _field_params(susceptibility, geometry, dt, b, dev, self._field_keep)
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
             want_positions=False, susceptibility=None):
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
                  want_positions=want_positions, susceptibility=susceptibility)
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
        if susceptibility is not None:
            raise NotImplementedError("the magnetisation-transfer walk takes no susceptibility "
                                      "field")
        return _simulate_bloch_mt(
            n_walkers, diffusivity, waveform, geometry, rf_events, T2=T2, T1=T1, M0=M0,
            off_resonance_hz=off_resonance_hz, seed=seed, echo_steps=echo_steps,
            return_mz=return_mz, crusher=crusher, surface_relaxivity=surface_relaxivity,
            kappa_MT=kappa_MT, dwell_time=dwell_time, T2_bound=T2_bound, T1_bound=T1_bound,
            off_resonance_bound=off_resonance_bound, sub_steps=sub_steps,
            return_bound_frac=return_bound_frac, equilibrate_binding=equilibrate_binding,
            require_gpu=require_gpu)
    _check_gpu(require_gpu)
    w, uniq, idx = _prepare(n_walkers, diffusivity, waveform, geometry, rf_events, T2=T2, T1=T1,
                            M0=M0, off_resonance_hz=off_resonance_hz, seed=seed,
                            echo_steps=echo_steps, return_mz=return_mz, crusher=crusher,
                            surface_relaxivity=surface_relaxivity, susceptibility=susceptibility)
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


# ---- magnetisation transfer ---------------------------------------------------------------------
# geometries whose reference class has a boundary log-weight rule (reflect_with_log_weight) and
# that the MT kernel walks
_MT_GEOMETRIES = frozenset({"Cylinder", "Sphere", "Ellipsoid", "Box1D", "PermeableSlab1D",
                            "PackedCylinders", "PackedSpheres"})


def _mt_radius(geometry):
    """The feature radius that sets the binding sub-step (bloch.py:344-353)."""
    for a in ("radius", "inner_radius", "_feature_radius"):
        v = getattr(geometry, a, None)
        if v is not None:
            try:
                return float(v)
            except (TypeError, ValueError):
                pass
    return None


def _mt_surface_to_volume(geometry):
    R = _mt_radius(geometry)
    if R is not None and R > 0.0:
        name = type(geometry).__name__
        if name == "Sphere":
            return 3.0 / R
        if name == "Cylinder":
            return 2.0 / R
    return None


def _mt_mode(equilibrate_binding, G, T2, T2_bound, geometry):
    """'off' | 'burnin' | 'fast' (bloch.py:375-401): 'fast' needs a known S/V and a read-out
    the mid-air bound start cannot bias (no gradient, or a bound pool dark against T2)."""
    eb = equilibrate_binding
    if eb in (None, False, 'off'):
        return 'off'
    if eb in ('auto', True, 'burnin'):
        return 'burnin'
    if eb == 'fast':
        if _mt_surface_to_volume(geometry) is None:
            warnings.warn("equilibrate_binding='fast' needs a known surface-to-volume "
                          "(analytic Sphere/Cylinder); falling back to 'burnin'.", stacklevel=3)
            return 'burnin'
        dark = T2 is None or float(T2_bound) <= 0.02 * float(T2)
        if np.any(G) and not dark:
            warnings.warn("equilibrate_binding='fast' is unsafe: a gradient is present and the "
                          "bound pool is not MR-dark (T2_bound not << T2), so the mid-air bound "
                          "positions would bias the signal; falling back to 'burnin'.",
                          stacklevel=3)
            return 'burnin'
        return 'fast'
    raise ValueError(f"equilibrate_binding must be 'auto'|'burnin'|'fast'|'off', got {eb!r}")


def _mt_rotations(flip, axis, carrier_rf, n_sub, dt, off_free, off_bound):
    """Per sample, the rotation of one sub-step for the free and the bound pool (n_t, 2, 3, 3):
    the exact rotation about k = (f cos ax, f sin ax, dphi) with f the sample's flip over n_sub
    and dphi the pool's carrier phase over one sub-step (bloch.py:462-465, 505-529), in the
    cancellation-free form cos|k| I + sinc|k| [k]x + (sinc(|k|/2)^2 / 2) k k^T."""
    f32 = np.float32
    inv = 1.0 / n_sub
    fs = np.asarray(flip, f32).astype(np.float64) * inv
    ax = np.asarray(axis, f32)
    kx = fs * np.cos(ax).astype(np.float64)
    ky = fs * np.sin(ax).astype(np.float64)
    free = (2.0 * np.pi * off_free * dt + np.asarray(carrier_rf, f32).astype(np.float64)) * inv
    bnd = 2.0 * np.pi * off_bound * dt * inv
    out = np.empty((len(fs), 2, 3, 3))
    for p, kz in enumerate((free, free + bnd)):
        th = np.sqrt(kx * kx + ky * ky + kz * kz)
        with np.errstate(invalid="ignore", divide="ignore"):
            sb = np.where(th > 1e-12, np.sin(th) / th, 1.0)
            half = 0.5 * th
            sh = np.where(half > 1e-12, np.sin(half) / half, 1.0)
        cb = 0.5 * sh * sh
        ca = np.cos(th)
        k = np.stack([kx, ky, kz], axis=1)                       # (n_t, 3)
        cross = np.zeros((len(fs), 3, 3))
        cross[:, 0, 1], cross[:, 0, 2] = -kz, ky
        cross[:, 1, 0], cross[:, 1, 2] = kz, -kx
        cross[:, 2, 0], cross[:, 2, 1] = -ky, kx
        out[:, p] = (ca[:, None, None] * np.eye(3) + sb[:, None, None] * cross
                     + cb[:, None, None] * k[:, :, None] * k[:, None, :])
    return out


class MTWalk:
    """Device buffers of one MT walk (``dmsim_bloch_mt``) over n walkers."""

    def __init__(self, geometry, n_walkers, D, dt, n_sub, seed, *, kappa_MT, dwell_time,
                 surface_relaxivity):
        name = type(geometry).__name__
        if name not in _MT_GEOMETRIES:
            raise TypeError(f"{name} has no reflect_with_log_weight; MT binding needs the "
                            "boundary-local-time channel (Sphere / Cylinder / Box1D / Ellipsoid "
                            "/ packed cylinders or spheres).")
        self.lib = _lib.load()
        dev = self.dev = _lib.device()
        self.n, self.n_sub, self.dt = int(n_walkers), int(n_sub), float(dt)
        dt_sub = self.dt / self.n_sub
        self.step_l = np.float32(np.sqrt(6.0 * D * dt_sub))
        self.gdesc, self._keep = geometry._desc(float(self.step_l), _lib.WALL_RELAX, 0.0, 0.0,
                                                dev)
        self.p = p = _lib.MtParams()
        p.n_walkers, p.seed = self.n, int(seed) & 0xFFFFFFFFFFFFFFFF
        p.n_sub = self.n_sub
        p.step_length = self.step_l
        p.kappa_mt_over_D = np.float32(kappa_MT / D)
        p.dwell_substeps = np.float32(dwell_time / dt_sub)
        p.rho_over_D = np.float32(float(surface_relaxivity or 0.0) / D)
        self.status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        p.status = self.status.data_ptr()
        self.r = torch.empty((self.n, 3), dtype=torch.float32, device=dev)
        self.r_next = torch.empty_like(self.r)
        self.brem = torch.zeros(self.n, dtype=torch.float32, device=dev)
        self.brem_next = torch.empty_like(self.brem)
        self.occ_total = torch.empty(self.n, dtype=torch.float32, device=dev)
        self.counter = 0

    def _run(self, n_t, spin, extra):
        p = self.p
        p.n_t, p.spin, p.substep_offset = int(n_t), int(spin), self.counter & 0xFFFFFFFF
        p.r0, p.r_end = self.r.data_ptr(), self.r_next.data_ptr()
        p.brem_in, p.brem_out = self.brem.data_ptr(), self.brem_next.data_ptr()
        p.occ_total = self.occ_total.data_ptr()
        for k, v in extra.items():
            setattr(p, k, v)
        nbytes = self.lib.dmsim_bloch_mt_workspace_bytes(p, self.gdesc)
        if nbytes == 0:
            _lib.check(-1, "dmsim_bloch_mt_workspace_bytes")
        ws = torch.empty(nbytes, dtype=torch.uint8, device=self.dev)
        _lib.check(self.lib.dmsim_bloch_mt(p, self.gdesc, _lib.ptr(ws), nbytes,
                                           _lib.stream_handle()), "dmsim_bloch_mt")
        torch.cuda.synchronize(self.dev)
        self.r, self.r_next = self.r_next, self.r
        self.brem, self.brem_next = self.brem_next, self.brem
        self.counter += int(n_t) * self.n_sub

    def burn_chunk(self, n_chunk, sub=None):
        """Walk n_chunk samples (of ``sub`` sub-steps, default the walk's) without RF, gradient
        or magnetisation; returns the mean bound occupancy."""
        self.p.n_meas = 1
        n_sub = self.n_sub
        if sub is not None:
            self.n_sub = self.p.n_sub = int(sub)
        try:
            self._run(n_chunk, 0, {"occ": None, "sums": None, "G": None, "rot": None,
                                   "crush": None, "n_echo": 0, "echo_idx": None,
                                   "traj": None, "dlog_free": None})
        finally:
            self.n_sub = self.p.n_sub = n_sub
        return float(self.occ_total.sum().item()) / (self.n * n_chunk)


def _mt_run(w, G, dt, rf_events, *, T2, T1, M0, off_resonance_hz, off_resonance_bound,
            T2_bound, T1_bound, echo_steps, return_mz, crusher, return_bound_frac):
    """The sequence on an MT walk from its current positions, dwell and Philox counter:
    returns the sums (n_echo, M, 3), the echo samples read, the caller's echo order and the
    per-sample bound fractions (n, n_t) when asked."""
    n_meas, n_t, _ = G.shape
    dev = w.dev
    n_sub = w.n_sub
    flip, axis, carrier = _build_rf_schedule(rf_events, dt, n_t)
    rate, has_crush = _build_crusher(crusher, dt, n_t)
    echo = None
    if echo_steps is not None:
        echo = np.asarray(echo_steps, dtype=np.int64).ravel()
        if np.any(echo >= n_t) or np.any(echo < -n_t):
            raise IndexError(f"echo step out of range for {n_t} samples")
        echo = np.where(echo < 0, echo + n_t, echo)
    want = set() if echo is None else set(echo.tolist())
    if echo is None or return_mz:
        want.add(n_t - 1)
    uniq = np.array(sorted(want), dtype=np.int32)
    echo_c = (ctypes.c_int32 * len(uniq))(*uniq.tolist())
    rot = torch.from_numpy(np.ascontiguousarray(
        _mt_rotations(flip, axis, carrier, n_sub, dt, float(off_resonance_hz),
                      float(off_resonance_bound)).reshape(n_t, 18))).to(dev)
    G_dev = torch.from_numpy(np.ascontiguousarray(G.transpose(1, 0, 2), np.float32)).to(dev)
    crush_dev = (torch.from_numpy(np.asarray(rate, np.float32)).to(dev) if has_crush else None)
    sums = torch.zeros((len(uniq), n_meas, 3), dtype=torch.float64, device=dev)
    occ = (torch.empty((w.n, n_t), dtype=torch.float32, device=dev)
           if return_bound_frac else None)
    dt_sub = dt / n_sub
    inv2 = [0.0 if T2 is None else 1.0 / T2, 1.0 / T2_bound]
    inv1 = [0.0 if T1 is None else 1.0 / T1, 1.0 / T1_bound]
    p = w.p
    p.n_meas = n_meas
    p.gamma_dt = GAMMA * dt
    p.m0 = float(M0)
    for k in range(2):
        p.e2h[k] = float(np.exp(-0.5 * dt_sub * inv2[k]))
        p.e1h[k] = float(np.exp(-0.5 * dt_sub * inv1[k]))
    w._run(n_t, 1, {"G": G_dev.data_ptr(), "rot": rot.data_ptr(),
                    "crush": None if crush_dev is None else crush_dev.data_ptr(),
                    "occ": None if occ is None else occ.data_ptr(), "sums": sums.data_ptr(),
                    "n_echo": len(uniq), "echo_idx": echo_c})
    return sums.cpu().numpy(), uniq, echo, occ


def _simulate_bloch_mt(n_walkers, diffusivity, waveform, geometry, rf_events, *, T2, T1, M0,
                       off_resonance_hz, seed, echo_steps, return_mz, crusher,
                       surface_relaxivity, kappa_MT, dwell_time, T2_bound, T1_bound,
                       off_resonance_bound, sub_steps, return_bound_frac, equilibrate_binding,
                       require_gpu=None):
    """The MT forward walk (bloch.py:556-671)."""
    if dwell_time <= 0.0:
        raise ValueError("dwell_time must be > 0 when kappa_MT > 0 (MT on).")
    name = type(geometry).__name__
    if name not in _MT_GEOMETRIES:
        raise TypeError(f"{name} has no reflect_with_log_weight; MT binding needs the "
                        "boundary-local-time channel (Sphere / Cylinder / Box1D / Ellipsoid / "
                        "packed cylinders or spheres).")
    D = float(diffusivity)
    if hasattr(waveform, 'waveform'):
        waveform = waveform.waveform
    G, _ = _waveform_arrays(waveform, geometry)
    n_t = G.shape[1]
    dt = float(waveform.dt)
    if sub_steps is None:
        # binding alters the walk: sub-steps of R/25 (bloch.py:578-583)
        R = _mt_radius(geometry)
        sub_steps = 1 if R is None else max(1, int(np.ceil(dt / (R ** 2 / (3750.0 * D)))))
    mode = _mt_mode(equilibrate_binding, G, T2, T2_bound, geometry)
    _check_gpu(require_gpu)
    w = MTWalk(geometry, n_walkers, D, dt, int(sub_steps), seed, kappa_MT=kappa_MT,
               dwell_time=dwell_time, surface_relaxivity=surface_relaxivity)
    r0 = geometry.init_positions(int(n_walkers), int(seed))
    w.r.copy_(torch.from_numpy(np.ascontiguousarray(
        _to_frame(geometry, np.asarray(r0, np.float32)), np.float32)))
    dwell_sub = float(w.p.dwell_substeps)
    S_V = _mt_surface_to_volume(geometry)
    P_eq = (kappa_MT * S_V) / (kappa_MT * S_V + 1.0 / dwell_time) if S_V is not None else None
    converged = True
    if mode == 'fast':
        rng = np.random.default_rng([int(seed) & 0xFFFFFFFF, 0xB0117E])
        u_state, u_dwell = rng.random((2, int(n_walkers)), dtype=np.float32)
        b0 = np.where(u_state < np.float32(P_eq),
                      -np.log(np.maximum(u_dwell, np.float32(1e-20))) * np.float32(dwell_sub),
                      np.float32(0.0)).astype(np.float32)
        w.brem.copy_(torch.from_numpy(b0))
    elif mode == 'burnin':
        # bloch.py:404-429: chunks of about one dwell, RF and gradient off, until the bound
        # occupancy changes by <= 1 % between chunks (at most 40)
        n_chunk = int(max(4, round(float(dwell_time) / dt)))
        prev, converged = -1.0, False
        for _ in range(40):
            occ = w.burn_chunk(n_chunk)
            if prev >= 0.0 and abs(occ - prev) <= 0.01 * max(occ, 1e-6):
                converged = True
                break
            prev = occ
    s, uniq, echo, occ = _mt_run(
        w, G, dt, rf_events, T2=T2, T1=T1, M0=M0, off_resonance_hz=off_resonance_hz,
        off_resonance_bound=off_resonance_bound, T2_bound=T2_bound, T1_bound=T1_bound,
        echo_steps=echo_steps, return_mz=return_mz, crusher=crusher,
        return_bound_frac=return_bound_frac)
    occ_run = float(w.occ_total.sum().item()) / (int(n_walkers) * n_t)
    if mode != 'off':
        if mode == 'burnin' and not converged:
            warnings.warn("equilibrate_binding: bound-pool occupancy did not plateau within the "
                          "burn-in cap (long-dwell / heterogeneous substrate?); the MT signal may "
                          "be under-equilibrated.", stacklevel=3)
        if P_eq is not None and abs(occ_run - P_eq) > max(0.05 * P_eq, 0.01):
            warnings.warn(f"equilibrate_binding='{mode}': bound occupancy during the sequence "
                          f"({occ_run:.3f}) differs from equilibrium k_f/(k_f+k_r)={P_eq:.3f}; "
                          "the MT bound pool may be off-equilibrium.", stacklevel=3)
    out = _finish(s, n_walkers, uniq, echo, return_mz)
    out = list(out) if isinstance(out, tuple) else [out]
    if return_bound_frac:
        out.append(occ.mean(dim=0, dtype=torch.float64).cpu().numpy())
    return out[0] if len(out) == 1 else tuple(out)

