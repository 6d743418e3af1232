"""Sequence builders for the vector-Bloch walk (pulse_sequence.py of dmipy-sim).

A :class:`BlochSequence` is what :func:`~dmipy_sim_gb300.bloch.simulate_bloch` consumes: the
PHYSICAL gradient on a ``dt`` grid, a finite-pulse RF event list, optional echo samples and an
optional voxel-scale crusher.  Builders: a gradient echo, a spin echo, the FEXI filter-exchange
stimulated echo, and an off-resonance saturation block prepended to any readout.
"""
from dataclasses import dataclass, replace
from types import SimpleNamespace

import numpy as np

from .bloch import simulate_bloch
from .constants import GAMMA

__all__ = ["BlochSequence", "gradient_echo", "spin_echo", "fexi", "prepend_mt_prep",
           "run_bloch_sequence", "emergent_z_spectrum"]


@dataclass
class BlochSequence:
    """One acquisition for the forward walk (pulse_sequence.py:26-44)."""
    G: np.ndarray                       # (n_meas, n_t, 3) physical gradient (T/m)
    dt: float                           # sample spacing (s)
    rf_events: list                     # [{t_s, flip_deg, axis_deg, duration_s, offset_hz}]
    complex_signal: bool = True         # read Mx + i My (False: the real part is the signal)
    echo_steps: list = None             # samples to read; None reads the last
    crusher: dict = None                # {'windows_s': [(t0, t1), ...], 'n_cycles': ...}
    family: str = "gre"
    notes: str = ""

    @property
    def n_t(self):
        return self.G.shape[1]

    @property
    def n_meas(self):
        return self.G.shape[0]


def _hard(t_s, flip, axis):
    return {'t_s': float(t_s), 'flip_deg': float(flip), 'axis_deg': float(axis),
            'duration_s': 0.0, 'offset_hz': 0.0}


def gradient_echo(TE, dt, *, n_meas=1, exc_axis_deg=90.0):
    """A hard 90 at t = 0, free evolution to TE (samples 0 .. round(TE/dt)), no gradient
    (pulse_sequence.py:47-59)."""
    n_t = int(round(TE / dt)) + 1
    return BlochSequence(G=np.zeros((n_meas, n_t, 3)), dt=dt,
                         rf_events=[_hard(0.0, 90.0, exc_axis_deg)], complex_signal=True,
                         family="gre", notes="90 + free evolution to TE (complex)")


def spin_echo(TE, dt, *, n_meas=1, exc_axis_deg=90.0):
    """A hard 90 at 0 and a hard 180 about x at TE/2; the echo forms at TE.  No gradient
    unless set on ``G`` (pulse_sequence.py:62-75)."""
    n_t = int(round(TE / dt)) + 1
    rf = [_hard(0.0, 90.0, exc_axis_deg), _hard(TE / 2.0, 180.0, 0.0)]
    return BlochSequence(G=np.zeros((n_meas, n_t, 3)), dt=dt, rf_events=rf,
                         complex_signal=False, family="se",
                         notes="90 - 180@TE/2 - echo (emergent refocusing)")


def fexi(delta, t_mix, dt, *, g_filter, g_detect, Delta=None, delta_detect=None,
         Delta_detect=None, direction=(1., 0., 0.), crush_cycles=32.0, exc_axis_deg=0.0):
    """FEXI filter-exchange stimulated echo (pulse_sequence.py:78-170).

    Timeline in samples: a bipolar filter (+g_filter for round(delta/dt) samples, a gap of
    max(1, round((Delta - delta)/dt)), -g_filter), a 90 that stores the magnetisation, the
    mixing time round(t_mix/dt) under a voxel crusher, a 90 that recalls it, a bipolar detection
    block (+g_detect[m], gap, -g_detect[m]) and one closing sample.  The three 90s share
    ``exc_axis_deg``.  One measurement per detection amplitude; ``.b_detect`` holds each one's
    b-value over the detection block, gamma^2 dt sum_t (dt sum_{t' <= t} G)^2."""
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    gd = np.atleast_1d(np.asarray(g_detect, dtype=np.float64))
    Delta = delta if Delta is None else Delta
    dd = delta if delta_detect is None else delta_detect
    Dd = Delta if Delta_detect is None else Delta_detect
    nf, gapf = int(round(delta / dt)), max(1, int(round((Delta - delta) / dt)))
    nd, gapd = int(round(dd / dt)), max(1, int(round((Dd - dd) / dt)))
    store = 2 * nf + gapf
    recall = store + int(round(t_mix / dt))
    n_t = recall + 2 * nd + gapd + 1
    G = np.zeros((len(gd), n_t, 3))
    G[:, :nf] = g_filter * d
    G[:, nf + gapf:store] = -g_filter * d
    for m, g in enumerate(gd):
        G[m, recall:recall + nd] = g * d
        G[m, recall + nd + gapd:recall + 2 * nd + gapd] = -g * d
    rf = [_hard(i * dt, 90.0, exc_axis_deg) for i in (0, store, recall)]
    crusher = {'windows_s': [((store + 1) * dt, (recall - 1) * dt)],
               'n_cycles': float(crush_cycles)}
    q = GAMMA * np.cumsum(G[:, recall:, :], axis=1) * dt       # (M, n, 3)
    b_detect = np.sum(q ** 2, axis=(1, 2)) * dt
    seq = BlochSequence(G=G, dt=dt, rf_events=rf, complex_signal=True, crusher=crusher,
                        family="fexi",
                        notes="PGSE filter - store - t_mix (exchange) - recall - PGSE detect")
    seq.b_detect = b_detect
    return seq


def prepend_mt_prep(seq, mt_prep):
    """Prepend an off-resonance saturation pulse and, after it, a crusher window to ``seq``
    (pulse_sequence.py:173-212).

    ``mt_prep``: ``offset_hz``, ``duration_s``, ``b1_hz`` (flip = 360 b1 duration degrees) or
    ``flip_deg``; optional ``axis_deg`` (0), ``spoiler_s`` (5e-4 s) and ``n_cycles`` (32).  The
    readout moves later by round(duration/dt) + round(spoiler/dt) samples (at least one for the
    pulse), with its RF times, echo samples and gradient; a zero-length spoiler keeps the
    readout's own crusher."""
    dt = seq.dt
    dur = float(mt_prep['duration_s'])
    flip = (float(mt_prep['flip_deg']) if mt_prep.get('flip_deg') is not None
            else 360.0 * float(mt_prep['b1_hz']) * dur)
    n_sat = max(1, int(round(dur / dt)))
    n_spoil = int(round(float(mt_prep.get('spoiler_s', 0.5e-3)) / dt))
    shift = n_sat + n_spoil
    G = np.concatenate([np.zeros((seq.n_meas, shift, 3), dtype=seq.G.dtype), seq.G], axis=1)
    sat = {'t_s': dur / 2.0, 'flip_deg': flip, 'axis_deg': float(mt_prep.get('axis_deg', 0.0)),
           'duration_s': dur, 'offset_hz': float(mt_prep['offset_hz'])}
    rf = [sat] + [dict(e, t_s=float(e['t_s']) + shift * dt) for e in seq.rf_events]
    echo = None if seq.echo_steps is None else [int(s) + shift for s in seq.echo_steps]
    crusher = seq.crusher
    if n_spoil > 0:
        crusher = {'windows_s': [(n_sat * dt, (n_sat + n_spoil) * dt)],
                   'n_cycles': float(mt_prep.get('n_cycles', 32.0))}
    return replace(seq, G=G, rf_events=rf, echo_steps=echo, crusher=crusher,
                   notes=seq.notes + f"; MT-prep {float(mt_prep['offset_hz']):.0f} Hz / "
                                     f"{dur * 1e3:.0f} ms")


def run_bloch_sequence(seq, n_walkers, diffusivity, geometry, *, seed=0, **kw):
    """``simulate_bloch`` on a :class:`BlochSequence` (its gradient, RF list, echo samples and
    crusher); further keywords pass through (pulse_sequence.py:215-226)."""
    wf = SimpleNamespace(G=np.asarray(seq.G), dt=float(seq.dt))
    return simulate_bloch(n_walkers, diffusivity, wf, geometry, seq.rf_events, seed=seed,
                          echo_steps=seq.echo_steps, crusher=seq.crusher, **kw)


def emergent_z_spectrum(offsets_hz, geometry, *, n_walkers, diffusivity, w1_hz, t_sat, dt,
                        T2, kappa_MT, dwell_time, T1=1.0, T2_bound=1e-5, T1_bound=1.0,
                        equilibrate_binding="auto", seed=0):
    """Final walker-mean Mz after a continuous-wave saturation of nutation rate ``w1_hz`` and
    length ``t_sat`` at each offset (pulse_sequence.py:229-281).  The bound pool needs the
    magnetisation-transfer walk (``kappa_MT > 0``), which this engine does not build."""
    offsets = np.atleast_1d(np.asarray(offsets_hz, dtype=float))
    n_t = int(round(float(t_sat) / float(dt))) + 1
    wf = SimpleNamespace(G=np.zeros((1, n_t, 3)), dt=float(dt))
    flip = 360.0 * float(w1_hz) * float(t_sat)
    mz = np.empty(offsets.shape)
    for i, off in enumerate(offsets):
        rf = [{'t_s': float(t_sat) / 2, 'flip_deg': flip, 'axis_deg': 0.0,
               'duration_s': float(t_sat), 'offset_hz': float(off)}]
        _, m = simulate_bloch(n_walkers, diffusivity, wf, geometry, rf, T2=T2, T1=T1,
                              kappa_MT=kappa_MT, dwell_time=dwell_time, T2_bound=T2_bound,
                              T1_bound=T1_bound, return_mz=True,
                              equilibrate_binding=equilibrate_binding, seed=seed)
        mz[i] = float(m[0])
    return mz
