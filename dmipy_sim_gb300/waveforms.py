"""Gradient waveforms: the ``Waveform`` object and the constructors the walk is driven by.

Same fields, units and conventions as dmipy-sim's ``waveforms.py`` (Waveform 39-90, pgse 93-163,
pgste 166-262, ogse 265-350, trapezoidal_ogse 353-455, b_trapezoidal_ogse 458-487,
calc_b 490-516, calc_btensor 519-543, btensor_invariants 546-595, ste 598-655, pte 658-720,
set_b 723-772, rotate_waveform 775-818, tile_waveform 821-848, cpmg 851-917): ``G`` is (n_meas, n_t, 3) float32
in T/m on a uniform time grid ``dt``; the second lobe of a spin echo carries the refocusing sign
(bipolar convention), so the phase is simply gamma * sum_t G(t) . r(t) * dt.  Host-side numpy only.
"""
from dataclasses import dataclass, replace
from warnings import warn

import numpy as np

from .constants import GAMMA, DEFAULT_SLEW_RATE, resolve_slew


@dataclass
class Waveform:
    """Gradient waveform: G (n_meas, n_t, 3) T/m, uniform step dt (s).

    ``echo_idx`` is the sample the signal is read at (the last one for a spin echo);
    ``echo_indices`` lists the echoes of a multi-echo train (CPMG); ``chi_perp`` is the (n_t,)
    transverse-coherence mask (1 transverse, 0 stored longitudinally; None = all transverse);
    ``stimulated_echo`` halves the signal.  ``rf_events`` and ``G_display`` are for display only.
    """
    G: np.ndarray
    dt: float
    echo_idx: int
    rf_events: list = None
    G_display: np.ndarray = None
    echo_indices: np.ndarray = None
    chi_perp: np.ndarray = None
    TM: float = None
    stimulated_echo: bool = False


def _lobe(arr, m, i0, n, amp, n_rise):
    """Write a rectangular (n_rise = 0) or trapezoidal lobe of peak ``amp`` into samples
    [i0, i0 + n) of measurement m (waveforms.py:15-29)."""
    n_rise = min(int(n_rise), n // 2)
    if n_rise > 0:
        ramp = np.arange(n_rise, dtype=np.float64) / n_rise
        arr[m, i0:i0 + n_rise] = ramp[:, None] * amp
        arr[m, i0 + n_rise:i0 + n - n_rise] = amp
        arr[m, i0 + n - n_rise:i0 + n] = (1.0 - ramp)[:, None] * amp
    else:
        arr[m, i0:i0 + n] = amp


def _ramp_samples(square, G_peak, slew_rate, dt, n):
    """Ramp length in samples of a slew-limited lobe (waveforms.py:32-36)."""
    if square or G_peak <= 0:
        return 0
    return min(max(0, round((G_peak / float(slew_rate)) / dt)), n // 2)


def _amplitudes(G_magnitude, n_meas):
    return np.broadcast_to(np.asarray(G_magnitude, dtype=np.float32), (n_meas,))


def pgse(delta, DELTA, G_magnitude, bvecs, n_t, slew_rate=DEFAULT_SLEW_RATE):
    """Pulsed-gradient spin echo over DELTA + delta seconds (waveforms.py:93-163).

    Lobes start at samples 0 and round(DELTA/dt), each max(1, round(delta/dt)) samples long; the
    second lobe is -G.  Slew-limited trapezoids by default, ``slew_rate=np.inf`` for squares.
    """
    bvecs = np.asarray(bvecs, dtype=np.float32)
    n_meas = bvecs.shape[0]
    amp = _amplitudes(G_magnitude, n_meas)
    dt = (DELTA + delta) / (n_t - 1)
    n_pulse = max(1, round(delta / dt))
    n_DELTA = round(DELTA / dt)
    _, square = resolve_slew(slew_rate)
    n_rise = _ramp_samples(square, float(np.max(np.abs(amp))), slew_rate, dt, n_pulse)
    G = np.zeros((n_meas, n_t, 3), dtype=np.float32)
    Gd = np.zeros((n_meas, n_t, 3), dtype=np.float32)
    for m in range(n_meas):
        g = amp[m] * bvecs[m]
        _lobe(G, m, 0, n_pulse, g, n_rise)
        _lobe(G, m, n_DELTA, n_pulse, -g, n_rise)
        _lobe(Gd, m, 0, n_pulse, g, n_rise)
        _lobe(Gd, m, n_DELTA, n_pulse, g, n_rise)
    mid = (n_pulse + n_DELTA) // 2
    rf = [{'t_s': 0.0, 'label': 'Mz→Mxy', 'flip_deg': 90},
          {'t_s': mid * dt, 'label': 'refocus', 'flip_deg': 180}]
    return Waveform(G=G, dt=float(dt), echo_idx=n_t - 1, rf_events=rf, G_display=Gd)


def pgste(delta, TM, G_magnitude, bvecs, n_t, slew_rate=DEFAULT_SLEW_RATE):
    """Pulsed-gradient stimulated echo: +G lobe, mixing time TM stored longitudinally (chi = 0),
    -G lobe; signal halved (waveforms.py:166-262)."""
    bvecs = np.asarray(bvecs, dtype=np.float32)
    n_meas = bvecs.shape[0]
    amp = _amplitudes(G_magnitude, n_meas)
    dt = (2.0 * delta + TM) / (n_t - 1)
    n_pulse = max(1, round(delta / dt))
    i_recall = n_pulse + round(TM / dt)
    _, square = resolve_slew(slew_rate)
    n_rise = _ramp_samples(square, float(np.max(np.abs(amp))), slew_rate, dt, n_pulse)
    G = np.zeros((n_meas, n_t, 3), dtype=np.float32)
    Gd = np.zeros((n_meas, n_t, 3), dtype=np.float32)
    n2 = min(n_pulse, n_t - i_recall)
    for m in range(n_meas):
        g = amp[m] * bvecs[m]
        _lobe(G, m, 0, n_pulse, g, n_rise)
        _lobe(G, m, i_recall, n2, -g, n_rise)
        _lobe(Gd, m, 0, n_pulse, g, n_rise)
        _lobe(Gd, m, i_recall, n2, g, n_rise)
    chi = np.ones(n_t, dtype=bool)
    chi[n_pulse:i_recall] = False
    rf = [{'t_s': 0.0, 'label': 'Mz→Mxy', 'flip_deg': 90},
          {'t_s': n_pulse * dt, 'label': 'store', 'flip_deg': 90},
          {'t_s': i_recall * dt, 'label': 'recall', 'flip_deg': 90}]
    return Waveform(G=G, dt=float(dt), echo_idx=n_t - 1, rf_events=rf, G_display=Gd,
                    chi_perp=chi, TM=float(TM), stimulated_echo=True)


def ogse(frequency, T_total, G_magnitude, bvecs, n_t, kind='cosine'):
    """Oscillating-gradient spin echo (waveforms.py:265-350).

    The frequency snaps to an integer number of periods per half echo, f = N / (T_total/2); the
    post-180 half is the negated time mirror of the first half, so the moment nulls at the echo.
    """
    bvecs = np.asarray(bvecs, dtype=np.float32)
    n_meas = bvecs.shape[0]
    amp = _amplitudes(G_magnitude, n_meas)
    dt = T_total / (n_t - 1)
    t = np.arange(n_t, dtype=np.float64) * dt
    half = T_total / 2.0
    n_per = max(1, int(round(frequency * half)))
    f_eff = n_per / half
    if abs(f_eff - frequency) > 0.1 * max(frequency, 1e-9):
        warn(f"ogse: frequency snapped {frequency:.1f} -> {f_eff:.1f} Hz "
             f"({n_per} periods per half-echo of {half * 1e3:.1f} ms) for a valid OGSE")
    if kind == 'cosine':
        env = np.cos(2 * np.pi * f_eff * t)
    elif kind == 'sine':
        env = np.sin(2 * np.pi * f_eff * t)
    else:
        raise ValueError(f"ogse kind must be 'cosine' or 'sine', got {kind!r}")
    mid = n_t // 2
    env[n_t - mid:] = -env[:mid][::-1]
    if n_t % 2 == 1:
        env[mid] = 0.0
    G = (amp[:, None, None] * env[None, :, None] * bvecs[:, None, :]).astype(np.float32)
    gap = (n_t - 1) // 2
    rf = [{'t_s': 0.0, 'label': 'Mz→Mxy', 'flip_deg': 90},
          {'t_s': gap * dt, 'label': 'refocus', 'flip_deg': 180}]
    return Waveform(G=G, dt=float(dt), echo_idx=n_t - 1, rf_events=rf)


def cpmg(n_echoes, TE, G_magnitude, bvecs, n_t_per_echo=100):
    """CPMG echo train with ideal 180s at (k + 1/2) TE and echoes at k TE (waveforms.py:851-917).

    ``G`` carries the sign flip of every refocusing pulse; ``echo_indices`` = k * n_t_per_echo.
    """
    bvecs = np.asarray(bvecs, dtype=np.float32)
    n_meas = bvecs.shape[0]
    amp = _amplitudes(G_magnitude, n_meas)
    n_t = n_echoes * n_t_per_echo + 1
    dt = n_echoes * TE / (n_t - 1)
    t = np.arange(n_t) * dt
    sign = np.ones(n_t, dtype=np.float32)
    for k in range(n_echoes):
        sign[t >= (k + 0.5) * TE] *= -1.0
    g = amp[:, None] * bvecs                                   # (n_meas, 3)
    G_phys = np.broadcast_to(g[:, None, :], (n_meas, n_t, 3)).astype(np.float32)
    G_eff = (sign[None, :, None] * g[:, None, :]).astype(np.float32)
    rf = [{'t_s': 0.0, 'label': 'Mz→Mxy', 'flip_deg': 90}]
    rf += [{'t_s': (k + 0.5) * TE, 'label': 'refocus', 'flip_deg': 180} for k in range(n_echoes)]
    return Waveform(G=G_eff, dt=float(dt), echo_idx=n_t - 1, rf_events=rf,
                    G_display=G_phys, echo_indices=np.arange(1, n_echoes + 1) * n_t_per_echo)


def _q(waveform):
    G = np.asarray(waveform.G)
    return np.cumsum(G * waveform.dt, axis=1) * GAMMA


def calc_b(waveform):
    """b-value per measurement (s/m^2): q(t) by the left-point rule, |q|^2 by the trapezoid rule,
    consistent with the walk's post-step phase sampling (waveforms.py:490-516)."""
    q = _q(waveform)
    return np.trapezoid(np.sum(q ** 2, axis=2), dx=waveform.dt, axis=1).astype(np.float64)


def calc_btensor(waveform):
    """B-tensor per measurement, B_ij = int q_i q_j dt, with trace(B) = calc_b (waveforms.py:519-543)."""
    q = _q(waveform)
    return np.trapezoid(q[:, :, :, None] * q[:, :, None, :], dx=waveform.dt,
                        axis=1).astype(np.float64)


def set_b(waveform, b_target):
    """Scale each measurement's G by sqrt(b_target / calc_b) (waveforms.py:723-772)."""
    import warnings
    b_now = calc_b(waveform)
    b_arr = np.asarray(b_target, dtype=np.float64).ravel()
    nz = b_arr[b_arr > 0]
    if nz.size > 0 and nz.max() < 1e5:
        warnings.warn(
            f"set_b: b_target values appear very small (max={nz.max():.4g} s/m²). "
            "Did you pass b-values in s/mm² instead of s/m²? Multiply by 1e6 to convert.",
            UserWarning, stacklevel=2)
    b_t = np.broadcast_to(np.asarray(b_target, dtype=np.float64), b_now.shape)
    scale = np.sqrt(b_t / b_now).astype(np.float32)
    G = (np.asarray(waveform.G) * scale[:, None, None]).astype(np.float32)
    Gd = waveform.G_display
    if Gd is not None:
        Gd = (np.asarray(Gd) * scale[:, None, None]).astype(np.float32)
    return replace(waveform, G=G, G_display=Gd)


def rotate_waveform(waveform, R=None, *, theta=None):
    """Rotate the gradient vectors, G_new = G @ R.T; ``theta`` rotates about y (waveforms.py:775-818)."""
    if (R is None) == (theta is None):
        raise ValueError("rotate_waveform: pass exactly one of R or theta.")
    if theta is not None:
        c, s = np.cos(float(theta)), np.sin(float(theta))
        R = np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]], dtype=np.float32)
    R = np.asarray(R, dtype=np.float32)
    G = np.einsum('mtj,ij->mti', np.asarray(waveform.G), R).astype(np.float32)
    return Waveform(G=G, dt=waveform.dt, echo_idx=waveform.echo_idx, rf_events=waveform.rf_events,
                    chi_perp=waveform.chi_perp, TM=waveform.TM,
                    stimulated_echo=waveform.stimulated_echo)


def tile_waveform(waveform, n_copies):
    """Stack n_copies of the waveform along the measurement axis (waveforms.py:821-848)."""
    G = np.tile(np.asarray(waveform.G), (n_copies, 1, 1)).astype(np.float32)
    return Waveform(G=G, dt=waveform.dt, echo_idx=waveform.echo_idx, rf_events=waveform.rf_events,
                    chi_perp=waveform.chi_perp, TM=waveform.TM,
                    stimulated_echo=waveform.stimulated_echo)


def trapezoidal_ogse(N, delta, DELTA, G_magnitude, bvecs, n_t, rise_time=None, slew_rate=200e3):
    """Trapezoidal N-lobe OGSE over DELTA + delta (waveforms.py:353-455): two blocks of N lobes,
    each delta/N long with linear ramps of ``rise_time`` (default: peak G / slew_rate), the first
    block starting at sample 0 with signs +,-,+,..., the second at round(DELTA/dt) with the signs
    flipped.  N = 1 is a trapezoidal PGSE."""
    bvecs = np.asarray(bvecs, dtype=np.float32)
    n_meas = bvecs.shape[0]
    amp = _amplitudes(G_magnitude, n_meas)
    g_peak = float(np.max(np.abs(amp)))
    if rise_time is None:
        rise_time = g_peak / slew_rate if g_peak > 0 else 0.0
    dt = (DELTA + delta) / (n_t - 1)
    n_lobe = max(1, round(delta / (N * dt)))
    n_rise = min(max(0, round(rise_time / dt)), n_lobe // 2)
    starts = (0, round(DELTA / dt))
    G = np.zeros((n_meas, n_t, 3), dtype=np.float32)
    for m in range(n_meas):
        for blk, b0 in enumerate(starts):
            for k in range(N):
                sgn = (-1) ** k if blk == 0 else -((-1) ** k)
                peak = sgn * amp[m]                        # float32, as the lobe's flat top
                i0, i1 = b0 + k * n_lobe, b0 + (k + 1) * n_lobe
                if n_rise > 0:
                    up = np.linspace(0.0, peak, n_rise, endpoint=False)
                    down = np.linspace(peak, 0.0, n_rise, endpoint=False)
                    G[m, i0:i0 + n_rise] = up[:, None] * bvecs[m]
                    G[m, i0 + n_rise:i1 - n_rise] = peak * bvecs[m]
                    G[m, i1 - n_rise:i1] = down[:, None] * bvecs[m]
                else:
                    G[m, i0:i1] = peak * bvecs[m]
    mid = (n_lobe * N + starts[1]) // 2
    rf = [{'t_s': 0.0, 'label': 'Mz→Mxy', 'flip_deg': 90},
          {'t_s': mid * dt, 'label': 'refocus', 'flip_deg': 180}]
    return Waveform(G=G, dt=float(dt), echo_idx=n_t - 1, rf_events=rf)


def b_trapezoidal_ogse(N, delta, DELTA, G, rise_time):
    """Closed-form b-value of the trapezoidal N-lobe OGSE (waveforms.py:458-487, Drobnjak et al.
    2016 Eq. 2): the oscillating part plus, for odd N, the cross-block term of the net lobe
    moment."""
    x = rise_time * N / delta
    osc = 2.0 * G ** 2 * GAMMA ** 2 * delta ** 3 / (15.0 * N ** 2) * (
        5.0 - 7.5 * x - 1.25 * x ** 2 + 4.0 * x ** 3)
    q_net = (1 - (-1) ** N) * (delta - N * rise_time) / (2.0 * N)
    return float(osc + G ** 2 * GAMMA ** 2 * (DELTA - delta) * q_net ** 2)


def btensor_invariants(B):
    """(b, b_delta, b_eta) of B-tensors (n_meas, 3, 3) (waveforms.py:546-595): b = trace,
    b_delta = normalised anisotropy (linear 1, spherical 0, planar -0.5) and b_eta = normalised
    asymmetry, in the prolate/oblate convention chosen by which extreme eigenvalue lies farther
    from b/3."""
    lam = np.linalg.eigvalsh(np.asarray(B))[:, ::-1]         # descending
    l1, l2, l3 = lam[:, 0], lam[:, 1], lam[:, 2]
    b = l1 + l2 + l3
    bs = np.where(b > 0, b, 1.0)
    prolate = np.abs(l1 - b / 3.0) >= np.abs(l3 - b / 3.0)
    b_delta = np.where(prolate, (l1 - (l2 + l3) / 2.0) / bs, (l3 - (l1 + l2) / 2.0) / bs)
    b_eta = np.where(prolate, (l2 - l3) / bs, (l1 - l2) / bs)
    return b, b_delta, b_eta


def _bipolar_axes(axes, total, G_magnitude, n_t, slew_rate):
    """One measurement of back-to-back bipolar lobe pairs, one pair per axis, each pair taking
    2 / (2 len(axes)) of the n_t samples (the tensor-encoding layout of waveforms.py:598-720)."""
    dt = total / (n_t - 1)
    n_seg = max(1, round(n_t / (2 * len(axes))))
    _, square = resolve_slew(slew_rate)
    n_rise = _ramp_samples(square, abs(float(G_magnitude)), slew_rate, dt, n_seg)
    G = np.zeros((1, n_t, 3), dtype=np.float32)
    for i, a in enumerate(axes):
        enc0 = 2 * i * n_seg
        enc1 = min((2 * i + 1) * n_seg, n_t)
        dec1 = min((2 * i + 2) * n_seg, n_t)
        g = (G_magnitude * np.asarray(a)).astype(np.float32)
        _lobe(G, 0, enc0, enc1 - enc0, g, n_rise)
        _lobe(G, 0, enc1, dec1 - enc1, -g, n_rise)
    return Waveform(G=G, dt=float(dt), echo_idx=n_t - 1,
                    rf_events=[{'t_s': 0.0, 'label': 'Mz→Mxy', 'flip_deg': 90}])


def ste(delta, DELTA, G_magnitude, n_t, slew_rate=DEFAULT_SLEW_RATE):
    """Spherical tensor encoding (b_delta = 0) over DELTA + delta (waveforms.py:598-655): bipolar
    pairs along x, y and z in turn, so every q_i(t) returns to zero before the next axis starts
    and B = (b/3) I."""
    return _bipolar_axes(np.eye(3, dtype=np.float32), DELTA + delta, G_magnitude, n_t, slew_rate)


def pte(delta, DELTA, G_magnitude, plane_normal, n_t, slew_rate=DEFAULT_SLEW_RATE):
    """Planar tensor encoding (b_delta = -0.5) over DELTA + delta (waveforms.py:658-720): bipolar
    pairs along two orthonormal in-plane axes u, v (Gram-Schmidt from x, or y when the normal is
    close to x, and v = n x u)."""
    n = np.asarray(plane_normal, dtype=np.float64)
    n = n / np.linalg.norm(n)
    ref = np.array([1.0, 0.0, 0.0]) if abs(n[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = ref - np.dot(ref, n) * n
    u /= np.linalg.norm(u)
    v = np.cross(n, u)
    v /= np.linalg.norm(v)
    return _bipolar_axes([u, v], DELTA + delta, G_magnitude, n_t, slew_rate)
