"""RF pulses as sampled transmit fields, and the Bloch integrator that plays them on spins.

A pulse is its complex field B1(t) = B1x + i B1y (Tesla) on a uniform raster (the interface of
dmipy-sim's rf.py:38-275).  The constructors build a pulse from a named envelope:

  hard        a constant complex amplitude
  sinc        sinc(x) on x in [-w, w], optionally Hamming-apodised
  sech        the hyperbolic-secant full passage sech(beta tau)^(1 + i mu)  (Silver, Joseph and
              Hoult, Phys. Rev. A 31, 1985)
  tanh / tan  the adiabatic half passage: amplitude tanh(beta tau), frequency sweep
              tan(kappa (1 - tau)) / tan(kappa)  (Garwood and Ke, J. Magn. Reson. 94, 1991), and
              BIR-4, four such segments with phase jumps of half the flip
  composite   hard sub-pulses at a common peak amplitude

and flip-prescribed envelopes are scaled so that the on-resonance flip gamma * dt * sum |B1|
equals the prescription.

``bloch_simulate`` integrates the Bloch equation in the rotating frame for an ensemble of spins
(off-resonance, B1+ scale): every raster step is a rotation by the step's effective-field vector
w = (gamma b B1x dt, gamma b B1y dt, 2 pi df dt) -- applied here as the unit quaternion
(cos(|w|/2), sin(|w|/2) w/|w|) -- followed by relaxation toward +z.  The flip is whatever the
field produces; nothing is renormalised.  The scanner deliverability check needs a vendor limits
catalogue that is not part of this package.
"""
from dataclasses import dataclass

import numpy as np

from .constants import GAMMA

__all__ = ["B1Pulse", "bloch_simulate", "slice_profile"]


# ------------------------------------------------------------------------------------------------
# envelopes (unscaled, on n raster samples)
# ------------------------------------------------------------------------------------------------
def _raster_len(duration, dt, least):
    """Samples of a pulse of the given duration: duration / dt rounded, at least ``least``."""
    return max(least, int(round(float(duration) / float(dt))))


def _sinc_envelope(n, half_width, hamming):
    x = np.linspace(-half_width, half_width, n)
    taper = 0.54 + 0.46 * np.cos(np.pi * x / half_width) if hamming else 1.0
    return np.sinc(x) * taper


def _sech_envelope(n, beta, mu):
    """sech(beta tau)^(1 + i mu) for tau in [-1, 1] (amplitude sech, phase mu log sech)."""
    sech = 1.0 / np.cosh(beta * np.linspace(-1.0, 1.0, n))
    return sech * np.exp(1j * mu * np.log(sech + 1e-300))


def _half_passage(n, beta, kappa, sweep_hz):
    """(amplitude, frequency in Hz) of one adiabatic half passage over tau in [0, 1]."""
    tau = np.linspace(0.0, 1.0, n)
    return np.tanh(beta * tau), sweep_hz * np.tan(kappa * (1.0 - tau)) / np.tan(kappa)


def _phase_of_sweep(freq_hz, dt):
    """Running phase (rad) of a frequency sweep: the left Riemann sum of 2 pi f dt."""
    return np.cumsum(2.0 * np.pi * np.asarray(freq_hz, float) * float(dt))


def _per_flip(envelope, flip_deg, dt):
    """The envelope scaled so that gamma * dt * sum |B1| is the flip (a zero envelope stays 0)."""
    area = GAMMA * float(dt) * float(np.sum(np.abs(envelope)))
    return envelope * (np.radians(float(flip_deg)) / area if area > 0.0 else 0.0)


def _rotated(envelope, phase_deg):
    return np.asarray(envelope, np.complex128) * np.exp(1j * np.radians(float(phase_deg)))


# ------------------------------------------------------------------------------------------------
# the pulse
# ------------------------------------------------------------------------------------------------
@dataclass
class B1Pulse:
    """Complex B1(t) in Tesla on raster ``dt``; ``flip_deg`` is the intended net flip when the
    constructor prescribes one (None otherwise)."""
    b1: np.ndarray
    dt: float
    label: str = ""
    flip_deg: float = None

    def __post_init__(self):
        arr = np.asarray(self.b1, dtype=np.complex128)
        if arr.ndim != 1:
            raise ValueError("b1 must be 1-D (n_samples,)")
        self.b1, self.dt = arr, float(self.dt)

    # ---- raster and field statistics ----------------------------------------------------------
    n = property(lambda self: int(self.b1.size))
    duration = property(lambda self: self.n * self.dt)
    times = property(lambda self: self.dt * np.arange(self.n))
    magnitude = property(lambda self: np.abs(self.b1))
    phase = property(lambda self: np.angle(self.b1))

    @property
    def peak_b1(self):
        """Largest |B1| (T)."""
        return float(self.magnitude.max()) if self.n else 0.0

    @property
    def b1_rms(self):
        """Root-mean-square |B1| over the pulse (T)."""
        return float(np.sqrt(np.mean(self.magnitude ** 2))) if self.n else 0.0

    @property
    def sar_proxy(self):
        """dt * sum |B1|^2 (T^2 s): proportional to the RF energy deposited."""
        return float(self.dt * np.sum(self.magnitude ** 2))

    @property
    def nominal_flip_rad(self):
        """gamma * dt * sum |B1|: the on-resonance flip of a pulse of constant phase."""
        return float(GAMMA * self.dt * np.sum(self.magnitude))

    @property
    def nominal_flip_deg(self):
        return float(np.degrees(self.nominal_flip_rad))

    @property
    def max_slew_b1(self):
        """Largest |B1| change per second between neighbouring samples (T/s)."""
        if self.n < 2:
            return 0.0
        return float(np.abs(np.diff(self.b1)).max() / self.dt)

    # ---- constructors ------------------------------------------------------------------------
    @classmethod
    def from_samples(cls, b1, dt, label=""):
        """A pulse from its complex samples (T)."""
        return cls(np.asarray(b1, np.complex128), dt, label)

    @classmethod
    def from_magnitude_phase(cls, mag_T, phase_rad, dt, label=""):
        """A pulse from |B1| (T) and its phase (rad; None for a constant zero phase)."""
        mag = np.asarray(mag_T, float)
        ph = np.zeros(mag.shape) if phase_rad is None else np.asarray(phase_rad, float)
        return cls(mag * np.exp(1j * ph), dt, label)

    @classmethod
    def hard(cls, flip_deg, duration, dt, phase_deg=0.0, label="hard"):
        """Constant amplitude over duration / dt samples (at least one), scaled to the flip."""
        n = _raster_len(duration, dt, 1)
        env = _per_flip(np.ones(n), flip_deg, dt)
        return cls(_rotated(env, phase_deg), dt, label, float(flip_deg))

    @classmethod
    def windowed_sinc(cls, flip_deg, duration, dt, time_bw=4.0, n_zeros=None, window="hamming",
                      phase_deg=0.0, label="sinc"):
        """sinc over +-(time_bw / 2) zero crossings (or ``n_zeros``), Hamming-apodised with
        ``window="hamming"`` or not (None / "none" / "rect"), at least 3 samples, scaled to the
        flip."""
        if window not in ("hamming", None, "none", "rect"):
            raise ValueError(f"unknown window {window!r}")
        n = _raster_len(duration, dt, 3)
        half = float(time_bw) / 2.0 if n_zeros is None else float(n_zeros)
        env = _per_flip(_sinc_envelope(n, half, window == "hamming"), flip_deg, dt)
        return cls(_rotated(env, phase_deg), dt, label, float(flip_deg))

    @classmethod
    def adiabatic_hs(cls, duration, dt, *, peak_b1, mu=4.0, beta=5.3, label="adiabatic_hs"):
        """Hyperbolic-secant inversion: peak_b1 sech(beta tau)^(1 + i mu), tau in [-1, 1]."""
        n = _raster_len(duration, dt, 3)
        return cls(peak_b1 * _sech_envelope(n, beta, mu), dt, label, 180.0)

    @classmethod
    def adiabatic_half_passage(cls, duration, dt, *, peak_b1, beta=6.0, kappa=np.arctan(20.0),
                               sweep_hz=1.0e4, label="ahp"):
        """Adiabatic 90: amplitude peak_b1 tanh(beta tau) under a frequency sweep from
        ``sweep_hz`` down to 0, the phase being the sweep's running integral."""
        n = _raster_len(duration, dt, 3)
        amp, freq = _half_passage(n, beta, kappa, sweep_hz)
        return cls(peak_b1 * amp * np.exp(1j * _phase_of_sweep(freq, dt)), dt, label, 90.0)

    @classmethod
    def bir4(cls, flip_deg, duration, dt, *, peak_b1, beta=6.0, kappa=np.arctan(20.0),
             sweep_hz=1.0e4, label="bir4"):
        """BIR-4 plane rotation: four half-passage segments of n // 4 samples (n at least 8),
        amplitudes forward / reversed / forward / reversed, sweeps +, -reversed, +, -reversed,
        and a phase jump of half the flip across the middle two segments."""
        q = _raster_len(duration, dt, 8) // 4
        a, f = _half_passage(q, beta, kappa, sweep_hz)
        segments = ((a, f, 0.0), (a[::-1], -f[::-1], 1.0), (a, f, 1.0), (a[::-1], -f[::-1], 0.0))
        amp = np.concatenate([s[0] for s in segments])
        freq = np.concatenate([s[1] for s in segments])
        jump = np.repeat([s[2] for s in segments], q) * np.radians(float(flip_deg) / 2.0)
        phase = _phase_of_sweep(freq, dt) + jump
        return cls(peak_b1 * amp * np.exp(1j * phase), dt, label, float(flip_deg))

    @classmethod
    def composite(cls, segments, dt, *, peak_b1, label="composite"):
        """Hard sub-pulses (flip_deg, phase_deg) played back to back at amplitude peak_b1: each
        lasts |flip| / (gamma peak_b1)."""
        pieces = []
        for flip, phase in segments:
            length = abs(np.radians(float(flip))) / (GAMMA * float(peak_b1))
            pieces.append(cls.hard(flip, length, dt, phase_deg=phase).b1)
        return cls(np.concatenate(pieces), dt, label)

    def deliverability(self, model, *, coil="body", tol=1.02):
        raise NotImplementedError("the vendor scanner-limits catalogue is not part of this "
                                  "package; compare peak_b1, b1_rms and dt with the limits "
                                  "directly")

    def is_deliverable(self, model, *, coil="body", tol=1.02):
        return self.deliverability(model, coil=coil, tol=tol)["deliverable"]


# ------------------------------------------------------------------------------------------------
# Bloch integration
# ------------------------------------------------------------------------------------------------
def _rotate(M, w):
    """Rotate the vectors M (3, E) by the rotation vectors w (3, E) (angle |w| about w / |w|,
    right-handed), through the unit quaternion (c, s u), c = cos(|w|/2), s = sin(|w|/2):
    M' = M + 2 c (v x M) + 2 v x (v x M) with v = s u.  A rotation below 1e-30 rad leaves M."""
    ang = np.sqrt(np.sum(w * w, axis=0))
    tiny = ang < 1e-30
    safe = np.where(tiny, 1.0, ang)
    half = 0.5 * safe
    v = w * (np.sin(half) / safe)
    c = np.cos(half)
    t = 2.0 * np.cross(v, M, axis=0)
    out = M + c * t + np.cross(v, t, axis=0)
    return np.where(tiny, M, out)


def bloch_simulate(pulse, df_hz=0.0, b1_scale=1.0, M0=None, T1=np.inf, T2=np.inf,
                   return_history=False):
    """Magnetisation after ``pulse`` for spins at off-resonance ``df_hz`` (Hz) with B1+ factor
    ``b1_scale`` (broadcast together into an ensemble of E spins), starting from ``M0`` ((3,) or
    (3, E); +z by default).  Per raster step: rotation by (gamma b B1x dt, gamma b B1y dt,
    2 pi df dt), then Mxy *= exp(-dt / T2), Mz <- Mz exp(-dt / T1) + 1 - exp(-dt / T1) (infinite
    times relax nothing).  Returns (Mxy (E,) complex, Mz (E,)) and, with ``return_history``, M at every
    step boundary (n + 1, 3, E)."""
    df, bs = np.broadcast_arrays(np.asarray(df_hz, float), np.asarray(b1_scale, float))
    df, bs = df.ravel().astype(float), bs.ravel().astype(float)
    E = df.size
    if M0 is None:
        M = np.vstack([np.zeros((2, E)), np.ones((1, E))])
    else:
        m0 = np.asarray(M0, float)
        M = np.array(np.broadcast_to(m0[:, None] if m0.ndim == 1 else m0, (3, E)), float)
    dt = pulse.dt
    keep_t2 = np.exp(-dt / T2) if np.isfinite(T2) else 1.0
    keep_t1 = np.exp(-dt / T1) if np.isfinite(T1) else 1.0
    wz = 2.0 * np.pi * dt * df
    history = [M.copy()] if return_history else None
    for b in pulse.b1:
        w = np.stack([GAMMA * dt * (b.real * bs), GAMMA * dt * (b.imag * bs), wz])
        M = _rotate(M, w)
        M[:2] *= keep_t2
        M[2] = M[2] * keep_t1 + (1.0 - keep_t1)
        if return_history:
            history.append(M.copy())
    mxy, mz = M[0] + 1j * M[1], M[2].copy()
    if return_history:
        return mxy, mz, np.stack(history)
    return mxy, mz


def slice_profile(pulse, slice_gradient, positions_m, df_hz=0.0, b1_scale=1.0, **kw):
    """(positions, Mxy, Mz) across a slice: the spin at z also sees gamma G_ss z / (2 pi) Hz of
    off-resonance (the interface of rf.py:366-377)."""
    z = np.asarray(positions_m, float)
    df = np.asarray(df_hz, float) + float(slice_gradient) * z * (GAMMA / (2.0 * np.pi))
    mxy, mz = bloch_simulate(pulse, df_hz=df, b1_scale=b1_scale, **kw)
    return z, mxy, mz
