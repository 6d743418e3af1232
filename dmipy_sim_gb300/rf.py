"""The RF pulse as its complex transmit field B1(t) = B1x + i B1y (Tesla) on a uniform raster,
and the single-spin Bloch integrator that maps it to magnetisation (rf.py of dmipy-sim).

Constructors: explicit samples, magnitude/phase, a hard (rectangular) pulse, an apodised sinc,
the hyperbolic-secant adiabatic full passage (Silver, Joseph & Hoult 1985), the adiabatic half
passage and BIR-4 (Garwood & Ke 1991), composite hard pulses.  ``bloch_simulate`` rotates each
spin of an ensemble (off-resonance, B1+ scale) per raster step about its effective field
(gamma B1x b, gamma B1y b, 2 pi df) dt and relaxes it toward +z; no flip is renormalised.
The scanner deliverability check reads a vendor limits catalogue that is not part of this
package.
"""
from dataclasses import dataclass

import numpy as np

from .constants import GAMMA

__all__ = ["B1Pulse", "bloch_simulate", "slice_profile"]


@dataclass
class B1Pulse:
    """Complex B1(t) in Tesla on raster ``dt`` (rf.py:38-275); ``flip_deg`` is the intended net
    flip when the constructor knows it."""
    b1: np.ndarray
    dt: float
    label: str = ""
    flip_deg: float = None

    def __post_init__(self):
        self.b1 = np.asarray(self.b1, dtype=np.complex128)
        if self.b1.ndim != 1:
            raise ValueError("b1 must be 1-D (n_samples,)")
        self.dt = float(self.dt)

    @property
    def n(self):
        return self.b1.shape[0]

    @property
    def duration(self):
        return self.n * self.dt

    @property
    def times(self):
        return np.arange(self.n) * self.dt

    @property
    def magnitude(self):
        return np.abs(self.b1)

    @property
    def phase(self):
        return np.angle(self.b1)

    @property
    def peak_b1(self):
        return float(np.max(np.abs(self.b1))) if self.n else 0.0

    @property
    def b1_rms(self):
        return float(np.sqrt(np.mean(np.abs(self.b1) ** 2))) if self.n else 0.0

    @property
    def sar_proxy(self):
        """sum |B1|^2 dt (T^2 s), proportional to the deposited RF energy."""
        return float(np.sum(np.abs(self.b1) ** 2) * self.dt)

    @property
    def nominal_flip_rad(self):
        """gamma sum |B1| dt: the on-resonance flip of a constant-phase pulse."""
        return float(GAMMA * np.sum(np.abs(self.b1)) * self.dt)

    @property
    def nominal_flip_deg(self):
        return np.degrees(self.nominal_flip_rad)

    @property
    def max_slew_b1(self):
        return float(np.max(np.abs(np.diff(self.b1))) / self.dt) if self.n >= 2 else 0.0

    @classmethod
    def from_samples(cls, b1, dt, label=""):
        return cls(b1=np.asarray(b1, dtype=np.complex128), dt=dt, label=label)

    @classmethod
    def from_magnitude_phase(cls, mag_T, phase_rad, dt, label=""):
        mag = np.asarray(mag_T, float)
        ph = np.zeros_like(mag) if phase_rad is None else np.asarray(phase_rad, float)
        return cls(b1=mag * np.exp(1j * ph), dt=dt, label=label)

    @classmethod
    def hard(cls, flip_deg, duration, dt, phase_deg=0.0, label="hard"):
        """round(duration/dt) samples (at least 1) of the amplitude whose discretised area
        gamma B1 n dt is the flip."""
        n = max(1, int(round(float(duration) / float(dt))))
        amp = np.deg2rad(float(flip_deg)) / (GAMMA * n * float(dt))
        b1 = np.full(n, amp, dtype=np.complex128) * np.exp(1j * np.deg2rad(phase_deg))
        return cls(b1=b1, dt=dt, label=label, flip_deg=float(flip_deg))

    @classmethod
    def windowed_sinc(cls, flip_deg, duration, dt, time_bw=4.0, n_zeros=None, window="hamming",
                      phase_deg=0.0, label="sinc"):
        """sinc(x) on x in [-z, z] (z = time_bw/2 zero crossings a side unless ``n_zeros``),
        Hamming-apodised (0.54 + 0.46 cos(pi x / z)) or not, scaled so gamma sum |B1| dt is
        the flip."""
        n = max(3, int(round(float(duration) / float(dt))))
        z = float(n_zeros) if n_zeros is not None else float(time_bw) / 2.0
        x = np.linspace(-z, z, n)
        env = np.sinc(x)
        if window == "hamming":
            env = env * (0.54 + 0.46 * np.cos(np.pi * x / z))
        elif window not in (None, "none", "rect"):
            raise ValueError(f"unknown window {window!r}")
        area = GAMMA * np.sum(np.abs(env)) * float(dt)
        amp = np.deg2rad(float(flip_deg)) / area if area > 0 else 0.0
        b1 = (env * amp).astype(np.complex128) * np.exp(1j * np.deg2rad(phase_deg))
        return cls(b1=b1, dt=dt, label=label, flip_deg=float(flip_deg))

    @classmethod
    def adiabatic_hs(cls, duration, dt, *, peak_b1, mu=4.0, beta=5.3, label="adiabatic_hs"):
        """Hyperbolic secant: peak_b1 sech(beta tau)^(1 + i mu), tau in [-1, 1]."""
        n = max(3, int(round(float(duration) / float(dt))))
        sech = 1.0 / np.cosh(beta * np.linspace(-1.0, 1.0, n))
        b1 = peak_b1 * sech * np.exp(1j * mu * np.log(sech + 1e-300))
        return cls(b1=b1.astype(np.complex128), dt=dt, label=label, flip_deg=180.0)

    @staticmethod
    def _half_passage(n, beta, kappa, sweep_hz):
        tau = np.linspace(0.0, 1.0, n)
        amp = np.tanh(beta * tau)
        freq = sweep_hz * np.tan(kappa * (1.0 - tau)) / np.tan(kappa)
        return amp, freq

    @classmethod
    def adiabatic_half_passage(cls, duration, dt, *, peak_b1, beta=6.0, kappa=np.arctan(20.0),
                               sweep_hz=1.0e4, label="ahp"):
        """Amplitude peak_b1 tanh(beta tau) while the frequency sweeps sweep_hz tan(kappa (1 -
        tau)) / tan(kappa) down to 0 (tau in [0, 1]); the phase is its running integral."""
        n = max(3, int(round(float(duration) / float(dt))))
        amp, freq = cls._half_passage(n, beta, kappa, sweep_hz)
        phase = np.cumsum(2.0 * np.pi * freq * float(dt))
        return cls(b1=(peak_b1 * amp * np.exp(1j * phase)).astype(np.complex128), dt=dt,
                   label=label, flip_deg=90.0)

    @classmethod
    def bir4(cls, flip_deg, duration, dt, *, peak_b1, beta=6.0, kappa=np.arctan(20.0),
             sweep_hz=1.0e4, label="bir4"):
        """Four half passages of n//4 samples (n = round(duration/dt), at least 8): amplitude
        forward, reversed, forward, reversed; the frequency likewise with signs +, -, +, -;
        phase jumps of flip/2 on the middle two segments."""
        n = max(8, int(round(float(duration) / float(dt))))
        q = n // 4
        amp0, fr0 = cls._half_passage(q, beta, kappa, sweep_hz)
        half = np.deg2rad(float(flip_deg) / 2.0)
        amp = np.concatenate([amp0, amp0[::-1], amp0, amp0[::-1]])
        fr = np.concatenate([fr0, -fr0[::-1], fr0, -fr0[::-1]])
        jump = np.concatenate([np.zeros(q), np.full(q, half), np.full(q, half), np.zeros(q)])
        ph = np.cumsum(2.0 * np.pi * fr * float(dt)) + jump
        b1 = peak_b1 * amp * np.exp(1j * ph)
        return cls(b1=b1.astype(np.complex128), dt=dt, label=label, flip_deg=float(flip_deg))

    @classmethod
    def composite(cls, segments, dt, *, peak_b1, label="composite"):
        """Hard sub-pulses (flip_deg, phase_deg) at peak_b1, each |flip| / (gamma peak_b1)
        long, concatenated."""
        parts = [cls.hard(f, abs(np.deg2rad(float(f))) / (GAMMA * float(peak_b1)), dt,
                          phase_deg=p).b1 for f, p in segments]
        return cls(b1=np.concatenate(parts).astype(np.complex128), dt=dt, label=label)

    def deliverability(self, model, *, coil="body", tol=1.02):
        raise NotImplementedError("the vendor scanner-limits catalogue is not part of this "
                                  "package; compare peak_b1, b1_rms and dt with the limits "
                                  "directly")

    def is_deliverable(self, model, *, coil="body", tol=1.02):
        return self.deliverability(model, coil=coil, tol=tol)["deliverable"]


def bloch_simulate(pulse, df_hz=0.0, b1_scale=1.0, M0=None, T1=np.inf, T2=np.inf,
                   return_history=False):
    """Magnetisation after ``pulse`` for an ensemble of spins (off-resonance ``df_hz``, B1+
    factor ``b1_scale``, broadcast together; start ``M0`` or +z).  Each raster step rotates by
    |n| about n = (gamma B1x b dt, gamma B1y b dt, 2 pi df dt) (the identity below 1e-30 rad)
    and relaxes: Mxy *= exp(-dt/T2), Mz -> Mz exp(-dt/T1) + 1 - exp(-dt/T1).  Returns
    (Mxy, Mz) and, with ``return_history``, M at every step (n + 1, 3, E) (rf.py:278-363)."""
    df = np.asarray(df_hz, float)
    bs = np.asarray(b1_scale, float)
    E = int(np.broadcast(df, bs).size)
    df = np.broadcast_to(df, (E,)).astype(float)
    bs = np.broadcast_to(bs, (E,)).astype(float)
    M = np.zeros((3, E))
    if M0 is None:
        M[2] = 1.0
    else:
        M0 = np.asarray(M0, float)
        M[:] = M0[:, None] if M0.ndim == 1 else M0
    dt = pulse.dt
    nz = 2.0 * np.pi * df * dt
    e1 = np.exp(-dt / T1) if np.isfinite(T1) else 1.0
    e2 = np.exp(-dt / T2) if np.isfinite(T2) else 1.0
    hist = None
    if return_history:
        hist = np.empty((pulse.n + 1, 3, E))
        hist[0] = M
    for k in range(pulse.n):
        nx = GAMMA * (pulse.b1[k].real * bs) * dt
        ny = GAMMA * (pulse.b1[k].imag * bs) * dt
        theta = np.sqrt(nx * nx + ny * ny + nz * nz)
        still = theta < 1e-30
        th = np.where(still, 1.0, theta)
        ux, uy, uz = nx / th, ny / th, nz / th
        c, s = np.cos(th), np.sin(th)
        omc = 1.0 - c
        Mx, My, Mz = M
        dot = ux * Mx + uy * My + uz * Mz
        rx = Mx * c + (uy * Mz - uz * My) * s + ux * dot * omc
        ry = My * c + (uz * Mx - ux * Mz) * s + uy * dot * omc
        rz = Mz * c + (ux * My - uy * Mx) * s + uz * dot * omc
        rx, ry, rz = (np.where(still, Mx, rx), np.where(still, My, ry), np.where(still, Mz, rz))
        M = np.stack([rx * e2, ry * e2, rz * e1 + (1.0 - e1)])
        if return_history:
            hist[k + 1] = M
    Mxy = M[0] + 1j * M[1]
    if return_history:
        return Mxy, M[2], hist
    return Mxy, M[2]


def slice_profile(pulse, slice_gradient, positions_m, df_hz=0.0, b1_scale=1.0, **kw):
    """(positions, Mxy, Mz) across a slice: a spin at z sees the extra off-resonance
    gamma G_ss z / (2 pi) Hz (rf.py:366-377)."""
    z = np.asarray(positions_m, float)
    df = (GAMMA / (2.0 * np.pi)) * float(slice_gradient) * z + np.asarray(df_hz, float)
    Mxy, Mz = bloch_simulate(pulse, df_hz=df, b1_scale=b1_scale, **kw)
    return z, Mxy, Mz
