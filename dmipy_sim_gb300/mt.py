"""Magnetisation transfer: the binding bookkeeping of the MT walk and the analytic two-pool
Bloch-McConnell model that validates it (mt.py of dmipy-sim).

A free spin that hits a reactive wall with penetration d_perp sticks with probability
p = min(1, 2 kappa_MT d_perp / D), stays bound for an exponential dwell of mean ``dwell_time`` and
relaxes meanwhile with the bound pool's T2 / T1.  In the well-mixed limit this is a two-pool
exchange with forward rate k_f = kappa_MT * S/V and backward rate k_r = 1 / dwell_time, whose
magnetisation obeys the Bloch-McConnell equations: per pool, precession about z at its offset,
nutation about the B1 axis, relaxation toward its M0, and exchange of every component at k_f
(free -> bound) and k_r (bound -> free).  With constant coefficients the 7-dimensional affine
system (Mxa, Mya, Mza, Mxb, Myb, Mzb, 1) evolves exactly by a matrix exponential.
"""
import warnings

import numpy as np

__all__ = [
    "stick_probability", "forward_rate", "backward_rate", "bound_fraction",
    "kappa_MT_from_forward_rate", "dwell_time_from_fraction", "surface_to_volume",
    "resolve_equilibrate_mode", "equilibrate_burnin_plateau", "two_pool_generator",
    "evolve_two_pool", "bloch_mcconnell_transverse", "bloch_mcconnell_longitudinal",
    "mt_z_spectrum",
]


def stick_probability(d_perp, kappa_MT, D):
    """min(1, 2 kappa_MT d_perp / D) for a hit of penetration ``d_perp`` (m)."""
    return np.minimum(1.0, 2.0 * (kappa_MT / D) * np.asarray(d_perp, dtype=float))


def forward_rate(kappa_MT, S_over_V):
    """k_f = kappa_MT * S/V (1/s)."""
    return float(kappa_MT) * float(S_over_V)


def backward_rate(dwell_time):
    """k_r = 1 / dwell_time (1/s)."""
    if dwell_time <= 0.0:
        raise ValueError(f"dwell_time must be > 0, got {dwell_time}")
    return 1.0 / float(dwell_time)


def bound_fraction(kappa_MT, dwell_time, S_over_V):
    """Equilibrium bound fraction k_f / (k_f + k_r)."""
    kf, kr = forward_rate(kappa_MT, S_over_V), backward_rate(dwell_time)
    return kf / (kf + kr) if kf + kr > 0 else 0.0


def kappa_MT_from_forward_rate(k_f, S_over_V):
    """kappa_MT = k_f / (S/V)."""
    if S_over_V <= 0.0:
        raise ValueError(f"S_over_V must be > 0, got {S_over_V}")
    return float(k_f) / float(S_over_V)


def dwell_time_from_fraction(f_bound, k_f):
    """The dwell time that gives an equilibrium bound fraction ``f_bound`` at forward rate
    ``k_f``: detailed balance k_f (1 - f_b) = k_r f_b."""
    if not 0.0 < f_bound < 1.0:
        raise ValueError(f"f_bound must be in (0,1), got {f_bound}")
    if k_f <= 0.0:
        raise ValueError(f"k_f must be > 0, got {k_f}")
    return f_bound / (k_f * (1.0 - f_bound))


def _radius(geometry):
    for a in ("radius", "sphere_radius"):
        v = getattr(geometry, a, None)
        if v is not None:
            return float(v)
    radii = getattr(geometry, "_radii_np", None)
    if radii is not None and len(radii):
        return float(np.min(radii))
    return None


def surface_to_volume(geometry):
    """S/V (1/m) of a Sphere (3/R) or an infinite Cylinder (2/R); None otherwise."""
    R = _radius(geometry)
    if R is not None and R > 0.0:
        name = type(geometry).__name__
        if name == "Sphere":
            return 3.0 / R
        if name == "Cylinder":
            return 2.0 / R
    return None


def resolve_equilibrate_mode(equilibrate_binding, geometry):
    """'off' | 'burnin' | 'fast' for an MT walk without a read-out: 'auto' means 'burnin';
    'fast' needs a known S/V and falls back to 'burnin' with a warning."""
    eb = equilibrate_binding
    if eb in (None, False, "off"):
        return "off"
    if eb in ("auto", True, "burnin"):
        return "burnin"
    if eb == "fast":
        if surface_to_volume(geometry) is None:
            warnings.warn("equilibrate_binding='fast' needs a known surface-to-volume "
                          "(analytic Sphere/Cylinder); falling back to 'burnin'.", stacklevel=2)
            return "burnin"
        return "fast"
    raise ValueError(f"equilibrate_binding must be 'auto'|'burnin'|'fast'|'off', got {eb!r}")


def equilibrate_burnin_plateau(chunk_fn, r0, keys, brem0, tol=0.01, max_chunks=40):
    """Advance ``chunk_fn(r, keys, brem) -> (r, keys, brem, occupancy)`` until the occupancy
    changes by at most ``tol`` relative between chunks (at most ``max_chunks``); returns
    ``(r, keys, brem, occupancy, converged)``."""
    r, k, brem = r0, keys, brem0
    prev = -1.0
    for _ in range(int(max_chunks)):
        r, k, brem, occ = chunk_fn(r, k, brem)
        occ = float(occ)
        if prev >= 0.0 and abs(occ - prev) <= tol * max(occ, 1e-6):
            return r, k, brem, occ, True
        prev = occ
    return r, k, brem, prev, False


def two_pool_generator(*, R1a, R2a, R1b, R2b, k_f, k_r, M0a=1.0, M0b=None, dw_a=0.0, dw_b=0.0,
                       w1=0.0, rf_phase=0.0):
    """The 7 x 7 generator A of dx/dt = A x, x = (Mxa, Mya, Mza, Mxb, Myb, Mzb, 1).

    Per pool: dM/dt = M x (0, 0, dw) + w1 u x M - R2 (Mx, My) - R1 (Mz - M0) with
    u = (cos rf_phase, sin rf_phase, 0); exchange: dMa/dt -= k_f Ma - k_r Mb and the reverse.
    ``M0b`` defaults to the detailed-balance size M0a k_f / k_r."""
    if M0b is None:
        M0b = M0a * (k_f / k_r) if k_r > 0 else 0.0
    ux, uy = np.cos(rf_phase), np.sin(rf_phase)

    def pool(R1, R2, dw, M0):
        B = np.array([[-R2, -dw, w1 * uy],
                      [dw, -R2, -w1 * ux],
                      [-w1 * uy, w1 * ux, -R1]], dtype=float)
        return B, np.array([0.0, 0.0, R1 * M0])

    Ba, ca = pool(R1a, R2a, dw_a, M0a)
    Bb, cb = pool(R1b, R2b, dw_b, M0b)
    I3 = np.eye(3)
    A = np.zeros((7, 7))
    A[:3, :3] = Ba - k_f * I3
    A[3:6, 3:6] = Bb - k_r * I3
    A[:3, 3:6] = k_r * I3
    A[3:6, :3] = k_f * I3
    A[:3, 6] = ca
    A[3:6, 6] = cb
    return A


def evolve_two_pool(state0, t, A):
    """exp(A t) state0."""
    from scipy.linalg import expm
    return expm(np.asarray(A, float) * float(t)) @ np.asarray(state0, dtype=float)


def _pools(M0a, M0b, k_f, k_r):
    return M0a, (M0a * (k_f / k_r) if k_r > 0 else 0.0) if M0b is None else M0b


def bloch_mcconnell_transverse(t, *, T2a, T2b, k_f, k_r, T1a=1.0, T1b=1.0, M0a=1.0, M0b=None,
                               dw_a=0.0, dw_b=0.0):
    """|Mxa + i Mya|(t) of the free pool after both pools were tipped onto x (no RF)."""
    M0a, M0b = _pools(M0a, M0b, k_f, k_r)
    A = two_pool_generator(R1a=1.0 / T1a, R2a=1.0 / T2a, R1b=1.0 / T1b, R2b=1.0 / T2b,
                           k_f=k_f, k_r=k_r, M0a=M0a, M0b=M0b, dw_a=dw_a, dw_b=dw_b)
    x0 = np.array([M0a, 0.0, 0.0, M0b, 0.0, 0.0, 1.0])
    ts = np.atleast_1d(np.asarray(t, dtype=float))
    out = np.array([np.hypot(*evolve_two_pool(x0, tt, A)[:2]) for tt in ts])
    return out if out.size > 1 else float(out[0])


def bloch_mcconnell_longitudinal(t, *, T1a, T1b, k_f, k_r, M0a=1.0, M0b=None, Mza0=None,
                                 Mzb0=None):
    """Mza(t) of the free pool under exchange without RF; both pools inverted unless
    ``Mza0`` / ``Mzb0`` are given."""
    M0a, M0b = _pools(M0a, M0b, k_f, k_r)
    A = two_pool_generator(R1a=1.0 / T1a, R2a=1e-9, R1b=1.0 / T1b, R2b=1e-9, k_f=k_f, k_r=k_r,
                           M0a=M0a, M0b=M0b)
    x0 = np.array([0.0, 0.0, -M0a if Mza0 is None else Mza0, 0.0, 0.0,
                   -M0b if Mzb0 is None else Mzb0, 1.0])
    ts = np.atleast_1d(np.asarray(t, dtype=float))
    out = np.array([evolve_two_pool(x0, tt, A)[2] for tt in ts])
    return out if out.size > 1 else float(out[0])


def mt_z_spectrum(offsets_hz, *, w1_hz, t_sat, T1a, T2a, T1b, T2b, k_f, k_r, M0a=1.0, M0b=None,
                  read_pool="a"):
    """Mz of the read pool ('a' free, 'b' bound) over its M0 after a continuous-wave pulse of
    nutation ``w1_hz`` and length ``t_sat`` at each offset (Hz) from thermal equilibrium."""
    M0a, M0b = _pools(M0a, M0b, k_f, k_r)
    offsets = np.atleast_1d(np.asarray(offsets_hz, dtype=float))
    idx, norm = (2, M0a) if read_pool == "a" else (5, M0b)
    x0 = np.array([0.0, 0.0, M0a, 0.0, 0.0, M0b, 1.0])
    out = np.empty(offsets.shape)
    for i, off in enumerate(offsets):
        dw = 2.0 * np.pi * off
        A = two_pool_generator(R1a=1.0 / T1a, R2a=1.0 / T2a, R1b=1.0 / T1b, R2b=1.0 / T2b,
                               k_f=k_f, k_r=k_r, M0a=M0a, M0b=M0b, dw_a=dw, dw_b=dw,
                               w1=2.0 * np.pi * float(w1_hz))
        out[i] = evolve_two_pool(x0, t_sat, A)[idx] / norm if norm > 0 else 0.0
    return out if out.size > 1 else float(out[0])
