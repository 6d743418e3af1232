"""Magnetic-susceptibility off-resonance fields dBz(r) (tesla) for the vector-Bloch walk and the
Bloch replay (susceptibility.py of dmipy-sim).

Providers, each with ``delta_bz_fn()`` returning a host callable r (..., 3) -> dBz (...), and
evaluated on the device by the Bloch walk (``simulate_bloch(susceptibility=...)``: the walker
precesses by gamma dBz(r) dt per sample at its position after the sample):

* ``SusceptibilitySources``: uniformly magnetised spheres (Schenck 1996), outside each
  (dchi B0 / 3) a^3 (3 cos^2 theta - 1) / r^3 with B0 along z, the distance clamped to a inside;
* ``MyelinSusceptibility``: hollow cylinders of anisotropic susceptibility (Wharton & Bowtell
  2012), closed form per axon summed over periodic images;
* ``GridSusceptibility``: any field solved on a grid (``dipole_field``: the Lorentz-corrected
  k-space dipole model of a chi-tensor grid), sampled trilinearly.
"""
from dataclasses import dataclass

import numpy as np

from .constants import GAMMA  # noqa: F401

__all__ = ["SusceptibilitySources", "MyelinSusceptibility", "GridSusceptibility",
           "myelin_susceptibility_tensor", "dipole_field", "radial_from_sdf", "sample_grid"]

# symmetric tensor components, in this order
_SYM6 = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


@dataclass
class SusceptibilitySources:
    """Magnetised-sphere perturbers: centres (P, 3) m, radii (P,) m, delta_chi (SI, scalar or
    per sphere), B0 tesla along +z (susceptibility.py:41-95)."""
    centers: np.ndarray
    radii: np.ndarray
    delta_chi: "float | np.ndarray" = 1e-6
    B0: float = 3.0

    def __post_init__(self):
        self.centers = np.asarray(self.centers, dtype=np.float64).reshape(-1, 3)
        self.radii = np.asarray(self.radii, dtype=np.float64).reshape(-1)
        if self.centers.shape[0] != self.radii.shape[0]:
            raise ValueError("centers and radii must have the same length")
        self.delta_chi = np.broadcast_to(np.asarray(self.delta_chi, np.float64),
                                          self.radii.shape).copy()
        if not np.all(self.radii > 0):
            raise ValueError("radii must be positive")

    @property
    def n_perturbers(self):
        return int(self.radii.shape[0])

    def _table(self):
        """(P, 5) float32 rows (cx, cy, cz, (dchi B0 / 3) a^3, a^2)."""
        t = np.empty((self.n_perturbers, 5), np.float32)
        t[:, :3] = self.centers
        t[:, 3] = (self.delta_chi * self.B0 / 3.0) * self.radii ** 3
        t[:, 4] = self.radii ** 2
        return t

    def delta_bz_fn(self):
        t = self._table()

        def delta_bz(r):
            r = np.asarray(r, np.float32)
            d = r[..., None, :] - t[:, :3]
            q = np.maximum(np.sum(d * d, axis=-1), t[:, 4])
            return np.sum(t[:, 3] * (3.0 * d[..., 2] ** 2 / q - 1.0) / q ** 1.5, axis=-1)

        return delta_bz


def _axis_to_z(axis):
    """The rotation taking the unit vector ``axis`` to +z."""
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    v = np.cross(a, [0.0, 0.0, 1.0])
    s, c = np.linalg.norm(v), float(a[2])
    if s < 1e-12:
        return np.eye(3) if c > 0 else np.diag([1.0, -1.0, -1.0])
    vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + vx + vx @ vx * ((1 - c) / (s * s))


@dataclass
class MyelinSusceptibility:
    """Hollow cylinders along z (inner radii a, outer b, centres (N, 2) in a periodic cell of
    side L), anisotropic susceptibility delta_chi_a in B0, fibre-to-B0 angle theta and B0
    azimuth alpha (susceptibility.py:98-205).  Per axon and image, with (dx, dy) from its centre
    and r^2 = dx^2 + dy^2: outside (r > b) Phi_C += (b^2 - a^2)(dx^2 - dy^2)/r^4 and Phi_S +=
    (b^2 - a^2) 2 dx dy / r^4; in the sheath the same with (r^4 - a^4)/(r^4 (b^2 + a^2)) and
    Phi_0 += ln(b/r); in the lumen Phi_0 += ln(b/a).  dBz = dchi_a B0 sin^2(theta)/2 (Phi_0 +
    cos 2alpha Phi_C + sin 2alpha Phi_S).  ``R`` optionally rotates lab positions into the
    fibre frame; positions wrap into the cell when ``periodic``."""
    centers: np.ndarray
    inner_radii: np.ndarray
    outer_radii: np.ndarray
    L: float
    delta_chi_a: float = -0.1e-6
    B0: float = 3.0
    theta: float = 0.0
    alpha: float = 0.0
    R: np.ndarray = None
    n_images: int = 2
    periodic: bool = True

    def __post_init__(self):
        self.centers = np.asarray(self.centers, dtype=np.float64).reshape(-1, 2)
        self.inner_radii = np.asarray(self.inner_radii, dtype=np.float64).reshape(-1)
        self.outer_radii = np.asarray(self.outer_radii, dtype=np.float64).reshape(-1)
        if not (self.centers.shape[0] == self.inner_radii.shape[0] == self.outer_radii.shape[0]):
            raise ValueError("centers, inner_radii, outer_radii must have the same length")
        if not np.all(self.outer_radii > self.inner_radii):
            raise ValueError("outer_radii must exceed inner_radii")

    @property
    def n_perturbers(self):
        return int(self.inner_radii.shape[0])

    @classmethod
    def from_geometry(cls, geom, delta_chi_a=-0.1e-6, B0=3.0, b0_dir=(0., 0., 1.), n_images=2):
        """From a packed myelinated-cylinder geometry and the lab B0 direction."""
        N = int(getattr(geom, 'N_actual', len(geom._inner_radii_np)))
        axis = np.asarray(getattr(geom, 'orientation', (0., 0., 1.)), float)
        axis = axis / np.linalg.norm(axis)
        b0 = np.asarray(b0_dir, float)
        b0 = b0 / np.linalg.norm(b0)
        theta = float(np.arccos(np.clip(abs(np.dot(axis, b0)), 0.0, 1.0)))
        bp = _axis_to_z(axis) @ b0
        return cls(centers=np.asarray(geom._centers_np)[:N],
                   inner_radii=np.asarray(geom._inner_radii_np)[:N],
                   outer_radii=np.asarray(geom._outer_radii_np)[:N], L=float(geom._L_float),
                   delta_chi_a=delta_chi_a, B0=B0, theta=theta,
                   alpha=float(np.arctan2(bp[1], bp[0])), R=None, n_images=n_images)

    def _table(self):
        """(N, 8) float32 rows (cx, cy, a^2, b^2, a^4, ln(b/a), 0, 0) and the scalars
        (L, scale, cos 2alpha, sin 2alpha)."""
        t = np.zeros((self.n_perturbers, 8), np.float32)
        t[:, :2] = self.centers
        t[:, 2] = self.inner_radii ** 2
        t[:, 3] = self.outer_radii ** 2
        t[:, 4] = self.inner_radii ** 4
        t[:, 5] = np.log(self.outer_radii / self.inner_radii)
        scale = np.float32(self.delta_chi_a * self.B0) * np.float32(np.sin(self.theta) ** 2 * 0.5)
        return t, (np.float32(self.L), scale, np.float32(np.cos(2 * self.alpha)),
                   np.float32(np.sin(2 * self.alpha)))

    def delta_bz_fn(self):
        t, (L, scale, c2a, s2a) = self._table()
        ims = np.arange(-self.n_images, self.n_images + 1, dtype=np.float32) * L
        ox, oy = [v.ravel() for v in np.meshgrid(ims, ims)]
        R = None if self.R is None else np.asarray(self.R, np.float32)
        wrap = bool(self.periodic)

        def delta_bz(r):
            r = np.asarray(r, np.float32)
            if R is not None:
                r = r @ R.T
            x, y = r[..., 0], r[..., 1]
            if wrap:
                x = np.mod(x + 0.5 * L, L) - 0.5 * L
                y = np.mod(y + 0.5 * L, L) - 0.5 * L
            dx = x[..., None, None] - (t[:, 0, None] + ox)
            dy = y[..., None, None] - (t[:, 1, None] + oy)
            a2, b2, a4, lba = (t[:, k, None] for k in (2, 3, 4, 5))
            r2 = dx * dx + dy * dy
            r4 = r2 * r2
            out = r2 > b2
            sheath = (r2 > a2) & ~out
            lumen = r2 < a2
            with np.errstate(divide="ignore", invalid="ignore"):
                f = np.where(out, (b2 - a2) / np.where(out, r4, 1.0), 0.0)
                f = f + np.where(sheath, (r4 - a4) / (np.where(sheath, r4, 1.0) * (b2 + a2)), 0.0)
                phi0 = np.where(sheath, -0.5 * np.log(np.where(sheath, r2, 1.0) / b2), 0.0)
            phi0 = phi0 + np.where(lumen, lba, 0.0)
            pc = np.sum(f * (dx * dx - dy * dy), axis=(-2, -1))
            ps = np.sum(f * 2.0 * dx * dy, axis=(-2, -1))
            return scale * np.sum(phi0, axis=(-2, -1)) + scale * (c2a * pc + s2a * ps)

        return delta_bz


def _voxel(voxel_size, ndim=3):
    vs = np.atleast_1d(np.asarray(voxel_size, float))
    if vs.size == 1:
        vs = np.repeat(vs, ndim)
    if vs.size != ndim:
        raise ValueError(f"voxel_size must be a scalar or length-{ndim}, got {vs}")
    return vs


def _unit(v, axis=-1, eps=1e-30):
    v = np.asarray(v, float)
    return v / np.maximum(np.linalg.norm(v, axis=axis, keepdims=True), eps)


def myelin_susceptibility_tensor(myelin_mask, radial_dir, chi_iso=0.0, chi_aniso=0.0):
    """Per voxel chi = mask (chi_iso I + chi_aniso (n n^T - I/3)), n the unit radial
    direction; (Nx, Ny, Nz, 6) in the order xx, yy, zz, xy, xz, yz."""
    m = np.asarray(myelin_mask, float)
    n = _unit(radial_dir, axis=-1)
    chi6 = np.zeros(m.shape + (6,))
    for c, (i, j) in enumerate(_SYM6):
        term = 0.0
        if chi_aniso != 0.0:
            term = term + chi_aniso * (n[..., i] * n[..., j] - (1.0 / 3.0 if i == j else 0.0))
        if chi_iso != 0.0 and i == j:
            term = term + chi_iso
        chi6[..., c] = m * term
    return chi6


def dipole_field(chi6, voxel_size, b0_dir, B0=1.0):
    """dBz (T) of a chi-tensor grid by the Lorentz-corrected k-space dipole model:
    dB(k)/B0 = H.chi(k).H / 3 - (H.k)(k.chi(k).H) with k the unit wave vector and the k = 0
    term zeroed; H the unit B0 direction in the grid frame (susceptibility.py:254-286)."""
    chi6 = np.asarray(chi6, float)
    shape = chi6.shape[:3]
    H = _unit(np.asarray(b0_dir, float).ravel())
    vs = _voxel(voxel_size, 3)
    K = np.meshgrid(*[2.0 * np.pi * np.fft.fftfreq(n, d=d) for n, d in zip(shape, vs)],
                    indexing="ij")
    k2 = sum(k ** 2 for k in K)
    dc = k2 == 0.0
    inv = np.where(dc, 0.0, 1.0 / np.sqrt(np.where(dc, 1.0, k2)))
    kh = [k * inv for k in K]
    ck = [np.fft.fftn(chi6[..., c]) for c in range(6)]
    comp = {}
    for c, (i, j) in enumerate(_SYM6):
        comp[(i, j)] = comp[(j, i)] = ck[c]
    chiH = [sum(comp[(i, j)] * H[j] for j in range(3)) for i in range(3)]
    HchiH = sum(H[i] * chiH[i] for i in range(3))
    kchiH = sum(kh[i] * chiH[i] for i in range(3))
    Hk = sum(H[i] * kh[i] for i in range(3))
    kern = (1.0 / 3.0) * HchiH - Hk * kchiH
    kern[dc] = 0.0
    return np.real(np.fft.ifftn(kern)) * float(B0)


def radial_from_sdf(sdf, voxel_size):
    """grad(sdf) / |grad(sdf)|, the local membrane normal."""
    vs = _voxel(voxel_size, 3)
    return _unit(np.stack(np.gradient(np.asarray(sdf, float), *vs, edge_order=2), axis=-1))


def _trilinear(grid, idx, periodic):
    """Order-1 interpolation at fractional voxel indices idx (M, 3): wrapped per axis when
    periodic, else edge values beyond the grid."""
    shape = np.asarray(grid.shape)
    i0 = np.floor(idx).astype(np.int64)
    f = idx - i0
    out = np.zeros(idx.shape[0])
    for corner in range(8):
        w = np.ones(idx.shape[0])
        ii = []
        for a in range(3):
            bit = (corner >> a) & 1
            j = i0[:, a] + bit
            w = w * (f[:, a] if bit else 1.0 - f[:, a])
            j = np.mod(j, shape[a]) if periodic[a] else np.clip(j, 0, shape[a] - 1)
            ii.append(j)
        out += w * grid[ii[0], ii[1], ii[2]]
    return out


def sample_grid(grid, positions, origin, voxel_size, periodic=False, order=1):
    """Trilinear sample of a field grid at positions (..., 3); voxel (0, 0, 0) has its corner at
    ``origin`` (centre at origin + voxel/2)."""
    if order != 1:
        raise NotImplementedError("only trilinear (order 1) sampling")
    pos = np.asarray(positions, float)
    lead = pos.shape[:-1]
    vs = _voxel(voxel_size, 3)
    idx = (pos.reshape(-1, 3) - np.asarray(origin, float).ravel()) / vs - 0.5
    per = (periodic,) * 3 if isinstance(periodic, bool) else tuple(periodic)
    for a in range(3):
        if per[a]:
            idx[:, a] = np.mod(idx[:, a], grid.shape[a])
    return _trilinear(np.asarray(grid, float), idx, per).reshape(lead)


@dataclass
class GridSusceptibility:
    """A solved field grid dB (Nx, Ny, Nz) T with the corner of voxel (0, 0, 0) at ``origin``,
    sampled trilinearly (periodic or edge-clamped) (susceptibility.py:320-365)."""
    dB: np.ndarray
    origin: np.ndarray
    voxel_size: "float | np.ndarray"
    periodic: bool = False

    @classmethod
    def from_source(cls, mask, radial_dir, voxel_size, origin, b0_dir, B0, chi_iso=0.0,
                    chi_aniso=0.0, periodic=False):
        chi6 = myelin_susceptibility_tensor(mask, radial_dir, chi_iso, chi_aniso)
        return cls(dB=dipole_field(chi6, voxel_size, b0_dir, B0),
                   origin=np.asarray(origin, float), voxel_size=voxel_size,
                   periodic=bool(periodic))

    def delta_bz_fn(self):
        grid = np.asarray(self.dB, np.float32).astype(np.float64)
        org = np.asarray(self.origin, np.float32).ravel().astype(np.float64)
        vs = _voxel(self.voxel_size, 3).astype(np.float32).astype(np.float64)
        per = (bool(self.periodic),) * 3

        def delta_bz(r):
            r = np.asarray(r, np.float64)
            lead = r.shape[:-1]
            idx = (r.reshape(-1, 3) - org) / vs - 0.5
            if per[0]:
                idx = np.mod(idx, np.asarray(grid.shape, float))
            return _trilinear(grid, idx, per).reshape(lead)

        return delta_bz
