"""Substrate geometries: host-side objects that describe the walls and build the device descriptor.

Same constructors, attribute names and conventions as dmipy-sim's geometries.py (FreeDiffusion
34-45, Sphere 143-424, Cylinder 427-844, pack_cylinders 1502-1601, PackedCylinders 1604-2242,
pack_spheres 2249-2340, PackedSpheres 2343-2786, _rotation_to_z 1466-1495).  The per-walker
``reflect`` / ``reflect_with_log_weight`` / ``permeate`` plug-ins of the reference are not Python
functions here: each geometry compiles to a POD ``dmsim_geometry`` descriptor (include/dmsim.h)
consumed by the CUDA step functions, and packed substrates additionally get a uniform cell list
(every object within reach of each cell, pre-shifted to its periodic image) on the device.
"""
import itertools

import numpy as np
import torch

from . import _lib

__all__ = ["Geometry", "FreeDiffusion", "Cylinder", "Sphere", "MyelinatedCylinder",
           "PackedMyelinatedCylinders", "pack_myelinated_cylinders", "Box1D", "PermeableSlab1D",
           "PermeableShell", "Ellipsoid",
           "pack_cylinders", "PackedCylinders", "pack_spheres", "PackedSpheres",
           "lattice_cylinders"]


def _rotation_to_z(v):
    """Rotation matrix R with R @ v = [0, 0, 1] (Rodrigues; geometries.py:1466-1495)."""
    v = np.asarray(v, dtype=np.float64)
    v = v / np.linalg.norm(v)
    k = np.array([0.0, 0.0, 1.0])
    dot = float(np.dot(v, k))
    if abs(dot - 1.0) < 1e-10:
        return np.eye(3)
    if abs(dot + 1.0) < 1e-10:
        return np.diag([1.0, -1.0, -1.0])
    axis = np.cross(v, k)
    axis = axis / np.linalg.norm(axis)
    ang = np.arccos(np.clip(dot, -1.0, 1.0))
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * (K @ K)


class Geometry:
    """Base class.  Subclasses provide ``_desc(...)`` (the device descriptor) and ``_frame()``
    (the lab -> walk-frame rotation, or None when the walk runs in the lab frame)."""

    surface_relaxivity_t2 = None
    permeability = None

    def _frame(self):
        return None

    def _wall_mode(self, with_weight_channel):
        if self.permeability is not None:
            return _lib.WALL_PERMEATE
        if with_weight_channel:
            return _lib.WALL_RELAX
        return _lib.WALL_REFLECT

    def _base_desc(self, kind, wall_mode, rho_over_D, kappa_over_D):
        g = _lib.Geometry()
        g.kind = kind
        g.wall_mode = wall_mode
        g.rho_over_D = float(rho_over_D)
        g.kappa_over_D = float(kappa_over_D)
        return g


class FreeDiffusion(Geometry):
    """Unbounded free diffusion; walkers start at the origin (geometries.py:34-45)."""

    def classify_position(self, r):
        return np.zeros(np.shape(r)[:-1], dtype=np.int32)

    def init_positions(self, n_walkers, key=None):
        return np.zeros((n_walkers, 3), dtype=np.float32)

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        return self._base_desc(_lib.GEOM_FREE, _lib.WALL_REFLECT, 0.0, 0.0), ()


def _opt_float(v):
    return float(v) if v is not None else None


def _host_rng(key):
    return np.random.default_rng(None if key is None else int(np.asarray(key).ravel()[-1]))


class Sphere(Geometry):
    """Reflecting (optionally relaxing / permeable) sphere of radius R at the origin
    (geometries.py:143-424).  Exchange time R/(3 kappa); surface T2 = R/(3 rho)."""

    def __init__(self, radius, surface_relaxivity_t2=None, permeability=None):
        self.radius = float(radius)
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)
        self.permeability = _opt_float(permeability)

    def volume(self):
        return (4.0 / 3.0) * np.pi * self.radius ** 3

    def surface_area(self):
        return 4.0 * np.pi * self.radius ** 2

    def classify_position(self, r):
        r = np.asarray(r, dtype=np.float32)
        return np.where(np.sum(r * r, axis=-1) < np.float32(self.radius) ** 2, 0, 1).astype(np.int32)

    def init_positions(self, n_walkers, key=None):
        """Uniform inside the sphere (host rejection sampling, geometries.py:186-195)."""
        rng = _host_rng(key)
        out = []
        while sum(len(a) for a in out) < n_walkers:
            p = rng.uniform(-self.radius, self.radius, (n_walkers * 4, 3))
            out.append(p[np.linalg.norm(p, axis=1) < self.radius])
        return np.concatenate(out)[:n_walkers].astype(np.float32)

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        g = self._base_desc(_lib.GEOM_SPHERE, wall_mode, rho_over_D, kappa_over_D)
        g.radius = self.radius
        g.eps_detect = np.float32(1e-7 * self.radius)
        g.nudge = np.float32(1e-4 * self.radius)
        return g, ()


class Cylinder(Geometry):
    """Infinite cylinder of radius R along ``orientation`` (geometries.py:427-844).

    The walk runs in the cylinder frame (``_R @ orientation = z``); gradients are rotated into it
    and positions out of it by the engine.
    """

    def __init__(self, radius, orientation, surface_relaxivity_t2=None, permeability=None):
        self.radius = float(radius)
        o = np.asarray(orientation, dtype=np.float64)
        self.orientation = (o / np.linalg.norm(o)).astype(np.float32)
        R = _rotation_to_z(self.orientation)
        self._R = R.astype(np.float32)
        self._R_inv = R.T.astype(np.float32)
        self._is_identity_rotation = bool(np.allclose(R, np.eye(3)))
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)
        self.permeability = _opt_float(permeability)

    def _frame(self):
        return None if self._is_identity_rotation else self._R.astype(np.float64)

    def classify_position(self, r):
        r = np.asarray(r, dtype=np.float32)
        rc = r if self._is_identity_rotation else r @ self._R.T
        return np.where(np.sum(rc[..., :2] ** 2, axis=-1) < np.float32(self.radius) ** 2,
                        0, 1).astype(np.int32)

    def init_positions(self, n_walkers, key=None):
        """Uniform in the cross-section, z = 0 in the cylinder frame (geometries.py:477-491)."""
        rng = _host_rng(key)
        out = []
        while sum(len(a) for a in out) < n_walkers:
            xy = rng.uniform(-self.radius, self.radius, (n_walkers * 2, 2))
            out.append(xy[np.linalg.norm(xy, axis=1) < self.radius])
        xy = np.concatenate(out)[:n_walkers].astype(np.float32)
        rc = np.concatenate([xy, np.zeros((n_walkers, 1), np.float32)], axis=1)
        return (rc @ self._R).astype(np.float32)

    def volume(self, L=1.0):
        return np.pi * self.radius ** 2 * float(L)

    def surface_area(self, L=1.0, include_caps=False):
        a = 2.0 * np.pi * self.radius * float(L)
        if include_caps:
            a += 2.0 * np.pi * self.radius ** 2
        return a

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        g = self._base_desc(_lib.GEOM_CYLINDER, wall_mode, rho_over_D, kappa_over_D)
        g.radius = self.radius
        g.eps_detect = np.float32(1e-7 * self.radius)
        g.nudge = np.float32(1e-4 * self.radius)
        return g, ()


class Ellipsoid(Geometry):
    """Reflecting (optionally relaxing / permeable) axis-aligned ellipsoid with semi-axes
    (a, b, c) along (x, y, z) at the origin (geometries.py:1137-1427); a = b = c = R is the
    sphere."""

    def __init__(self, semiaxes, surface_relaxivity_t2=None, permeability=None):
        self.semiaxes = np.asarray(semiaxes, dtype=np.float64)
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)
        self.permeability = _opt_float(permeability)

    def _inv2(self):
        s = self.semiaxes.astype(np.float32)
        return np.float32(1.0) / (s * s)

    def init_positions(self, n_walkers, key=None):
        """Uniform in the unit ball scaled by the semi-axes (geometries.py:1167-1182)."""
        rng = _host_rng(key)
        out = []
        while sum(len(a) for a in out) < n_walkers:
            p = rng.uniform(-1.0, 1.0, (n_walkers * 4, 3))
            out.append(p[np.linalg.norm(p, axis=1) < 1.0])
        return (np.concatenate(out)[:n_walkers] * self.semiaxes).astype(np.float32)

    def classify_position(self, r):
        r = np.asarray(r, dtype=np.float32)
        return np.where(np.sum(r * self._inv2() * r, axis=-1) < np.float32(1.0), 0,
                        1).astype(np.int32)

    def volume(self):
        a, b, c = self.semiaxes
        return (4.0 / 3.0) * np.pi * a * b * c

    def surface_area(self):
        """Thomsen's approximation (p = 1.6075, relative error < 1.061 %)."""
        p = 1.6075
        a, b, c = self.semiaxes ** p
        return 4.0 * np.pi * ((a * b + a * c + b * c) / 3.0) ** (1.0 / p)

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        g = self._base_desc(_lib.GEOM_ELLIPSOID, wall_mode, rho_over_D, kappa_over_D)
        m = float(np.min(self.semiaxes))
        g.radius = m
        g.eps_detect = np.float32(1e-7 * m)
        g.nudge = np.float32(1e-4 * m)
        g.ell_inv2[:] = [float(v) for v in self._inv2()]
        return g, ()


class Box1D(Geometry):
    """1-D reflecting slab, walls at x = 0 and x = length, free along y and z
    (geometries.py:48-140); surface relaxivity weights each wall overshoot."""

    def __init__(self, length, surface_relaxivity_t2=None):
        self.length = float(length)
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)

    def volume(self):
        return self.length

    def surface_area(self):
        return 2.0

    def classify_position(self, r):
        return np.zeros(np.shape(r)[:-1], dtype=np.int32)

    def init_positions(self, n_walkers, key=None):
        x = _host_rng(key).uniform(0.0, self.length, n_walkers)
        return np.stack([x, np.zeros(n_walkers), np.zeros(n_walkers)], 1).astype(np.float32)

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        g = self._base_desc(_lib.GEOM_BOX1D, wall_mode, rho_over_D, 0.0)
        g.L = np.float32(self.length)
        return g, ()


class PermeableSlab1D(Geometry):
    """Closed two-compartment slab: a permeable membrane at x = length/2 between reflecting
    walls at 0 and length (geometries.py:3221-3300); every walker starts in compartment A
    (x < length/2), so f_A(t) = 1/2 + 1/2 exp(-4 kappa t / length)."""

    def __init__(self, length, permeability, surface_relaxivity_t2=None):
        self.length = float(length)
        self.permeability = float(permeability)
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)
        self.radius = float(length) / 2.0

    def volume(self):
        return self.length / 2.0

    def surface_area(self):
        return 1.0

    def classify_position(self, r):
        r = np.asarray(r, dtype=np.float32)
        return np.where(r[..., 0] < np.float32(self.length / 2.0), 0, 1).astype(np.int32)

    def init_positions(self, n_walkers, key=None):
        x = _host_rng(key).uniform(0.0, self.length / 2.0, n_walkers)
        return np.stack([x, np.zeros(n_walkers), np.zeros(n_walkers)], 1).astype(np.float32)

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        g = self._base_desc(_lib.GEOM_SLAB, wall_mode, rho_over_D, kappa_over_D)
        g.L = np.float32(self.length)
        g.radius = np.float32(self.length / 2.0)
        return g, ()


class PermeableShell(Geometry):
    """Closed radial two-compartment shell: a permeable membrane at r = r_inner inside a
    reflecting wall at r = r_outer (geometries.py:3303-3431); ``kind='sphere'`` measures r from the
    origin, ``'cylinder'`` from the axis along ``orientation`` (walked in the axis frame)."""

    def __init__(self, r_inner, r_outer, permeability, kind="sphere", orientation=(0.0, 0.0, 1.0),
                 surface_relaxivity_t2=None):
        if kind not in ("sphere", "cylinder"):
            raise ValueError("kind must be 'sphere' or 'cylinder'")
        self.r_inner, self.r_outer = float(r_inner), float(r_outer)
        self.permeability = float(permeability)
        self.kind = kind
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)
        self.radius = float(r_inner)
        o = np.asarray(orientation, dtype=np.float64)
        self._o = o / np.linalg.norm(o)
        R = _rotation_to_z(self._o)
        self._R = R.astype(np.float32)
        self._is_identity_rotation = kind == "sphere" or bool(np.allclose(R, np.eye(3)))

    def _frame(self):
        return None if self._is_identity_rotation else self._R.astype(np.float64)

    def _radial(self, r):
        r = np.asarray(r, dtype=np.float64)
        if self.kind == "sphere":
            return r
        return r - (r @ self._o)[..., None] * self._o

    def volume(self):
        if self.kind == "sphere":
            return (4.0 / 3.0) * np.pi * self.r_inner ** 3
        return np.pi * self.r_inner ** 2

    def surface_area(self):
        if self.kind == "sphere":
            return 4.0 * np.pi * self.r_inner ** 2
        return 2.0 * np.pi * self.r_inner

    def classify_position(self, r):
        rad = np.linalg.norm(self._radial(r), axis=-1)
        return np.where(rad < self.r_inner, 0, 1).astype(np.int32)

    def init_positions(self, n_walkers, key=None):
        """Uniform in compartment A; a cylindrical shell spreads the axial coordinate over
        [0, r_inner) (geometries.py:3343-3358)."""
        rng = _host_rng(key)
        v = rng.normal(size=(n_walkers, 3))
        if self.kind == "cylinder":
            v -= (v @ self._o)[:, None] * self._o
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        dim = 3.0 if self.kind == "sphere" else 2.0
        pos = v * (rng.uniform(size=n_walkers) ** (1.0 / dim) * self.r_inner)[:, None]
        if self.kind == "cylinder":
            pos += (rng.uniform(size=n_walkers) * self.r_inner)[:, None] * self._o
        return pos.astype(np.float32)

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        g = self._base_desc(_lib.GEOM_SHELL, wall_mode, rho_over_D, kappa_over_D)
        g.radius = self.r_inner
        g.shell_r_out = self.r_outer
        g.shell_cyl = 1 if self.kind == "cylinder" else 0
        g.eps_detect = np.float32(1e-7 * self.r_inner)
        g.nudge = np.float32(1e-4 * self.r_inner)
        return g, ()


# water per unit myelin volume, the default proton density of the myelin compartment
# (substrate/biophysical_constants.py: myelin_water_proton_density)
MYELIN_WATER_PROTON_DENSITY = 0.40


class MyelinatedCylinder(Geometry):
    """Three-compartment myelinated cylinder along ``orientation`` (geometries.py:847-1134): intra-
    axonal (r < inner_radius), myelin sheath (inner_radius <= r < outer_radius) and extra-axonal
    space, each with its own isotropic diffusivity, optional T2, and water proton density
    (``water_fractions``, the signal weight of a walker by its starting compartment); the two walls
    have independent permeabilities.  Walked by its own step rule (physics.py:420-680): one step
    per waveform sample of the compartment's length, mirror reflection at a wall unless a Powles
    draw lets the walker through, then a clamp onto its compartment's side.
    """

    _is_myelinated = True

    def __init__(self, inner_radius, outer_radius, orientation, D_intra, D_extra, D_myelin=0.0,
                 kappa_inner=None, kappa_outer=None, T2_intra=None, T2_myelin=None,
                 T2_extra=None, water_fractions=None):
        if outer_radius <= inner_radius:
            raise ValueError("outer_radius must be > inner_radius")
        self.inner_radius = float(inner_radius)
        self.outer_radius = float(outer_radius)
        self.radius = self.inner_radius
        self.D_intra, self.D_myelin, self.D_extra = float(D_intra), float(D_myelin), float(D_extra)
        self.kappa_inner = _opt_float(kappa_inner)
        self.kappa_outer = _opt_float(kappa_outer)
        self.T2_intra = _opt_float(T2_intra)
        self.T2_myelin = _opt_float(T2_myelin)
        self.T2_extra = _opt_float(T2_extra)
        if water_fractions is None:
            water_fractions = (1.0, MYELIN_WATER_PROTON_DENSITY, 1.0)
        self.water_fractions = tuple(float(w) for w in water_fractions)
        o = np.asarray(orientation, dtype=np.float64)
        self.orientation = (o / np.linalg.norm(o)).astype(np.float32)
        R = _rotation_to_z(self.orientation)
        self._R = R.astype(np.float32)
        self._R_inv = R.T.astype(np.float32)
        self._is_identity_rotation = bool(np.allclose(R, np.eye(3)))
        self._init_compartments = None

    def _frame(self):
        return None if self._is_identity_rotation else self._R.astype(np.float64)

    def _wall_mode(self, with_weight_channel=False):
        permeable = self.kappa_inner is not None or self.kappa_outer is not None
        return _lib.WALL_PERMEATE if permeable else _lib.WALL_REFLECT

    # ---- compartments -------------------------------------------------------------------------
    def _areas(self):
        ri, ro = self.inner_radius, self.outer_radius
        return np.pi * ri ** 2, np.pi * (ro ** 2 - ri ** 2), np.pi * ((2 * ro) ** 2 - ro ** 2)

    def seed_counts(self, n_walkers):
        """Walkers seeded per compartment, proportional to the compartment areas with the
        extra-axonal space taken out to 2 outer_radius (geometries.py:935-952)."""
        a = self._areas()
        tot = sum(a)
        n0 = int(round(n_walkers * a[0] / tot))
        n1 = int(round(n_walkers * a[1] / tot))
        return n0, n1, n_walkers - n0 - n1

    def classify_position(self, r):
        """0 intra-axonal, 1 myelin, 2 extra-axonal by the squared distance from the axis
        (geometries.py:1018-1029)."""
        r = np.asarray(r, dtype=np.float32)
        rc = r if self._is_identity_rotation else r @ self._R.T
        q = np.sum(rc[..., :2] ** 2, axis=-1)
        ri2, ro2 = np.float32(self.inner_radius) ** 2, np.float32(self.outer_radius) ** 2
        return np.where(q < ri2, 0, np.where(q < ro2, 1, 2)).astype(np.int32)

    def init_positions(self, n_walkers, key=None):
        """Host sampler: the compartment counts of :meth:`seed_counts`, uniform in the disc and the
        annuli (geometries.py:928-1006); sets ``_init_compartments``."""
        rng = _host_rng(key)
        counts = self.seed_counts(n_walkers)
        bounds = ((0.0, self.inner_radius), (self.inner_radius, self.outer_radius),
                  (self.outer_radius, 2.0 * self.outer_radius))
        pos, comp = [], []
        for c, (n, (lo, hi)) in enumerate(zip(counts, bounds)):
            got = np.zeros((0, 2))
            while len(got) < n:
                xy = rng.uniform(-hi, hi, (n * 3 + 8, 2))
                rr = np.linalg.norm(xy, axis=1)
                got = np.concatenate([got, xy[(rr >= lo) & (rr < hi)]])
            pos.append(got[:n])
            comp.append(np.full(n, c, np.int32))
        xy = np.concatenate(pos).astype(np.float32)
        rc = np.concatenate([xy, np.zeros((n_walkers, 1), np.float32)], axis=1)
        self._init_compartments = np.concatenate(comp)
        return (rc @ self._R).astype(np.float32)

    def spin_weight_sum(self, n_walkers, r0=None):
        """Sum over the walkers of their compartment's water proton density: the normaliser of
        the signal sum (core.py:426-427)."""
        wf = np.asarray(self.water_fractions, np.float64)
        if r0 is not None:
            return float(np.sum(wf[self.classify_position(r0)]))
        return float(np.dot(self.seed_counts(n_walkers), wf))

    def volume(self, compartment, L=1.0):
        a = dict(zip(("intra", "myelin", "extra"), self._areas()))
        if compartment not in a:
            raise ValueError(f"compartment must be 'intra', 'myelin', or 'extra'; got {compartment!r}")
        return a[compartment] * float(L)

    def surface_area(self, compartment, L=1.0):
        ri, ro = self.inner_radius, self.outer_radius
        a = {"intra": ri, "myelin": ri + ro, "extra": ro}
        if compartment not in a:
            raise ValueError(f"compartment must be 'intra', 'myelin', or 'extra'; got {compartment!r}")
        return 2.0 * np.pi * a[compartment] * float(L)

    def volume_fraction(self, compartment):
        return self.volume(compartment) / (np.pi * (2.0 * self.outer_radius) ** 2)

    # ---- device descriptor --------------------------------------------------------------------
    def _myelin_desc(self, dt, n_total):
        """Descriptor of a walk with time step ``dt`` over ``n_total`` walkers (global indices):
        per-compartment step lengths sqrt(6 D dt), kappa/D of the compartment left, dt/T2, log
        spin weights and the seeding ranges, in the reference's float32 arithmetic
        (physics.py:451-503)."""
        g = self._base_desc(_lib.GEOM_MYELIN, self._wall_mode(), 1.0, 0.0)
        g.radius = self.inner_radius
        g.myelin_r_out = self.outer_radius
        g.eps_detect = np.float32(1e-7 * self.inner_radius)
        g.nudge = np.float32(1e-4 * self.inner_radius)
        dt32 = np.float32(dt)
        D = np.array([self.D_intra, self.D_myelin, self.D_extra], np.float32)
        g.myelin_step[:] = [float(np.sqrt(np.float32(6.0) * d * dt32)) for d in D]
        Dl = np.maximum(D, np.float32(1e-30))
        ki = np.float32(self.kappa_inner or 0.0)
        ko = np.float32(self.kappa_outer or 0.0)
        g.myelin_kin_over_D[:] = [float(ki / d) for d in Dl]
        g.myelin_kout_over_D[:] = [float(ko / d) for d in Dl]
        T2 = (self.T2_intra, self.T2_myelin, self.T2_extra)
        if any(t is not None for t in T2):
            g.myelin_t2dec[:] = [float(dt32 / np.float32(t if t is not None else 1e6)) for t in T2]
        with np.errstate(divide="ignore"):
            g.myelin_logw0[:] = [float(np.log(np.float32(w))) for w in self.water_fractions]
        n0, n1, _ = self.seed_counts(n_total)
        g.myelin_seed_n[:] = [n0, n0 + n1]
        return g

    def _has_weight(self):
        return (any(t is not None for t in (self.T2_intra, self.T2_myelin, self.T2_extra))
                or any(w != 1.0 for w in self.water_fractions))


def pack_myelinated_cylinders(inner_radii, g_ratios, target_packing, cell_size=None, seed=0,
                              max_attempts=100_000):
    """RSA of myelinated cylinders (outer radius = inner / g-ratio) in a periodic square cell,
    largest first, outer walls not overlapping -- the same draws as geometries.py:2787-2857, so a
    seed gives the same packing.  Returns (inner_radii, g_ratios, centers (N, 2))."""
    inner_radii = np.asarray(inner_radii, dtype=np.float64).ravel()
    N = len(inner_radii)
    g = np.broadcast_to(np.asarray(g_ratios, dtype=np.float64).ravel(), (N,)).copy()
    outer = inner_radii / g
    if cell_size is None:
        if target_packing is None:
            raise ValueError("Provide either cell_size or target_packing.")
        cell_size = float(np.sqrt(np.pi * np.sum(outer ** 2) / target_packing))
    L = float(cell_size)
    rng = np.random.default_rng(int(seed))
    order = np.argsort(outer)[::-1]
    out_s = outer[order]
    cs = np.zeros((N, 2))
    for i, r in enumerate(out_s):
        for _ in range(max_attempts):
            c = rng.uniform(-L / 2.0, L / 2.0, 2)
            dq = c - cs[:i]
            dq -= L * np.round(dq / L)
            if i == 0 or not np.any(np.linalg.norm(dq, axis=1) < r + out_s[:i]):
                cs[i] = c
                break
        else:
            raise RuntimeError(f"RSA failed after {max_attempts} attempts placing cylinder {i}.")
    centers = np.empty_like(cs)
    centers[order] = cs
    return inner_radii, g, centers


class PackedMyelinatedCylinders(Geometry):
    """Myelinated axons in a periodic square cell (geometries.py:2860-3218), three compartments:
    extra-axonal (id 0), intra-axonal of axon k (id 1 + k), myelin of axon k (id N_max + 1 + k).
    Per-axon diffusivities and wall permeabilities, per-compartment T2 (axon 0's values, as the
    reference's step reads them), surface relaxivity at the myelin walls.  Walked by its own step
    rule (physics.py:682-1062): a step of the walker's compartment along a unit direction,
    mirror reflection or Powles transmission at its axon's walls, an extra-axonal walker pushed out
    of whichever sheath it entered, clamps, reclassification; the phase reads the periodic-
    unwrapped position and myelin water carries the myelin proton density as its spin weight.
    """

    _is_packed_myelinated = True

    def __init__(self, inner_radii, g_ratios, centers, cell_size, N_max=128,
                 orientation=(0.0, 0.0, 1.0), D_intra=2e-9, D_myelin=0.0, D_extra=2e-9,
                 T2_intra=None, T2_myelin=None, T2_extra=None, kappa_inner=0.0, kappa_outer=0.0,
                 rho_inner=0.0, rho_outer=0.0):
        inner = np.asarray(inner_radii, dtype=np.float64).ravel()
        N = len(inner)
        g = np.broadcast_to(np.asarray(g_ratios, dtype=np.float64).ravel(), (N,)).copy()
        centers = np.asarray(centers, dtype=np.float64)
        if centers.shape != (N, 2):
            raise ValueError(f"centers shape {centers.shape} must be ({N}, 2)")
        if N_max < N:
            raise ValueError(f"N_max={N_max} < N_actual={N}")
        self.N_actual, self.N_max = N, int(N_max)
        self._cell_size = self._L_float = float(cell_size)
        self._myelin_proton_density = MYELIN_WATER_PROTON_DENSITY

        def bc(x, name, opt=False):
            if x is None:
                if opt:
                    return None
                x = 0.0
            x = np.asarray(x, dtype=np.float64).ravel()
            if x.size == 1:
                return np.full(N, float(x[0]))
            if x.size != N:
                raise ValueError(f"{name} must be scalar or length {N}, got {x.size}")
            return x.copy()

        def pad(a, fill=0.0):
            out = np.full(self.N_max, fill, dtype=np.float64)
            out[:N] = a
            return out
        self._inner_radii_np = pad(inner)
        self._outer_radii_np = pad(inner / g)
        cen = np.zeros((self.N_max, 2))
        cen[:N] = centers
        self._centers_np = cen
        self._D = {k: pad(bc(v, k)) for k, v in (("intra", D_intra), ("myelin", D_myelin),
                                                  ("extra", D_extra))}
        T2 = {k: bc(v, k, opt=True) for k, v in (("intra", T2_intra), ("myelin", T2_myelin),
                                                  ("extra", T2_extra))}
        self._has_t2 = any(v is not None for v in T2.values())
        self._T2 = {k: (pad(v) if v is not None else np.full(self.N_max, 1e6))
                    for k, v in T2.items()}
        self._kappa_inner = pad(bc(kappa_inner, "kappa_inner"))
        self._kappa_outer = pad(bc(kappa_outer, "kappa_outer"))
        self._rho_inner = pad(bc(rho_inner, "rho_inner"))
        self._rho_outer = pad(bc(rho_outer, "rho_outer"))
        o = np.asarray(orientation, dtype=np.float64)
        self.orientation = (o / np.linalg.norm(o)).astype(np.float32)
        R = _rotation_to_z(self.orientation)
        self._R = R.astype(np.float32)
        self._R_inv = R.T.astype(np.float32)
        self._is_identity_rotation = bool(np.allclose(R, np.eye(3)))
        nz = self._inner_radii_np[self._inner_radii_np > 0]
        ref_r = float(np.min(nz)) if len(nz) else 1e-6
        self._eps = np.float32(1e-7 * ref_r)
        self._nudge = np.float32(1e-4 * ref_r)
        self.min_gap = self._compute_min_gap()
        self._init_compartments = None
        self._dev_cache = {}

    def _frame(self):
        return None if self._is_identity_rotation else self._R.astype(np.float64)

    def _wall_mode(self, with_weight_channel=False):
        permeable = np.any(self._kappa_inner > 0) or np.any(self._kappa_outer > 0)
        return _lib.WALL_PERMEATE if permeable else _lib.WALL_REFLECT

    def _compute_min_gap(self):
        N, L = self.N_actual, self._L_float
        c, o = self._centers_np[:N], self._outer_radii_np[:N]
        gap = float("inf")
        for i in range(N):
            dq = c[i] - c[i + 1:]
            dq -= L * np.round(dq / L)
            if len(dq):
                gap = min(gap, float(np.min(np.linalg.norm(dq, axis=1) - o[i] - o[i + 1:])))
            gap = min(gap, L - 2.0 * o[i])
        return gap

    def volume_fraction(self, compartment):
        L, N = self._L_float, self.N_actual
        i, o = self._inner_radii_np[:N], self._outer_radii_np[:N]
        if compartment == "intra":
            return float(np.pi * np.sum(i ** 2) / L ** 2)
        if compartment == "myelin":
            return float(np.pi * np.sum(o ** 2 - i ** 2) / L ** 2)
        if compartment == "extra":
            return float((L ** 2 - np.pi * np.sum(o ** 2)) / L ** 2)
        raise ValueError(f"compartment must be 'intra', 'myelin', or 'extra'; got {compartment!r}")

    # ---- seeding ------------------------------------------------------------------------------
    def seed_counts(self, n_walkers):
        """(n_intra (N,), n_myelin (N,), n_extra): area-proportional counts, extra-axonal space
        taking the remainder, intra counts trimmed in order when rounding overshoots
        (geometries.py:3100-3125)."""
        L, N = self._L_float, self.N_actual
        i, o = self._inner_radii_np[:N], self._outer_radii_np[:N]
        a_in, a_my = np.pi * i ** 2, np.pi * (o ** 2 - i ** 2)
        a_ex = L * L - np.pi * np.sum(o ** 2)
        tot = a_ex + np.sum(a_in) + np.sum(a_my)
        n_in = np.array([int(round(n_walkers * a / tot)) for a in a_in], dtype=np.int64)
        n_my = np.array([int(round(n_walkers * a / tot)) for a in a_my], dtype=np.int64)
        n_ex = n_walkers - int(n_in.sum()) - int(n_my.sum())
        if n_ex < 0:
            excess = -n_ex
            for k in range(N):
                trim = min(excess, int(n_in[k]))
                n_in[k] -= trim
                excess -= trim
                if excess == 0:
                    break
            n_ex = 0
        return n_in, n_my, n_ex

    def to3(self, comp):
        """Encoded compartment ids -> 0 intra, 1 myelin, 2 extra (core.py:548-550)."""
        comp = np.asarray(comp)
        return np.where(comp == 0, 2, np.where(comp > self.N_max, 1, 0)).astype(np.int32)

    def classify_position(self, r):
        """Encoded compartment of positions (lab frame) by their min-image distance to each axon:
        intra of the axon whose inner disc holds it, else myelin of the axon whose sheath holds
        it, else extra-axonal (0)."""
        r = np.atleast_2d(np.asarray(r, dtype=np.float32))
        rc = r if self._is_identity_rotation else r @ self._R.T
        L, N = np.float32(self._L_float), self.N_actual
        out = np.zeros(len(rc), np.int32)
        for k in range(N - 1, -1, -1):
            q = rc[:, :2] - self._centers_np[k].astype(np.float32)
            q = q - L * np.floor(q / L + np.float32(0.5))
            d2 = np.sum(q * q, axis=1)
            ri, ro = np.float32(self._inner_radii_np[k]), np.float32(self._outer_radii_np[k])
            out = np.where(d2 < ro * ro, self.N_max + 1 + k, out)
        for k in range(N - 1, -1, -1):
            q = rc[:, :2] - self._centers_np[k].astype(np.float32)
            q = q - L * np.floor(q / L + np.float32(0.5))
            d2 = np.sum(q * q, axis=1)
            ri = np.float32(self._inner_radii_np[k])
            out = np.where(d2 < ri * ri, 1 + k, out)
        return out

    def init_positions(self, n_walkers, key=None):
        """Host sampler of the reference (geometries.py:3084-3214): the counts of
        :meth:`seed_counts`, uniform in each inner disc, sheath and in the extra-axonal space;
        sets ``_init_compartments`` (encoded ids)."""
        rng = _host_rng(key)
        L, N = self._L_float, self.N_actual
        n_in, n_my, n_ex = self.seed_counts(n_walkers)
        pos, comp = [], []
        for kind, counts in ((0, n_in), (1, n_my)):
            for k in range(N):
                nk = int(counts[k])
                if nk == 0:
                    continue
                ri, ro = self._inner_radii_np[k], self._outer_radii_np[k]
                lo, hi = (0.0, ri) if kind == 0 else (ri, ro)
                got = np.zeros((0, 2))
                while len(got) < nk:
                    xy = rng.uniform(-hi, hi, (max(nk * 4, 64), 2))
                    d = np.linalg.norm(xy, axis=1)
                    got = np.concatenate([got, xy[(d >= lo) & (d < hi)]])
                pos.append(got[:nk] + self._centers_np[k])
                comp.append(np.full(nk, (1 + k) if kind == 0 else (self.N_max + 1 + k), np.int32))
        if n_ex > 0:
            got = np.zeros((0, 2))
            while len(got) < n_ex:
                xy = rng.uniform(-L / 2.0, L / 2.0, (max(n_ex * 4, 1024), 2))
                ok = np.ones(len(xy), bool)
                for k in range(N):
                    d = xy - self._centers_np[k]
                    d -= L * np.round(d / L)
                    ok &= np.sum(d ** 2, axis=1) > self._outer_radii_np[k] ** 2
                got = np.concatenate([got, xy[ok]])
            pos.append(got[:n_ex])
            comp.append(np.zeros(n_ex, np.int32))
        xy = np.concatenate(pos).astype(np.float32)
        rc = np.concatenate([xy, np.zeros((n_walkers, 1), np.float32)], axis=1)
        self._init_compartments = np.concatenate(comp)
        return (rc @ self._R).astype(np.float32)

    def spin_weight_sum(self, n_walkers):
        """Walkers seeded in a sheath weigh the myelin proton density, the others 1."""
        n_in, n_my, n_ex = self.seed_counts(n_walkers)
        return float(n_in.sum() + n_ex) + float(n_my.sum()) * self._myelin_proton_density

    # ---- the walk -----------------------------------------------------------------------------
    def _rho_D(self):
        f = np.float32
        rho = max(float(np.max(self._rho_inner.astype(f))), float(np.max(self._rho_outer.astype(f))))
        D_ref = float(max(np.max(self._D["intra"].astype(f)), np.max(self._D["extra"].astype(f))))
        return rho, D_ref

    def sub_steps(self, dt):
        """One walk step per sample; with surface relaxivity, sub-steps to the extra-axonal pore
        scale (physics.py:1009-1022)."""
        from .core import surface_sub_steps
        rho, D_ref = self._rho_D()
        return surface_sub_steps(self, D_ref, dt) if rho > 0.0 else 1

    def _pmyelin_desc(self, dt_sub, n_total, dev):
        """Descriptor and device tables of a walk with sub-step ``dt_sub`` (physics.py:705-740,
        995-1025), in the reference's float32 arithmetic."""
        f = np.float32
        N = self.N_actual
        dt32 = f(dt_sub)
        tab = np.zeros((max(N, 1), 16), np.float32)
        tab[:N, 0:2] = self._centers_np[:N].astype(f)
        tab[:N, 2] = self._inner_radii_np[:N].astype(f)
        tab[:N, 3] = self._outer_radii_np[:N].astype(f)
        for j, c in enumerate(("intra", "myelin", "extra")):
            Dc = self._D[c][:N].astype(f)
            tab[:N, 4 + j] = np.sqrt(f(6.0) * Dc * dt32)
            Dl = np.maximum(Dc, f(1e-30))
            tab[:N, 7 + j] = self._kappa_inner[:N].astype(f) / Dl
            tab[:N, 10 + j] = self._kappa_outer[:N].astype(f) / Dl
        n_in, n_my, n_ex = self.seed_counts(n_total)
        ends = np.cumsum(np.concatenate([n_in, n_my, [n_ex]])).astype(np.int64)
        t_tab = torch.from_numpy(tab).to(dev)
        t_seed = torch.from_numpy(ends).to(dev)
        g = self._base_desc(_lib.GEOM_PMYELIN, self._wall_mode(), 1.0, 0.0)
        g.radius = float(np.min(self._inner_radii_np[:N]))
        g.L = self._L_float
        g.eps_detect = self._eps
        g.nudge = self._nudge
        g.pmy_n, g.pmy_nmax = N, self.N_max
        g.pmy_cyl, g.pmy_seed = t_tab.data_ptr(), t_seed.data_ptr()
        if self._has_t2:
            g.pmy_t2dec[:] = [float(dt32 / f(self._T2[c][0])) for c in ("intra", "myelin", "extra")]
        rho, D_ref = self._rho_D()
        g.pmy_rho_over_D = float(f(rho / D_ref)) if rho > 0.0 else 0.0
        g.pmy_logw_myelin = float(np.log(f(self._myelin_proton_density)))
        return g, (t_tab, t_seed)

    def _has_weight(self):
        return self._has_t2 or self._rho_D()[0] > 0.0 or self._myelin_proton_density != 1.0


# ------------------------------------------------------------------------------------------------
# Random sequential addition packers
# ------------------------------------------------------------------------------------------------
def _rsa(radii, dim, L, seed, max_attempts, what):
    """RSA in a periodic box, largest objects first; the same draws as geometries.py:1570-1595 so a
    seed gives the same packing."""
    rng = np.random.default_rng(int(seed))
    order = np.argsort(radii)[::-1]
    rs = radii[order]
    cs = np.zeros((len(radii), dim))
    for i, r_new in enumerate(rs):
        placed = False
        for _ in range(max_attempts):
            c = rng.uniform(-L / 2.0, L / 2.0, dim)
            if i:
                dq = c - cs[:i]
                dq -= L * np.round(dq / L)
                if np.any(np.linalg.norm(dq, axis=1) < r_new + rs[:i]):
                    continue
            cs[i] = c
            placed = True
            break
        if not placed:
            raise RuntimeError(
                f"RSA failed after {max_attempts} attempts placing {what} {i} "
                f"(r = {r_new * 1e6:.2f} µm).  The target packing fraction may exceed what RSA can "
                f"achieve; try reducing target_vf or increasing max_attempts.")
    out = np.empty_like(cs)
    out[order] = cs
    return out


def _check_pack_args(radii, target_vf, L):
    radii = np.asarray(radii, dtype=np.float64).ravel()
    if len(radii) == 0:
        raise ValueError("radii must contain at least one element.")
    if np.any(radii <= 0):
        raise ValueError("All radii must be positive.")
    if (target_vf is None) == (L is None):
        raise ValueError("Provide exactly one of target_vf or L.")
    if target_vf is not None and not 0.0 < float(target_vf) < 1.0:
        raise ValueError(f"target_vf must be in (0, 1), got {target_vf}.")
    return radii


def pack_cylinders(radii, target_vf=None, L=None, seed=0, max_attempts=100_000):
    """Pack parallel cylinders in a periodic square (geometries.py:1502-1601).

    Returns ``(centers (N, 2), L, achieved_vf)``.
    """
    radii = _check_pack_args(radii, target_vf, L)
    L = float(np.sqrt(np.pi * np.sum(radii ** 2) / float(target_vf))) if target_vf is not None \
        else float(L)
    if np.any(radii > L / 2.0):
        raise ValueError(f"Largest radius ({np.max(radii) * 1e6:.2f} µm) exceeds L/2 "
                         f"({L / 2.0 * 1e6:.2f} µm).  Reduce target_vf or supply a larger L.")
    centers = _rsa(radii, 2, L, seed, max_attempts, "cylinder")
    return centers, L, float(np.pi * np.sum(radii ** 2) / L ** 2)


def pack_spheres(radii, target_vf=None, L=None, seed=0, max_attempts=100_000):
    """Pack spheres in a periodic cube (geometries.py:2249-2340).

    Returns ``(centers (N, 3), L, achieved_vf)``.
    """
    radii = _check_pack_args(radii, target_vf, L)
    L = float(((4.0 / 3.0) * np.pi * np.sum(radii ** 3) / float(target_vf)) ** (1.0 / 3.0)) \
        if target_vf is not None else float(L)
    if np.any(radii > L / 2.0):
        raise ValueError(f"Largest radius ({np.max(radii) * 1e6:.2f} µm) exceeds L/2 "
                         f"({L / 2.0 * 1e6:.2f} µm).  Reduce target_vf or supply a larger L.")
    centers = _rsa(radii, 3, L, seed, max_attempts, "sphere")
    return centers, L, float((4.0 / 3.0) * np.pi * np.sum(radii ** 3) / L ** 3)


def lattice_cylinders(n_side, target_vf, radius_mean, radius_sd, seed=0, gap=0.05):
    """Cylinders on an n_side x n_side periodic square lattice with lognormal radii.

    The substrate of the packed-cylinder workload (volume fraction up to ~0.7 with polydisperse
    radii, beyond what random sequential addition reaches).  Radii are drawn lognormal with the
    given mean and standard deviation, every radius is clipped to (1 - gap) * a / 2 so neighbours
    never touch, and the lattice spacing ``a`` is solved (bisection) so that
    sum(pi r^2) / L^2 = target_vf.  Returns ``(radii, centers (n, 2), L)``.
    """
    rng = np.random.default_rng(int(seed))
    s2 = np.log(1.0 + (radius_sd / radius_mean) ** 2)
    raw = rng.lognormal(np.log(radius_mean) - 0.5 * s2, np.sqrt(s2), n_side * n_side)

    def vf(a):
        r = np.minimum(raw, 0.5 * (1.0 - gap) * a)
        return np.pi * np.sum(r ** 2) / (n_side * a) ** 2, r

    lo, hi = 1e-9, 100.0 * radius_mean
    if vf(lo)[0] < target_vf:
        raise ValueError(f"target_vf {target_vf} is not reachable on a square lattice with "
                         f"gap {gap} (maximum {np.pi / 4 * (1 - gap) ** 2:.3f})")
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if vf(mid)[0] > target_vf:
            lo = mid
        else:
            hi = mid
    a = 0.5 * (lo + hi)
    radii = vf(a)[1]
    L = n_side * a
    ij = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij"), -1)
    centers = ((ij.reshape(-1, 2) + 0.5) * a - L / 2).astype(np.float64)
    return radii, centers, L


def _min_gap(centers, radii, L):
    n = len(radii)
    gap = float("inf")
    for i in range(n):
        dq = centers[i] - centers[i + 1:]
        dq -= L * np.round(dq / L)
        if len(dq):
            gap = min(gap, float(np.min(np.linalg.norm(dq, axis=1) - radii[i] - radii[i + 1:])))
    return min(gap, float(np.min(L - 2.0 * radii)))


def build_cell_list(centers, radii, L, reach, max_bytes=96 * 1024, min_cell=None):
    """Uniform cell list over the periodic cell [-L/2, L/2)^d.

    Cell c lists every periodic image (within one box) of every object whose disc/ball of radius
    R + reach meets the cell, ordered by object index then image, as float32 (cx, cy, cz, R).
    The grid is as fine as the table budget ``max_bytes`` allows (no finer than ``min_cell``).
    Returns ``(n, cell_start uint32 (padded to 16 B), cand float32 (n_cand, 4), cand_obj int32)``.
    """
    centers = np.asarray(centers, dtype=np.float64)
    radii = np.asarray(radii, dtype=np.float64)
    K, dim = centers.shape
    c0 = centers - L * np.floor(centers / L + 0.5)
    Rr = radii + reach
    shifts = np.array(list(itertools.product((-1, 0, 1), repeat=dim)), dtype=np.float64)
    if min_cell is None:
        min_cell = max(reach, 0.25 * float(np.mean(radii)))
    n = max(1, int(L // min_cell))
    while True:
        h = L / n
        cells, objs, imgs = [], [], []
        for si, s in enumerate(shifts):
            cs = c0 + L * s                                           # (K, dim)
            lo = np.floor((cs - Rr[:, None] + L / 2) / h).astype(np.int64)
            hi = np.floor((cs + Rr[:, None] + L / 2) / h).astype(np.int64)
            lo = np.clip(lo, 0, n - 1)
            hi = np.clip(hi, 0, n - 1)
            inside_box = np.all((cs + Rr[:, None] + L / 2 >= 0) & (cs - Rr[:, None] + L / 2 <= L),
                                axis=1)
            span = int(np.max(hi - lo + 1)) if K else 1
            grids = np.stack(np.meshgrid(*[np.arange(span)] * dim, indexing="ij"),
                             axis=-1).reshape(-1, dim)                 # (B, dim)
            idx = lo[:, None, :] + grids[None, :, :]                   # (K, B, dim)
            ok = np.all(idx <= hi[:, None, :], axis=2) & inside_box[:, None]
            edge_lo = -L / 2 + idx * h
            d = np.maximum(np.maximum(edge_lo - cs[:, None, :], 0.0),
                           cs[:, None, :] - (edge_lo + h))
            ok &= np.sum(d * d, axis=2) <= (Rr[:, None] * (1 + 1e-9)) ** 2
            kk, bb = np.nonzero(ok)
            cid = np.zeros(len(kk), dtype=np.int64)
            for a in reversed(range(dim)):
                cid = cid * n + idx[kk, bb, a]
            cells.append(cid)
            objs.append(kk)
            imgs.append(np.full(len(kk), si))
        cells = np.concatenate(cells)
        objs = np.concatenate(objs)
        imgs = np.concatenate(imgs)
        n_cells = n ** dim
        nbytes = (n_cells + 4) * 4 + len(cells) * 16
        if nbytes <= max_bytes or n == 1:
            break
        n = max(1, int(n / 1.25))
    order = np.lexsort((imgs, objs, cells))
    cells, objs, imgs = cells[order], objs[order], imgs[order]
    counts = np.bincount(cells, minlength=n_cells)
    start = np.zeros(((n_cells + 1 + 3) // 4) * 4, dtype=np.uint32)
    start[1:n_cells + 1] = np.cumsum(counts)
    start[n_cells + 1:] = start[n_cells]
    pos = c0[objs] + L * shifts[imgs]
    cand = np.zeros((len(objs), 4), dtype=np.float32)
    cand[:, :dim] = pos
    cand[:, 3] = radii[objs]
    return n, start, cand, objs.astype(np.int32)


class _Packed(Geometry):
    """Shared machinery of PackedCylinders / PackedSpheres (periodic objects + cell list)."""

    _dim = 2
    _kind = None

    def _setup(self, radii, centers, L, surface_relaxivity_t2, permeability):
        self.surface_relaxivity_t2 = _opt_float(surface_relaxivity_t2)
        self.permeability = _opt_float(permeability)
        self._L_float = float(L)
        self._radii_np = radii.copy()
        self._centers_np = centers.copy()
        self._centers_jax = centers.astype(np.float32)    # name kept for duck-typed callers
        self._radii_jax = radii.astype(np.float32)
        self._L_jax = np.float32(L)
        min_r = float(np.min(radii))
        self._eps_detect = np.float32(1e-7 * min_r)
        self._nudge = np.float32(1e-4 * min_r)
        self.min_gap = _min_gap(centers, radii, float(L))
        self._dev_cache = {}

    def _classify_frame(self, rc):
        L = np.float32(self._L_float)
        q = rc[..., None, :self._dim] - self._centers_jax
        q = q - L * np.floor(q / L + np.float32(0.5))
        inside = np.sum(q * q, axis=-1) < self._radii_jax ** 2
        ids = np.arange(1, len(self._radii_np) + 1, dtype=np.int32)
        return np.max(np.where(inside, ids, 0), axis=-1).astype(np.int32)

    # Byte budget of the cell list (cell offsets + candidates): the grid is as fine as this
    # allows.  Lists within the walk's shared-memory budget are staged on chip.
    cell_list_bytes = 96 * 1024

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        reach = float(step_length) * 1.05 + 8.0 * float(self._nudge)
        key = (round(reach, 15), str(dev), int(self.cell_list_bytes))
        if key not in self._dev_cache:
            n, start, cand, obj = build_cell_list(self._centers_np, self._radii_np, self._L_float,
                                                  reach, max_bytes=int(self.cell_list_bytes))
            t_start = torch.from_numpy(start.view(np.int32)).to(dev)
            t_cand = torch.from_numpy(cand).to(dev)
            t_obj = torch.from_numpy(obj if len(obj) else np.zeros(1, np.int32)).to(dev)
            # lists are sorted by cell then object: a repeated (cell, object) pair means two
            # images of one object share a cell, and only then must candidates be min-image tested
            n_cells = n ** self._dim
            cell_of = np.repeat(np.arange(n_cells), np.diff(start[:n_cells + 1].astype(np.int64)))
            need_mi = bool(np.any((cell_of[1:] == cell_of[:-1]) & (obj[1:] == obj[:-1])))
            max_cand = int(np.max(np.diff(start[:n_cells + 1].astype(np.int64)))) if n_cells else 0
            self._dev_cache = {key: (n, reach, t_start, t_cand, t_obj, len(obj), need_mi,
                                     max_cand)}
        n, reach, t_start, t_cand, t_obj, n_cand, need_mi, max_cand = self._dev_cache[key]
        g = self._base_desc(self._kind, wall_mode, rho_over_D, kappa_over_D)
        g.radius = float(np.min(self._radii_np))
        g.eps_detect = self._eps_detect
        g.nudge = self._nudge
        g.L = np.float32(self._L_float)
        g.n_objects = len(self._radii_np)
        g.grid_n = n
        g.cell_h = self._L_float / n
        g.reach = reach
        g.n_cand = n_cand
        g.need_min_image = 1 if need_mi else 0
        g.max_cell_cand = max_cand
        g.cell_start = t_start.data_ptr()
        g.cand = t_cand.data_ptr()
        g.cand_obj = t_obj.data_ptr()
        return g, (t_start, t_cand, t_obj)

    def volume_fraction(self):
        if self._dim == 2:
            return float(np.pi * np.sum(self._radii_np ** 2) / self._L_float ** 2)
        return float((4.0 / 3.0) * np.pi * np.sum(self._radii_np ** 3) / self._L_float ** 3)


class PackedCylinders(_Packed):
    """Extra-axonal diffusion among parallel cylinders in a periodic square (geometries.py:1604-2242).

    Positions stay unfolded for the phase; detection uses the minimum image; one specular
    reflection per sub-step plus the fold-first safety clamp; permeable walls transmit with the
    Powles probability.
    """

    _dim = 2
    _kind = _lib.GEOM_PACKED_CYLINDERS

    def __init__(self, radii, centers, L, orientation=(0., 0., 1.), surface_relaxivity_t2=None,
                 permeability=None):
        radii = np.asarray(radii, dtype=np.float64).ravel()
        centers = np.asarray(centers, dtype=np.float64)
        if centers.shape != (len(radii), 2):
            raise ValueError(f"centers shape {centers.shape} does not match ({len(radii)}, 2) for "
                             f"{len(radii)} cylinders.")
        if np.any(radii <= 0):
            raise ValueError("All radii must be positive.")
        o = np.asarray(orientation, dtype=np.float64)
        self.orientation = (o / np.linalg.norm(o)).astype(np.float32)
        R = _rotation_to_z(self.orientation)
        self._R = R.astype(np.float32)
        self._R_inv = R.T.astype(np.float32)
        self._is_identity_rotation = bool(np.allclose(R, np.eye(3)))
        self._setup(radii, centers, L, surface_relaxivity_t2, permeability)

    def _frame(self):
        return None if self._is_identity_rotation else self._R.astype(np.float64)

    def classify_position(self, r):
        """0 = extra-axonal, k = inside cylinder k (1-based)."""
        r = np.asarray(r, dtype=np.float32)
        rc = r if self._is_identity_rotation else r @ self._R.T
        return self._classify_frame(rc)

    def init_positions(self, n_walkers, key=None):
        """Uniform in the periodic box outside every cylinder, z = 0 (geometries.py:1717-1744)."""
        rng = _host_rng(key)
        L = self._L_float
        out, have = [], 0
        while have < n_walkers:
            xy = rng.uniform(-L / 2.0, L / 2.0, (max(n_walkers * 4, 1024), 2))
            ok = np.ones(len(xy), bool)
            for k in range(len(self._radii_np)):
                d = xy - self._centers_np[k]
                d -= L * np.round(d / L)
                ok &= np.sum(d * d, axis=1) > self._radii_np[k] ** 2
            out.append(xy[ok])
            have = sum(len(a) for a in out)
        xy = np.concatenate(out)[:n_walkers].astype(np.float32)
        rc = np.concatenate([xy, np.zeros((n_walkers, 1), np.float32)], axis=1)
        return (rc @ self._R).astype(np.float32)

    def volume(self, L=1.0):
        return float(np.pi * np.sum(self._radii_np ** 2) * float(L))

    def surface_area(self, L=1.0):
        return float(2.0 * np.pi * np.sum(self._radii_np) * float(L))


class PackedSpheres(_Packed):
    """Extra-cellular diffusion among spheres in a periodic cube (geometries.py:2343-2786)."""

    _dim = 3
    _kind = _lib.GEOM_PACKED_SPHERES

    def __init__(self, radii, centers, L, surface_relaxivity_t2=None, permeability=None):
        radii = np.asarray(radii, dtype=np.float64).ravel()
        centers = np.asarray(centers, dtype=np.float64)
        if centers.shape != (len(radii), 3):
            raise ValueError(f"centers shape {centers.shape} does not match ({len(radii)}, 3) for "
                             f"{len(radii)} spheres.")
        if np.any(radii <= 0):
            raise ValueError("All radii must be positive.")
        self._setup(radii, centers, L, surface_relaxivity_t2, permeability)

    def classify_position(self, r):
        """0 = extra-cellular, k = inside sphere k (1-based)."""
        return self._classify_frame(np.asarray(r, dtype=np.float32))

    def init_positions(self, n_walkers, key=None):
        """Uniform in the periodic cube outside every sphere (geometries.py:2421-2443)."""
        rng = _host_rng(key)
        L = self._L_float
        out, have = [], 0
        while have < n_walkers:
            p = rng.uniform(-L / 2.0, L / 2.0, (max(n_walkers * 4, 1024), 3))
            ok = np.ones(len(p), bool)
            for k in range(len(self._radii_np)):
                d = p - self._centers_np[k]
                d -= L * np.round(d / L)
                ok &= np.sum(d * d, axis=1) > self._radii_np[k] ** 2
            out.append(p[ok])
            have = sum(len(a) for a in out)
        return np.concatenate(out)[:n_walkers].astype(np.float32)

    def volume(self):
        return float((4.0 / 3.0) * np.pi * np.sum(self._radii_np ** 3))

    def surface_area(self):
        return float(4.0 * np.pi * np.sum(self._radii_np ** 2))
