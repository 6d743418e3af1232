"""Seeded synthetic studies: substrates, free gradient waveforms and tissue parameters drawn from
fixed ranges, as batched-walk instances and as the surrogate's training set.

Ranges: mean radius 0.5-5 um, volume fraction 0.3-0.8 (clamped to what the packer reaches:
random sequential addition up to 0.5 for cylinders, a polydisperse square lattice above that up
to 0.70; 0.38 for spheres, stepped down where 16 spheres jam first), permeability 0-1e-4 m/s, surface relaxivity 0-5e-6 m/s, diffusivity
1-3e-9 m^2/s, walkers log-uniform 1e4-1e6, 300-3000 waveform samples, 8-96 measurements.

A free waveform set is built from a few smooth refocused shapes: q(t) = sum_k c_k sin(pi k t/TE)
vanishes at t = 0 and at the echo, and the gradient is its derivative / gamma.  Each measurement
applies one shape along a random direction, scaled to a b-value drawn from [0, b_max].  The set
therefore has a shape basis of rank <= the number of shapes (the batched kernel's basis form).
"""
import numpy as np

from .batched import Instance
from .constants import GAMMA
from .geometries import PackedCylinders, PackedSpheres, lattice_cylinders, pack_cylinders, \
    pack_spheres
from .waveforms import Waveform, calc_b

RANGES = {"radius": (0.5e-6, 5e-6), "f": (0.3, 0.8), "kappa": (0.0, 1e-4),
          "rho": (0.0, 5e-6), "D": (1e-9, 3e-9)}
F_MAX = {"PackedCylinders": 0.70, "PackedSpheres": 0.38}


def free_shapes(n_shapes, n_t, rng, n_harm=4):
    """(n_shapes, n_t) unit-peak gradient shapes whose dephasing q(t) is refocused at the last
    sample."""
    t = np.linspace(0.0, 1.0, n_t)
    out = np.empty((n_shapes, n_t))
    k = np.arange(1, n_harm + 1)
    for i in range(n_shapes):
        c = rng.normal(size=n_harm) / k
        g = np.sum(c[:, None] * (np.pi * k[:, None]) * np.cos(np.pi * k[:, None] * t[None, :]), 0)
        g -= g.mean()            # the sampled moment sum_t g(t) dt is exactly zero
        out[i] = g / np.max(np.abs(g))
    return out


def free_waveform_set(n_meas, n_t, TE, rng, n_shapes=None, b_max=3e9):
    """A Waveform of n_meas free measurements; returns (waveform, shape index, direction,
    b-values)."""
    n_shapes = int(n_shapes or rng.integers(1, 4))
    shapes = free_shapes(n_shapes, n_t, rng)
    dt = TE / (n_t - 1)
    idx = rng.integers(0, n_shapes, n_meas)
    dirs = rng.normal(size=(n_meas, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    b = rng.uniform(0.0, b_max, n_meas)
    G = shapes[idx][:, :, None] * dirs[:, None, :] * 0.05          # 50 mT/m peak, then scale
    wf = Waveform(G.astype(np.float32), dt, n_t - 1)
    b0 = calc_b(wf)
    s = np.sqrt(np.divide(b, b0, out=np.zeros_like(b), where=b0 > 0))
    wf = Waveform((G * s[:, None, None]).astype(np.float32), dt, n_t - 1)
    return wf, idx, dirs, b


def q_encoding(wf, n_samples=32, t_max=0.08, axis=(0.0, 0.0, 1.0)):
    """Waveform encoding of each measurement: the dephasing q(t) = gamma int_0^t g dt' at
    n_samples absolute times (the midpoints of [0, t_max] cut into n_samples; q = 0 after the
    waveform ends), split into its component along ``axis`` and its magnitude across it (signed
    by the component along the transverse direction of largest reach), in rad/um:
    (n_meas, 2 n_samples).  Absolute times keep the diffusion-time information that a
    resampling on [0, TE] would lose."""
    G = np.asarray(wf.G, np.float64)
    M, n_t, _ = G.shape
    q = GAMMA * np.cumsum(G, axis=1) * wf.dt                      # q after sample i, rad/m
    tq = (np.arange(n_t) + 1.0) * wf.dt
    ts = (np.arange(n_samples) + 0.5) * (t_max / n_samples)
    # linear interpolation on the shared time grid (0 before the first sample, 0 after the end)
    i = np.searchsorted(tq, ts, side="right")
    inside = (i > 0) & (ts <= tq[-1])
    hi = np.clip(i, 1, n_t - 1)
    lo = hi - 1
    w = np.clip((ts - tq[lo]) / (tq[hi] - tq[lo]), 0.0, 1.0)
    exact_end = ts == tq[-1]
    w[exact_end] = 1.0
    qs = q[:, lo] * (1.0 - w)[None, :, None] + q[:, hi] * w[None, :, None]
    qs[:, ~inside] = 0.0
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    par = qs @ a
    perp = qs - par[..., None] * a
    mag = np.linalg.norm(perp, axis=-1)
    ref = perp[np.arange(M), np.argmax(mag, axis=1)]
    sign = np.sign(np.einsum("mtk,mk->mt", perp, ref))
    sign[sign == 0] = 1.0
    return np.concatenate([par, mag * sign], axis=1) * 1e-6


def packed_substrate(kind, radius, f, rng, n_objects=16, rho=0.0, kappa=0.0):
    """A packed substrate of ``n_objects`` with mean radius ``radius`` at volume fraction ``f``
    (clamped to the packer's reach).  Returns (geometry, achieved f)."""
    seed = int(rng.integers(0, 2 ** 31))
    kw = {"surface_relaxivity_t2": rho or None, "permeability": kappa or None}
    if kind == "PackedCylinders":
        f = min(f, F_MAX[kind])
        if f <= 0.5:
            radii = np.clip(rng.normal(radius, 0.1 * radius, n_objects), 0.5 * radius,
                            1.5 * radius)
            centers, L, fa = pack_cylinders(radii, target_vf=f, seed=seed)
        else:
            n_side = int(round(np.sqrt(n_objects)))
            radii, centers, L = lattice_cylinders(n_side, f, radius, 0.1 * radius, seed=seed)
            fa = float(np.pi * np.sum(radii ** 2) / L ** 2)
        return PackedCylinders(radii, centers, L, **kw), fa
    if kind == "PackedSpheres":
        f = min(f, F_MAX[kind])
        radii = np.clip(rng.normal(radius, 0.1 * radius, n_objects), 0.5 * radius, 1.5 * radius)
        while True:   # a few spheres jam below the large-system RSA limit: step f down
            try:
                centers, L, fa = pack_spheres(radii, target_vf=f, seed=seed, max_attempts=20000)
                break
            except RuntimeError:
                f -= 0.02
        return PackedSpheres(radii, centers, L, **kw), fa
    raise ValueError(f"unknown packed kind {kind!r}")


def ellipsoid_cell_mesh(n_cells=200, faces_per_cell=2500, seed=0, box=None,
                        radius_range=(2e-6, 5e-6), permeable=True):
    """The periodic mesh substrate of ``n_cells`` random ellipsoid cells (about
    n_cells x faces_per_cell triangles); returns (mesh, intracellular volume fraction)."""
    import warnings
    from .mesh import Mesh, random_ellipsoid_cells
    if box is None:
        box = 60e-6 * (n_cells / 200.0) ** (1.0 / 3.0)
    V, F = random_ellipsoid_cells(n_cells, box, radius_range, seed=seed,
                                  faces_per_cell=faces_per_cell)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        m = Mesh(V, F, periodic=True, voxel_min=[-box / 2] * 3, voxel_max=[box / 2] * 3,
                 feature_radius=radius_range[0], permeability=1e-5 if permeable else None)
    tri = V[F]
    vol = np.einsum("ij,ij->i", tri[:, 0], np.cross(tri[:, 1], tri[:, 2])).sum() / 6.0
    return m, float(vol / box ** 3)


def instance_mix(n=256, seed=0, kinds=("PackedCylinders", "PackedSpheres", "Mesh"),
                 walkers=(1e4, 1e6), n_t=(300, 3000), n_meas=(8, 96), TE=(0.03, 0.08),
                 walker_scale=1.0, mesh=None, b_max=3e9):
    """``n`` batched-walk instances drawn with ``numpy.random.default_rng(seed)``.  Returns
    (instances, parameters): one dict per instance with kind, radius, f, kappa, rho, D,
    n_walkers, n_t, n_meas, TE.  ``walker_scale`` multiplies every walker count (a reduced
    copy of the same study); ``mesh`` = (Mesh, f) reuses a built mesh substrate."""
    rng = np.random.default_rng(int(seed))
    insts, params = [], []
    for i in range(n):
        kind = kinds[int(rng.integers(0, len(kinds)))]
        r = rng.uniform(*RANGES["radius"])
        f = rng.uniform(*RANGES["f"])
        kappa = rng.uniform(*RANGES["kappa"])
        rho = rng.uniform(*RANGES["rho"])
        D = rng.uniform(*RANGES["D"])
        nw = int(np.exp(rng.uniform(np.log(walkers[0]), np.log(walkers[1]))))
        nt = int(rng.integers(n_t[0], n_t[1] + 1))
        M = int(rng.integers(n_meas[0], n_meas[1] + 1))
        te = rng.uniform(*TE)
        wf, _, _, _ = free_waveform_set(M, nt, te, rng, b_max=b_max)
        if kind == "Mesh":
            if mesh is None:
                mesh = ellipsoid_cell_mesh()
            geom = mesh[0].with_walls(rho or None, kappa or None)
            fa, r = mesh[1], mesh[0].radius
        else:
            geom, fa = packed_substrate(kind, r, f, rng, rho=rho, kappa=kappa)
        insts.append(Instance(max(1, int(nw * walker_scale)), D, wf, geom, seed=1000 + i))
        params.append(dict(kind=kind, radius=r, f=fa, kappa=kappa, rho=rho, D=D,
                           n_walkers=nw, n_t=nt, n_meas=M, TE=te))
    return insts, params
