"""Triangle-mesh substrate: host-side construction of the device tables.

Same constructor, attributes and conventions as dmipy-sim's ``mesh.py`` (Mesh 257-907, load_ply
136-180): optional 3-D periodicity with ghost triangles replicated across the periodic faces,
area-weighted smooth vertex normals, a uniform grid with cell = 4 x the diffusion step
(R/6, or R/25 when permeable), the float32 collision epsilon 1e-7 * min(box), the nudge
max(1e-4 * step, 16 * eps), the graze lift 1e-4 and a 10-bounce budget.  The grid is stored as
CSR lists (the reference pads every cell to the largest occupancy); each cell lists its triangles
in index order, so the 27-cell gather visits candidates in the reference's order.

The walk itself (``mesh.py`` reflect 637-671 / reflect_with_log_weight 673-705 / permeate
707-743 / classify 227-254 / leak guard 578-597) runs in the CUDA kernels; seeding draws uniform
points in the box and keeps those whose ray-crossing parity says inside (or outside), on the GPU.
"""
import copy
import itertools
import struct
import warnings
from collections import defaultdict

import numpy as np
import torch

from . import _lib
from .geometries import Geometry

_PERM_EDGE_RATIO_MAX = 0.05


def _rotation_from_z(axis):
    """Rotation R (mesh -> lab) with R @ z = axis / |axis| (Rodrigues)."""
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    z = np.array([0.0, 0.0, 1.0])
    v = np.cross(z, a)
    c = float(np.dot(z, a))
    if np.linalg.norm(v) < 1e-12:
        return np.eye(3) if c > 0 else np.diag([1.0, -1.0, -1.0])
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + K + K @ K * (1.0 / (1.0 + c))


def smooth_vertex_normals(V, F):
    """Area-weighted vertex normals (n_vertices, 3)."""
    tri = V[F]
    cr = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    vn = np.zeros((len(V), 3))
    for k in range(3):
        np.add.at(vn, F[:, k], cr)
    return vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)


def load_ply(path, scale=1.0, recenter=False):
    """Vertices (metres, float64) and triangle faces (int64) of an ASCII or binary PLY file.

    Vertex properties other than x/y/z are skipped; faces must be triangles.  The index type the
    header declares is honoured for binary files; ASCII payloads are read as decimal text (so an
    undersized declared index type cannot truncate them).
    """
    with open(path, "rb") as fh:
        raw = fh.read()
    end = raw.find(b"end_header")
    if end < 0:
        raise ValueError(f"{path}: not a PLY file")
    header = raw[:end].decode("ascii", "replace").splitlines()
    body = raw[raw.find(b"\n", end) + 1:]
    fmt = next((h.split()[1] for h in header if h.startswith("format")), "ascii")
    elems, cur = [], None
    for h in header:
        t = h.split()
        if t[:1] == ["element"]:
            cur = [t[1], int(t[2]), []]
            elems.append(cur)
        elif t[:1] == ["property"] and cur is not None:
            cur[2].append(t[1:])
    types = {"char": "b", "int8": "b", "uchar": "B", "uint8": "B", "short": "h", "int16": "h",
             "ushort": "H", "uint16": "H", "int": "i", "int32": "i", "uint": "I", "uint32": "I",
             "float": "f", "float32": "f", "double": "d", "float64": "d"}
    V = F = None
    if fmt == "ascii":
        tok = body.split()
        pos = 0
        for name, n, props in elems:
            if name == "vertex":
                width = len(props)
                arr = np.asarray(tok[pos:pos + n * width], dtype=np.float64).reshape(n, width)
                names = [p[-1] for p in props]
                V = arr[:, [names.index("x"), names.index("y"), names.index("z")]]
                pos += n * width
            elif name == "face":
                F = np.empty((n, 3), np.int64)
                for i in range(n):
                    k = int(tok[pos])
                    if k != 3:
                        raise ValueError(f"{path}: only triangle faces are supported")
                    F[i] = [int(x) for x in tok[pos + 1:pos + 4]]
                    pos += 4
            else:
                pos += n * len(props)
    else:
        endian = "<" if "little" in fmt else ">"
        off = 0
        for name, n, props in elems:
            if name == "vertex":
                dt = np.dtype([(p[-1], endian + types[p[0]]) for p in props])
                arr = np.frombuffer(body, dtype=dt, count=n, offset=off)
                V = np.stack([arr["x"], arr["y"], arr["z"]], 1).astype(np.float64)
                off += dt.itemsize * n
            elif name == "face":
                cnt_t, idx_t = types[props[0][1]], types[props[0][2]]
                F = np.empty((n, 3), np.int64)
                cs, isz = struct.calcsize(cnt_t), struct.calcsize(idx_t)
                for i in range(n):
                    k = struct.unpack_from(endian + cnt_t, body, off)[0]
                    off += cs
                    if k != 3:
                        raise ValueError(f"{path}: only triangle faces are supported")
                    F[i] = struct.unpack_from(endian + idx_t * 3, body, off)
                    off += 3 * isz
            else:
                dt = np.dtype([(p[-1], endian + types[p[0]]) for p in props])
                off += dt.itemsize * n
    if V is None or F is None:
        raise ValueError(f"{path}: no vertex or face element")
    if recenter:
        V = V - 0.5 * (V.min(0) + V.max(0))
    return V * scale, F


def icosphere(radius, subdivisions=2):
    """Geodesic sphere: an icosahedron (convex hull of the 12 golden-ratio vertices, faces
    oriented outward) refined by splitting every triangle into four, projected onto the sphere."""
    from scipy.spatial import ConvexHull
    p = (1.0 + 5.0 ** 0.5) / 2.0
    base = []
    for a, b in itertools.product((-1.0, 1.0), repeat=2):
        base += [(0.0, a, b * p), (a, b * p, 0.0), (b * p, 0.0, a)]
    V = np.asarray(base)
    F = ConvexHull(V).simplices.astype(np.int64)
    for f in F:                                      # orient outward
        a, b, c = V[f]
        if np.dot(np.cross(b - a, c - a), a + b + c) < 0:
            f[1], f[2] = f[2], f[1]
    for _ in range(int(subdivisions)):
        Vl = [tuple(v) for v in V]
        mids = {}

        def mid(i, j):
            key = (min(i, j), max(i, j))
            if key not in mids:
                mids[key] = len(Vl)
                Vl.append(tuple(0.5 * (V[i] + V[j])))
            return mids[key]
        nf = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        V = np.asarray(Vl)
        F = np.asarray(nf, np.int64)
    V = V / np.linalg.norm(V, axis=1, keepdims=True) * radius
    return V, F


def uv_sphere(radius, n_lat, n_lon):
    """Latitude-longitude sphere: two poles and n_lat - 1 rings of n_lon vertices, 2 n_lon
    (n_lat - 1) outward-oriented triangles."""
    th = np.pi * np.arange(1, n_lat) / n_lat
    ph = 2.0 * np.pi * np.arange(n_lon) / n_lon
    ring = np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :],
                     np.sin(th)[:, None] * np.sin(ph)[None, :],
                     np.repeat(np.cos(th)[:, None], n_lon, axis=1)], axis=-1).reshape(-1, 3)
    V = np.concatenate([[[0.0, 0.0, 1.0]], ring, [[0.0, 0.0, -1.0]]])
    south = len(V) - 1

    def vid(i, j):
        return 1 + i * n_lon + (j % n_lon)
    F = []
    for j in range(n_lon):
        F.append((0, vid(0, j), vid(0, j + 1)))
        F.append((south, vid(n_lat - 2, j + 1), vid(n_lat - 2, j)))
        for i in range(n_lat - 2):
            a, b = vid(i, j), vid(i, j + 1)
            c, d = vid(i + 1, j), vid(i + 1, j + 1)
            F.append((a, c, d))
            F.append((a, d, b))
    F = np.asarray(F, np.int64)
    tri = V[F]
    out = np.einsum("ij,ij->i", np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]),
                    tri.sum(1)) < 0
    F[out] = F[out][:, [0, 2, 1]]
    return V * radius, F


def random_ellipsoid_cells(n_cells, box, radius_range, subdivisions=3, seed=0, max_tries=20000,
                           faces_per_cell=None):
    """A substrate of ``n_cells`` closed ellipsoidal cells placed without overlap inside the cubic
    box [-box/2, box/2)^3 (a margin from every face, so each surface stays closed), with random
    semi-axes in ``radius_range`` and random orientations.  Each cell is an icosphere of the
    given subdivision level, or, with ``faces_per_cell``, a latitude-longitude sphere of about
    that many triangles.  Returns ``(V, F)``."""
    rng = np.random.default_rng(int(seed))
    Vs, Fs, cent, bound = [], [], [], []
    if faces_per_cell:
        n_lat = max(3, int(round(np.sqrt(faces_per_cell / 4.0))))
        n_lon = max(3, int(round(faces_per_cell / (2.0 * (n_lat - 1)))))
        base_V, base_F = uv_sphere(1.0, n_lat, n_lon)
    else:
        base_V, base_F = icosphere(1.0, subdivisions)
    off = 0
    for _ in range(max_tries):
        if len(cent) == n_cells:
            break
        axes = rng.uniform(radius_range[0], radius_range[1], 3)
        rmax = float(np.max(axes))
        c = rng.uniform(-box / 2 + 1.05 * rmax, box / 2 - 1.05 * rmax, 3)
        if cent and np.any(np.linalg.norm(np.asarray(cent) - c, axis=1) <
                           1.05 * (np.asarray(bound) + rmax)):
            continue
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        Rq = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                       [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                       [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        Vs.append((base_V * axes) @ Rq.T + c)
        Fs.append(base_F + off)
        off += len(base_V)
        cent.append(c)
        bound.append(rmax)
    if len(cent) < n_cells:
        raise RuntimeError(f"placed only {len(cent)} of {n_cells} cells in the box")
    return np.concatenate(Vs), np.concatenate(Fs)


def _closed_surface(F):
    """Every edge shared by exactly two faces."""
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e, axis=0, return_counts=True)
    return bool(np.all(cnt == 2))


def hit_reach(step_length, cell_size):
    """The reach (a float32 value) of the hit lists that serve steps of ``step_length``: at least
    1.001 x the step, rounded up to the ladder cell_size x 2^(q/16); None when that is not below
    the cell size or the step is not a positive number."""
    if not (step_length > 0.0) or not np.isfinite(step_length):
        return None
    q = int(np.ceil(16.0 * np.log2(step_length * 1.001 / cell_size)))
    reach = float(np.float32(cell_size * 2.0 ** (q / 16.0)))
    if reach < step_length * 1.001:
        reach = float(np.nextafter(np.float32(step_length * 1.001), np.float32(np.inf)))
    return reach if reach < cell_size else None


class Mesh(Geometry):
    """Reflecting / relaxing / permeable triangle-mesh substrate (mesh.py:257-907).

    Parameters as the reference: ``vertices``, ``faces``, ``periodic``, ``voxel_min/voxel_max``,
    ``feature_radius``, ``surface_relaxivity_t2``, ``permeability`` (float or
    ``{"intra_to_extra", "extra_to_intra"}``), ``intra``/``extra`` per-side surface relaxivity,
    ``orientation``/``R`` (acquisition rotation), ``cell_size``, ``max_bounces``.  Per-compartment
    bulk D/T2/T1 are not supported by this engine.

    ``use_hit_lists`` (default True): the nearest-hit search of a step reads, per grid cell, only
    the candidates within the step's reach of the cell (``dmsim_mesh_hit_lists``) instead of the
    whole 27-cell gather; the walk is the same either way.
    """

    use_hit_lists = True

    def __init__(self, vertices, faces, *, periodic=False, voxel_min=None, voxel_max=None,
                 feature_radius=None, surface_relaxivity_t2=None, permeability=None, intra=None,
                 extra=None, orientation=None, R=None, cell_size=None, cap=None, max_bounces=10):
        V = np.asarray(vertices, np.float64)
        F = np.asarray(faces, np.int64)
        self.vertices, self.faces = V, F
        if isinstance(periodic, bool):
            periodic = (periodic,) * 3
        self.periodic = tuple(bool(p) for p in periodic)
        if any(self.periodic) and (voxel_min is None or voxel_max is None):
            raise ValueError("a periodic Mesh needs voxel_min and voxel_max (the periodic box)")
        lo, hi = V.min(0), V.max(0)
        self.vmin = np.asarray(voxel_min, np.float64) if voxel_min is not None else lo.copy()
        self.vmax = np.asarray(voxel_max, np.float64) if voxel_max is not None else hi.copy()
        self.L = self.vmax - self.vmin
        if feature_radius is None:
            sides = self.L
            feature_radius = 0.5 * float(np.min(sides[sides > 0]))
        self.radius = float(feature_radius)
        self.reject_escape = True

        intra = dict(intra or {})
        extra = dict(extra or {})
        for side, dct in (("intra", intra), ("extra", extra)):
            bad = set(dct) - {"surface_relaxivity_t2", "D", "T2", "T1"}
            if bad:
                raise NotImplementedError(f"Mesh {side}={sorted(bad)}: supported per-compartment "
                                          "properties are ['D', 'T1', 'T2', 'surface_relaxivity_t2'].")
            if any(k in dct for k in ("D", "T2", "T1")):
                raise NotImplementedError("per-compartment D/T2/T1 on a Mesh is not supported by "
                                          "this engine")
        rho_i = intra.get("surface_relaxivity_t2", surface_relaxivity_t2)
        rho_e = extra.get("surface_relaxivity_t2", surface_relaxivity_t2)
        rho_i = float(rho_i) if rho_i is not None else 0.0
        rho_e = float(rho_e) if rho_e is not None else 0.0
        rho_nom = max(rho_i, rho_e)
        self.surface_relaxivity_t2 = rho_nom if rho_nom > 0 else None
        self._rho_mult_intra = np.float32(rho_i / rho_nom if rho_nom > 0 else 1.0)
        self._rho_mult_extra = np.float32(rho_e / rho_nom if rho_nom > 0 else 1.0)
        if isinstance(permeability, dict):
            k_out = float(permeability.get("intra_to_extra", 0.0))
            k_in = float(permeability.get("extra_to_intra", 0.0))
        elif permeability is not None:
            k_out = k_in = float(permeability)
        else:
            k_out = k_in = 0.0
        k_nom = max(k_out, k_in)
        self.permeability = k_nom if k_nom > 0 else None
        self._kappa_mult_out = np.float32(k_out / k_nom if k_nom > 0 else 1.0)
        self._kappa_mult_in = np.float32(k_in / k_nom if k_nom > 0 else 1.0)
        self._D_comp = self._T2_comp = self._T1_comp = None

        self.orientation = orientation
        if R is not None:
            Rm = np.asarray(R, np.float64).reshape(3, 3)
        elif orientation is not None:
            Rm = _rotation_from_z(orientation)
        else:
            Rm = None
        self._orient_R = None if Rm is None else np.ascontiguousarray(Rm, np.float32)

        e = V[F]
        edge = np.concatenate([np.linalg.norm(e[:, 1] - e[:, 0], axis=1),
                               np.linalg.norm(e[:, 2] - e[:, 1], axis=1),
                               np.linalg.norm(e[:, 0] - e[:, 2], axis=1)])
        self.edge_median = float(np.median(edge))
        self.edge_p90 = float(np.percentile(edge, 90))
        self.edge_feature_ratio = self.edge_median / self.radius
        if self.permeability is not None and self.edge_feature_ratio > _PERM_EDGE_RATIO_MAX:
            warnings.warn(f"Mesh is likely too coarse for MC-noise-accurate PERMEABILITY: median "
                          f"edge / feature_radius = {self.edge_feature_ratio:.3f} (need <~ "
                          f"{_PERM_EDGE_RATIO_MAX}).", stacklevel=2)

        step_l = self.radius / (25.0 if self.permeability is not None else 6.0)
        self.cell_size = float(cell_size) if cell_size is not None else 4.0 * step_l
        self.margin = self.cell_size

        vn = smooth_vertex_normals(V, F)
        tri_v, tri_vn = V[F], vn[F]
        tmin, tmax = tri_v.min(1), tri_v.max(1)
        all_tri, all_vn = [tri_v], [tri_vn]
        for combo in itertools.product((-1, 0, 1), repeat=3):     # periodic ghosts
            if all(c == 0 for c in combo) or any(combo[a] and not self.periodic[a]
                                                  for a in range(3)):
                continue
            keep = np.ones(len(F), bool)
            shift = np.zeros(3)
            for a in range(3):
                if combo[a] == -1:
                    keep &= tmax[:, a] > self.vmax[a] - self.margin
                    shift[a] = -self.L[a]
                elif combo[a] == 1:
                    keep &= tmin[:, a] < self.vmin[a] + self.margin
                    shift[a] = self.L[a]
            if keep.any():
                all_tri.append(tri_v[keep] + shift)
                all_vn.append(tri_vn[keep])
        tri_all = np.concatenate(all_tri)
        vn_all = np.concatenate(all_vn)
        self.n_ghost = len(tri_all) - len(F)
        nrm = np.cross(tri_all[:, 1] - tri_all[:, 0], tri_all[:, 2] - tri_all[:, 0])
        nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)

        self.grid_min = self.vmin - self.margin
        self.dims = np.maximum(1, np.ceil((self.vmax + self.margin - self.grid_min) /
                                          self.cell_size).astype(int))
        cs = self.cell_size
        lo_c = np.clip(np.floor((tri_all.min(1) - self.grid_min) / cs).astype(int), 0,
                       self.dims - 1)
        hi_c = np.clip(np.floor((tri_all.max(1) - self.grid_min) / cs).astype(int), 0,
                       self.dims - 1)
        cells, tris = [], []
        span = hi_c - lo_c + 1
        for sx in range(int(span[:, 0].max())):
            for sy in range(int(span[:, 1].max())):
                for sz in range(int(span[:, 2].max())):
                    ok = (sx < span[:, 0]) & (sy < span[:, 1]) & (sz < span[:, 2])
                    t = np.nonzero(ok)[0]
                    c = ((lo_c[t, 0] + sx) * self.dims[1] + lo_c[t, 1] + sy) * self.dims[2] + \
                        lo_c[t, 2] + sz
                    cells.append(c)
                    tris.append(t)
        cells = np.concatenate(cells)
        tris = np.concatenate(tris)
        order = np.lexsort((tris, cells))
        cells, tris = cells[order], tris[order]
        n_cells = int(np.prod(self.dims))
        counts = np.bincount(cells, minlength=n_cells)
        self.C = self.max_occ = int(counts.max()) if len(counts) else 0
        self.overflow = 0
        if cap is not None and self.max_occ > int(cap):
            keep = np.ones(len(cells), bool)
            first = np.searchsorted(cells, np.arange(n_cells))
            rank = np.arange(len(cells)) - first[cells]
            keep = rank < int(cap)
            self.overflow = int((~keep).sum())
            cells, tris = cells[keep], tris[keep]
            counts = np.bincount(cells, minlength=n_cells)
            self.C = int(cap)
        self._cell_start = np.zeros(n_cells + 1, np.uint32)
        self._cell_start[1:] = np.cumsum(counts)
        self._cell_tri = tris.astype(np.uint32)
        self._tri_all = tri_all.astype(np.float32)
        self._vn_all = vn_all.astype(np.float32)
        self._nrm_all = nrm.astype(np.float32)
        self._n_orig = len(F)
        scale = float(np.min(self.L))
        self._EPS = np.float32(1e-7 * scale)
        self._NUDGE = np.float32(max(1e-4 * step_l, 16.0 * float(self._EPS)))
        self._GRAZE = np.float32(1e-4)
        self._MAX_BOUNCES = int(max_bounces)
        self._closed = None
        self._dev_cache = {}

    def with_walls(self, surface_relaxivity_t2=None, permeability=None):
        """The same surface with other (uniform) wall properties: a view that shares this mesh's
        triangles, grid and device tables.  The grid stays the one this mesh was built with."""
        self._surface_is_closed()   # computed once, shared by every view
        m = copy.copy(self)
        m.surface_relaxivity_t2 = (float(surface_relaxivity_t2)
                                   if surface_relaxivity_t2 else None)
        m._rho_mult_intra = m._rho_mult_extra = np.float32(1.0)
        m.permeability = float(permeability) if permeability else None
        m._kappa_mult_out = m._kappa_mult_in = np.float32(1.0)
        return m

    # -------------------------------------------------------------------------------------------
    def _surface_is_closed(self):
        if self._closed is None:
            self._closed = _closed_surface(self.faces)
        return self._closed

    def _tables(self, dev):
        key = str(dev)
        if key not in self._dev_cache:
            t = self._tri_all
            A = t[:, 0]
            E1 = t[:, 1] - A            # float32 differences, as the reference forms them per step
            E2 = t[:, 2] - A
            cent = (t.astype(np.float64).mean(1)).astype(np.float32)
            rec = np.zeros((len(t), 16), np.float32)
            rec[:, 0:3], rec[:, 3:6], rec[:, 6:9] = A, E1, E2
            rec[:, 9:12], rec[:, 12:15] = self._nrm_all, cent
            rec[:, 15] = (np.arange(len(t)) < self._n_orig).astype(np.float32)  # 1 = not a ghost
            vn = np.zeros((len(t), 12), np.float32)
            vn[:, 0:9] = self._vn_all.reshape(-1, 9)
            # bounding sphere of each float32 triangle about its float32 centroid, widened so
            # that rounding in the walk's segment test can never reject a true hit
            c64 = cent.astype(np.float64)
            rb = np.max(np.linalg.norm(t.astype(np.float64) - c64[:, None, :], axis=2), axis=1)
            bs = np.zeros((len(t), 4), np.float32)
            bs[:, 0:3] = cent
            bs[:, 3] = (rb * (1.0 + 1e-3) + 1e-9).astype(np.float32)
            tt = {
                "tri": torch.from_numpy(rec).to(dev),
                "vn": torch.from_numpy(vn).to(dev),
                "bs": torch.from_numpy(bs).to(dev),
                "cs": torch.from_numpy(self._cell_start.view(np.int32)).to(dev),
                "ct": torch.from_numpy((self._cell_tri if len(self._cell_tri)
                                        else np.zeros(1, np.uint32)).view(np.int32)).to(dev),
            }
            self._neighbourhoods(tt, dev)
            self._dev_cache[key] = tt
        return self._dev_cache[key]

    def _neighbourhoods(self, tt, dev):
        """Per grid cell, the distinct triangles of its 27-cell gather, built on the device
        (dmsim_mesh_neighbourhoods): the walk then visits each candidate once."""
        lib = _lib.load()
        g = _lib.Geometry()
        g.mesh_dims[:] = [int(x) for x in self.dims]
        g.mesh_cell_start = tt["cs"].data_ptr()
        g.mesh_cell_tri = tt["ct"].data_ptr()
        n_cells = int(np.prod(self.dims))
        start = torch.zeros(n_cells + 1, dtype=torch.int64, device=dev)
        counts = torch.empty(n_cells + 1, dtype=torch.int32, device=dev)
        s = _lib.stream_handle()
        _lib.check(lib.dmsim_mesh_neighbourhoods(g, _lib.ptr(counts), None, s),
                   "dmsim_mesh_neighbourhoods")
        start[1:] = torch.cumsum(counts[:n_cells].to(torch.int64), 0)
        total = int(start[-1].item())
        if total >= 2 ** 31:
            raise RuntimeError("mesh neighbourhood lists exceed 2^31 entries")
        nb_start = start.to(torch.int32)
        nb_tri = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
        _lib.check(lib.dmsim_mesh_neighbourhoods(g, _lib.ptr(nb_start), _lib.ptr(nb_tri), s),
                   "dmsim_mesh_neighbourhoods")
        tt["nbs"], tt["nbt"] = nb_start, nb_tri
        # each entry's centroid record in list order: the classification reads it beside the
        # list position instead of through the triangle index
        tt["nbc"] = tt["tri"][nb_tri.to(torch.int64), 12:16].contiguous() if total else \
            torch.zeros((1, 4), dtype=torch.float32, device=dev)
        self.n_neighbourhood_entries = total

    def _hit_lists(self, tt, step_length):
        """The hit lists for steps up to ``step_length`` (dmsim_mesh_hit_lists), built for a
        reach rounded up to a ladder of 1/16 octave steps from the grid cell, so that walks of
        similar step lengths share one set; None when the reach is not below the cell size (the
        neighbourhood lists then serve)."""
        reach = hit_reach(step_length, float(self.cell_size))
        if reach is None:
            return None
        cache = tt.setdefault("hit", {})
        if reach not in cache:
            lib = _lib.load()
            g = _lib.Geometry()
            g.mesh_dims[:] = [int(x) for x in self.dims]
            g.grid_min[:] = [float(np.float32(x)) for x in self.grid_min]
            g.mesh_cell = float(np.float32(self.cell_size))
            g.tri = tt["tri"].data_ptr()
            g.tri_bs = tt["bs"].data_ptr()
            g.mesh_nb_start = tt["nbs"].data_ptr()
            g.mesh_nb_tri = tt["nbt"].data_ptr()
            n_cells = int(np.prod(self.dims))
            dev = tt["tri"].device
            counts = torch.empty(n_cells + 1, dtype=torch.int32, device=dev)
            s = _lib.stream_handle()
            _lib.check(lib.dmsim_mesh_hit_lists(g, reach, _lib.ptr(counts), None, None, s),
                       "dmsim_mesh_hit_lists")
            start = torch.zeros(n_cells + 1, dtype=torch.int64, device=dev)
            start[1:] = torch.cumsum(counts[:n_cells].to(torch.int64), 0)
            total = int(start[-1].item())
            hs = start.to(torch.int32)
            ht = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
            hb = torch.empty((max(total, 1), 4), dtype=torch.float32, device=dev)
            _lib.check(lib.dmsim_mesh_hit_lists(g, reach, _lib.ptr(hs), _lib.ptr(ht),
                                                _lib.ptr(hb), s), "dmsim_mesh_hit_lists")
            cache[reach] = (hs, ht, hb, total)
        return reach, cache[reach]

    def _desc(self, step_length, wall_mode, rho_over_D, kappa_over_D, dev):
        tt = self._tables(dev)
        g = self._base_desc(_lib.GEOM_MESH, wall_mode, rho_over_D, kappa_over_D)
        g.radius = self.radius
        g.n_tri = len(self._tri_all)
        g.mesh_dims[:] = [int(x) for x in self.dims]
        g.periodic[:] = [int(p) for p in self.periodic]
        g.max_bounces = self._MAX_BOUNCES
        g.grid_min[:] = [float(np.float32(x)) for x in self.grid_min]
        g.mesh_cell = float(np.float32(self.cell_size))
        g.vmin[:] = [float(np.float32(x)) for x in self.vmin]
        g.box[:] = [float(np.float32(x)) for x in self.L]
        g.mesh_eps = self._EPS
        g.mesh_nudge = self._NUDGE
        g.mesh_graze = self._GRAZE
        g.rho_mult_intra = self._rho_mult_intra
        g.rho_mult_extra = self._rho_mult_extra
        g.kappa_mult_out = self._kappa_mult_out
        g.kappa_mult_in = self._kappa_mult_in
        g.reject_escape = 1 if self.reject_escape else 0
        g.seed_parity = 1 if self._surface_is_closed() else 0
        g.seed_inside = 1
        g.tri = tt["tri"].data_ptr()
        g.tri_vn = tt["vn"].data_ptr()
        g.tri_bs = tt["bs"].data_ptr()
        g.mesh_cell_start = tt["cs"].data_ptr()
        g.mesh_cell_tri = tt["ct"].data_ptr()
        g.mesh_nb_start = tt["nbs"].data_ptr()
        g.mesh_nb_tri = tt["nbt"].data_ptr()
        g.mesh_nb_cent = tt["nbc"].data_ptr()
        hl = self._hit_lists(tt, float(step_length)) if self.use_hit_lists else None
        if hl is not None:
            reach, (hs, ht, hb, total) = hl
            g.mesh_hit_start = hs.data_ptr()
            g.mesh_hit_tri = ht.data_ptr()
            g.mesh_hit_bs = hb.data_ptr()
            g.mesh_hit_reach = reach
            self.n_hit_entries = total
        return g, (tt,)

    def classify_position(self, r):
        """0 = interior (inside a cell), 1 = exterior, from the nearest triangle centroid in the
        27-cell gather (mesh.py:227-254); host-side numpy."""
        r = np.atleast_2d(np.asarray(r, np.float64))
        out = np.empty(len(r), np.int32)
        rw = np.where(np.asarray(self.periodic)[None, :],
                      self.vmin + np.mod(r - self.vmin, self.L), r)
        cent = self._tri_all.astype(np.float64).mean(1)
        for i, p in enumerate(rw):
            cand = self._gather(p)
            if len(cand) == 0:
                out[i] = 1
                continue
            d = np.linalg.norm(p - cent[cand], axis=1)
            k = cand[int(np.argmin(d))]
            out[i] = 0 if np.dot(p - cent[k], self._nrm_all[k]) < 0 else 1
        return out

    def _gather(self, p):
        c = np.clip(np.floor((p - self.grid_min) / self.cell_size).astype(int), 0, self.dims - 1)
        out = []
        for d in itertools.product((-1, 0, 1), repeat=3):
            nb = np.clip(c + np.asarray(d), 0, self.dims - 1)
            cid = (nb[0] * self.dims[1] + nb[1]) * self.dims[2] + nb[2]
            out.append(self._cell_tri[self._cell_start[cid]:self._cell_start[cid + 1]])
        return np.concatenate(out).astype(np.int64)

    def init_positions(self, n_walkers, key=None, intra=True):
        """Uniform in the box, inside (``intra``) or outside the closed surface, by ray-crossing
        parity (host numpy; the walk seeds on the GPU)."""
        rng = np.random.default_rng(None if key is None else int(np.asarray(key).ravel()[-1]))
        out, need = [], n_walkers
        while need > 0:
            pts = rng.uniform(self.vmin, self.vmax, (max(need * 4, 1024), 3))
            ins = mesh_contains(self.vertices, self.faces, pts)
            out.append(pts[ins if intra else ~ins])
            need = n_walkers - sum(len(a) for a in out)
        return np.concatenate(out)[:n_walkers].astype(np.float32)

    def quality_report(self, verbose=True):
        ratio = self.edge_feature_ratio
        rep = {"n_vertices": int(len(self.vertices)), "n_faces": int(len(self.faces)),
               "n_ghost_faces": int(self.n_ghost), "feature_radius": self.radius,
               "edge_median": self.edge_median, "edge_p90": self.edge_p90,
               "edge_feature_ratio": ratio, "grid_dims": tuple(int(x) for x in self.dims),
               "grid_max_occupancy": int(self.max_occ), "grid_overflow": int(self.overflow),
               "periodic": self.periodic, "watertight": self._surface_is_closed(),
               "diffusion_noise_floor": True, "relaxivity_noise_floor": True,
               "permeability_noise_floor": bool(ratio <= _PERM_EDGE_RATIO_MAX)}
        if verbose:
            for k, v in rep.items():
                print(f"  {k:26s}: {v}")
        return rep

    @classmethod
    def from_ply(cls, path, scale=1.0, recenter=False, **kwargs):
        V, F = load_ply(path, scale=scale, recenter=recenter)
        return cls(V, F, **kwargs)


def mesh_contains(V, F, pts):
    """Inside a closed surface, by the parity of ray crossings (host numpy).  The ray leaves along
    a direction slightly off the +x axis so that it does not thread vertices or edges of meshes
    built on axis-aligned lattices."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    pts = np.atleast_2d(np.asarray(pts, np.float64))
    A, B, Cc = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    e1, e2 = B - A, Cc - A
    d = np.array([1.0, 0.0123456789, 0.0271828183])
    d /= np.linalg.norm(d)
    P = np.cross(d, e2)
    det = np.sum(P * e1, 1)
    ok = np.abs(det) > 1e-300
    out = np.zeros(len(pts), bool)
    for i in range(0, len(pts), 256):
        p = pts[i:i + 256]
        T = p[:, None, :] - A[None]
        u = np.sum(P[None] * T, 2) / np.where(ok, det, 1)[None]
        Q = np.cross(T, e1[None])
        v = (Q @ d) / np.where(ok, det, 1)[None]
        t = np.sum(Q * e2[None], 2) / np.where(ok, det, 1)[None]
        hit = ok[None] & (u >= 0) & (v >= 0) & (u + v <= 1) & (t > 0)
        out[i:i + 256] = (hit.sum(1) % 2) == 1
    return out
