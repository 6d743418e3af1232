"""Python handle on the CPU oracle (oracle/oracle.c) — TEST INFRASTRUCTURE ONLY.

Imported by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg as the checker;
the product package never imports it.  ``walk`` runs the restated reference walk on the host
cores (FP32 or FP64); ``plugin`` runs one reference geometry plug-in call (lab frame).
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

(FREE, CYLINDER, SPHERE, PACKED_CYLINDERS, PACKED_SPHERES, MESH, MYELIN, PMYELIN, BOX1D, SLAB,
 SHELL, ELLIPSOID) = range(12)
REFLECT, RELAX, PERMEATE = range(3)


class OrMesh(C.Structure):
    _fields_ = [("n_tri", C.c_int32), ("n_cells", C.c_int32), ("dims", C.c_int32 * 3),
                ("per", C.c_int32 * 3), ("gmin", C.c_double * 3), ("cs", C.c_double),
                ("vmin", C.c_double * 3), ("box", C.c_double * 3), ("eps", C.c_double),
                ("nudge", C.c_double), ("graze", C.c_double), ("max_bounces", C.c_int32),
                ("reject", C.c_int32), ("rho_mult_intra", C.c_double),
                ("rho_mult_extra", C.c_double), ("kappa_mult_out", C.c_double),
                ("kappa_mult_in", C.c_double), ("tri", C.c_void_p), ("vn", C.c_void_p),
                ("nrm", C.c_void_p), ("cent", C.c_void_p), ("cell_start", C.c_void_p),
                ("cell_tri", C.c_void_p)]


class OrMyelin(C.Structure):
    _fields_ = [("r_in", C.c_double), ("r_out", C.c_double), ("nudge", C.c_double),
                ("step", C.c_double * 3), ("kin", C.c_double * 3), ("kout", C.c_double * 3),
                ("t2dec", C.c_double * 3), ("logw0", C.c_double * 3)]


class OrPMyelin(C.Structure):
    _fields_ = [("n", C.c_int32), ("nmax", C.c_int32), ("L", C.c_double), ("nudge", C.c_double),
                ("rho_over_D", C.c_double), ("logw_myelin", C.c_double),
                ("t2dec", C.c_double * 3), ("cyl", C.c_void_p)]


class OrGeom(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_objects", C.c_int32), ("radius", C.c_double),
                ("L", C.c_double), ("rmin", C.c_double), ("objects", C.c_void_p),
                ("rot", C.c_double * 9), ("rot_identity", C.c_int32), ("pad", C.c_int32),
                ("mesh", C.c_void_p), ("myelin", C.c_void_p), ("pmyelin", C.c_void_p),
                ("r_out", C.c_double), ("cyl", C.c_int32), ("pad2", C.c_int32),
                ("semi", C.c_double * 3)]


class OrWalk(C.Structure):
    _fields_ = [("n_walkers", C.c_int64), ("walker_offset", C.c_int64), ("seed", C.c_uint64),
                ("n_t", C.c_int32), ("n_meas", C.c_int32), ("sub_steps", C.c_int32),
                ("phase_per_substep", C.c_int32), ("has_weight", C.c_int32), ("wall", C.c_int32),
                ("n_echo", C.c_int32), ("f16_positions", C.c_int32),
                ("echo_idx", C.POINTER(C.c_int32)), ("step_length", C.c_double),
                ("gamma_dt", C.c_double), ("t2_decay", C.c_double), ("t1_decay", C.c_double),
                ("rho_over_D", C.c_double), ("kappa_over_D", C.c_double)]


class OrBloch(C.Structure):
    _fields_ = [("rf_flip", C.c_void_p), ("rf_axis", C.c_void_p), ("carrier", C.c_void_p),
                ("crush", C.c_void_p), ("m0", C.c_double), ("e2", C.c_double),
                ("e1", C.c_double)]


class OrMt(C.Structure):
    _fields_ = [("n_walkers", C.c_int64), ("seed", C.c_uint64), ("s0", C.c_uint32),
                ("n_t", C.c_int32), ("n_meas", C.c_int32), ("n_sub", C.c_int32),
                ("n_echo", C.c_int32), ("echo_idx", C.POINTER(C.c_int32)),
                ("step_length", C.c_double), ("kod_mt", C.c_double),
                ("dwell_substeps", C.c_double), ("rho_over_D", C.c_double),
                ("gamma_dt", C.c_double), ("m0", C.c_double), ("dt", C.c_double),
                ("T2", C.c_double * 2), ("T1", C.c_double * 2), ("off", C.c_double * 2),
                ("G", C.c_void_p), ("rf_flip", C.c_void_p), ("rf_axis", C.c_void_p),
                ("carrier", C.c_void_p), ("crush", C.c_void_p), ("r0", C.c_void_p),
                ("brem0", C.c_void_p), ("r_end", C.c_void_p), ("brem_end", C.c_void_p),
                ("occ_total", C.c_void_p)]


_lib = None


def build():
    """Compile the oracle with gcc (oracle/build.sh)."""
    subprocess.run(["sh", str(HERE / "build.sh")], check=True)


def load():
    global _lib
    if _lib is None:
        src = [HERE / "oracle.c", HERE / "oracle_impl.inc", HERE / "oracle.h"]
        if not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in src):
            build()
        lib = C.CDLL(str(LIB))
        for suf in ("_f32", "_f64"):
            f = getattr(lib, "or_plugin" + suf)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrGeom), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                          C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double),
                          C.POINTER(C.c_double)]
            f = getattr(lib, "or_walk" + suf)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrGeom), C.POINTER(OrWalk), C.c_void_p, C.c_void_p, C.c_void_p,
                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        lib.or_philox.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                  C.POINTER(C.c_uint32)]
        for suf in ("_f32", "_f64"):
            f = getattr(lib, "or_bloch_mt" + suf)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrGeom), C.POINTER(OrMt), C.c_void_p, C.c_int]
        for suf in ("_f32", "_f64"):
            f = getattr(lib, "or_bloch" + suf)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrGeom), C.POINTER(OrWalk), C.POINTER(OrBloch), C.c_void_p,
                          C.c_void_p, C.c_void_p, C.c_int]
        for suf in ("_f32", "_f64"):
            f = getattr(lib, "or_pmyelin_plugin" + suf)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrGeom), C.POINTER(C.c_double), C.POINTER(C.c_double),
                          C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double),
                          C.POINTER(C.c_int), C.POINTER(C.c_double)]
        for suf in ("_f32", "_f64"):
            f = getattr(lib, "or_myelin_plugin" + suf)
            f.restype = C.c_int
            f.argtypes = [C.POINTER(OrGeom), C.POINTER(C.c_double), C.POINTER(C.c_double),
                          C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double),
                          C.POINTER(C.c_int), C.POINTER(C.c_double)]
        _lib = lib
    return _lib


def geom(kind, radius=0.0, L=0.0, objects=None, rot=None):
    """Oracle geometry.  ``objects`` (K, 4) = (cx, cy, cz, R); ``rot`` lab -> cylinder frame."""
    g = OrGeom()
    g.kind = kind
    g.radius = float(radius)
    g.L = float(L)
    keep = None
    if objects is not None:
        keep = np.ascontiguousarray(objects, dtype=np.float64)
        g.n_objects = len(keep)
        g.objects = keep.ctypes.data
        g.rmin = float(np.min(keep[:, 3]))
    R = np.eye(3) if rot is None else np.asarray(rot, dtype=np.float64)
    g.rot[:] = R.ravel().tolist()
    g.rot_identity = int(np.allclose(R, np.eye(3)))
    g._keep = keep
    return g


def _vertex_normals(V, F):
    """Area-weighted unit vertex normals (mesh.py:75-84)."""
    tv = V[F]
    cr = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
    vn = np.zeros((len(V), 3))
    for c in range(3):
        np.add.at(vn, F[:, c], cr)
    return vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)


def mesh_geom(vertices, faces, *, periodic=False, voxel_min=None, voxel_max=None,
              feature_radius=None, rho_mult=(1.0, 1.0), kappa_mult=(1.0, 1.0), permeable=False,
              cell_size=None, max_bounces=10, reject=True):
    """Oracle mesh, built from the surface the way the reference's Mesh constructor builds its
    tables (mesh.py:311-546): the box and feature radius, ghost copies of the triangles near each
    periodic face, unit face normals, area-weighted vertex normals, the uniform grid over the box
    plus one cell of margin with each triangle listed in every cell its bounding box overlaps, and
    the float32 constants EPS = 1e-7 min(L), NUDGE = max(1e-4 step, 16 EPS), GRAZE = 1e-4.
    ``rho_mult`` = (intra, extra) and ``kappa_mult`` = (out, in) are the side multipliers."""
    import itertools
    V = np.asarray(vertices, np.float64)
    F = np.asarray(faces, np.int64)
    per = (bool(periodic),) * 3 if isinstance(periodic, (bool, np.bool_)) else \
        tuple(bool(p) for p in periodic)
    vmin = np.asarray(voxel_min, np.float64) if voxel_min is not None else V.min(0)
    vmax = np.asarray(voxel_max, np.float64) if voxel_max is not None else V.max(0)
    L = vmax - vmin
    radius = float(feature_radius) if feature_radius is not None else 0.5 * float(np.min(L[L > 0]))
    step_l = radius / (25.0 if permeable else 6.0)
    cs = float(cell_size) if cell_size is not None else 4.0 * step_l
    tv, tn = V[F], _vertex_normals(V, F)[F]
    lo_t, hi_t = tv.min(1), tv.max(1)
    tris, vns = [tv], [tn]
    for combo in itertools.product((-1, 0, 1), repeat=3):
        if combo == (0, 0, 0) or any(c != 0 and not per[a] for a, c in enumerate(combo)):
            continue
        keep = np.ones(len(F), bool)
        shift = np.zeros(3)
        for a, c in enumerate(combo):
            if c < 0:
                keep &= hi_t[:, a] > vmax[a] - cs
                shift[a] = -L[a]
            elif c > 0:
                keep &= lo_t[:, a] < vmin[a] + cs
                shift[a] = L[a]
        if keep.any():
            tris.append(tv[keep] + shift)
            vns.append(tn[keep])
    tri = np.concatenate(tris)
    vn = np.concatenate(vns)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    gmin = vmin - cs
    dims = np.maximum(1, np.ceil((vmax + cs - gmin) / cs).astype(int))
    lo = np.clip(np.floor((tri.min(1) - gmin) / cs).astype(int), 0, dims - 1)
    hi = np.clip(np.floor((tri.max(1) - gmin) / cs).astype(int), 0, dims - 1)
    cells = [[] for _ in range(int(np.prod(dims)))]
    for t in range(len(tri)):
        for ix in range(lo[t, 0], hi[t, 0] + 1):
            for iy in range(lo[t, 1], hi[t, 1] + 1):
                for iz in range(lo[t, 2], hi[t, 2] + 1):
                    cells[(ix * dims[1] + iy) * dims[2] + iz].append(t)
    start = np.zeros(len(cells) + 1, np.int32)
    start[1:] = np.cumsum([len(c) for c in cells])
    ctri = np.array([t for c in cells for t in c] or [0], np.int32)
    f32 = lambda x: np.asarray(x, np.float32).astype(np.float64)   # noqa: E731
    keep = {"tri": np.ascontiguousarray(f32(tri).reshape(-1, 9)),
            "vn": np.ascontiguousarray(f32(vn).reshape(-1, 9)),
            "nrm": np.ascontiguousarray(f32(nrm)), "cent": np.ascontiguousarray(f32(tri.mean(1))),
            "start": start, "ctri": ctri}
    m = OrMesh()
    m.n_tri, m.n_cells = len(tri), len(cells)
    m.dims[:] = [int(x) for x in dims]
    m.per[:] = [int(p) for p in per]
    m.gmin[:] = f32(gmin).tolist()
    m.cs = float(np.float32(cs))
    m.vmin[:] = f32(vmin).tolist()
    m.box[:] = f32(L).tolist()
    eps = np.float32(1e-7 * float(np.min(L)))
    m.eps = float(eps)
    m.nudge = float(np.float32(max(1e-4 * step_l, 16.0 * float(eps))))
    m.graze = float(np.float32(1e-4))
    m.max_bounces = int(max_bounces)
    m.reject = int(bool(reject))
    m.rho_mult_intra, m.rho_mult_extra = (float(np.float32(x)) for x in rho_mult)
    m.kappa_mult_out, m.kappa_mult_in = (float(np.float32(x)) for x in kappa_mult)
    m.tri, m.vn = keep["tri"].ctypes.data, keep["vn"].ctypes.data
    m.nrm, m.cent = keep["nrm"].ctypes.data, keep["cent"].ctypes.data
    m.cell_start, m.cell_tri = start.ctypes.data, ctri.ctypes.data
    g = OrGeom()
    g.kind = MESH
    g.radius = radius
    g.rot[:] = np.eye(3).ravel().tolist()
    g.rot_identity = 1
    g.mesh = C.addressof(m)
    g._keep = (m, keep)
    return g


def mesh_sides(rho_intra=None, rho_extra=None, kappa_out=None, kappa_in=None):
    """(rho_mult, kappa_mult, permeable) of per-side surface properties: each multiplier is the
    side's value over the larger of the two (mesh.py:349-371)."""
    ri, re_ = float(rho_intra or 0.0), float(rho_extra or 0.0)
    ko, ki = float(kappa_out or 0.0), float(kappa_in or 0.0)
    rn, kn = max(ri, re_), max(ko, ki)
    rho = (ri / rn, re_ / rn) if rn > 0 else (1.0, 1.0)
    kap = (ko / kn, ki / kn) if kn > 0 else (1.0, 1.0)
    return rho, kap, kn > 0


def myelin_geom(inner_radius, outer_radius, D, dt, kappa_inner=None, kappa_outer=None,
                T2=(None, None, None), water_fractions=(1.0, 0.4, 1.0)):
    """Oracle myelinated cylinder for a walk with time step ``dt``: the float32 constants of
    make_myelin_step_fn (physics.py:451-503) -- step sqrt(6 D_c dt), kappa / max(D_c, 1e-30) of
    the compartment left, dt / T2_c (T2 1e6 s where unset, 0 without any), nudge 1e-4 R_in -- and
    the log water proton densities.  ``D`` = (D_intra, D_myelin, D_extra)."""
    f = np.float32
    m = OrMyelin()
    m.r_in, m.r_out = float(f(inner_radius)), float(f(outer_radius))
    m.nudge = float(f(1e-4 * inner_radius))
    dt32 = f(dt)
    Df = [f(x) for x in D]
    m.step[:] = [float(np.sqrt(f(6.0) * d * dt32)) for d in Df]
    ki, ko = f(kappa_inner or 0.0), f(kappa_outer or 0.0)
    m.kin[:] = [float(ki / max(d, f(1e-30))) for d in Df]
    m.kout[:] = [float(ko / max(d, f(1e-30))) for d in Df]
    if any(t is not None for t in T2):
        m.t2dec[:] = [float(dt32 / f(t if t is not None else 1e6)) for t in T2]
    m.logw0[:] = [float(np.log(w)) if w > 0 else -np.inf for w in water_fractions]
    g = OrGeom()
    g.kind = MYELIN
    g.radius = float(inner_radius)
    g.rot[:] = np.eye(3).ravel().tolist()
    g.rot_identity = 1
    g.myelin = C.addressof(m)
    g._keep = (m,)
    return g


def pmyelin_geom(inner_radii, outer_radii, centers, L, dt_sub, D, kappa_inner, kappa_outer,
                 N_max=128, T2=None, rho=(None, None), myelin_proton_density=0.4):
    """Oracle packed myelinated cylinders for sub-step ``dt_sub``: the float32 per-axon tables of
    make_packed_myelin_traj_step_fn (physics.py:705-740) -- steps sqrt(6 D dt_sub) of intra /
    myelin / extra water, kappa / max(D, 1e-30) for each -- T2 of axon 0 (physics.py:995-1001),
    rho / D_ref with D_ref the largest intra or extra D (1009-1018), nudge 1e-4 of the smallest
    inner radius.  ``D`` = (D_intra, D_myelin, D_extra), each scalar or per axon; ``T2`` a
    (T2_intra, T2_myelin, T2_extra) triple of scalars or None."""
    f = np.float32
    ri = np.asarray(inner_radii, np.float64)
    ro = np.asarray(outer_radii, np.float64)
    n = len(ri)
    Ds = [np.broadcast_to(np.asarray(x, np.float64), (n,)).astype(f) for x in D]
    def per_axon(x):
        return np.broadcast_to(np.asarray(0.0 if x is None else x, np.float64), (n,)).astype(f)
    ki, ko = per_axon(kappa_inner), per_axon(kappa_outer)
    dt32 = f(dt_sub)
    tab = np.zeros((n, 16))
    tab[:, 0:2] = np.asarray(centers, np.float64).astype(f)
    tab[:, 2], tab[:, 3] = ri.astype(f), ro.astype(f)
    for j, Dc in enumerate(Ds):
        tab[:, 4 + j] = np.sqrt(f(6.0) * Dc * dt32)
        Dl = np.maximum(Dc, f(1e-30))
        tab[:, 7 + j] = ki / Dl
        tab[:, 10 + j] = ko / Dl
    m = OrPMyelin()
    m.n, m.nmax = n, int(N_max)
    m.L = float(f(L))
    m.nudge = float(f(1e-4 * float(np.min(ri[ri > 0]))))
    if T2 is not None and any(t is not None for t in T2):
        m.t2dec[:] = [float(dt32 / f(t if t is not None else 1e6)) for t in T2]
    r_i, r_o = (float(np.max(per_axon(x))) for x in rho)
    rr = max(r_i, r_o)
    D_ref = float(max(np.max(Ds[0]), np.max(Ds[2])))
    m.rho_over_D = float(f(rr / D_ref)) if rr > 0 else 0.0
    m.logw_myelin = float(np.log(f(myelin_proton_density)))
    tab = np.ascontiguousarray(tab)
    m.cyl = tab.ctypes.data
    g = OrGeom()
    g.kind = PMYELIN
    g.radius = float(np.min(ri))
    g.rot[:] = np.eye(3).ravel().tolist()
    g.rot_identity = 1
    g.pmyelin = C.addressof(m)
    g._keep = (m, tab)
    return g


def pmyelin_plugin(g, r, unit, comp, u1=0.0, u2=0.0, permeate=False, fp64=False):
    """One sub-step of the packed myelin walk rule; returns (r_new (3,), comp_new, unit dlog)."""
    lib = load()
    f = lib.or_pmyelin_plugin_f64 if fp64 else lib.or_pmyelin_plugin_f32
    ri = (C.c_double * 3)(*map(float, r))
    ui = (C.c_double * 3)(*map(float, unit))
    ro = (C.c_double * 3)()
    co = C.c_int()
    dl = C.c_double()
    if f(C.byref(g), ri, ui, int(comp), int(bool(permeate)), float(u1), float(u2), ro,
         C.byref(co), C.byref(dl)) != 0:
        raise RuntimeError("oracle packed myelin step failed")
    return np.array(ro[:]), co.value, dl.value


def slab_geom(kind, length):
    """Oracle Box1D (``kind`` BOX1D) or permeable slab (SLAB, membrane at length/2)."""
    g = geom(kind, L=float(np.float32(length)))
    g.radius = float(np.float32(length / 2.0))
    return g


def shell_geom(r_inner, r_outer, cylinder=False):
    """Oracle permeable shell (membrane r_inner, reflecting wall r_outer), in the frame whose z
    axis is the cylinder's."""
    g = geom(SHELL, radius=float(np.float32(r_inner)))
    g.r_out = float(np.float32(r_outer))
    g.cyl = int(bool(cylinder))
    return g


def ellipsoid_geom(semiaxes):
    """Oracle axis-aligned ellipsoid with semi-axes (a, b, c) along x, y, z."""
    g = geom(ELLIPSOID)
    g.semi[:] = [float(x) for x in semiaxes]
    return g


def geom_from(geometry, dt=None):
    """Oracle geometry of a dmipy_sim_gb300 geometry object (walk frame)."""
    name = type(geometry).__name__
    if name == "FreeDiffusion":
        return geom(FREE)
    if name == "Cylinder":
        return geom(CYLINDER, radius=geometry.radius, rot=geometry._R)
    if name == "Sphere":
        return geom(SPHERE, radius=geometry.radius)
    if name in ("PackedCylinders", "PackedSpheres"):
        c = np.asarray(geometry._centers_np, dtype=np.float64)
        objs = np.zeros((len(c), 4))
        objs[:, :c.shape[1]] = c
        objs[:, 3] = geometry._radii_np
        objs[:, :3] = objs[:, :3].astype(np.float32)        # the device tables are float32
        kind = PACKED_CYLINDERS if name == "PackedCylinders" else PACKED_SPHERES
        return geom(kind, L=np.float32(geometry._L_float), objects=objs,
                    rot=getattr(geometry, "_R", None))
    if name == "Ellipsoid":
        return ellipsoid_geom(geometry.semiaxes)
    if name == "Box1D":
        return slab_geom(BOX1D, geometry.length)
    if name == "PermeableSlab1D":
        return slab_geom(SLAB, geometry.length)
    if name == "PermeableShell":
        return shell_geom(geometry.r_inner, geometry.r_outer, geometry.kind == "cylinder")
    if name == "PackedMyelinatedCylinders":
        if dt is None:
            raise ValueError("the oracle's packed myelin needs the walk's sub-step")
        n = geometry.N_actual
        T2 = tuple(geometry._T2[c][0] for c in ("intra", "myelin", "extra")) \
            if geometry._has_t2 else None
        return pmyelin_geom(geometry._inner_radii_np[:n], geometry._outer_radii_np[:n],
                            geometry._centers_np[:n], geometry._L_float, dt,
                            tuple(geometry._D[c][:n] for c in ("intra", "myelin", "extra")),
                            geometry._kappa_inner[:n], geometry._kappa_outer[:n],
                            N_max=geometry.N_max, T2=T2,
                            rho=(geometry._rho_inner[:n], geometry._rho_outer[:n]),
                            myelin_proton_density=geometry._myelin_proton_density)
    if name == "MyelinatedCylinder":
        if dt is None:
            raise ValueError("the oracle's myelinated cylinder needs the walk's time step")
        return myelin_geom(geometry.inner_radius, geometry.outer_radius,
                           (geometry.D_intra, geometry.D_myelin, geometry.D_extra), dt,
                           geometry.kappa_inner, geometry.kappa_outer,
                           (geometry.T2_intra, geometry.T2_myelin, geometry.T2_extra),
                           geometry.water_fractions)
    if name == "Mesh":
        return mesh_geom(geometry.vertices, geometry.faces, periodic=geometry.periodic,
                         voxel_min=geometry.vmin, voxel_max=geometry.vmax,
                         feature_radius=geometry.radius,
                         rho_mult=(geometry._rho_mult_intra, geometry._rho_mult_extra),
                         kappa_mult=(geometry._kappa_mult_out, geometry._kappa_mult_in),
                         permeable=geometry.permeability is not None,
                         cell_size=geometry.cell_size, max_bounces=geometry._MAX_BOUNCES,
                         reject=geometry.reject_escape)
    raise NotImplementedError(f"no oracle geometry for {name}")


def plugin(g, mode, r, step, rho_over_D=0.0, kappa_over_D=0.0, u=0.0, fp64=False):
    """One reference plug-in call; returns (r_new (3,), dlog)."""
    lib = load()
    f = lib.or_plugin_f64 if fp64 else lib.or_plugin_f32
    ri = (C.c_double * 3)(*map(float, r))
    si = (C.c_double * 3)(*map(float, step))
    ro = (C.c_double * 3)()
    dl = C.c_double()
    rc = f(C.byref(g), int(mode), ri, si, float(rho_over_D), float(kappa_over_D), float(u), ro,
           C.byref(dl))
    if rc != 0:
        raise RuntimeError("oracle plugin failed")
    return np.array(ro[:]), dl.value


def myelin_plugin(g, r, unit, comp, u1=0.0, u2=0.0, permeate=False, fp64=False):
    """One step of the myelinated cylinder's walk rule; returns (r_new (3,), comp_new, dt/T2)."""
    lib = load()
    f = lib.or_myelin_plugin_f64 if fp64 else lib.or_myelin_plugin_f32
    ri = (C.c_double * 3)(*map(float, r))
    ui = (C.c_double * 3)(*map(float, unit))
    ro = (C.c_double * 3)()
    co = C.c_int()
    t2 = C.c_double()
    if f(C.byref(g), ri, ui, int(comp), int(bool(permeate)), float(u1), float(u2), ro,
         C.byref(co), C.byref(t2)) != 0:
        raise RuntimeError("oracle myelin step failed")
    return np.array(ro[:]), co.value, t2.value


def walk(g, *, n_walkers, G, dt, sub_steps, phase_per_substep, seed, wall=REFLECT, chi=None,
         T2=None, T1=None, rho_over_D=0.0, kappa_over_D=0.0, D=2e-9, echo_idx=None, r0=None,
         walker_offset=0, fp64=False, f16_positions=False, want_walkers=False, n_threads=0,
         has_weight=None, step_length=None):
    """Restated reference walk.  ``G`` is (M, n_t, 3) in the walk frame.  Returns a dict with
    ``sums`` (n_echo, M, 3) and, with ``want_walkers``, ``pos``, ``log_w``, ``phi``.
    ``has_weight`` / ``step_length`` override the defaults (the myelinated cylinder walks unit
    directions scaled per compartment and weights by its own T2 and spin weights)."""
    from dmipy_sim_gb300.constants import GAMMA
    lib = load()
    G = np.asarray(G, dtype=np.float32)
    M, n_t, _ = G.shape
    Gt = np.ascontiguousarray(G.transpose(1, 0, 2))
    S = int(sub_steps)
    dt_sub = float(dt) / S
    echo = np.asarray([n_t - 1] if echo_idx is None else echo_idx, dtype=np.int32)
    p = OrWalk()
    p.n_walkers = int(n_walkers)
    p.walker_offset = int(walker_offset)
    p.seed = int(seed)
    p.n_t, p.n_meas, p.sub_steps = n_t, M, S
    p.phase_per_substep = int(bool(phase_per_substep))
    p.has_weight = int(T2 is not None or T1 is not None or rho_over_D != 0.0
                       or wall == PERMEATE) if has_weight is None else int(bool(has_weight))
    p.wall = int(wall)
    p.n_echo = len(echo)
    p.f16_positions = int(bool(f16_positions))
    echo_c = (C.c_int32 * len(echo))(*echo.tolist())
    p.echo_idx = echo_c
    step_l = np.float32(np.sqrt(6.0 * D * dt_sub)) if step_length is None else \
        np.float32(step_length)
    p.step_length = float(step_l)
    p.gamma_dt = float(np.float32(GAMMA * (dt_sub if phase_per_substep else float(dt))))
    p.t2_decay = float(np.float32(dt_sub / T2)) if T2 is not None else 0.0
    p.t1_decay = float(np.float32(dt_sub / T1)) if T1 is not None else 0.0
    p.rho_over_D = float(np.float32(rho_over_D))
    p.kappa_over_D = float(np.float32(kappa_over_D))
    chi_a = None if chi is None else np.ascontiguousarray(chi, dtype=np.float32)
    r0_a = None if r0 is None else np.ascontiguousarray(r0, dtype=np.float32)
    sums = np.zeros((len(echo), M, 3), dtype=np.float64)
    out = {"sums": sums}
    ptrs = [None, None, None]
    comp_ptr = None
    if want_walkers:
        out["pos"] = np.zeros((n_walkers, 3), np.float32)
        out["log_w"] = np.zeros(n_walkers, np.float32)
        out["phi"] = np.zeros((n_walkers, M), np.float32)
        out["comp"] = np.zeros(n_walkers, np.int32)
        ptrs = [out["pos"].ctypes.data, out["log_w"].ctypes.data, out["phi"].ctypes.data]
        comp_ptr = out["comp"].ctypes.data
    f = lib.or_walk_f64 if fp64 else lib.or_walk_f32
    rc = f(C.byref(g), C.byref(p), Gt.ctypes.data, None if chi_a is None else chi_a.ctypes.data,
           None if r0_a is None else r0_a.ctypes.data, sums.ctypes.data, *ptrs, int(n_threads),
           comp_ptr)
    if rc != 0:
        raise RuntimeError("oracle walk failed")
    norm = max(n_walkers, 1)
    if g.kind == PMYELIN:
        m = OrPMyelin.from_address(g.pmyelin)
        tab = g._keep[1]
        rr = np.asarray(r0, np.float32)
        L = np.float32(m.L)
        ci = np.full(len(rr), -1)
        cm = np.full(len(rr), -1)
        for j in range(m.n - 1, -1, -1):
            q = rr[:, :2] - tab[j, :2].astype(np.float32)
            q = q - L * np.floor(q / L + np.float32(0.5))
            d2 = np.sum(q * q, axis=1)
            ci = np.where(d2 < np.float32(tab[j, 2]) ** 2, j, ci)
            cm = np.where(d2 < np.float32(tab[j, 3]) ** 2, j, cm)
        myel = (ci < 0) & (cm >= 0)
        norm = float(np.sum(np.where(myel, np.exp(m.logw_myelin), 1.0)))
    if g.kind == MYELIN:
        # the ensemble is normalised by the sum of the spin weights (core.py:426-427)
        m = OrMyelin.from_address(g.myelin)
        q = np.sum(np.asarray(r0, np.float32)[:, :2] ** 2, axis=1)
        comp = np.where(q < np.float32(m.r_in) ** 2, 0,
                        np.where(q < np.float32(m.r_out) ** 2, 1, 2))
        norm = float(np.sum(np.exp(np.asarray(m.logw0[:]))[comp]))
    out["signal"] = sums[..., 0] / norm
    return out


def bloch(g, *, n_walkers, G, dt, sub_steps, seed, rf_flip, rf_axis, carrier=None, crush=None,
          wall=REFLECT, T2=None, T1=None, M0=1.0, rho_over_D=0.0, kappa_over_D=0.0, D=2e-9,
          echo_idx=None, r0=None, fp64=False, n_threads=0):
    """Restated vector-Bloch walk (bloch.py:109-131, 180-198).  ``G`` (M, n_t, 3) in the walk
    frame; per-sample ``rf_flip`` / ``rf_axis`` / ``carrier`` / ``crush`` in rad.  Returns the
    sums (n_echo, M, 3) of Mx, My, Mz over the walkers."""
    from dmipy_sim_gb300.constants import GAMMA
    lib = load()
    G = np.asarray(G, dtype=np.float32)
    M, n_t, _ = G.shape
    Gt = np.ascontiguousarray(G.transpose(1, 0, 2))
    S = int(sub_steps)
    dt = float(dt)
    echo = np.asarray([n_t - 1] if echo_idx is None else echo_idx, dtype=np.int32)
    p = OrWalk()
    p.n_walkers, p.seed = int(n_walkers), int(seed)
    p.n_t, p.n_meas, p.sub_steps, p.phase_per_substep = n_t, M, S, 1
    p.wall, p.n_echo = int(wall), len(echo)
    echo_c = (C.c_int32 * len(echo))(*echo.tolist())
    p.echo_idx = echo_c
    p.step_length = float(np.float32(np.sqrt(6.0 * D * dt / S)))
    p.gamma_dt = float(np.float32(GAMMA * dt / S))
    p.rho_over_D = float(np.float32(rho_over_D))
    p.kappa_over_D = float(np.float32(kappa_over_D))
    arrs = [None if a is None else np.ascontiguousarray(a, np.float32)
            for a in (rf_flip, rf_axis, carrier, crush)]
    b = OrBloch()
    b.rf_flip, b.rf_axis, b.carrier, b.crush = [None if a is None else a.ctypes.data
                                                for a in arrs]
    b.m0 = float(M0)
    b.e2 = float(np.float32(np.exp(-dt / T2))) if T2 is not None else 1.0
    b.e1 = float(np.float32(np.exp(-dt / T1))) if T1 is not None else 1.0
    r0_a = None if r0 is None else np.ascontiguousarray(r0, dtype=np.float32)
    sums = np.zeros((len(echo), M, 3), dtype=np.float64)
    f = lib.or_bloch_f64 if fp64 else lib.or_bloch_f32
    rc = f(C.byref(g), C.byref(p), C.byref(b), Gt.ctypes.data,
           None if r0_a is None else r0_a.ctypes.data, sums.ctypes.data, int(n_threads))
    if rc != 0:
        raise RuntimeError("oracle Bloch walk failed")
    return sums


def bloch_mt(g, *, n_walkers, G, dt, n_sub, seed, r0, rf_flip, rf_axis, carrier=None,
             crush=None, kappa_MT, dwell_time, D=2e-9, T2=None, T1=None, T2_bound=1e-5,
             T1_bound=1.0, off_resonance_hz=0.0, off_resonance_bound=0.0, rho=0.0, M0=1.0,
             echo_idx=None, brem0=None, s0=0, fp64=False, n_threads=0):
    """Restated magnetisation-transfer walk (bloch.py:468-553).  Returns a dict with ``sums``
    (n_echo, M, 3) of Mx, My, Mz and the walkers' ``r_end``, ``brem`` and ``occ_total``."""
    from dmipy_sim_gb300.constants import GAMMA
    lib = load()
    G = np.asarray(G, dtype=np.float32)
    M, n_t, _ = G.shape
    Gt = np.ascontiguousarray(G.transpose(1, 0, 2))
    dt = float(dt)
    dt_sub = dt / int(n_sub)
    echo = np.asarray([n_t - 1] if echo_idx is None else echo_idx, dtype=np.int32)
    p = OrMt()
    p.n_walkers, p.seed, p.s0 = int(n_walkers), int(seed), int(s0)
    p.n_t, p.n_meas, p.n_sub, p.n_echo = n_t, M, int(n_sub), len(echo)
    echo_c = (C.c_int32 * len(echo))(*echo.tolist())
    p.echo_idx = echo_c
    p.step_length = float(np.float32(np.sqrt(6.0 * D * dt_sub)))
    p.kod_mt = float(np.float32(kappa_MT / D))
    p.dwell_substeps = float(np.float32(dwell_time / dt_sub))
    p.rho_over_D = float(rho) / D
    p.gamma_dt = GAMMA * dt
    p.m0, p.dt = float(M0), dt
    p.T2[0], p.T2[1] = (0.0 if T2 is None else T2), T2_bound
    p.T1[0], p.T1[1] = (0.0 if T1 is None else T1), T1_bound
    p.off[0], p.off[1] = off_resonance_hz, off_resonance_bound
    keep = [Gt] + [None if a is None else np.ascontiguousarray(a, np.float32)
                   for a in (rf_flip, rf_axis, carrier, crush, r0, brem0)]
    p.G = Gt.ctypes.data
    p.rf_flip, p.rf_axis, p.carrier, p.crush, p.r0, p.brem0 = [
        None if a is None else a.ctypes.data for a in keep[1:]]
    out = {"r_end": np.zeros((n_walkers, 3), np.float32), "brem": np.zeros(n_walkers, np.float32),
           "occ_total": np.zeros(n_walkers, np.float32)}
    p.r_end, p.brem_end = out["r_end"].ctypes.data, out["brem"].ctypes.data
    p.occ_total = out["occ_total"].ctypes.data
    sums = np.zeros((len(echo), M, 3), dtype=np.float64)
    f = lib.or_bloch_mt_f64 if fp64 else lib.or_bloch_mt_f32
    if f(C.byref(g), C.byref(p), sums.ctypes.data, int(n_threads)) != 0:
        raise RuntimeError("oracle MT walk failed")
    out["sums"] = sums
    return out


def philox(seed, walker, stream, j):
    lib = load()
    o = (C.c_uint32 * 4)()
    lib.or_philox(int(seed), int(walker), int(stream), int(j), o)
    return list(o)
