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

FREE, CYLINDER, SPHERE, PACKED_CYLINDERS, PACKED_SPHERES = range(5)
REFLECT, RELAX, PERMEATE = range(3)


class OrGeom(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_objects", C.c_int32), ("radius", C.c_double),
                ("L", C.c_double), ("rmin", C.c_double), ("objects", C.c_void_p),
                ("rot", C.c_double * 9), ("rot_identity", C.c_int32), ("pad", C.c_int32)]


class OrWalk(C.Structure):
    _fields_ = [("n_walkers", C.c_int64), ("walker_offset", C.c_int64), ("seed", C.c_uint64),
                ("n_t", C.c_int32), ("n_meas", C.c_int32), ("sub_steps", C.c_int32),
                ("phase_per_substep", C.c_int32), ("has_weight", C.c_int32), ("wall", C.c_int32),
                ("n_echo", C.c_int32), ("f16_positions", C.c_int32),
                ("echo_idx", C.POINTER(C.c_int32)), ("step_length", C.c_double),
                ("gamma_dt", C.c_double), ("t2_decay", C.c_double), ("t1_decay", C.c_double),
                ("rho_over_D", C.c_double), ("kappa_over_D", C.c_double)]


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
                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.or_philox.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32,
                                  C.POINTER(C.c_uint32)]
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


def geom_from(geometry):
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


def walk(g, *, n_walkers, G, dt, sub_steps, phase_per_substep, seed, wall=REFLECT, chi=None,
         T2=None, T1=None, rho_over_D=0.0, kappa_over_D=0.0, D=2e-9, echo_idx=None, r0=None,
         walker_offset=0, fp64=False, f16_positions=False, want_walkers=False, n_threads=0):
    """Restated reference walk.  ``G`` is (M, n_t, 3) in the walk frame.  Returns a dict with
    ``sums`` (n_echo, M, 3) and, with ``want_walkers``, ``pos``, ``log_w``, ``phi``."""
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
                       or wall == PERMEATE)
    p.wall = int(wall)
    p.n_echo = len(echo)
    p.f16_positions = int(bool(f16_positions))
    echo_c = (C.c_int32 * len(echo))(*echo.tolist())
    p.echo_idx = echo_c
    step_l = np.float32(np.sqrt(6.0 * D * dt_sub))
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
    if want_walkers:
        out["pos"] = np.zeros((n_walkers, 3), np.float32)
        out["log_w"] = np.zeros(n_walkers, np.float32)
        out["phi"] = np.zeros((n_walkers, M), np.float32)
        ptrs = [out["pos"].ctypes.data, out["log_w"].ctypes.data, out["phi"].ctypes.data]
    f = lib.or_walk_f64 if fp64 else lib.or_walk_f32
    rc = f(C.byref(g), C.byref(p), Gt.ctypes.data, None if chi_a is None else chi_a.ctypes.data,
           None if r0_a is None else r0_a.ctypes.data, sums.ctypes.data, *ptrs, int(n_threads))
    if rc != 0:
        raise RuntimeError("oracle walk failed")
    out["signal"] = sums[..., 0] / max(n_walkers, 1)
    return out


def philox(seed, walker, stream, j):
    lib = load()
    o = (C.c_uint32 * 4)()
    lib.or_philox(int(seed), int(walker), int(stream), int(j), o)
    return list(o)
