"""ctypes binding of ``libdmsim.so`` (the C ABI declared in ``include/dmsim.h``).

The structures below mirror the C structs field for field.  Device memory is owned by PyTorch;
only raw pointers cross the boundary.  There is no CPU fallback: a missing library or a missing
GPU raises.
"""
import ctypes as C
import os
from pathlib import Path

import torch

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libdmsim.so"

DMSIM_ABI_VERSION = 13
TILE_WALKERS = 320

(GEOM_FREE, GEOM_CYLINDER, GEOM_SPHERE, GEOM_PACKED_CYLINDERS, GEOM_PACKED_SPHERES, GEOM_MESH,
 GEOM_MYELIN, GEOM_PMYELIN, GEOM_BOX1D, GEOM_SLAB, GEOM_SHELL, GEOM_ELLIPSOID) = range(12)
WALL_REFLECT, WALL_RELAX, WALL_PERMEATE = range(3)
SCHED_LOCKSTEP, SCHED_FREE_FLIGHT, SCHED_SCAN_EVERY = range(3)
SCHEDULES = {"lockstep": SCHED_LOCKSTEP, "free_flight": SCHED_FREE_FLIGHT,
             "scan_every": SCHED_SCAN_EVERY}

STATUS_NAMES = ("nonfinite", "clamped", "init_fail", "bounce_budget", "escape_reject",
                "wait_timeout", "graze_fp64", "transmit")
STATUS_WORDS = len(STATUS_NAMES)

# Symbols every build of the library exports (the C ABI of include/dmsim.h).
EXPORTED = ("dmsim_version", "dmsim_last_error", "dmsim_walk_workspace_bytes", "dmsim_walk",
            "dmsim_walk_noalloc", "dmsim_step_kat", "dmsim_replay_workspace_bytes",
            "dmsim_replay", "dmsim_batch_create", "dmsim_batch_bind", "dmsim_batch_launch",
            "dmsim_batch_info", "dmsim_batch_destroy", "dmsim_gemm_bf16", "dmsim_mlp_forward",
            "dmsim_mlp_pack",
            "dmsim_mlp_head", "dmsim_rowdot_bf16", "dmsim_sum_f32", "dmsim_adamw",
            "dmsim_adam_advance", "dmsim_mesh_neighbourhoods", "dmsim_mesh_hit_lists",
            "dmsim_project_modes",
            "dmsim_bloch_workspace_bytes", "dmsim_bloch", "dmsim_bloch_mt_workspace_bytes",
            "dmsim_bloch_mt", "dmsim_replay_bloch_workspace_bytes", "dmsim_replay_bloch",
            "dmsim_fp32_fma_peak")

EPI_STORE_F32, EPI_BIAS_GELU, EPI_GELU_BWD = range(3)


class Geometry(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("wall_mode", C.c_int32),
        ("radius", C.c_float), ("eps_detect", C.c_float), ("nudge", C.c_float),
        ("kappa_over_D", C.c_float), ("rho_over_D", C.c_float), ("L", C.c_float),
        ("n_objects", C.c_int32), ("grid_n", C.c_int32), ("cell_h", C.c_float),
        ("reach", C.c_float), ("n_cand", C.c_int32), ("need_min_image", C.c_int32),
        ("max_cell_cand", C.c_int32), ("pad2", C.c_int32),
        ("cell_start", C.c_void_p), ("cand", C.c_void_p), ("cand_obj", C.c_void_p),
        ("n_tri", C.c_int32), ("mesh_dims", C.c_int32 * 3), ("periodic", C.c_int32 * 3),
        ("max_bounces", C.c_int32), ("grid_min", C.c_float * 3), ("mesh_cell", C.c_float),
        ("vmin", C.c_float * 3), ("box", C.c_float * 3), ("mesh_eps", C.c_float),
        ("mesh_nudge", C.c_float), ("mesh_graze", C.c_float), ("rho_mult_intra", C.c_float),
        ("rho_mult_extra", C.c_float), ("kappa_mult_out", C.c_float),
        ("kappa_mult_in", C.c_float), ("reject_escape", C.c_int32), ("seed_parity", C.c_int32),
        ("seed_inside", C.c_int32), ("pad1", C.c_int32),
        ("tri", C.c_void_p), ("tri_vn", C.c_void_p), ("mesh_cell_start", C.c_void_p),
        ("mesh_cell_tri", C.c_void_p), ("mesh_nb_start", C.c_void_p), ("mesh_nb_tri", C.c_void_p),
        ("tri_bs", C.c_void_p), ("mesh_hit_start", C.c_void_p), ("mesh_hit_tri", C.c_void_p),
        ("mesh_hit_bs", C.c_void_p), ("mesh_nb_cent", C.c_void_p), ("mesh_hit_reach", C.c_float),
        ("mesh_hit_pad", C.c_int32),
        ("myelin_r_out", C.c_float), ("myelin_step", C.c_float * 3),
        ("myelin_kin_over_D", C.c_float * 3), ("myelin_kout_over_D", C.c_float * 3),
        ("myelin_t2dec", C.c_float * 3), ("myelin_logw0", C.c_float * 3),
        ("myelin_seed_n", C.c_int64 * 2),
        ("pmy_n", C.c_int32), ("pmy_nmax", C.c_int32), ("pmy_cyl", C.c_void_p),
        ("pmy_seed", C.c_void_p), ("pmy_t2dec", C.c_float * 3), ("pmy_rho_over_D", C.c_float),
        ("pmy_logw_myelin", C.c_float), ("pmy_pad", C.c_float),
        ("shell_r_out", C.c_float), ("shell_cyl", C.c_int32),
        ("ell_inv2", C.c_float * 3), ("ell_pad", C.c_float),
    ]


class WalkParams(C.Structure):
    _fields_ = [
        ("n_walkers", C.c_int64), ("walker_offset", C.c_int64), ("seed", C.c_uint64),
        ("n_t", C.c_int32), ("n_meas", C.c_int32), ("sub_steps", C.c_int32),
        ("phase_per_substep", C.c_int32), ("step_length", C.c_float), ("gamma_dt", C.c_float),
        ("t2_decay", C.c_float), ("t1_decay", C.c_float), ("has_weight", C.c_int32),
        ("n_echo", C.c_int32), ("echo_idx", C.POINTER(C.c_int32)), ("G", C.c_void_p),
        ("chi", C.c_void_p), ("r0", C.c_void_p), ("basis_rank", C.c_int32),
        ("schedule", C.c_int32), ("basis_V", C.c_void_p), ("basis_C", C.c_void_p),
    ]


class WalkOutputs(C.Structure):
    _fields_ = [
        ("sums", C.c_void_p), ("status", C.c_void_p), ("final_pos", C.c_void_p),
        ("log_w", C.c_void_p), ("phi", C.c_void_p), ("comp0", C.c_void_p),
        ("comp_end", C.c_void_p), ("traj", C.c_void_p), ("traj_f16", C.c_int32),
        ("pad0", C.c_int32), ("dlog_unit", C.c_void_p), ("comp_occ", C.c_void_p),
    ]


class BlochParams(C.Structure):
    _fields_ = [
        ("rf_flip", C.c_void_p), ("rf_axis", C.c_void_p), ("carrier", C.c_void_p),
        ("crush", C.c_void_p), ("m0", C.c_float), ("t1_sample", C.c_float),
        ("field_kind", C.c_int32), ("field_n", C.c_int32), ("field_tab", C.c_void_p),
        ("field_rot", C.c_float * 9), ("field_par", C.c_float * 8),
        ("field_dims", C.c_int32 * 3), ("field_gamma_dt", C.c_float),
    ]


class MtParams(C.Structure):
    _fields_ = [
        ("n_walkers", C.c_int64), ("seed", C.c_uint64), ("substep_offset", C.c_uint32),
        ("n_t", C.c_int32), ("n_meas", C.c_int32), ("n_sub", C.c_int32), ("n_echo", C.c_int32),
        ("spin", C.c_int32), ("echo_idx", C.POINTER(C.c_int32)), ("step_length", C.c_float),
        ("kappa_mt_over_D", C.c_float), ("dwell_substeps", C.c_float), ("rho_over_D", C.c_float),
        ("gamma_dt", C.c_double), ("m0", C.c_double), ("e2h", C.c_double * 2),
        ("e1h", C.c_double * 2), ("G", C.c_void_p), ("rot", C.c_void_p), ("crush", C.c_void_p),
        ("r0", C.c_void_p), ("brem_in", C.c_void_p), ("brem_out", C.c_void_p),
        ("r_end", C.c_void_p), ("occ", C.c_void_p), ("occ_total", C.c_void_p),
        ("sums", C.c_void_p), ("status", C.c_void_p), ("traj", C.c_void_p),
        ("traj_f16", C.c_int32), ("pad0", C.c_int32), ("dlog_free", C.c_void_p),
    ]


class ReplayBlochParams(C.Structure):
    _fields_ = [
        ("n_walkers", C.c_int64), ("n_t", C.c_int32), ("n_meas", C.c_int32),
        ("n_echo", C.c_int32), ("traj_f16", C.c_int32), ("traj", C.c_void_p), ("G", C.c_void_p),
        ("gamma_dt", C.c_double), ("dt_traj", C.c_double), ("e2", C.c_double),
        ("e1", C.c_double), ("inv_t2", C.c_double), ("inv_t1", C.c_double),
        ("comp", C.c_void_p), ("inv_t2_comp", C.c_void_p), ("inv_t1_comp", C.c_void_p),
        ("bound_frac", C.c_void_p), ("inv_t2_bound", C.c_double),
        ("inv_t1_bound", C.c_double), ("dphi_bound", C.c_double), ("dlog", C.c_void_p),
        ("rho_over_D", C.c_double), ("extra_phase", C.c_void_p), ("rf_start", C.c_void_p),
        ("rf_flip", C.c_void_p), ("rf_axis", C.c_void_p), ("rf_offset", C.c_void_p),
        ("rf_active", C.c_void_p), ("b1_scale", C.c_void_p), ("slice_dphi", C.c_void_p),
        ("weights", C.c_void_p), ("echo_idx", C.c_void_p), ("sums", C.c_void_p),
        ("echo_walker", C.c_void_p), ("m_last", C.c_void_p),
    ]


class BatchTuning(C.Structure):
    _fields_ = [
        ("blocks_per_sm", C.c_int32), ("tiles_per_item", C.c_int32), ("order", C.c_int32),
        ("concurrent_groups", C.c_int32), ("tab_smem_bytes", C.c_int64),
    ]


class Gemm(C.Structure):
    _fields_ = [
        ("A", C.c_void_p), ("B", C.c_void_p), ("M", C.c_int64), ("N", C.c_int32),
        ("K", C.c_int32), ("lda", C.c_int64), ("ldb", C.c_int64), ("epilogue", C.c_int32),
        ("splits", C.c_int32), ("C", C.c_void_p), ("bias", C.c_void_p), ("P", C.c_void_p),
        ("H", C.c_void_p), ("HT", C.c_void_p), ("ldht", C.c_int64), ("err", C.c_void_p),
    ]


class MlpFwd(C.Structure):
    _fields_ = [
        ("x", C.c_void_p), ("rows", C.c_int64), ("n_in", C.c_int32), ("depth", C.c_int32),
        ("shift", C.c_void_p), ("scale", C.c_void_p), ("W", C.c_void_p * 8),
        ("bias", C.c_void_p * 8), ("w_head", C.c_void_p), ("b_head", C.c_void_p),
        ("y", C.c_void_p), ("err", C.c_void_p),
    ]


_lib = None


def load():
    """Load libdmsim.so (building it first if it is missing); raises if that is impossible."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() or os.environ.get("DMSIM_REBUILD"):
        from .build import build
        build()
    lib = C.CDLL(str(LIB_PATH))
    lib.dmsim_version.restype = C.c_int
    lib.dmsim_last_error.restype = C.c_char_p
    lib.dmsim_walk_workspace_bytes.restype = C.c_size_t
    lib.dmsim_walk_workspace_bytes.argtypes = [C.POINTER(WalkParams), C.POINTER(Geometry)]
    lib.dmsim_walk.restype = C.c_int
    lib.dmsim_walk.argtypes = [C.POINTER(WalkParams), C.POINTER(Geometry), C.POINTER(WalkOutputs),
                               C.c_void_p, C.c_size_t, C.c_void_p]
    lib.dmsim_bloch_workspace_bytes.restype = C.c_size_t
    lib.dmsim_bloch_workspace_bytes.argtypes = [C.POINTER(WalkParams), C.POINTER(Geometry)]
    lib.dmsim_bloch.restype = C.c_int
    lib.dmsim_bloch.argtypes = [C.POINTER(WalkParams), C.POINTER(Geometry),
                                C.POINTER(BlochParams), C.POINTER(WalkOutputs), C.c_void_p,
                                C.c_size_t, C.c_void_p]
    lib.dmsim_bloch_mt_workspace_bytes.restype = C.c_size_t
    lib.dmsim_bloch_mt_workspace_bytes.argtypes = [C.POINTER(MtParams), C.POINTER(Geometry)]
    lib.dmsim_bloch_mt.restype = C.c_int
    lib.dmsim_bloch_mt.argtypes = [C.POINTER(MtParams), C.POINTER(Geometry), C.c_void_p,
                                   C.c_size_t, C.c_void_p]
    lib.dmsim_replay_bloch_workspace_bytes.restype = C.c_size_t
    lib.dmsim_replay_bloch_workspace_bytes.argtypes = [C.POINTER(ReplayBlochParams)]
    lib.dmsim_replay_bloch.restype = C.c_int
    lib.dmsim_replay_bloch.argtypes = [C.POINTER(ReplayBlochParams), C.c_void_p, C.c_size_t,
                                       C.c_void_p]
    lib.dmsim_fp32_fma_peak.restype = C.c_int
    lib.dmsim_fp32_fma_peak.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.dmsim_walk_noalloc.restype = C.c_int
    lib.dmsim_walk_noalloc.argtypes = [C.POINTER(WalkParams), C.POINTER(Geometry),
                                       C.POINTER(WalkOutputs), C.c_void_p]
    lib.dmsim_step_kat.restype = C.c_int
    lib.dmsim_step_kat.argtypes = [C.POINTER(Geometry), C.c_int64, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.dmsim_replay_workspace_bytes.restype = C.c_size_t
    lib.dmsim_replay_workspace_bytes.argtypes = [C.c_int64, C.c_int32, C.c_int32]
    lib.dmsim_replay.restype = C.c_int
    lib.dmsim_replay.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_int32, C.c_void_p,
                                 C.c_int32, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_size_t, C.c_void_p]
    lib.dmsim_batch_create.restype = C.c_int
    lib.dmsim_batch_create.argtypes = [C.c_int32, C.POINTER(WalkParams), C.POINTER(Geometry),
                                       C.POINTER(WalkOutputs), C.POINTER(BatchTuning),
                                       C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
    lib.dmsim_batch_bind.restype = C.c_int
    lib.dmsim_batch_bind.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.dmsim_batch_launch.restype = C.c_int
    lib.dmsim_batch_launch.argtypes = [C.c_void_p, C.c_void_p]
    lib.dmsim_batch_info.restype = C.c_int
    lib.dmsim_batch_info.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    lib.dmsim_batch_destroy.restype = None
    lib.dmsim_batch_destroy.argtypes = [C.c_void_p]
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    lib.dmsim_gemm_bf16.restype = C.c_int
    lib.dmsim_gemm_bf16.argtypes = [C.POINTER(Gemm), vp]
    lib.dmsim_mlp_forward.restype = C.c_int
    lib.dmsim_mlp_forward.argtypes = [C.POINTER(MlpFwd), vp]
    lib.dmsim_mlp_pack.restype = C.c_int
    lib.dmsim_mlp_pack.argtypes = [vp, i64, i32, i32, vp, vp, vp, vp, i64, vp]
    lib.dmsim_mlp_head.restype = C.c_int
    lib.dmsim_mlp_head.argtypes = [vp, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64, vp]
    lib.dmsim_rowdot_bf16.restype = C.c_int
    lib.dmsim_rowdot_bf16.argtypes = [vp, i64, i64, i64, vp, vp, vp]
    lib.dmsim_sum_f32.restype = C.c_int
    lib.dmsim_sum_f32.argtypes = [vp, i64, vp, vp]
    lib.dmsim_adamw.restype = C.c_int
    lib.dmsim_adamw.argtypes = [vp, vp, vp, vp, i32, i64, i32, vp, vp, vp, i32, vp]
    lib.dmsim_mesh_neighbourhoods.restype = C.c_int
    lib.dmsim_mesh_neighbourhoods.argtypes = [C.POINTER(Geometry), vp, vp, vp]
    lib.dmsim_mesh_hit_lists.restype = C.c_int
    lib.dmsim_mesh_hit_lists.argtypes = [C.POINTER(Geometry), C.c_float, vp, vp, vp, vp]
    lib.dmsim_adam_advance.restype = C.c_int
    lib.dmsim_adam_advance.argtypes = [vp, vp]
    lib.dmsim_project_modes.restype = C.c_int
    lib.dmsim_project_modes.argtypes = [vp, i32, i64, i32, i32, vp, i32, vp, vp, vp, vp]
    if lib.dmsim_version() != DMSIM_ABI_VERSION:
        raise RuntimeError(f"libdmsim ABI {lib.dmsim_version()} != {DMSIM_ABI_VERSION}")
    _lib = lib
    return lib


def device():
    """The CUDA device the walk runs on; raises when no GPU is visible (no CPU fallback)."""
    if not torch.cuda.is_available():
        raise RuntimeError("dmipy_sim_gb300 needs a CUDA GPU: the Monte-Carlo walk has no CPU path")
    return torch.device("cuda", torch.cuda.current_device())


def ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def check(rc, what):
    if rc != 0:
        msg = load().dmsim_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed (code {rc}): {msg}")


def stream_handle():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)
