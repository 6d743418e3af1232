"""Simulation entry points: ``simulate``, ``simulate_cpmg``, ``simulate_trajectories``.

Same signatures, routing and return conventions as dmipy-sim's core.py (simulate 193-762,
_replay_gap 77-106, _simulate_via_replay 115-190, _simulate_in_walker_batches 765-818,
simulate_cpmg 861-969, simulate_trajectories 972-1529), with the walk itself executed by the CUDA
kernels of libdmsim.so (one persistent launch per call; no JAX, no CPU fallback).

Engine semantics reproduced here:
  * ``engine="replay"`` (and "auto" where the reference routes to replay): the walk uses the
    producer's sub-step rule (step <= R/6, or R/25 when permeable; core.py:1089-1120) and the phase
    samples the position once per waveform sample, phi = gamma*dt*sum_t G(t).r(t)
    (trajectories.py:550-552).  The walk-once/replay split of the reference is fused into one
    kernel pass; no trajectory is materialised.
  * ``engine="fused"``: sub-steps from make_step_fn (physics.py:276-415: permeable R/25, surface
    relaxivity pore/8, meshes the collision rule, otherwise 1) and the phase accumulated at every
    sub-step with gamma*dt_sub.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .constants import GAMMA

_REPLAY_AUTO_GEOM_NAMES = frozenset({
    "FreeDiffusion", "Box1D", "Sphere", "Cylinder", "Ellipsoid", "PackedCylinders",
    "PackedSpheres", "Mesh",
})


# ------------------------------------------------------------------------------------------------
# Sub-step rules (physics.py:15-188, core.py:1089-1120)
# ------------------------------------------------------------------------------------------------
def _geometry_radius(geometry):
    """Smallest geometric radius of a geometry, or None (physics.py:15-32)."""
    R = getattr(geometry, 'radius', None)
    if R is None:
        R = getattr(geometry, 'sphere_radius', None)
    if R is None:
        radii = getattr(geometry, '_radii_np', None)
        if radii is not None and len(radii) > 0:
            R = float(np.min(radii))
    if R is None:
        inner = getattr(geometry, '_inner_radii_np', None)
        if inner is not None and len(inner) > 0 and np.any(inner > 0):
            R = float(np.min(inner[inner > 0]))
    return float(R) if R is not None else None


def permeable_sub_steps(geometry, diffusivity, dt):
    """Sub-steps so a permeable walk has step <= R/25 (physics.py:35-48)."""
    R = _geometry_radius(geometry)
    if R is None:
        return 1
    return max(1, int(np.ceil(dt / (R ** 2 / (3750.0 * diffusivity)))))


def _surface_char_radius(geometry):
    """Extra-axonal pore radius (cell area minus axons over their perimeter), else R
    (physics.py:51-69)."""
    outer = getattr(geometry, '_outer_radii_np', None)
    cell = getattr(geometry, '_cell_size', None)
    if outer is not None and cell is not None:
        outer = np.asarray(outer, float)
        outer = outer[outer > 0]
        area = float(cell) ** 2 - float(np.sum(np.pi * outer ** 2))
        perim = float(np.sum(2.0 * np.pi * outer))
        if perim > 0 and area > 0:
            return area / perim
    return _geometry_radius(geometry)


def collision_sub_steps(geometry, diffusivity, dt, frac=0.9):
    """Sub-steps so a step cannot outrun a mesh's 27-cell candidate gather (physics.py:72-95)."""
    cs = getattr(geometry, "cell_size", None)
    if cs is None or not np.isfinite(cs) or cs <= 0:
        return 1
    L = float(np.sqrt(6.0 * float(diffusivity) * float(dt)))
    ratio = L / (float(frac) * float(cs))
    return int(max(1, np.ceil(ratio ** 2))) if ratio > 1.0 else 1


def surface_sub_steps(geometry, diffusivity, dt, frac=8.0):
    """Sub-steps so the surface-relaxivity walk has step <= pore/frac (physics.py:163-188)."""
    g_frac = getattr(geometry, 'surface_substep_frac', None)
    if g_frac is not None:
        frac = g_frac
    if not frac or frac <= 0:
        return 1
    Rc = _surface_char_radius(geometry)
    if Rc is None:
        return 1
    return max(1, int(np.ceil(dt / ((Rc / frac) ** 2 / (6.0 * diffusivity)))))


def mt_sub_steps(geometry, diffusivity, dt, dwell_time, frac=8.0, dwell_frac=20.0):
    """Sub-steps of a magnetisation-transfer walk (physics.py:98-160): a mesh's collision rule,
    else steps of R/frac (the boundary local time's accuracy), and at least dwell_frac
    sub-steps per mean dwell."""
    if getattr(geometry, 'cell_size', None):
        n = collision_sub_steps(geometry, diffusivity, dt)
    else:
        R = _geometry_radius(geometry)
        n = 1 if R is None else max(1, int(np.ceil(dt / ((R / float(frac)) ** 2
                                                         / (6.0 * diffusivity)))))
    if dwell_time and dwell_time > 0:
        n = max(n, int(np.ceil(dt * float(dwell_frac) / float(dwell_time))))
    return max(1, int(n))


def replay_sub_steps(geometry, diffusivity, dt):
    """Producer-walk sub-steps: step <= R/6 (216), or R/25 (3750) when permeable (core.py:1089-1120)."""
    R = getattr(geometry, 'radius', None)
    if R is None:
        R = getattr(geometry, 'sphere_radius', None)
    if R is None:
        R = getattr(geometry, 'length', None)
    if R is None:
        radii = getattr(geometry, '_radii_np', None)
        if radii is not None and len(radii) > 0:
            R = float(np.min(radii))
    if R is None:
        inner = getattr(geometry, '_inner_radii_np', None)
        if inner is not None and len(inner) > 0:
            R = float(np.min(inner[inner > 0])) if np.any(inner > 0) else None
    if R is None:
        return 1
    div = 3750.0 if getattr(geometry, 'permeability', None) is not None else 216.0
    return max(1, int(np.ceil(dt / (float(R) ** 2 / (div * diffusivity)))))


def fused_sub_steps(geometry, diffusivity, dt):
    """The fused engine's sub-step count for this geometry (physics.py:276-415 branch order); a
    myelinated cylinder takes one step per sample (physics.py:420-680)."""
    if getattr(geometry, '_is_myelinated', False):
        return 1
    if getattr(geometry, '_is_packed_myelinated', False):
        return geometry.sub_steps(dt)
    if getattr(geometry, 'permeability', None) is not None:
        return permeable_sub_steps(geometry, diffusivity, dt)
    if getattr(geometry, 'surface_relaxivity_t2', None) is not None:
        return surface_sub_steps(geometry, diffusivity, dt)
    return collision_sub_steps(geometry, diffusivity, dt)


# ------------------------------------------------------------------------------------------------
# Routing (core.py:77-112)
# ------------------------------------------------------------------------------------------------
def _replay_gap(geometry, *, return_positions, return_compartments, return_walker_signals,
                diffusivity):
    if return_positions is not False:
        return "return_positions is a fused single-pass internal (no replay equivalent)"
    if return_compartments is not False:
        return "return_compartments is a fused single-pass internal (no replay equivalent)"
    if return_walker_signals:
        return "return_walker_signals is a fused single-pass internal (no replay equivalent)"
    if getattr(geometry, '_is_myelinated', False):
        return "MyelinatedCylinder uses a dedicated fused step kernel (no replay walk)"
    if getattr(geometry, '_is_packed_myelinated', False):
        return ("PackedMyelinatedCylinders fused single-reflection kernel is not "
                "position-parity with the multi-bounce replay walk")
    if getattr(geometry, 'permeability', None) is not None:
        return ("membrane permeability is single-pass walk semantics "
                "(fused-only; scalar replay has no exchange reservoir)")
    if getattr(geometry, '_D_comp', None) is not None:
        return "per-compartment diffusivity (Mesh intra/extra D) alters the walk (fused-only)"
    if diffusivity is None:
        return "replay needs an explicit diffusivity for the sub-step auto-tune"
    return None


def _replay_auto_allowed(geometry):
    return type(geometry).__name__ in _REPLAY_AUTO_GEOM_NAMES


# ------------------------------------------------------------------------------------------------
# The walk call
# ------------------------------------------------------------------------------------------------
class WalkResult:
    """Raw result of one device walk: FP64 ensemble sums and optional per-walker outputs."""

    def __init__(self, sums, n_walkers, status, extras):
        self.sums = sums              # (n_echo, M, 3) float64: sum w cos, sum w sin, sum (w cos)^2
        self.n_walkers = n_walkers
        self.status = status          # dict of anomaly counters
        self.extras = extras          # dict of device tensors

    @property
    def signal(self):
        return self.sums[..., 0] / max(self.n_walkers, 1)

    @property
    def stderr(self):
        n = max(self.n_walkers, 1)
        m = self.sums[..., 0] / n
        return np.sqrt(np.maximum(self.sums[..., 2] / n - m * m, 0.0) / n)


def _waveform_arrays(waveform, geometry):
    G = np.asarray(waveform.G, dtype=np.float32)                  # (M, n_t, 3)
    orient = getattr(geometry, '_orient_R', None)                 # Mesh placement (core.py:417-419)
    if orient is not None:
        G = G @ np.asarray(orient, dtype=np.float32)
    frame = geometry._frame()
    if frame is not None:                                         # g.r_lab = (R g).r_frame
        G = (G.astype(np.float64) @ frame.T).astype(np.float32)
    n_meas, n_t, _ = G.shape
    chi = getattr(waveform, 'chi_perp', None)
    chi = None if chi is None else np.asarray(chi, dtype=np.float32).reshape(n_t)
    return G, chi


def waveform_basis(G, max_rank=8, tol=1e-5):
    """Factor a measurement set into a few time shapes: G[m, t, k] = sum_j C[m, k, j] V[j, t].

    Protocols are built from a handful of waveform shapes (one PGSE lobe pair scaled and rotated
    per direction and b-value, one OGSE per frequency), so the (measurement, axis) rows of G are
    scalar multiples of at most ``max_rank`` shapes.  Each nonzero row is normalised by its value
    at its largest-magnitude sample and matched to the shapes found so far (max deviation
    <= tol).  Returns ``(V (n_t, r) float32, C (M, 3, r) float32)``, or None when more shapes are
    needed or the reconstruction misses G by more than tol * max|G| (the walk then accumulates
    every measurement's phase directly).
    """
    G = np.asarray(G, dtype=np.float64)
    M, n_t, _ = G.shape
    rows = G.transpose(0, 2, 1).reshape(M * 3, n_t)
    gmax = float(np.max(np.abs(rows))) if rows.size else 0.0
    if gmax == 0.0:
        return np.zeros((n_t, 1), np.float32), np.zeros((M, 3, 1), np.float32)
    shapes, coef = [], np.zeros((M * 3, max_rank))
    for i in range(M * 3):
        r = rows[i]
        piv = int(np.argmax(np.abs(r)))
        if abs(r[piv]) <= 1e-12 * gmax:
            continue
        s = r / r[piv]
        for j, v in enumerate(shapes):
            if np.max(np.abs(s - v)) <= tol:
                coef[i, j] = r[piv]
                break
        else:
            if len(shapes) == max_rank:
                return None
            shapes.append(s)
            coef[i, len(shapes) - 1] = r[piv]
    r_ = len(shapes)
    V = np.stack(shapes, 1)                                           # (n_t, r)
    C = coef[:, :r_]                                                  # (M*3, r)
    if np.max(np.abs(C @ V.T - rows)) > tol * gmax:
        return None
    return V.astype(np.float32), C.reshape(M, 3, r_).astype(np.float32)


class PreparedWalk:
    """A walk with every device buffer allocated once: ``launch()`` enqueues the kernels on the
    current stream (asynchronous, CUDA-graph capturable), ``result()`` synchronises and reads
    the sums back.  ``G`` is (M, n_t, 3) in the geometry's walk frame; ``r0`` (n, 3) in the walk
    frame."""

    def __init__(self, geometry, *, n_walkers, diffusivity, G, dt, sub_steps, phase_per_substep,
                 seed, chi=None, T2=None, T1=None, echo_idx=None, r0=None, walker_offset=0,
                 want_positions=False, want_walker_signals=False, want_compartments=False,
                 traj=None, traj_f16=True, want_dlog=False, want_comp_occ=False,
                 use_basis=True, allocate_workspace=True, total_walkers=None, schedule="lockstep"):
        self.lib = _lib.load()
        dev = self.dev = _lib.device()
        G = np.asarray(G, dtype=np.float32)
        n_meas, n_t, _ = G.shape
        dt = float(dt)
        S = int(sub_steps)
        dt_sub = dt / S
        gamma_dt = np.float32(GAMMA * (dt_sub if phase_per_substep else dt))
        self.myelin = bool(getattr(geometry, '_is_myelinated', False))
        self.pmyelin = bool(getattr(geometry, '_is_packed_myelinated', False))
        if self.pmyelin:
            # unit directions scaled per compartment and axon on the device; the per-step
            # log-weight (T2 per compartment, surface relaxivity) comes from the geometry
            step_l = np.float32(1.0)
            T2 = None
            want_w = geometry._has_weight() or T1 is not None
            self.gdesc, self._keep = geometry._pmyelin_desc(
                dt_sub, int(total_walkers or (n_walkers + walker_offset)), dev)
        elif self.myelin:
            # unit directions scaled per compartment on the device; T2 per compartment only (the
            # reference's myelin step ignores simulate's T2, physics.py:420-505)
            if S != 1:
                raise ValueError("a myelinated cylinder takes one step per waveform sample")
            step_l = np.float32(1.0)
            T2 = None
            want_w = geometry._has_weight() or T1 is not None
            self.gdesc = geometry._myelin_desc(dt, int(total_walkers or
                                                       (n_walkers + walker_offset)))
            self._keep = ()
        else:
            D = float(diffusivity)
            step_l = np.float32(np.sqrt(6.0 * D * dt_sub))
            rho = getattr(geometry, 'surface_relaxivity_t2', None)
            kappa = getattr(geometry, 'permeability', None)
            rho_over_D = np.float32(rho / D) if rho is not None else np.float32(0.0)
            kappa_over_D = np.float32(kappa / D) if kappa is not None else np.float32(0.0)
            want_w = (rho is not None) or (kappa is not None) or (T2 is not None) or (T1 is not None)
            wall = geometry._wall_mode(rho is not None or want_dlog)
            self.gdesc, self._keep = geometry._desc(float(step_l), wall, rho_over_D, kappa_over_D,
                                                    dev)
        echo = np.asarray([n_t - 1] if echo_idx is None else echo_idx, dtype=np.int32).ravel()
        self._echo_c = (ctypes.c_int32 * len(echo))(*echo.tolist())
        self.G_dev = torch.from_numpy(np.ascontiguousarray(G.transpose(1, 0, 2))).to(dev)
        self.chi_dev = None if chi is None else torch.from_numpy(
            np.asarray(chi, np.float32)).to(dev)
        self.r0_dev = None
        if r0 is not None:
            r0 = np.asarray(r0, dtype=np.float32)
            if r0.shape != (n_walkers, 3):
                raise ValueError(f"r0 must have shape ({n_walkers}, 3), got {r0.shape}")
            self.r0_dev = torch.from_numpy(np.ascontiguousarray(r0)).to(dev)
        p = self.p = _lib.WalkParams()
        p.n_walkers = int(n_walkers)
        p.walker_offset = int(walker_offset)
        p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        p.n_t = n_t
        p.n_meas = n_meas
        p.sub_steps = S
        p.phase_per_substep = 1 if phase_per_substep else 0
        p.step_length = step_l
        p.gamma_dt = gamma_dt
        p.t2_decay = np.float32(dt_sub / T2) if T2 is not None else 0.0
        p.t1_decay = np.float32(dt_sub / T1) if T1 is not None else 0.0
        p.has_weight = 1 if want_w else 0
        p.n_echo = len(echo)
        p.echo_idx = self._echo_c
        p.G = self.G_dev.data_ptr()
        basis = waveform_basis(G) if use_basis else None
        self.basis_rank = 0
        if basis is not None:
            V, Cb = basis
            self.V_dev = torch.from_numpy(np.ascontiguousarray(V)).to(dev)
            self.C_dev = torch.from_numpy(np.ascontiguousarray(Cb)).to(dev)
            p.basis_rank = self.basis_rank = V.shape[1]
            p.basis_V = self.V_dev.data_ptr()
            p.basis_C = self.C_dev.data_ptr()
        # packed cylinders in the basis form: "lockstep" (default) walks every lane of a warp on
        # the same sub-step; "free_flight" lets lanes step independently and skips the wall scan
        # while a walker stays inside a wall-free disc; "scan_every" is that kernel scanning every
        # sub-step (bit-identical to "free_flight")
        if schedule not in _lib.SCHEDULES:
            raise ValueError(f"schedule must be one of {sorted(_lib.SCHEDULES)}")
        p.schedule = _lib.SCHEDULES[schedule]
        p.chi = None if self.chi_dev is None else self.chi_dev.data_ptr()
        p.r0 = None if self.r0_dev is None else self.r0_dev.data_ptr()
        self.sums = torch.zeros((len(echo), n_meas, 3), dtype=torch.float64, device=dev)
        self.status = torch.zeros(_lib.STATUS_WORDS, dtype=torch.int32, device=dev)
        o = self.o = _lib.WalkOutputs()
        o.sums = self.sums.data_ptr()
        o.status = self.status.data_ptr()
        ex = self.extras = {}
        if want_positions:
            ex["pos"] = torch.empty((n_walkers, 3), dtype=torch.float32, device=dev)
            o.final_pos = ex["pos"].data_ptr()
        if want_walker_signals:
            ex["log_w"] = torch.zeros(n_walkers, dtype=torch.float32, device=dev)
            ex["phi"] = torch.empty((n_walkers, n_meas), dtype=torch.float32, device=dev)
            o.log_w = ex["log_w"].data_ptr()
            o.phi = ex["phi"].data_ptr()
        if want_compartments:
            ex["comp0"] = torch.empty(n_walkers, dtype=torch.int32, device=dev)
            ex["comp_end"] = torch.empty(n_walkers, dtype=torch.int32, device=dev)
            o.comp0 = ex["comp0"].data_ptr()
            o.comp_end = ex["comp_end"].data_ptr()
        if traj is not None:
            o.traj = traj.data_ptr()
            o.traj_f16 = 1 if traj_f16 else 0
        if want_dlog:
            ex["dlog"] = torch.empty((n_walkers, n_t), dtype=torch.float32, device=dev)
            o.dlog_unit = ex["dlog"].data_ptr()
        if want_comp_occ:
            ex["comp_occ"] = torch.empty((n_walkers, n_t), dtype=torch.float32, device=dev)
            o.comp_occ = ex["comp_occ"].data_ptr()
        self.ws_bytes = self.lib.dmsim_walk_workspace_bytes(p, self.gdesc)
        if self.ws_bytes == 0:
            _lib.check(-1, "dmsim_walk_workspace_bytes")
        # a walk that joins a batch gets its scratch from the batch's workspace instead
        self.ws = (torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
                   if allocate_workspace else None)
        self.n_walkers = int(n_walkers)
        self.n_meas, self.n_t, self.sub_steps = n_meas, n_t, S

    @property
    def launches_per_call(self):
        """Kernels one launch() enqueues: waveform re-layout, the walk (one per 64-measurement
        pass in the direct form) and the cross-block reduction."""
        if self.basis_rank:
            return 3
        mt = 16 if self.n_meas <= 16 else 32 if self.n_meas <= 32 else 64
        return 2 + (self.n_meas + mt - 1) // mt

    def launch(self):
        rc = self.lib.dmsim_walk(self.p, self.gdesc, self.o, _lib.ptr(self.ws), self.ws_bytes,
                                 _lib.stream_handle())
        _lib.check(rc, "dmsim_walk")

    def result(self):
        torch.cuda.synchronize(self.dev)
        st = self.status.cpu().numpy().astype(np.uint32)
        return WalkResult(self.sums.cpu().numpy(), self.n_walkers,
                          dict(zip(_lib.STATUS_NAMES, st.tolist())), self.extras)


def run_walk(geometry, **kw):
    """One device walk (see :class:`PreparedWalk` for the arguments); returns a
    :class:`WalkResult`."""
    w = PreparedWalk(geometry, **kw)
    w.launch()
    return w.result()


def step_kat(geometry, r, steps, u=None, wall=None, diffusivity=2e-9):
    """One device sub-step (the walk kernel's step functions) for each (r, step, u) in the walk
    frame; returns ``(r_new (n, 3), dlog_unit (n,))``.  The known-answer counterpart of one
    reference plug-in call (reflect / reflect_with_log_weight / permeate)."""
    lib = _lib.load()
    dev = _lib.device()
    r = np.ascontiguousarray(r, dtype=np.float32)
    steps = np.ascontiguousarray(steps, dtype=np.float32)
    n = len(r)
    rho = getattr(geometry, 'surface_relaxivity_t2', None)
    kappa = getattr(geometry, 'permeability', None)
    if wall is None:
        wall = geometry._wall_mode(rho is not None)
    kod = np.float32(kappa / diffusivity) if kappa is not None else 0.0
    reach = float(np.max(np.linalg.norm(steps, axis=1))) if n else 0.0
    gdesc, keep = geometry._desc(reach, wall, 0.0, kod, dev)
    t_r = torch.from_numpy(r).to(dev)
    t_s = torch.from_numpy(steps).to(dev)
    t_u = None if u is None else torch.from_numpy(np.ascontiguousarray(u, np.float32)).to(dev)
    out = torch.empty_like(t_r)
    dl = torch.empty(n, dtype=torch.float32, device=dev)
    rc = lib.dmsim_step_kat(gdesc, n, _lib.ptr(t_r), _lib.ptr(t_s), _lib.ptr(t_u), _lib.ptr(out),
                            _lib.ptr(dl), _lib.stream_handle())
    _lib.check(rc, "dmsim_step_kat")
    torch.cuda.synchronize(dev)
    del keep
    return out.cpu().numpy(), dl.cpu().numpy()


def _to_lab(geometry, pos):
    frame = geometry._frame()
    if frame is None:
        return pos
    return (pos.astype(np.float64) @ frame).astype(np.float32)


def _to_frame(geometry, r):
    frame = geometry._frame()
    r = np.asarray(r, dtype=np.float32)
    if frame is None:
        return r
    return (r.astype(np.float64) @ frame.T).astype(np.float32)


def _check_gpu(require_gpu):
    if require_gpu is False:
        return
    _lib.device()


# ------------------------------------------------------------------------------------------------
# Public API
# ------------------------------------------------------------------------------------------------
def simulate(n_walkers, diffusivity=None, waveform=None, geometry=None, seed=123, T2=None, T1=None,
             return_positions=False, return_compartments=False, return_walker_signals=False,
             r0=None, walker_batch_size=None, require_gpu=None, engine="auto"):
    """Monte-Carlo diffusion signal (core.py:193-762).

    Returns ``signals`` (n_meas,) float32 = Re<exp(log_w) exp(i phi)> (x0.5 for a stimulated echo),
    followed, as requested, by positions ((n, 3) final or (n, n_t, 3) 'full'), compartment
    (origin, final or full) and per-walker (log_w (n,), phi (n, n_meas)).
    """
    if return_compartments not in (False, 'final', 'full'):
        raise ValueError("return_compartments must be False, 'final', or 'full'; "
                         f"got {return_compartments!r}")
    if return_positions not in (False, True, 'full'):
        raise ValueError(f"return_positions must be False, True, or 'full'; got {return_positions!r}")
    if engine not in ("auto", "replay", "fused"):
        raise ValueError(f"engine must be 'auto', 'replay', or 'fused'; got {engine!r}")
    if hasattr(waveform, 'waveform'):
        waveform = waveform.waveform
    myelin = bool(getattr(geometry, '_is_myelinated', False))
    pmyelin = bool(getattr(geometry, '_is_packed_myelinated', False))
    if pmyelin and r0 is not None:
        raise NotImplementedError(
            "simulate(r0=...) is unsupported for PackedMyelinatedCylinders; it initialises walkers "
            "(and their compartments) from `seed`")
    if diffusivity is None and not (myelin or pmyelin):
        raise NotImplementedError(
            "simulate() without an explicit diffusivity is only defined for geometries carrying "
            "their own D (MyelinatedCylinder)")
    if return_compartments == 'full':
        raise NotImplementedError("return_compartments='full' is not supported by this engine")

    gap = _replay_gap(geometry, return_positions=return_positions,
                      return_compartments=return_compartments,
                      return_walker_signals=return_walker_signals, diffusivity=diffusivity)
    if engine == "replay" and gap is not None:
        raise NotImplementedError(f"engine='replay' cannot serve this run: {gap}. "
                                  "Use engine='fused' (or 'auto').")
    use_replay = engine == "replay" or (engine == "auto" and gap is None
                                        and _replay_auto_allowed(geometry))
    _check_gpu(require_gpu)

    G, chi = _waveform_arrays(waveform, geometry)
    dt = float(waveform.dt)
    if use_replay:
        S = replay_sub_steps(geometry, diffusivity, dt)
    else:
        S = fused_sub_steps(geometry, diffusivity, dt)
        if walker_batch_size is not None and walker_batch_size < n_walkers:
            return _simulate_in_walker_batches(
                n_walkers, walker_batch_size, seed=seed, diffusivity=diffusivity,
                waveform=waveform, geometry=geometry, T2=T2, T1=T1, r0=r0,
                return_positions=return_positions, return_compartments=return_compartments,
                return_walker_signals=return_walker_signals)

    n_t = G.shape[1]
    traj = None
    if return_positions == 'full':
        traj = torch.empty((n_walkers, n_t, 3), dtype=torch.float32, device=_lib.device())
    res = run_walk(geometry, n_walkers=n_walkers, diffusivity=diffusivity, G=G, dt=dt,
                   sub_steps=S, phase_per_substep=not use_replay, seed=seed, chi=chi, T2=T2, T1=T1,
                   r0=None if r0 is None else _to_frame(geometry, r0),
                   want_positions=return_positions is True,
                   want_walker_signals=bool(return_walker_signals),
                   want_compartments=return_compartments is not False, traj=traj, traj_f16=False)
    signals = res.signal[0].astype(np.float32)
    if myelin or pmyelin:
        # the walkers' log-weights start at log(spin weight): normalise by the weight sum
        # instead of the walker count (core.py:426-427)
        sw = (geometry.spin_weight_sum(n_walkers, r0) if myelin
              else geometry.spin_weight_sum(n_walkers))
        signals = (signals.astype(np.float64) * n_walkers / sw).astype(np.float32)
    if getattr(waveform, 'stimulated_echo', False):
        signals = signals * np.float32(0.5)
    out = [signals]
    if return_positions == 'full':
        out.append(_to_lab(geometry, traj.cpu().numpy().reshape(-1, 3)).reshape(n_walkers, n_t, 3))
    elif return_positions:
        out.append(_to_lab(geometry, res.extras["pos"].cpu().numpy()))
    if return_compartments is not False:
        out.append(res.extras["comp0"].cpu().numpy())
        out.append(res.extras["comp_end"].cpu().numpy())
    if return_walker_signals:
        out.append(res.extras["log_w"].cpu().numpy())
        out.append(res.extras["phi"].cpu().numpy())
    return out[0] if len(out) == 1 else tuple(out)


def _simulate_in_walker_batches(n_walkers, walker_batch_size, *, seed, diffusivity, waveform,
                                geometry, T2, T1, r0, return_positions, return_compartments,
                                return_walker_signals):
    """Walker chunks with sub-seeds seed + 1 + b, recombined as a size-weighted mean
    (core.py:765-818)."""
    n_b = (n_walkers + walker_batch_size - 1) // walker_batch_size
    acc = None
    extra = []
    for b in range(n_b):
        s0 = b * walker_batch_size
        nb = min(walker_batch_size, n_walkers - s0)
        out = simulate(nb, diffusivity, waveform, geometry, seed=seed + 1 + b, T2=T2, T1=T1,
                       return_positions=return_positions,
                       return_compartments=return_compartments,
                       return_walker_signals=return_walker_signals,
                       r0=None if r0 is None else r0[s0:s0 + nb], walker_batch_size=None,
                       require_gpu=False, engine="fused")
        items = list(out) if isinstance(out, tuple) else [out]
        sig = np.asarray(items.pop(0))
        acc = sig * nb if acc is None else acc + sig * nb
        extra.append(items)
    res = [acc / n_walkers]
    for k in range(len(extra[0])):
        res.append(np.concatenate([e[k] for e in extra], axis=0))
    return res[0] if len(res) == 1 else tuple(res)


def simulate_mixture(compartments, waveform, seed=123):
    """Compartments without exchange (core.py:821-858): each dict (``fraction``, ``n_walkers``,
    ``diffusivity``, ``geometry``) is walked on its own by ``simulate`` with seed + its index,
    and the signals are summed weighted by the fractions, which must sum to 1."""
    total = sum(c['fraction'] for c in compartments)
    if abs(total - 1.0) > 1e-6:
        raise ValueError(f"Compartment fractions must sum to 1, got {total}")
    signal = None
    for i, c in enumerate(compartments):
        s = c['fraction'] * simulate(n_walkers=c['n_walkers'], diffusivity=c['diffusivity'],
                                     waveform=waveform, geometry=c['geometry'], seed=seed + i)
        signal = s if signal is None else signal + s
    return signal


def simulate_cpmg(n_walkers, diffusivity, waveform, geometry, *, T2=None, seed=123,
                  walker_batch_size=None, require_gpu=None):
    """Multi-echo CPMG signal (n_echoes, n_meas) from one walk (core.py:861-969): the ensemble is
    reduced only at the echo samples instead of materialising the (n, n_t, n_meas) trace."""
    _check_gpu(require_gpu)
    if getattr(geometry, '_is_myelinated', False) or getattr(geometry, '_is_packed_myelinated',
                                                            False):
        raise NotImplementedError("myelinated cylinders are walked by simulate() only (the "
                                  "reference's CPMG path has no myelin step rule)")
    if hasattr(waveform, 'waveform'):
        waveform = waveform.waveform
    echo = getattr(waveform, 'echo_indices', None)
    if echo is None:
        raise ValueError("simulate_cpmg needs a multi-echo waveform with echo_indices set; "
                         "build it with dmipy_sim.cpmg(...).")
    echo = np.asarray(echo, dtype=int)
    if walker_batch_size is not None and walker_batch_size < n_walkers:
        n_b = (n_walkers + walker_batch_size - 1) // walker_batch_size
        acc = None
        for b in range(n_b):
            nb = min(walker_batch_size, n_walkers - b * walker_batch_size)
            s = simulate_cpmg(nb, diffusivity, waveform, geometry, T2=T2, seed=seed + 1 + b,
                              walker_batch_size=None, require_gpu=False)
            acc = s * nb if acc is None else acc + s * nb
        return acc / n_walkers
    G, chi = _waveform_arrays(waveform, geometry)
    S = fused_sub_steps(geometry, diffusivity, float(waveform.dt))
    order = np.argsort(echo, kind="stable")
    uniq, inv = np.unique(echo[order], return_inverse=True)
    res = run_walk(geometry, n_walkers=n_walkers, diffusivity=diffusivity, G=G,
                   dt=float(waveform.dt), sub_steps=S, phase_per_substep=True, seed=seed, chi=chi,
                   T2=T2, echo_idx=uniq)
    sig = res.signal.astype(np.float32)                 # (n_unique, M)
    out = np.empty((len(echo), G.shape[0]), dtype=np.float32)
    out[order] = sig[inv]
    return out


def simulate_trajectories(n_walkers, diffusivity, geometry, T_max, dt_save, seed=42,
                          walker_batch_size=50_000, save_relaxation_data=False, require_gpu=None,
                          r0=None, kappa_MT=0.0, dwell_time=0.0, equilibrate_binding="auto",
                          compress=None):
    """Walk once and return the positions after every saved step (core.py:972-1529).

    Returns ``(trajectories (n, n_t, 3) float16, dt_actual, sub_steps, dt_sim)`` and, with
    ``save_relaxation_data``, also ``dlog_boundary_unit (n, n_t) float16`` and ``comp_traj``
    (float16 occupancy of compartment 1 for a permeable Cylinder/Sphere, int8 zeros otherwise).

    ``compress=K`` returns a compressed master instead (core.py:1370-1407, 1503-1517): the first
    K orthonormal DCT-II bands of every walker's float32 path (``pos_modes`` (n, K, 3)) and, with
    ``save_relaxation_data``, the boundary channel as its cumulative endpoint and detrended bands
    (``blt_endpoint`` (n,), ``blt_modes`` (n, K)) plus the raw ``comp_traj``.  The projection
    runs on the GPU per walker batch; the raw trajectory never leaves the device.
    """
    if kappa_MT and kappa_MT > 0:
        raise NotImplementedError("magnetisation-transfer binding walks are not supported")
    if getattr(geometry, '_is_myelinated', False) or getattr(geometry, '_is_packed_myelinated',
                                                            False):
        raise NotImplementedError("myelinated cylinders are walked by simulate() only (the packed "
                                  "producer's magnetisation-transfer walk is not built here)")
    if compress is not None:
        return _simulate_trajectories_compressed(
            n_walkers, diffusivity, geometry, T_max, dt_save, seed, walker_batch_size,
            save_relaxation_data, require_gpu, r0, int(compress))
    _check_gpu(require_gpu)
    n_t = int(round(T_max / dt_save)) + 1
    dt_actual = T_max / (n_t - 1)
    S = replay_sub_steps(geometry, diffusivity, dt_actual)
    dt_sim = dt_actual / S
    dev = _lib.device()
    traj = torch.empty((n_walkers, n_t, 3), dtype=torch.float16, device=dev)
    perm2 = (getattr(geometry, 'permeability', None) is not None
             and type(geometry).__name__ in ("Cylinder", "Sphere"))
    G = np.zeros((1, n_t, 3), dtype=np.float32)
    res = run_walk(geometry, n_walkers=n_walkers, diffusivity=diffusivity, G=G, dt=dt_actual,
                   sub_steps=S, phase_per_substep=False, seed=seed,
                   r0=None if r0 is None else _to_frame(geometry, r0), traj=traj, traj_f16=True,
                   want_dlog=save_relaxation_data and hasattr(geometry, "_desc"),
                   want_comp_occ=save_relaxation_data and perm2)
    t = traj.float().cpu().numpy()
    t = _to_lab(geometry, t.reshape(-1, 3)).reshape(n_walkers, n_t, 3).astype(np.float16)
    if not save_relaxation_data:
        return t, dt_actual, S, dt_sim
    dlog = res.extras["dlog"].cpu().numpy().astype(np.float16)
    if perm2:
        comp = res.extras["comp_occ"].cpu().numpy().astype(np.float16)
    else:
        comp = np.zeros((n_walkers, n_t), dtype=np.int8)
    return t, dt_actual, S, dt_sim, dlog, comp


def _simulate_trajectories_compressed(n_walkers, diffusivity, geometry, T_max, dt_save, seed,
                                      walker_batch_size, save_relaxation_data, require_gpu, r0,
                                      K):
    """simulate_trajectories(compress=K): walk each walker batch with a float32 trajectory
    export, project it onto the DCT-II bands on the device (dmsim_project_modes), keep only the
    bands.  Walkers are keyed by their global index, so the batches partition one walk."""
    from . import compression as _cx
    if K < 1:
        raise ValueError(f"compress must be a positive mode count, got {K}")
    _check_gpu(require_gpu)
    n_t = int(round(T_max / dt_save)) + 1
    dt_actual = T_max / (n_t - 1)
    S = replay_sub_steps(geometry, diffusivity, dt_actual)
    dev = _lib.device()
    Kc = min(K, n_t)
    batch = max(1, int(walker_batch_size or n_walkers))
    perm2 = (getattr(geometry, 'permeability', None) is not None
             and type(geometry).__name__ in ("Cylinder", "Sphere"))
    want_dlog = save_relaxation_data and hasattr(geometry, "_desc")
    r0f = None if r0 is None else _to_frame(geometry, r0)
    G = np.zeros((1, n_t, 3), dtype=np.float32)
    pos_modes = np.empty((n_walkers, Kc, 3), np.float32)
    blt_end = np.zeros(n_walkers, np.float32) if save_relaxation_data else None
    blt_modes = np.zeros((n_walkers, Kc), np.float32) if save_relaxation_data else None
    comp = None
    if save_relaxation_data:
        comp = np.zeros((n_walkers, n_t), np.float16 if perm2 else np.int8)
    for b0 in range(0, n_walkers, batch):
        nb = min(batch, n_walkers - b0)
        traj = torch.empty((nb, n_t, 3), dtype=torch.float32, device=dev)
        res = run_walk(geometry, n_walkers=nb, diffusivity=diffusivity, G=G, dt=dt_actual,
                       sub_steps=S, phase_per_substep=False, seed=seed, walker_offset=b0,
                       r0=None if r0f is None else r0f[b0:b0 + nb], traj=traj, traj_f16=False,
                       want_dlog=want_dlog, want_comp_occ=save_relaxation_data and perm2)
        modes = _cx.project_modes(traj, Kc).cpu().numpy()
        pos_modes[b0:b0 + nb] = _to_lab(geometry, modes.reshape(-1, 3)).reshape(nb, Kc, 3)
        del traj
        if save_relaxation_data:
            if want_dlog:
                e, m = _cx.project_modes(res.extras["dlog"], Kc, cumulative=True)
                blt_end[b0:b0 + nb] = e.cpu().numpy()
                blt_modes[b0:b0 + nb] = m.cpu().numpy()
            if perm2:
                comp[b0:b0 + nb] = res.extras["comp_occ"].cpu().numpy().astype(np.float16)
    master = {"compressed": True, "method": "temporal_dct", "K": int(Kc), "n_t": int(n_t),
              "dt_traj": dt_actual, "sub_steps": S, "dt_sim": dt_actual / S,
              "pos_modes": pos_modes}
    if save_relaxation_data:
        master["blt_endpoint"] = blt_end
        master["blt_modes"] = blt_modes
        master["comp_traj"] = comp
    return master
