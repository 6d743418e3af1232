/*
 * dmsim.h — C ABI of the GB300 Monte-Carlo diffusion-MRI forward walk.
 *
 * The library replaces the per-walker JAX step loop of dmipy-sim:
 *   - the fused scan body   physics.py:191-417 (make_step_fn) driven by core.py:572-727 (simulate)
 *     and core.py:861-969 (simulate_cpmg),
 *   - the walk-once producer core.py:972-1529 (simulate_trajectories),
 *   - the replay operator    trajectories.py:360-641 (replay),
 *   - the per-walker geometry plug-ins geometries.py:14-31 (reflect / reflect_with_log_weight /
 *     permeate / classify_position / init_positions) of Sphere (143-424), Cylinder (427-844),
 *     PackedCylinders (1604-2242), PackedSpheres (2343-2786) and mesh.py:257-907 (Mesh).
 *
 * Conventions
 *   - Every pointer inside the structs is a DEVICE pointer unless the field says otherwise.
 *     The caller allocates and owns every buffer, including the workspace sized by
 *     dmsim_walk_workspace_bytes(); the library allocates nothing.
 *   - Geometry-frame coordinates: the kernels walk in the geometry's native frame (cylinder axis
 *     along z, mesh native frame).  The caller rotates gradients INTO that frame and positions out
 *     of it (dmipy-sim does the same for meshes, core.py:417-419).
 *   - Return value: 0 on success, a negative DMSIM_E* code on failure; dmsim_last_error() gives a
 *     thread-local message.  Device-side anomalies never trap: they are counted in the status
 *     words (DMSIM_STATUS_*) that the caller reads back.
 *   - Streams: every call is asynchronous on the given cudaStream_t (passed as void*), re-entrant,
 *     and touches no global mutable state except the thread-local error string.
 */
#ifndef DMSIM_H
#define DMSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DMSIM_ABI_VERSION 13

/* ---- error codes ---------------------------------------------------------------------------- */
#define DMSIM_OK 0
#define DMSIM_EINVAL (-1)     /* bad argument (sizes, null pointers, unsupported combination)   */
#define DMSIM_ECUDA (-2)      /* a CUDA runtime call failed                                     */
#define DMSIM_EWORKSPACE (-3) /* workspace smaller than dmsim_walk_workspace_bytes()            */
#define DMSIM_ETOOBIG (-4)    /* a size beyond a documented maximum                             */

/* ---- device status words (uint32 counters written by the kernels) --------------------------- */
#define DMSIM_STATUS_NONFINITE 0      /* walkers whose position became NaN/Inf                  */
#define DMSIM_STATUS_CLAMPED 1        /* safety-clamp projections (geometries.py:556-559 etc.)  */
#define DMSIM_STATUS_INIT_FAIL 2      /* walkers whose rejection seeding ran out of attempts    */
#define DMSIM_STATUS_BOUNCE_BUDGET 3  /* mesh steps whose bounce budget ran out (mesh.py:662)   */
#define DMSIM_STATUS_ESCAPE_REJECT 4  /* mesh steps rejected by the leak guard (mesh.py:669)    */
#define DMSIM_STATUS_WAIT_TIMEOUT 5   /* bounded mbarrier waits that gave up                    */
#define DMSIM_STATUS_GRAZE_FP64 6     /* wall roots re-solved in FP64 at a grazing hit          */
#define DMSIM_STATUS_TRANSMIT 7       /* membrane transmissions (Powles crossings)              */
#define DMSIM_STATUS_WORDS 8

/* ---- geometry descriptor -------------------------------------------------------------------- */
enum dmsim_geom_kind {
  DMSIM_GEOM_FREE = 0,             /* geometries.py:34-45                                      */
  DMSIM_GEOM_CYLINDER = 1,         /* geometries.py:427-844, axis along frame z                */
  DMSIM_GEOM_SPHERE = 2,           /* geometries.py:143-424, centred at the origin             */
  DMSIM_GEOM_PACKED_CYLINDERS = 3, /* geometries.py:1604-2242, periodic square cell, axis z    */
  DMSIM_GEOM_PACKED_SPHERES = 4,   /* geometries.py:2343-2786, periodic cubic cell             */
  DMSIM_GEOM_MESH = 5,             /* mesh.py:257-907                                          */
  DMSIM_GEOM_MYELIN = 6,           /* geometries.py:847-1134 + physics.py:420-680, axis frame z */
  DMSIM_GEOM_PMYELIN = 7,          /* geometries.py:2860-3218 + physics.py:682-1062, periodic   */
  DMSIM_GEOM_BOX1D = 8,            /* geometries.py:48-140, walls at x = 0 and x = L           */
  DMSIM_GEOM_SLAB = 9,             /* geometries.py:3221-3300, membrane at x = L/2 in [0, L]   */
  DMSIM_GEOM_SHELL = 10,           /* geometries.py:3303-3431, membrane R_in, wall R_out       */
  DMSIM_GEOM_ELLIPSOID = 11        /* geometries.py:1137-1427, axis-aligned at the origin      */
};

enum dmsim_wall_mode {
  DMSIM_WALL_REFLECT = 0,  /* reflect()                  */
  DMSIM_WALL_RELAX = 1,    /* reflect_with_log_weight()  */
  DMSIM_WALL_PERMEATE = 2  /* permeate()                 */
};

typedef struct dmsim_geometry {
  int32_t kind;      /* enum dmsim_geom_kind */
  int32_t wall_mode; /* enum dmsim_wall_mode */
  float radius;      /* Cylinder/Sphere R; packed: R_min (m) */
  float eps_detect;  /* crossing threshold, 1e-7*R (geometries.py:219)        */
  float nudge;       /* post-collision nudge, 1e-4*R (geometries.py:220)      */
  float kappa_over_D;
  float rho_over_D; /* used only by the RELAX/PERMEATE weight channel; the walk kernel scales
                       the unit (rho/D = 1) boundary log-weight by this value */
  float L;          /* packed: periodic cell side (m) */

  /* packed objects: uniform cell list over the periodic cell [-L/2, L/2)^d.  cell c covers
     candidates cand[cell_start[c] .. cell_start[c+1]); each candidate is a float4
     (cx, cy, cz, R) already shifted to the periodic image nearest the cell.  Every object whose
     disc/ball comes within `reach` of the cell is listed. */
  int32_t n_objects;
  int32_t grid_n; /* cells per axis */
  float cell_h;   /* L / grid_n */
  float reach;    /* maximum step length + margin the lists were built for */
  int32_t n_cand;
  int32_t need_min_image; /* 1 if a cell lists two images of one object (then each candidate is
                             checked to be its object's minimum image from the walker) */
  int32_t max_cell_cand;  /* most candidates any cell lists (0: unknown).  When it is 2, every
                             walker of a warp scans two slots (a shorter list is padded with an
                             unreachable dummy), so the scan has no divergent trip count */
  int32_t pad2;
  const uint32_t* cell_start; /* grid_n^d + 1 */
  const float* cand;          /* n_cand x 4 */
  const int32_t* cand_obj;    /* n_cand: object index of each candidate (classification) */

  /* mesh (DMSIM_GEOM_MESH): triangles incl. periodic ghosts, uniform grid (CSR) */
  int32_t n_tri;
  int32_t mesh_dims[3];
  int32_t periodic[3];
  int32_t max_bounces;
  float grid_min[3];
  float mesh_cell;
  float vmin[3];
  float box[3];
  float mesh_eps;
  float mesh_nudge;
  float mesh_graze;
  float rho_mult_intra;
  float rho_mult_extra;
  float kappa_mult_out;
  float kappa_mult_in;
  int32_t reject_escape;
  int32_t seed_parity;           /* seed by ray-crossing parity (closed surface), else by the
                                    nearest-centroid classifier                              */
  int32_t seed_inside;           /* seed inside (1) or outside (0) the surface                */
  int32_t pad1;
  const float* tri;              /* n_tri x 16: A, E1 = B - A, E2 = C - A, geometric normal,
                                    centroid, 1 for an original / 0 for a periodic ghost      */
  const float* tri_vn;           /* n_tri x 12: smooth normals at A, B, C (+3 padding)        */
  const uint32_t* mesh_cell_start; /* prod(mesh_dims) + 1 (CSR)                              */
  const uint32_t* mesh_cell_tri;   /* triangle indices, each cell in increasing order         */
  const uint32_t* mesh_nb_start;   /* optional (NULL: the 27 cells are visited one by one):   */
  const uint32_t* mesh_nb_tri;     /* per cell, the distinct triangles of its 27-cell gather,
                                      from dmsim_mesh_neighbourhoods()                        */
  const float* tri_bs;             /* optional n_tri x 4: a bounding sphere (centre, radius) of
                                      each triangle; a candidate whose sphere misses the step's
                                      segment is skipped before the Moller-Trumbore test.  The
                                      radius must cover the float32 vertices (it only prunes). */
  const uint32_t* mesh_hit_start;  /* optional hit lists (NULL: the neighbourhood lists serve  */
  const uint32_t* mesh_hit_tri;    /* the hit search too): per cell, the neighbourhood list's
                                      triangles that come within mesh_hit_reach of the cell,
                                      in the same order, from dmsim_mesh_hit_lists().  Used by
                                      the nearest-hit search of a step no longer than the reach;
                                      classification always reads the neighbourhood lists.    */
  const float* mesh_hit_bs;        /* optional: tri_bs of each hit-list entry, in list order
                                      (4 floats per entry), read beside the index             */
  const float* mesh_nb_cent;       /* optional: the centroid record (tri[16 k + 12 .. 16]) of
                                      each neighbourhood-list entry, in list order, for the
                                      nearest-centroid classification                         */
  float mesh_hit_reach;            /* the reach (m) the hit lists were built for              */
  int32_t mesh_hit_pad;

  /* myelinated cylinder (DMSIM_GEOM_MYELIN): compartments 0 intra-axonal (r < radius), 1 myelin
     (radius <= r < myelin_r_out), 2 extra-axonal, r the distance from the frame z axis.  Each
     walker carries its compartment; a step is the unit direction times its compartment's
     step length, mirrored at a boundary it crosses unless a Powles draw lets it through (wall
     mode PERMEATE; REFLECT when neither boundary is permeable).  rho_over_D must be 1: the
     kernel adds -myelin_t2dec[c] (times the coherence flag) to the log-weight each step. */
  float myelin_r_out;
  float myelin_step[3];        /* sqrt(6 D_c dt) per compartment (m)                           */
  float myelin_kin_over_D[3];  /* kappa_inner / max(D_c, 1e-30), c = the compartment left        */
  float myelin_kout_over_D[3]; /* kappa_outer / max(D_c, 1e-30)                                  */
  float myelin_t2dec[3];       /* dt / T2_c (0 without per-compartment T2)                       */
  float myelin_logw0[3];       /* log of each compartment's water proton density (spin weight)   */
  int64_t myelin_seed_n[2];    /* seeding without r0: global walkers [0, n0) intra, [n0, n1)
                                  myelin, [n1, ...) extra, uniform in the disc / annuli up to
                                  2 myelin_r_out (geometries.py:928-1006)                        */

  /* packed myelinated cylinders (DMSIM_GEOM_PMYELIN): pmy_n axons in the periodic square cell of
     side L (cell [-L/2, L/2)^2, axis along frame z).  Compartment ids as the reference's: 0
     extra-axonal, 1 + k intra-axonal of axon k, pmy_nmax + 1 + k myelin of axon k.  pmy_cyl holds
     16 floats per axon: cx, cy, R_in, R_out, the step sqrt(6 D dt_sub) of its intra / myelin /
     extra water, kappa_inner / max(D, 1e-30) and kappa_outer / max(D, 1e-30) for each of the
     three, and 3 unused.  nudge is 1e-4 of the smallest R_in; rho_over_D must be 1 (the step
     returns the whole per-step log-weight). */
  int32_t pmy_n;
  int32_t pmy_nmax;
  const float* pmy_cyl;        /* pmy_n x 16 */
  const int64_t* pmy_seed;     /* 2 pmy_n + 1 range ends of the global walker index seeded
                                  intra of axon 0..n-1, then myelin of axon 0..n-1, then extra  */
  float pmy_t2dec[3];          /* dt_sub / T2 (intra, myelin, extra), 0 without T2             */
  float pmy_rho_over_D;        /* surface relaxivity rho / D_ref (0: none)                     */
  float pmy_logw_myelin;       /* log of the myelin water proton density (spin weight)          */
  float pmy_pad;

  /* the validation slabs and shell: Box1D and PermeableSlab1D use L (slab length); the shell
     uses radius (R_in, the permeable membrane), shell_r_out (the reflecting outer wall) and
     shell_cyl (1: radii measured from the frame z axis, 0: from the origin) */
  float shell_r_out;
  int32_t shell_cyl;

  /* ellipsoid (DMSIM_GEOM_ELLIPSOID): 1 / a^2, 1 / b^2, 1 / c^2 of the semi-axes along x, y, z;
     radius = the smallest semi-axis (eps_detect = 1e-7, nudge = 1e-4 of it) */
  float ell_inv2[3];
  float ell_pad;
} dmsim_geometry;

/* Walk schedules of packed cylinders in the basis phase form (dmsim_walk_params.schedule).
   LOCKSTEP (the default): every lane of a warp on the same sub-step, a wall scan on each.
   FREE_FLIGHT: lanes step independently and skip the wall scan while the walker stays inside the
   wall-free disc of its last scan; SCAN_EVERY: the same kernel with a scan on every sub-step
   (bit-identical walks: the check of the skip).  On GB300 the lock-step kernel is the faster one
   on dense packings: the independent lanes' divergence costs more than the skipped scans.
   Other geometries and forms always walk lock-step. */
enum dmsim_schedule {
  DMSIM_SCHED_LOCKSTEP = 0,
  DMSIM_SCHED_FREE_FLIGHT = 1,
  DMSIM_SCHED_SCAN_EVERY = 2
};

/* ---- walk parameters -------------------------------------------------------------------------- */
typedef struct dmsim_walk_params {
  int64_t n_walkers;     /* walkers in this call                                                */
  int64_t walker_offset; /* global index of the first walker (Philox counter; shard offset)   */
  uint64_t seed;
  int32_t n_t;               /* waveform samples                                               */
  int32_t n_meas;            /* measurements M                                                 */
  int32_t sub_steps;         /* physics sub-steps per waveform sample, S                       */
  int32_t phase_per_substep; /* 1: phi += gamma*dt_sub*g.r after every sub-step (fused engine,
                                physics.py:313); 0: phi += gamma*dt*g.r at the sample's last
                                sub-step only (walk-once + replay, trajectories.py:550-552)    */
  float step_length;         /* sqrt(6 D dt_sub)                                               */
  float gamma_dt;            /* gamma*dt_sub (fused) or gamma*dt (replay)                       */
  float t2_decay;            /* dt_sub/T2 per sub-step, 0 if none                               */
  float t1_decay;            /* dt_sub/T1 per sub-step, 0 if none                               */
  int32_t has_weight;        /* track log_w (surface relaxivity, permeability, T2, T1)          */
  int32_t n_echo;            /* emitted samples: 1 for simulate (the last), n_echoes for CPMG   */
  const int32_t* echo_idx;   /* HOST array of n_echo ascending sample indices                   */
  const float* G;            /* (n_t, n_meas, 3) float, geometry frame, T/m                     */
  const float* chi;          /* (n_t) transverse mask or NULL (all ones)                        */
  const float* r0;           /* (n_walkers, 3) geometry-frame start positions or NULL           */
  /* Shape basis of the waveform set (optional).  When basis_rank r > 0 (r <= 8, n_meas <= 512)
     the measurements are built from r time shapes, G[t, m, k] = sum_j C[m, k, j] V[t, j], and the
     walk accumulates 3 r phase moments instead of n_meas phases; G is then ignored. */
  int32_t basis_rank;
  int32_t schedule;          /* enum dmsim_schedule: how packed cylinders in the basis form are
                                walked (0, the default, is lock-step)                          */
  const float* basis_V;      /* (n_t, basis_rank)                                               */
  const float* basis_C;      /* (n_meas, 3, basis_rank)                                         */
} dmsim_walk_params;

/* ---- outputs ---------------------------------------------------------------------------------- */
typedef struct dmsim_walk_outputs {
  double* sums;      /* (n_echo, n_meas, 3): sum w cos(phi), sum w sin(phi), sum (w cos(phi))^2 */
  uint32_t* status;  /* DMSIM_STATUS_WORDS counters (accumulated, not cleared)                 */
  float* final_pos;  /* optional (n_walkers, 3) geometry frame, unfolded                         */
  float* log_w;      /* optional (n_walkers)                                                     */
  float* phi;        /* optional (n_walkers, n_meas)                                             */
  int32_t* comp0;    /* optional (n_walkers) compartment at t=0                                 */
  int32_t* comp_end; /* optional (n_walkers) compartment at the end                              */
  void* traj;        /* optional (n_walkers, n_t, 3) positions after each sample                 */
  int32_t traj_f16;  /* 1: traj is float16 (as core.py:1426-1449), 0: float32                   */
  int32_t pad0;
  float* dlog_unit;  /* optional (n_walkers, n_t) boundary log-weight per sample at rho/D = 1     */
  float* comp_occ;   /* optional (n_walkers, n_t) mean compartment id over the sample's sub-steps */
} dmsim_walk_outputs;

/* ---- entry points ----------------------------------------------------------------------------- */

/* Library ABI version (DMSIM_ABI_VERSION). */
int dmsim_version(void);

/* Thread-local message for the last failing call on this thread. */
const char* dmsim_last_error(void);

/* Measurement helper, no counterpart in the reference: enqueues one launch of a kernel that runs
   8 independent FP32 fused-multiply-add chains per thread, iters x 16 times each, on blocks x
   threads threads (threads a multiple of 32, at most 256), and stores one float into sink.  FLOPs
   per launch = blocks * threads * iters * 256; timed with events on the stream it gives this
   GPU's measured FP32 FMA rate, the denominator of the walk kernels' roofline fraction. */
int dmsim_fp32_fma_peak(int blocks, int threads, int iters, float* sink, void* stream);

/* Workspace bytes dmsim_walk() needs for these parameters on the current device
   (per-block FP64 partials of the ensemble sums).  Replaces the device memory XLA allocated for
   the vmapped scan carry (core.py:700-727). */
size_t dmsim_walk_workspace_bytes(const dmsim_walk_params* p, const dmsim_geometry* g);

/* One Monte-Carlo walk of p->n_walkers walkers through g, accumulating the ensemble sums at
   every echo sample.  Replaces the vmap(lax.scan(step_fn)) of core.py:700-727 (simulate),
   core.py:944-969 (simulate_cpmg, n_echo > 1) and the producer walk of core.py:1243-1309
   (simulate_trajectories, when o->traj is set).  o->sums is overwritten; the signal for echo e,
   measurement m is sums[(e*M+m)*3+0] / n_walkers (core.py:426-429). */
int dmsim_walk(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_walk_outputs* o,
               void* workspace, size_t workspace_bytes, void* stream);

/* The same walk as dmsim_walk for callers that cannot allocate device memory (an XLA custom call
   that only gets the buffers XLA hands it, a plug-in under a fixed device-memory budget).  It has
   no counterpart in the reference.  The caller passes inputs and outputs only; the scratch lives
   in one library-owned device array of DMSIM_NOALLOC_SCRATCH_BYTES (16 MiB) that every GPU which
   loads the library keeps until exit.  The first call on a device (with that device current)
   looks the array's address up once: make it before any stream capture.  That address holds
   until the device's context is reset (cudaDeviceReset): after a reset, do not call this entry
   point on that device again in the same process.  Calls share the array
   and it keeps the last call's contents, so calls that overlap on the GPU race: serialise them.
   A walk whose workspace (dmsim_walk_workspace_bytes) exceeds the array returns DMSIM_ETOOBIG
   without launching anything.  Allocates nothing. */
#define DMSIM_NOALLOC_SCRATCH_BYTES (16u << 20)
int dmsim_walk_noalloc(const dmsim_walk_params* p, const dmsim_geometry* g,
                       const dmsim_walk_outputs* o, void* stream);

/* Known-answer entry point of the device step functions: one geometry sub-step for each of n
   (position, step, uniform) triples, through exactly the code the walk kernel runs.  Counterpart
   of a single reference plug-in call (geometries.py: Cylinder/Sphere/PackedCylinders/PackedSpheres
   .reflect / .reflect_with_log_weight / .permeate) applied to a batch.  r_in (n, 3) are unfolded
   geometry-frame positions, steps (n, 3), u (n) the Powles uniforms (PERMEATE; may be NULL
   otherwise); writes r_out (n, 3) and dlog_unit (n) = -2 * sum of d_perp (rho/D = 1).  The cell
   list of a packed geometry must have been built with reach >= every |step|. */
int dmsim_step_kat(const dmsim_geometry* g, int64_t n, const float* r_in, const float* steps,
                   const float* u, float* r_out, float* dlog_unit, void* stream);

/* Neighbourhood lists of a mesh grid (g->mesh_dims, mesh_cell_start, mesh_cell_tri): for each
   cell, the triangles of its 27 neighbour cells (indices clamped to the grid) without repeats,
   in the order the 27-cell gather of mesh.py:208-215 visits them (neighbours in x-major order,
   each cell's triangles in increasing order, the first occurrence kept).  The walk visits each
   candidate once instead of once per grid cell it overlaps, with the same result.  Two calls:
   with nb_tri == NULL it writes each cell's list length to nb_start[0 .. n_cells); the caller
   turns the lengths into offsets (exclusive prefix sum, nb_start[n_cells] = total) and calls
   again with nb_tri of `total` entries. */
int dmsim_mesh_neighbourhoods(const dmsim_geometry* g, uint32_t* nb_start, uint32_t* nb_tri,
                              void* stream);

/* Hit lists of a mesh grid for steps no longer than `reach` (m): for each cell, the entries of its
   neighbourhood list (g->mesh_nb_start / mesh_nb_tri, from dmsim_mesh_neighbourhoods) whose
   triangle (g->tri: A, A + E1, A + E2) overlaps the cell's box widened on every side by reach
   plus a rounding margin, by a separating-axis test in float64; the cells on the grid's faces
   (which also hold the positions clamped into the grid) keep their whole list.  A step's path,
   bounces included, stays within its length of its start, so every triangle the 27-cell gather
   of mesh.py:208-215 could report as hit within the step is kept, in the gather's order.  Two
   calls, as dmsim_mesh_neighbourhoods: with hit_tri == NULL the list lengths go to
   hit_start[0 .. n_cells); then with the offsets in hit_start and hit_tri of `total` entries,
   and hit_bs (4 x `total` floats, or NULL) for the entries' bounding spheres from g->tri_bs. */
int dmsim_mesh_hit_lists(const dmsim_geometry* g, float reach, uint32_t* hit_start,
                         uint32_t* hit_tri, float* hit_bs, void* stream);

/* Replay operator on saved trajectories, trajectories.py:360-641 without relaxation terms:
   phi[m,w] = gamma_dt * sum_t G[t,m,:] . traj[w,t,:]  (trajectories.py:550-552) and
   sums[m] = (sum_w e^{log_w[w]} cos phi, sum e^{log_w} sin phi, sum (e^{log_w} cos phi)^2).
   traj is (n_walkers, n_t, 3) float16 (traj_f16=1) or float32; log_w is (n_walkers) or NULL
   (all zero); phi_out is optional (n_walkers, n_meas).  Workspace from
   dmsim_replay_workspace_bytes(). */
size_t dmsim_replay_workspace_bytes(int64_t n_walkers, int32_t n_t, int32_t n_meas);
int dmsim_replay(const void* traj, int32_t traj_f16, int64_t n_walkers, int32_t n_t,
                 const float* G, int32_t n_meas, float gamma_dt, const float* log_w,
                 double* sums, float* phi_out, void* workspace, size_t workspace_bytes,
                 void* stream);

/* ---- vector Bloch ------------------------------------------------------------------------------
   The forward vector-Bloch walk of bloch.py:212-340 (simulate_bloch without magnetisation
   transfer; a susceptibility field is optional, below): every walker carries M_m = (Mx, My, Mz)
   for each measurement m,
   starting from (0, 0, m0), and each waveform sample t applies, after the move of the walk
   (the same walk, stream and sub-steps as dmsim_walk for the same parameters):
     an RF rotation by rf_flip[t] about (cos rf_axis[t], sin rf_axis[t], 0)    (bloch.py:44-57),
     free precession of Mxy by phi_t + carrier[t] + crush[t] * u_w, with phi_t the gradient
       phase of the sample as in dmsim_walk (gamma_dt, phase_per_substep) and u_w the walker's
       crusher coordinate, uniform in [0, 1) from Philox stream 2 (bloch.py:126),
     Mxy *= exp(log-weight of the sample) (t2_decay per sub-step, rho_over_D x the boundary
       log-weight), Mz -> m0 + (Mz - m0) exp(-t1_sample)                      (bloch.py:129-131).
   p->chi must be NULL, p->t1_decay 0 and p->basis_rank 0; myelinated geometries are refused.
   o->sums (n_echo, n_meas, 3) receives sum_w Mx, sum_w My, sum_w Mz at each echo sample (after
   that sample's update); o->phi must be NULL; the other per-walker outputs are as dmsim_walk's. */
typedef struct dmsim_bloch_params {
  const float* rf_flip;  /* DEVICE (n_t): flip of the sample (rad), 0 = no pulse                 */
  const float* rf_axis;  /* DEVICE (n_t): B1 phase of the sample (rad; 0 = x, pi/2 = y)          */
  const float* carrier;  /* DEVICE (n_t) extra precession (rad: off-resonance, pulse carrier) or
                            NULL                                                                  */
  const float* crush;    /* DEVICE (n_t) crusher rate (rad per unit coordinate) or NULL          */
  float m0;              /* equilibrium longitudinal magnetisation                                */
  float t1_sample;       /* dt/T1 per waveform sample, 0 if none                                  */
  /* susceptibility field (bloch.py:126-128, susceptibility.py): evaluated at the walker's
     position after each sample, rotated into the field frame by field_rot (row-major), and added
     to its precession as field_gamma_dt * dBz.  field_kind 0 none; 1 magnetised spheres, table
     (field_n, 5) = (cx, cy, cz, (dchi B0/3) a^3, a^2); 2 hollow myelin cylinders, table
     (field_n, 8) = (cx, cy, a^2, b^2, a^4, ln(b/a), 0, 0), field_par = (L, dchi_a B0 sin^2/2,
     cos 2 alpha, sin 2 alpha, images per side, periodic); 3 a grid of field_dims (x-major,
     C order), field_par = (origin xyz, voxel xyz, periodic), trilinear. */
  int32_t field_kind, field_n;
  const float* field_tab; /* DEVICE table or grid                                                 */
  float field_rot[9];
  float field_par[8];
  int32_t field_dims[3];
  float field_gamma_dt;   /* gamma * dt                                                           */
} dmsim_bloch_params;

size_t dmsim_bloch_workspace_bytes(const dmsim_walk_params* p, const dmsim_geometry* g);
int dmsim_bloch(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_bloch_params* b,
                const dmsim_walk_outputs* o, void* workspace, size_t workspace_bytes,
                void* stream);

/* ---- magnetisation-transfer Bloch walk ---------------------------------------------------------
   The binding walk of bloch.py:343-671 (simulate_bloch with kappa_MT > 0): every sample of dt is
   n_sub sub-steps; in each a free walker takes a reflecting step of step_length (the boundary
   log-weight dl = -2 sum d_perp of the wall hits, geometries' reflect_with_log_weight), sticks
   with probability min(1, kappa_mt_over_D * (-dl)) on the third uniform of its Philox draw and
   then stays put for -ln(max(u4, 1e-20)) * dwell_substeps sub-steps (u4 the fourth uniform); a
   bound walker counts its dwell down.  With spin = 1 each walker's magnetisation M_m (FP64) is
   carried through every sub-step by a Strang split -- half relaxation with the walker's current
   pool (e2h, e1h [free, bound]), the rotation rot[t][pool] (RF nutation and off-resonance over
   one sub-step, row-major 3x3), the second half relaxation and, for a free walker that did not
   just bind, Mxy *= exp(rho_over_D * dl) -- and, after the sample's sub-steps, Mxy is rotated by
   gamma_dt * G[t, m] . r + crush[t] * u_w (u_w from Philox stream 2, as dmsim_bloch).  The
   uniforms of sub-step s come from Philox stream 0, counter substep_offset + s, so a burn-in
   (spin = 0) continued by the sequence's walk draws the walk the reference's carried keys draw.
   Geometries: cylinder, sphere, ellipsoid, Box1D, PermeableSlab1D and packed cylinders / spheres
   (their walls always reflect here).  Outputs: sums (n_echo, n_meas, 3) of Mx, My, Mz at each
   echo sample (after its update); per walker the end position, the residual dwell, the bound
   fraction per sample and its sum over the samples. */
typedef struct dmsim_mt_params {
  int64_t n_walkers;
  uint64_t seed;
  uint32_t substep_offset;  /* Philox counter of the first sub-step                             */
  int32_t n_t, n_meas, n_sub, n_echo;
  int32_t spin;             /* 1: evolve the magnetisation; 0: walk and binding only (burn-in)  */
  const int32_t* echo_idx;  /* HOST array of n_echo ascending sample indices (spin = 1)          */
  float step_length;        /* sqrt(6 D dt / n_sub)                                             */
  float kappa_mt_over_D;    /* binding reactivity over D (1/m)                                  */
  float dwell_substeps;     /* mean dwell in sub-steps                                          */
  float rho_over_D;         /* transverse surface relaxivity over D at free wall contacts       */
  double gamma_dt;          /* gamma * dt                                                       */
  double m0;                /* equilibrium longitudinal magnetisation                           */
  double e2h[2], e1h[2];    /* exp(-dt_sub / (2 T2)), exp(-dt_sub / (2 T1)): free, bound         */
  const float* G;           /* DEVICE (n_t, n_meas, 3) walk frame, T/m (spin = 1)               */
  const double* rot;        /* DEVICE (n_t, 2, 9) per-sub-step rotation, free / bound (spin = 1)*/
  const float* crush;       /* DEVICE (n_t) crusher rate or NULL                                */
  const float* r0;          /* DEVICE (n_walkers, 3) walk-frame start positions                 */
  const float* brem_in;     /* DEVICE (n_walkers) residual dwell at the start, or NULL (free)    */
  float* brem_out;          /* DEVICE (n_walkers) residual dwell at the end, or NULL            */
  float* r_end;             /* DEVICE (n_walkers, 3) end positions (unfolded) or NULL           */
  float* occ;               /* DEVICE (n_walkers, n_t) bound fraction of each sample, or NULL   */
  float* occ_total;         /* DEVICE (n_walkers) sum of the samples' bound fractions, or NULL  */
  double* sums;             /* DEVICE (n_echo, n_meas, 3), overwritten (spin = 1)               */
  uint32_t* status;         /* DEVICE DMSIM_STATUS_WORDS counters                               */
  /* the saved walk of mt_walk.py:43-239 (simulate_mt_trajectories), each optional: positions
     after every sample (unfolded), and the free-pool boundary log-weight of every sample (the
     dl of the sub-steps on which the walker was free and did not bind) */
  void* traj;               /* DEVICE (n_walkers, n_t, 3) float16 (traj_f16 = 1) or float32    */
  int32_t traj_f16;
  int32_t pad0;
  float* dlog_free;         /* DEVICE (n_walkers, n_t) or NULL                                   */
} dmsim_mt_params;

size_t dmsim_bloch_mt_workspace_bytes(const dmsim_mt_params* p, const dmsim_geometry* g);
int dmsim_bloch_mt(const dmsim_mt_params* p, const dmsim_geometry* g, void* workspace,
                   size_t workspace_bytes, void* stream);

/* ---- vector-Bloch replay of a stored walk --------------------------------------------------------
   trajectories.py:734-949 (replay_bloch): every walker's magnetisation M_m, starting at
   (0, 0, 1), is carried through the samples of its saved positions in the order: the sample's RF
   increments rf_start[t] .. rf_start[t+1] (rotation by rf_flip * b1_scale[w] about
   (cos rf_axis, sin rf_axis, 0)); precession of Mxy by gamma_dt * G[t, m] . r(t) + extra_phase
   + bound_frac * dphi_bound + rf_offset[t] + (rf_active[t] ? slice_dphi[w] : 0); Mxy *=
   exp(rho_over_D * dlog); Mxy *= E2, Mz *= E1 with E = exp(-dt_traj * rate), the rate the
   compartment's (comp, inv_t*_comp) or the constant one, blended toward the bound pool by
   bound_frac (without compartments or bound_frac, e2 / e1 are used as given).  All FP64.  At
   each echo sample sums[m][e] = (sum_w weight_w Mx, sum_w weight_w My); optional per-walker
   echoes and the last measurement's final magnetisation.  Per-walker-sample arrays are
   (n_walkers, n_t); every pointer is DEVICE memory.  The library checks counts and pointers
   only, not the contents of the device tables: the caller guarantees echo_idx strictly ascending
   in [0, n_t), rf_start non-decreasing from 0 with rf_start[n_t] <= the length of rf_flip and
   rf_axis, and every comp id < the length of inv_t2_comp / inv_t1_comp.  The Python wrapper
   (trajectories.replay_bloch) builds and checks them on the host before the upload. */
typedef struct dmsim_replay_bloch_params {
  int64_t n_walkers;
  int32_t n_t, n_meas, n_echo, traj_f16;
  const void* traj;            /* (n_walkers, n_t, 3) float16 or float32                        */
  const double* G;             /* (n_t, n_meas, 3) on the walk's sample grid                    */
  double gamma_dt, dt_traj;
  double e2, e1;               /* per-sample factors without per-sample rates                  */
  double inv_t2, inv_t1;       /* base rates (1/s) blended with bound_frac                      */
  const int32_t* comp;         /* compartment per walker-sample or NULL                         */
  const double* inv_t2_comp;   /* rates per compartment                                         */
  const double* inv_t1_comp;
  const float* bound_frac;     /* bound-pool occupancy per walker-sample or NULL                */
  double inv_t2_bound, inv_t1_bound, dphi_bound;
  const float* dlog;           /* boundary log-weight at rho/D = 1 per walker-sample or NULL     */
  double rho_over_D;
  const double* extra_phase;   /* per walker-sample phase (rad) or NULL                         */
  const int32_t* rf_start;     /* (n_t + 1) offsets into rf_flip / rf_axis                      */
  const double* rf_flip;
  const double* rf_axis;
  const double* rf_offset;     /* (n_t) pulse carrier per sample or NULL                        */
  const uint8_t* rf_active;    /* (n_t) 1 while a pulse is on                                    */
  const double* b1_scale;      /* (n_walkers) or NULL                                           */
  const double* slice_dphi;    /* (n_walkers) slice-select phase per sample, or NULL            */
  const double* weights;       /* (n_walkers) or NULL (all 1)                                   */
  const int32_t* echo_idx;     /* (n_echo) ascending sample indices                             */
  double* sums;                /* (n_meas, n_echo, 2)                                           */
  double* echo_walker;         /* (n_meas, n_echo, n_walkers, 2) or NULL                        */
  double* m_last;              /* (3, n_walkers) of the last measurement, or NULL               */
} dmsim_replay_bloch_params;

size_t dmsim_replay_bloch_workspace_bytes(const dmsim_replay_bloch_params* p);
int dmsim_replay_bloch(const dmsim_replay_bloch_params* p, void* workspace,
                       size_t workspace_bytes, void* stream);

/* Temporal-mode projection, the compressed trajectory export of simulate_trajectories(compress=K)
   (core.py:1370-1407) and the temporal_dct / boundary_dct codecs of compression.py:55-62, 224-249:
   out[w,k,c] = sum_t basis[k,t] * x[w,t,c] with x (n_walkers, n_t, n_ch) float16 (x_f16 = 1) or
   float32, n_ch 1 or 3, basis (K, n_t) float32, out (n_walkers, K, n_ch) float32.  With ramp
   (n_t floats; n_ch must be 1) the series is replaced by its detrended running sum
   B_t - B_{n_t-1} ramp_t before the projection and B_{n_t-1} is written to endpoint[w].
   Kahan-compensated FP32 sums; no workspace. */
int dmsim_project_modes(const void* x, int32_t x_f16, int64_t n_walkers, int32_t n_t, int32_t n_ch,
                        const float* basis, int32_t K, const float* ramp, float* endpoint,
                        float* out, void* stream);

/* ---- batched walks ---------------------------------------------------------------------------
   Many independent walks (instances: geometry, waveform, rho, kappa, n_walkers, n_t, seed each
   their own) in one enqueue.  No counterpart in the reference, where each instance is one
   simulate() call (core.py:193-762) and a study loops over them on the host.

   Instances whose waveform comes as a shape basis (basis_rank > 0) are walked by persistent
   kernels, one per (geometry kind, wall mode, basis width, cell list in shared memory) group,
   whose blocks pull work items -- DMSIM_TILE_WALKERS x tiles_per_item walkers of one instance --
   from a queue in device memory until it is empty; groups run on forked streams so the tail of
   one overlaps the next.  Each work item owns a partial-sum slice, and a final kernel reduces
   every instance's slices in a fixed order: the sums do not depend on the schedule, and an
   instance gives exactly the sums a dmsim_walk() of the same parameters gives.  Instances
   without a basis run as plain dmsim_walk() launches inside the same enqueue.

   Lifecycle: dmsim_batch_create() validates and plans (host only; returns the workspace size),
   dmsim_batch_bind() uploads the instance tables into the caller's workspace (once),
   dmsim_batch_launch() enqueues the whole batch (asynchronous, no host synchronisation, no
   allocation: capturable in a CUDA graph), dmsim_batch_destroy() frees the host plan.
   Every device pointer of the p / g / o arrays must stay valid while the plan is in use (their
   contents may change between launches); echo_idx is read at create time. */
#define DMSIM_TILE_WALKERS 320

typedef struct dmsim_batch_tuning {
  int32_t blocks_per_sm;     /* resident blocks per SM of each persistent grid; 0 = occupancy max */
  int32_t tiles_per_item;    /* walker tiles per work item; 0 = 1                               */
  int32_t order;             /* 0 = the given instance order; 1 = costliest instances first     */
  int32_t concurrent_groups; /* 1 = groups on forked streams; 0 = one after another            */
  int64_t tab_smem_bytes;    /* cell lists up to this size are staged in shared memory; 0 = 96 KiB */
} dmsim_batch_tuning;

typedef struct dmsim_batch dmsim_batch; /* opaque host-side plan */

int dmsim_batch_create(int32_t n, const dmsim_walk_params* p, const dmsim_geometry* g,
                       const dmsim_walk_outputs* o, const dmsim_batch_tuning* tuning,
                       dmsim_batch** out, size_t* workspace_bytes);
int dmsim_batch_bind(dmsim_batch* b, void* workspace, size_t workspace_bytes, void* stream);
int dmsim_batch_launch(const dmsim_batch* b, void* stream);
/* Plan summary: persistent kernel groups, instances on the plain path, work items, and the
   kernels one dmsim_batch_launch() enqueues. */
int dmsim_batch_info(const dmsim_batch* b, int32_t* n_groups, int32_t* n_single, int64_t* n_items,
                     int32_t* n_kernels);
void dmsim_batch_destroy(dmsim_batch* b);

/* ---- surrogate MLP ---------------------------------------------------------------------------
   Building blocks of the learned surrogate (an MLP from substrate parameters and a waveform
   encoding to the signal).  No counterpart in the reference.  The GEMM runs on the tcgen05 tensor
   cores: C[M, N] = A[M, K] . B[N, K]^T with A, B row-major bf16 (K contiguous), fp32
   accumulation in tensor memory, and one of these fused epilogues:
     STORE_F32  C (M, N) fp32; with `splits` > 1, split s of K writes C + s*M*N;
     BIAS_GELU  P = acc + bias[n] (fp32, stored when P is given), H = gelu(P) as bf16 (M, N) and,
                when HT is given, its transpose (N, ldht);
     GELU_BWD   H = acc * gelu'(P[m, n]) as bf16 (M, N) (+ transpose), P read-only (M, N) fp32.
   GELU is x * Phi(x) with the exact normal CDF.  N must be a multiple of 128, K of 64;
   row strides are in elements.  `err` is a device word incremented by a CTA whose bounded waits
   gave up (zero after a healthy run). */
#define DMSIM_EPI_STORE_F32 0
#define DMSIM_EPI_BIAS_GELU 1
#define DMSIM_EPI_GELU_BWD 2

typedef struct dmsim_gemm {
  const void* A;  /* bf16 (M, lda) */
  const void* B;  /* bf16 (N, ldb) */
  int64_t M;
  int32_t N, K;
  int64_t lda, ldb;
  int32_t epilogue;
  int32_t splits;
  float* C;
  const float* bias;
  float* P;
  void* H;   /* bf16 (M, N) */
  void* HT;  /* bf16 (N, ldht) or NULL */
  int64_t ldht;
  uint32_t* err;
} dmsim_gemm;

int dmsim_gemm_bf16(const dmsim_gemm* g, void* stream);

/* The surrogate's whole forward pass in one launch (no counterpart in the reference: the learned
   surrogate is this project's own): y = head(gelu(... gelu(pack(x) W_0^T + b_0) ...)) for depth
   hidden layers of width 256 (GELU in its tanh form), on 128-row tiles kept on chip -- packed
   inputs and activations in shared memory, the accumulator in tensor memory, the bf16 weights
   streamed from L2 by TMA.  x (rows, n_in) fp32 with n_in <= 128, normalised as
   (x - shift) * scale (either may be NULL) and zero padded to 128 columns; W[0] bf16 (256, 128),
   W[l > 0] bf16 (256, 256), all 16-byte aligned; bias[l] and w_head fp32 (256), 16-byte
   aligned; b_head one fp32 value in device memory; y (rows) fp32.  A tensor-core pipeline that
   stalls past its bounded waits adds 1 to *err (device memory). */
typedef struct dmsim_mlp_fwd {
  const float* x;
  int64_t rows;
  int32_t n_in, depth;
  const float* shift;
  const float* scale;
  const void* W[8];
  const float* bias[8];
  const float* w_head;
  const float* b_head;
  float* y;
  uint32_t* err;
} dmsim_mlp_fwd;

int dmsim_mlp_forward(const dmsim_mlp_fwd* f, void* stream);

/* Input packing: out[r, c] = bf16((x[r, c] - shift[c]) * scale[c]) for c < features, 0 up to kp;
   out_t (kp, ldt) is the optional transpose.  shift / scale may be NULL. */
int dmsim_mlp_pack(const float* x, int64_t rows, int32_t features, int32_t kp, const float* shift,
                   const float* scale, void* out, void* out_t, int64_t ldt, void* stream);

/* Linear head y = H w + b over the last hidden layer H (rows, n) bf16.  With a target: the
   squared-error gradient dy = 2 (y - target) / rows, sqerr = (y - target)^2 and the seed
   gradient dP = dy * w * gelu'(P) of the last layer (bf16 (rows, n) and optional transpose). */
int dmsim_mlp_head(const void* H, int64_t rows, int32_t n, const float* w, const float* b,
                   float* y, const float* target, float* dy, float* sqerr, const float* P,
                   void* dP, void* dP_t, int64_t ldt, void* stream);

/* out[i] = sum_j X[i, j] * v[j] (v NULL: plain row sums) over bf16 X (rows, ld); fixed order. */
int dmsim_rowdot_bf16(const void* X, int64_t rows, int64_t cols, int64_t ld, const float* v,
                      float* out, void* stream);

/* out[0] = sum of x[0..n) in a fixed order (FP64 accumulation). */
int dmsim_sum_f32(const float* x, int64_t n, float* out, void* stream);

/* AdamW (decoupled weight decay) on fp32 master weights p with moments m, v; the gradient is the
   sum of `splits` consecutive partial buffers of n values.  hp (device) = [lr, beta1, beta2, eps,
   weight_decay, step]; dmsim_adam_advance adds 1 to the step.  W (rows, cols) and WT (cols, rows)
   receive the bf16 copies when given. */
int dmsim_adamw(float* p, float* m, float* v, const float* grad, int32_t splits, int64_t n,
                int32_t cols, const float* hp, void* W, void* WT, int32_t rows, void* stream);
int dmsim_adam_advance(float* hp, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DMSIM_H */
