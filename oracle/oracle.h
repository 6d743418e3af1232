/*
 * CPU oracle of the dmipy-sim Monte-Carlo walk — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-walker algorithm, used by tests/, smoke() and the
 * bench's CPU baseline as the checker; the product (libdmsim.so) never links or calls it.
 * Compiled twice: *_f32 restates the reference's FP32 arithmetic statement by statement, *_f64
 * is the same algorithm in FP64 (the "FP64 rerun" that the GPU's FP32 error is stated against).
 *
 * What it follows (paths inside the dmipy-sim source tree):
 *   step direction / sub-steps / phase / log-weight   physics.py:191-417
 *   Sphere reflect / reflect_with_log_weight / permeate   geometries.py:197-264, 266-318, 320-424
 *   Cylinder reflect / reflect_with_log_weight / permeate geometries.py:493-563, 565-653, 655-801
 *   PackedCylinders reflect / rwlw / permeate             geometries.py:1746-1884, 1886-2016, 2018-2183
 *   PackedSpheres reflect / rwlw / permeate               geometries.py:2445-2537, 2539-2631, 2633-2756
 *   Mesh reflect / reflect_with_log_weight / permeate     mesh.py:637-671, 673-705, 707-743
 *   MyelinatedCylinder step (own walk rule)               physics.py:506-677
 *   PackedMyelinatedCylinders step + fused weights         physics.py:742-930, 1034-1056
 *   Box1D reflect / reflect_with_log_weight               geometries.py:90-140
 *   PermeableSlab1D reflect / rwlw / permeate             geometries.py:3270-3300
 *   PermeableShell permeate / reflect                     geometries.py:3366-3431
 *   Ellipsoid reflect / rwlw / permeate                   geometries.py:1184-1392
 *     (wrap 203-206, 27-cell gather 208-215, Moller-Trumbore 561-569, bounce 599-635,
 *      nearest-centroid classification 227-254, leak guard 578-597)
 *   ensemble Re<w e^{i phi}>                              core.py:426-429; replay FP64 phase
 *                                                         trajectories.py:550-552, 634
 * It tests every object of a packed substrate (no cell list) with the reference's min-image
 * arithmetic on unfolded positions, exactly as the reference does.  Random numbers come from the
 * Philox stream contract of dmipy_sim_gb300/csrc/philox.cuh so a walk here and on the GPU is the
 * same walk, walker for walker.
 */
#ifndef DMSIM_ORACLE_H
#define DMSIM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_FREE = 0, OR_CYLINDER = 1, OR_SPHERE = 2, OR_PACKED_CYLINDERS = 3, OR_PACKED_SPHERES = 4,
       OR_MESH = 5, OR_MYELIN = 6, OR_PMYELIN = 7, OR_BOX1D = 8, OR_SLAB = 9, OR_SHELL = 10,
       OR_ELLIPSOID = 11 };
enum { OR_REFLECT = 0, OR_RELAX = 1, OR_PERMEATE = 2 };

/* A triangle mesh as the reference's Mesh holds it (mesh.py:311-546): every triangle including the
   periodic ghosts, float32 values stored as double; the uniform grid's cell lists in CSR form (each
   cell's triangles in increasing order, as the reference's buckets are filled). */
typedef struct {
  int32_t n_tri, n_cells;
  int32_t dims[3], per[3];
  double gmin[3], cs, vmin[3], box[3];
  double eps, nudge, graze;
  int32_t max_bounces, reject;
  double rho_mult_intra, rho_mult_extra, kappa_mult_out, kappa_mult_in;
  const double* tri;         /* n_tri x 9: vertices A, B, C */
  const double* vn;          /* n_tri x 9: smooth normals at A, B, C */
  const double* nrm;         /* n_tri x 3: unit geometric normal */
  const double* cent;        /* n_tri x 3: centroid */
  const int32_t* cell_start; /* n_cells + 1 */
  const int32_t* cell_tri;
} or_mesh;

/* A myelinated cylinder (geometries.py:847-1134) as make_myelin_step_fn sees it (physics.py:451-
   503): inner / outer radius, nudge 1e-4 R_in, and per compartment (intra, myelin, extra) the step
   length sqrt(6 D dt), kappa_inner / max(D, 1e-30), kappa_outer / max(D, 1e-30), dt / T2 (0
   without T2) and the log of the water proton density (float32 values stored as double). */
typedef struct {
  double r_in, r_out, nudge;
  double step[3], kin[3], kout[3], t2dec[3], logw0[3];
} or_myelin;

/* Packed myelinated cylinders (geometries.py:2860-3218) as make_packed_myelin_traj_step_fn and
   make_packed_myelin_step_fn see them (physics.py:705-740, 995-1025): n axons in the periodic
   cell of side L, compartment ids 0 extra / 1 + k intra / nmax + 1 + k myelin; per axon 16
   numbers: cx, cy, R_in, R_out, the intra / myelin / extra steps sqrt(6 D dt_sub), and
   kappa_inner / max(D, 1e-30), kappa_outer / max(D, 1e-30) for intra, myelin, extra water
   (float32 values stored as double). */
typedef struct {
  int32_t n, nmax;
  double L, nudge, rho_over_D, logw_myelin;
  double t2dec[3];   /* dt_sub / T2 of intra, myelin, extra (axon 0's values), 0 without T2 */
  const double* cyl; /* n x 16 */
} or_pmyelin;

typedef struct {
  int32_t kind;
  int32_t n_objects;
  double radius;      /* Cylinder/Sphere radius */
  double L;           /* packed cell side */
  double rmin;        /* packed: smallest radius (sets EPS and NUDGE) */
  const double* objects; /* n_objects x 4: (cx, cy, cz, R) */
  double rot[9];      /* lab -> cylinder frame (row-major), used by or_plugin only */
  int32_t rot_identity;
  int32_t pad;
  const or_mesh* mesh;   /* OR_MESH only */
  const or_myelin* myelin; /* OR_MYELIN only */
  const or_pmyelin* pmyelin; /* OR_PMYELIN only */
  double r_out;   /* OR_SHELL: the reflecting outer wall (radius = the permeable membrane) */
  int32_t cyl;    /* OR_SHELL: radii from the frame z axis (1) or the origin (0) */
  int32_t pad2;
  double semi[3]; /* OR_ELLIPSOID: semi-axes along x, y, z */
} or_geom;

typedef struct {
  int64_t n_walkers, walker_offset;
  uint64_t seed;
  int32_t n_t, n_meas, sub_steps, phase_per_substep;
  int32_t has_weight, wall, n_echo, f16_positions; /* f16: replay phase from float16-rounded positions */
  const int32_t* echo_idx;
  double step_length, gamma_dt, t2_decay, t1_decay, rho_over_D, kappa_over_D;
} or_walk_params;

/* One reference plug-in call in the LAB frame: mode OR_REFLECT (reflect), OR_RELAX
   (reflect_with_log_weight with rho_over_D) or OR_PERMEATE (permeate with kappa_over_D,
   rho_over_D and the Bernoulli uniform u).  Returns 0 on success. */
int or_plugin_f32(const or_geom* g, int mode, const double* r, const double* step,
                  double rho_over_D, double kappa_over_D, double u, double* r_out, double* dlog);
int or_plugin_f64(const or_geom* g, int mode, const double* r, const double* step,
                  double rho_over_D, double kappa_over_D, double u, double* r_out, double* dlog);

/* One step of the myelinated cylinder's own walk rule (physics.py:528-677) in its frame: start r in
   compartment comp, unit direction `unit`, Powles uniforms u1 (inner) / u2 (outer) when permeate.
   Writes the end point, the new compartment and dt/T2 of the new compartment. */
int or_myelin_plugin_f32(const or_geom* g, const double* r, const double* unit, int comp,
                         int permeate, double u1, double u2, double* r_out, int* comp_out,
                         double* t2dec);
int or_myelin_plugin_f64(const or_geom* g, const double* r, const double* unit, int comp,
                         int permeate, double u1, double u2, double* r_out, int* comp_out,
                         double* t2dec);

/* One sub-step of the packed myelin walk rule (physics.py:742-930) in the cylinder frame:
   in-cell start r, encoded compartment comp, unit direction, Powles uniforms u1 / u2 (permeate).
   Writes the in-cell end point, the new compartment and the unit boundary log-weight. */
int or_pmyelin_plugin_f32(const or_geom* g, const double* r, const double* unit, int comp,
                          int permeate, double u1, double u2, double* r_out, int* comp_out,
                          double* dlog);
int or_pmyelin_plugin_f64(const or_geom* g, const double* r, const double* unit, int comp,
                          int permeate, double u1, double u2, double* r_out, int* comp_out,
                          double* dlog);

/* A full walk in the geometry frame.  G is (n_t, n_meas, 3) float32, chi (n_t) or NULL, r0
   (n_walkers, 3) or NULL (seeded on the Philox seeding stream; a mesh needs r0).  sums (n_echo, n_meas, 3) is
   overwritten with sum w cos(phi), sum w sin(phi), sum (w cos(phi))^2.  final_pos (n, 3), log_w
   (n), phi (n, n_meas) are optional.  n_threads <= 0 uses every core.  comp_end (n) is optional:
   the walker's final compartment for the myelinated geometries (0 intra, 1 myelin, 2 extra). */
int or_walk_f32(const or_geom* g, const or_walk_params* p, const float* G, const float* chi,
                const float* r0, double* sums, float* final_pos, float* log_w, float* phi,
                int n_threads, int32_t* comp_end);
int or_walk_f64(const or_geom* g, const or_walk_params* p, const float* G, const float* chi,
                const float* r0, double* sums, float* final_pos, float* log_w, float* phi,
                int n_threads, int32_t* comp_end);

/* Vector-Bloch walk (bloch.py:109-131, 180-198 with the RF rotation of bloch.py:44-57): the walk
   of or_walk (same draws, sub-steps and steps; p->chi, t1_decay and t2_decay unused) with each
   walker's magnetisation of every measurement updated at every sample in the reference's order:
   RF rotation, precession by the sample's gradient phase plus carrier[t] + crush[t] * u_w,
   Mxy *= e2 * exp(-2 rho_over_D sum d_perp), Mz -> m0 + (Mz - m0) e1.  u_w is the walker's
   crusher coordinate (Philox stream 2, counter 0, first word).  The per-sample arrays are host
   arrays of n_t floats; carrier and crush may be NULL.  sums (n_echo, M, 3) receives sum Mx,
   sum My, sum Mz at each echo sample. */
typedef struct {
  const float* rf_flip;
  const float* rf_axis;
  const float* carrier;
  const float* crush;
  double m0, e2, e1;
} or_bloch_params;
int or_bloch_f32(const or_geom* g, const or_walk_params* p, const or_bloch_params* b,
                 const float* G, const float* r0, double* sums, int n_threads);
int or_bloch_f64(const or_geom* g, const or_walk_params* p, const or_bloch_params* b,
                 const float* G, const float* r0, double* sums, int n_threads);

/* Magnetisation-transfer Bloch walk (bloch.py:468-553), restated eagerly: per sub-step one
   Philox draw (stream 0, counter s0 + s: x, y the direction, z the binding test, w the dwell); a
   free walker takes a reflecting step with its boundary log-weight dl and sticks with
   min(1, kod_mt * (-dl)), then stays put for -ln(max(w, 1e-20)) * dwell_substeps sub-steps; the
   FP64 magnetisation takes half relaxation of the walker's pool, the exact rotation about
   (f cos ax, f sin ax, dphi_pool) (f = flip / n_sub, dphi the pool's carrier over a sub-step),
   the second half relaxation and, for a free walker that did not just bind, the factor
   exp(rho_over_D dl); after the sub-steps Mxy turns by gamma_dt G.r + crush u_w.  T2/T1 of 0
   mean none.  Per-sample arrays are host arrays of n_t floats (carrier, crush may be NULL);
   r0 is required, brem0 optional.  sums (n_echo, M, 3): sum Mx, My, Mz at each echo sample. */
typedef struct {
  int64_t n_walkers;
  uint64_t seed;
  uint32_t s0;
  int32_t n_t, n_meas, n_sub, n_echo;
  const int32_t* echo_idx;
  double step_length, kod_mt, dwell_substeps, rho_over_D, gamma_dt, m0, dt;
  double T2[2], T1[2], off[2];  /* free, bound */
  const float* G;               /* (n_t, M, 3) */
  const float* rf_flip;
  const float* rf_axis;
  const float* carrier;
  const float* crush;
  const float* r0;
  const float* brem0;
  float* r_end;
  float* brem_end;
  float* occ_total;
} or_mt_params;
int or_bloch_mt_f32(const or_geom* g, const or_mt_params* p, double* sums, int n_threads);
int or_bloch_mt_f64(const or_geom* g, const or_mt_params* p, double* sums, int n_threads);

/* Philox4x32-10 draw (for cross-checking the stream contract). */
void or_philox(uint64_t seed, uint64_t walker, uint32_t stream, uint32_t j, uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
