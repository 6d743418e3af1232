// Host side of the C ABI (include/dmsim.h): argument checks, launch planning, workspace layout,
// the waveform re-layout kernel, the deterministic cross-block reduction, and the replay kernel.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "dmsim.h"
#include "mt_kernel.cuh"
#include "walk_kernel.cuh"
#include "walk_ff.cuh"
#include "walk_wide.cuh"

namespace dmsim {
WalkFn walk_fn_free(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_cyl(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_sph(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_pcyl(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_psph(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_mesh(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_myelin(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_pmyelin(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_box1d(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_slab(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_shell(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_box1d(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_slab(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_shell(int wall, int pm, int width, bool tsm);
WalkFn walk_fn_ellipsoid(int wall, int pm, int width, bool tsm);
WideFn wide_fn_pcyl_reflect(int rt, bool psub, int nt);
WideFn wide_fn_pcyl_relax(int rt, bool psub, int nt);
WideFn wide_fn_pcyl_permeate(int rt, bool psub, int nt);
FfFn ff_fn_pcyl_reflect(int rt, bool psub, int nt);
FfFn ff_fn_pcyl_relax(int rt, bool psub, int nt);
FfFn ff_fn_pcyl_permeate(int rt, bool psub, int nt);
WalkFn walk_batch_fn_ellipsoid(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_free(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_cyl(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_sph(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_pcyl(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_psph(int wall, int pm, int width, bool tsm);
WalkFn walk_batch_fn_mesh(int wall, int pm, int width, bool tsm);
cudaError_t launch_project_modes(const void* x, bool f16, int64_t n_walkers, int n_t, int n_ch,
                                 const float* basis, int K, const float* ramp, float* endpoint,
                                 float* out, cudaStream_t st);
}  // namespace dmsim

using namespace dmsim;

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
size_t pad16(size_t v) { return (v + 15) & ~(size_t)15; }

// Largest shared-memory footprint for which the cell list is staged into shared memory; larger
// lists are read through L1 from global memory.
constexpr size_t kTabSmemBudget = 96 * 1024;
constexpr size_t kWideSmemMax = 227 * 1024;  // dynamic shared memory one block may take
constexpr size_t kFfPartialMax = (size_t)32 << 20;  // largest per-warp partial buffer (bytes)

// Free-flight walk: lanes that wait for a wall scan, a hit resolution and a sample update before
// the warp runs that stage.  DMSIM_FF_QUORUM="scan,hit,sample" overrides them, and
// DMSIM_FF_BLOCK (512 or 1024) the block size tried first (tuning knobs).
struct FfTuning {
  int q[3] = {12, 6, 8};
  int block = 0;
  FfTuning() {
    if (const char* v = getenv("DMSIM_FF_QUORUM")) {
      int a = 0, b = 0, c = 0;
      if (sscanf(v, "%d,%d,%d", &a, &b, &c) == 3 && a >= 1 && b >= 1 && c >= 1 && a <= 32 &&
          b <= 32 && c <= 32) {
        q[0] = a;
        q[1] = b;
        q[2] = c;
      }
    }
    if (const char* v = getenv("DMSIM_FF_BLOCK")) {
      const int n = atoi(v);
      if (n == 512 || n == 1024) block = n;
    }
  }
};
const FfTuning& ff_tuning() {
  static const FfTuning t;
  return t;
}
int ff_block_override() { return ff_tuning().block; }

// Direct form: measurements per pass.  Basis form: shapes held per thread.
int pick_mt(int M) {
  if (M <= 16) return 16;
  if (M <= 32) return 32;
  return 64;
}
int pick_rt(int r) { return r <= 2 ? 2 : (r <= 4 ? 4 : 8); }
constexpr int kMaxBasisRank = 8;
constexpr int kMaxBasisMeas = 512;

struct Plan {
  WalkFn fn = nullptr;
  WideFn wide = nullptr;  // packed cylinders, basis form: the wide-block kernel
  int grid_wide = 0, nt_wide = 0;
  size_t smem_wide = 0;
  FfFn ff = nullptr;  // packed cylinders, basis form, free flight: the free-flight kernel
  int grid_ff = 0, nt_ff = 0;
  size_t smem_ff = 0;
  int pm = 0;      // 0 direct, 1 basis, 2 vector Bloch (direct waveform)
  int width = 0;   // MT (direct) or RT (basis)
  int mt = 0;      // measurements per pass (direct) or 1 (basis: a single pass of all M)
  int row = 0;     // floats per staged waveform sample
  int n_pass = 0, n_chunks = 0, grid = 0;
  bool tsm = false;
  size_t smem = 0, tab_cs = 0, tab_cand = 0;
  size_t off_gp = 0, off_act = 0, off_cp = 0, off_part = 0, total = 0;
  SmemLayout lay;
};

int make_plan(const dmsim_walk_params* p, const dmsim_geometry* g, Plan* pl,
              size_t tab_budget = kTabSmemBudget, bool bloch = false) {
  if (!p || !g) return fail(DMSIM_EINVAL, "null params or geometry");
  if (bloch) {
    if (g->kind == DMSIM_GEOM_MYELIN || g->kind == DMSIM_GEOM_PMYELIN)
      return fail(DMSIM_EINVAL, "the Bloch walk does not take myelinated geometries");
    if (p->chi || p->t1_decay != 0.f || p->basis_rank != 0)
      return fail(DMSIM_EINVAL, "the Bloch walk takes no chi, t1_decay or waveform basis");
  }
  if (p->n_walkers < 0) return fail(DMSIM_EINVAL, "n_walkers < 0");
  if (p->n_t < 1 || p->n_meas < 1 || p->sub_steps < 1)
    return fail(DMSIM_EINVAL, "n_t, n_meas and sub_steps must be >= 1");
  if (p->n_echo < 1 || p->n_echo > kMaxEcho)
    return fail(DMSIM_ETOOBIG, "n_echo must be in [1, %d]", kMaxEcho);
  if (!p->echo_idx) return fail(DMSIM_EINVAL, "echo_idx is null");
  for (int e = 0; e < p->n_echo; ++e) {
    if (p->echo_idx[e] < 0 || p->echo_idx[e] >= p->n_t)
      return fail(DMSIM_EINVAL, "echo index %d out of range", p->echo_idx[e]);
    if (e > 0 && p->echo_idx[e] <= p->echo_idx[e - 1])
      return fail(DMSIM_EINVAL, "echo indices must be strictly ascending");
  }
  const bool packed = g->kind == DMSIM_GEOM_PACKED_CYLINDERS || g->kind == DMSIM_GEOM_PACKED_SPHERES;
  if (g->kind < 0 || g->kind > DMSIM_GEOM_ELLIPSOID)
    return fail(DMSIM_EINVAL, "unsupported geometry kind %d", g->kind);
  if (g->kind == DMSIM_GEOM_ELLIPSOID &&
      !(g->radius > 0.f && g->ell_inv2[0] > 0.f && g->ell_inv2[1] > 0.f && g->ell_inv2[2] > 0.f))
    return fail(DMSIM_EINVAL, "ellipsoid needs positive semi-axes");
  if ((g->kind == DMSIM_GEOM_BOX1D || g->kind == DMSIM_GEOM_SLAB) && !(g->L > 0.f))
    return fail(DMSIM_EINVAL, "slab geometry needs its length L > 0");
  if (g->kind == DMSIM_GEOM_BOX1D && g->wall_mode == DMSIM_WALL_PERMEATE)
    return fail(DMSIM_EINVAL, "Box1D walls are not permeable");
  if (g->kind == DMSIM_GEOM_SHELL && !(g->radius > 0.f && g->shell_r_out > g->radius))
    return fail(DMSIM_EINVAL, "shell needs 0 < R_in < R_out");
  if (g->kind == DMSIM_GEOM_PMYELIN) {
    if (g->pmy_n < 1 || g->pmy_nmax < g->pmy_n || !g->pmy_cyl || !g->pmy_seed || !(g->L > 0.f))
      return fail(DMSIM_EINVAL, "packed myelinated cylinders need their axon and seeding tables");
    if (((uintptr_t)g->pmy_cyl & 15) || ((uintptr_t)g->pmy_seed & 7))
      return fail(DMSIM_EINVAL, "packed myelin tables must be 16-byte aligned");
    if (g->wall_mode == DMSIM_WALL_RELAX)
      return fail(DMSIM_EINVAL, "packed myelin walls reflect or permeate");
    if (g->rho_over_D != 1.f || p->step_length != 1.f)
      return fail(DMSIM_EINVAL, "packed myelin walks unit directions with rho_over_D = 1");
  }
  if (g->kind == DMSIM_GEOM_MYELIN) {
    if (!(g->radius > 0.f) || !(g->myelin_r_out > g->radius))
      return fail(DMSIM_EINVAL, "myelinated cylinder needs 0 < inner radius < outer radius");
    if (g->wall_mode == DMSIM_WALL_RELAX)
      return fail(DMSIM_EINVAL, "myelinated cylinder walls reflect or permeate");
    if (g->rho_over_D != 1.f)
      return fail(DMSIM_EINVAL, "myelinated cylinder: rho_over_D must be 1 (T2 per compartment)");
    for (int c = 0; c < 3; ++c)
      if (!(g->myelin_step[c] >= 0.f)) return fail(DMSIM_EINVAL, "negative myelin step length");
    if (p->step_length != 1.f)
      return fail(DMSIM_EINVAL, "myelinated cylinder walks unit directions (step_length = 1)");
  }
  if (g->kind == DMSIM_GEOM_MESH) {
    if (!g->tri || !g->tri_vn || !g->mesh_cell_start || !g->mesh_cell_tri)
      return fail(DMSIM_EINVAL, "mesh geometry needs its triangle and grid tables");
    if (g->mesh_dims[0] < 1 || g->mesh_dims[1] < 1 || g->mesh_dims[2] < 1 ||
        !(g->mesh_cell > 0.f) || g->max_bounces < 1 || g->max_bounces > 64)
      return fail(DMSIM_EINVAL, "bad mesh grid or bounce budget");
    for (int a = 0; a < 3; ++a)
      if (g->periodic[a] && !(g->box[a] > 0.f))
        return fail(DMSIM_EINVAL, "periodic mesh axis with an empty box");
  }
  if (g->wall_mode < 0 || g->wall_mode > 2) return fail(DMSIM_EINVAL, "bad wall_mode");
  if (g->kind == DMSIM_GEOM_FREE && g->wall_mode != DMSIM_WALL_REFLECT)
    return fail(DMSIM_EINVAL, "free diffusion has no walls");
  if (packed) {
    if (!g->cell_start || !g->cand || g->grid_n < 1 || g->n_cand < 0 || !(g->L > 0.f))
      return fail(DMSIM_EINVAL, "packed geometry needs a cell list");
    if (!(g->reach >= p->step_length))
      return fail(DMSIM_EINVAL, "cell list reach %g is shorter than the step %g", g->reach,
                  p->step_length);
    if (((uintptr_t)g->cell_start & 15) || ((uintptr_t)g->cand & 15))
      return fail(DMSIM_EINVAL, "cell list arrays must be 16-byte aligned");
  }
  if (p->basis_rank < 0 || p->basis_rank > kMaxBasisRank)
    return fail(DMSIM_EINVAL, "basis_rank must be in [0, %d]", kMaxBasisRank);
  if (p->schedule < DMSIM_SCHED_LOCKSTEP || p->schedule > DMSIM_SCHED_SCAN_EVERY)
    return fail(DMSIM_EINVAL, "schedule must be one of DMSIM_SCHED_*");
  if (bloch) {
    if (p->G == nullptr) return fail(DMSIM_EINVAL, "G is null");
    pl->pm = 2;
    pl->width = pl->mt = p->n_meas <= 4 ? 4 : 16;
    pl->n_pass = (p->n_meas + pl->mt - 1) / pl->mt;
    pl->row = 3 * pl->mt;
  } else if (p->basis_rank > 0) {
    if (!p->basis_V || !p->basis_C) return fail(DMSIM_EINVAL, "basis_V / basis_C is null");
    if (p->n_meas > kMaxBasisMeas)
      return fail(DMSIM_ETOOBIG, "the basis form handles at most %d measurements", kMaxBasisMeas);
    pl->pm = 1;
    pl->width = pick_rt(p->basis_rank);
    pl->mt = 1;
    pl->n_pass = 1;
    pl->row = pl->width;
  } else {
    if (p->G == nullptr) return fail(DMSIM_EINVAL, "G is null");
    pl->pm = 0;
    pl->width = pl->mt = pick_mt(p->n_meas);
    pl->n_pass = (p->n_meas + pl->mt - 1) / pl->mt;
    pl->row = 3 * pl->mt;
  }
  pl->n_chunks = (p->n_t + kTC - 1) / kTC;
  size_t cells = 0;
  if (packed) {
    cells = (size_t)g->grid_n * g->grid_n * (g->kind == DMSIM_GEOM_PACKED_SPHERES ? g->grid_n : 1);
    pl->tab_cs = pad16((cells + 1) * 4);
    pl->tab_cand = (size_t)g->n_cand * 16;
    pl->tsm = pl->tab_cs + pl->tab_cand <= tab_budget;
  }
  switch (g->kind) {
    case DMSIM_GEOM_FREE: pl->fn = walk_fn_free(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_CYLINDER: pl->fn = walk_fn_cyl(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_SPHERE: pl->fn = walk_fn_sph(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_PACKED_CYLINDERS:
      pl->fn = walk_fn_pcyl(g->wall_mode, pl->pm, pl->width, pl->tsm);
      break;
    case DMSIM_GEOM_PACKED_SPHERES:
      pl->fn = walk_fn_psph(g->wall_mode, pl->pm, pl->width, pl->tsm);
      break;
    case DMSIM_GEOM_MESH: pl->fn = walk_fn_mesh(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_MYELIN:
      pl->fn = walk_fn_myelin(g->wall_mode, pl->pm, pl->width, false);
      break;
    case DMSIM_GEOM_PMYELIN:
      pl->fn = walk_fn_pmyelin(g->wall_mode, pl->pm, pl->width, false);
      break;
    case DMSIM_GEOM_BOX1D: pl->fn = walk_fn_box1d(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_SLAB: pl->fn = walk_fn_slab(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_SHELL: pl->fn = walk_fn_shell(g->wall_mode, pl->pm, pl->width, false); break;
    case DMSIM_GEOM_ELLIPSOID:
      pl->fn = walk_fn_ellipsoid(g->wall_mode, pl->pm, pl->width, false);
      break;
  }
  if (!pl->fn) return fail(DMSIM_EINVAL, "no kernel for this geometry/wall combination");
  pl->lay = walk_smem_layout(pl->pm, pl->width, p->n_meas);
  pl->smem = pl->lay.off_tab + (pl->tsm ? pl->tab_cs + pl->tab_cand : 0) +
             (g->kind == DMSIM_GEOM_MESH ? kWarps * kMeshScratchBytes : 0);

  int dev = 0, n_sm = 0, nb = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(DMSIM_ECUDA, "cudaGetDevice failed");
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(DMSIM_ECUDA, "cudaDeviceGetAttribute failed");
  if (cudaFuncSetAttribute((const void*)pl->fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)pl->smem) != cudaSuccess)
    return fail(DMSIM_ECUDA, "cudaFuncSetAttribute(%zu B shared) failed", pl->smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)pl->fn, kBlock, pl->smem) !=
          cudaSuccess ||
      nb < 1)
    return fail(DMSIM_ECUDA, "kernel does not fit on an SM (%zu B shared)", pl->smem);
  const int64_t n_tiles = (p->n_walkers + kBlock - 1) / kBlock;
  int64_t grid = (int64_t)nb * n_sm;
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  pl->grid = (int)grid;
  // Packed cylinders in the basis form with the cell list on chip walk on the wide-block kernel
  // (walk_wide.cuh: one block of 1024, else 512, threads per SM) when launch_single sees no
  // trajectory, boundary-weight or occupancy export.  The partial buffer is sized for the larger
  // of the two grids.
  int64_t grid_part = grid;
  if (g->kind == DMSIM_GEOM_PACKED_CYLINDERS && pl->tsm && pl->pm == 1 && !bloch) {
    const bool psub = p->phase_per_substep != 0;
    for (int nt : {1024, 512}) {
      WideFn fn = g->wall_mode == DMSIM_WALL_REFLECT ? wide_fn_pcyl_reflect(pl->width, psub, nt)
                  : g->wall_mode == DMSIM_WALL_RELAX ? wide_fn_pcyl_relax(pl->width, psub, nt)
                                                     : wide_fn_pcyl_permeate(pl->width, psub, nt);
      const size_t smem = wide_layout(nt, pl->width, p->n_meas, pl->tab_cs + pl->tab_cand).total;
      int nbw = 0;
      if (!fn || smem > kWideSmemMax ||
          cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbw, (const void*)fn, nt, smem) !=
              cudaSuccess ||
          nbw < 1) {
        cudaGetLastError();
        continue;
      }
      const int64_t tiles_w = (p->n_walkers + nt - 1) / nt;
      int64_t gw = (int64_t)nbw * n_sm;
      if (gw > tiles_w) gw = tiles_w;
      if (gw < 1) gw = 1;
      pl->wide = fn;
      pl->nt_wide = nt;
      pl->smem_wide = smem;
      pl->grid_wide = (int)gw;
      grid_part = std::max(grid_part, gw);
      break;
    }
    // The free-flight kernel (walk_ff.cuh), when asked for, walks the same walkers with fewer
    // wall scans; it keeps one FP64 partial slice per warp, so it is taken while those slices
    // stay small.
    if (pl->wide && p->schedule != DMSIM_SCHED_LOCKSTEP) {
      for (int nt : {ff_block_override(), 1024, 512}) {
        if (nt <= 0) continue;
        FfFn fn = g->wall_mode == DMSIM_WALL_REFLECT ? ff_fn_pcyl_reflect(pl->width, psub, nt)
                  : g->wall_mode == DMSIM_WALL_RELAX ? ff_fn_pcyl_relax(pl->width, psub, nt)
                                                     : ff_fn_pcyl_permeate(pl->width, psub, nt);
        const size_t smem = ff_layout(nt, pl->width, p->n_meas, pl->tab_cs + pl->tab_cand).total;
        int nbf = 0;
        if (!fn || smem > kWideSmemMax ||
            cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbf, (const void*)fn, nt, smem) !=
                cudaSuccess ||
            nbf < 1) {
          cudaGetLastError();
          continue;
        }
        const int64_t blocks = (p->n_walkers + nt - 1) / nt;
        int64_t gf = (int64_t)nbf * n_sm;
        if (gf > blocks) gf = blocks;
        if (gf < 1) gf = 1;
        const int64_t slots = gf * (nt / 32);
        if ((size_t)slots * p->n_echo * p->n_meas * 3 * 8 > kFfPartialMax) break;
        pl->ff = fn;
        pl->nt_ff = nt;
        pl->smem_ff = smem;
        pl->grid_ff = (int)gf;
        grid_part = std::max(grid_part, slots);
        break;
      }
    }
  }
  const int Mp = pl->pm == 1 ? p->n_meas : pl->n_pass * pl->mt;
  size_t off = 0;
  pl->off_gp = off;
  off = align256(off + (size_t)pl->n_pass * pl->n_chunks * kTC * pl->row * 4);
  pl->off_act = off;
  off = align256(off + (size_t)pl->n_pass * p->n_t);
  pl->off_cp = off;
  off = align256(off + (pl->pm == 1 ? (size_t)p->n_meas * 3 * pl->width * 4 : 0));
  pl->off_part = off;
  off = align256(off + (size_t)grid_part * p->n_echo * Mp * 3 * 8);
  pl->total = off;
  return DMSIM_OK;
}

// Waveform re-layout: G (n_t, M, 3) -> per pass (n_chunks*kTC, MT, 3), zero padded, plus a
// per-sample flag telling whether any gradient of the pass is on (the walk skips the phase
// update otherwise).
__global__ void k_prep(const float* __restrict__ G, int n_t, int M, int mt, int n_pass, int t_pad,
                       float* __restrict__ Gp, uint8_t* __restrict__ act) {
  const int64_t n = (int64_t)n_pass * t_pad;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int pass = (int)(i / t_pad), t = (int)(i % t_pad);
    float* dst = Gp + ((size_t)pass * t_pad + t) * mt * 3;
    bool any = false;
    for (int j = 0; j < mt; ++j) {
      const int m = pass * mt + j;
      for (int k = 0; k < 3; ++k) {
        float v = 0.f;
        if (t < n_t && m < M) v = G[((size_t)t * M + m) * 3 + k];
        dst[j * 3 + k] = v;
        any |= (v != 0.f);
      }
    }
    if (t < n_t) act[(size_t)pass * n_t + t] = any ? 1 : 0;
  }
}

// Basis form: V (n_t, r) -> (n_chunks*kTC, RT) and C (M, 3, r) -> (M, 3, RT), zero padded, plus
// the per-sample activity flag.
__global__ void k_prep_basis(const float* __restrict__ V, const float* __restrict__ C, int n_t,
                             int M, int r, int rt, int t_pad, float* __restrict__ Vp,
                             uint8_t* __restrict__ act, float* __restrict__ Cp) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t_pad; i += stride) {
    const int t = (int)i;
    bool any = false;
    for (int j = 0; j < rt; ++j) {
      const float v = (t < n_t && j < r) ? V[(size_t)t * r + j] : 0.f;
      Vp[(size_t)t * rt + j] = v;
      any |= (v != 0.f);
    }
    if (t < n_t) act[t] = any ? 1 : 0;
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)M * 3 * rt;
       i += stride) {
    const int j = (int)(i % rt);
    const int64_t mk = i / rt;
    Cp[i] = j < r ? C[mk * r + j] : 0.f;
  }
}

// Deterministic reduction of the per-block FP64 partials (fixed block order).
__global__ void k_reduce(const double* __restrict__ part, int grid, int n_echo, int Mp, int M,
                         double* __restrict__ sums) {
  const int n = n_echo * M * 3;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int e = i / (M * 3), r = i % (M * 3);
    double acc = 0.0;
    for (int b = 0; b < grid; ++b) acc += part[((size_t)b * n_echo + e) * Mp * 3 + r];
    sums[i] = acc;
  }
}

// ---- replay (trajectories.py:550-552, 634): phase of saved trajectories ------------------------
constexpr int kRB = 128;   // walkers per block
constexpr int kRT = 8;     // samples per staged step
constexpr int kRM = 16;    // measurements per register tile

template <bool F16>
__global__ void __launch_bounds__(kRB) k_replay(const void* __restrict__ traj, int64_t n_walkers,
                                                int n_t, const float* __restrict__ G, int M,
                                                float gamma_dt, const float* __restrict__ log_w,
                                                double* __restrict__ part, float* __restrict__ phi_out) {
  __shared__ float Gs[kRT * kRM * 3];
  __shared__ float red[kRB / 32][kRM * 3];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_mt = (M + kRM - 1) / kRM;
  const int64_t n_tiles = (n_walkers + kRB - 1) / kRB;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t w = tile * kRB + tid;
    const bool act = w < n_walkers;
    const float wgt = act ? (log_w ? expf(log_w[w]) : 1.f) : 0.f;
    for (int mt = 0; mt < n_mt; ++mt) {
      float phi[kRM], kc[kRM];
#pragma unroll
      for (int j = 0; j < kRM; ++j) phi[j] = kc[j] = 0.f;
      for (int t0 = 0; t0 < n_t; t0 += kRT) {
        __syncthreads();
        for (int i = tid; i < kRT * kRM * 3; i += kRB) {
          const int tt = i / (kRM * 3), r = i % (kRM * 3), m = mt * kRM + r / 3;
          Gs[i] = (t0 + tt < n_t && m < M) ? G[((size_t)(t0 + tt) * M + m) * 3 + r % 3] : 0.f;
        }
        __syncthreads();
        for (int tt = 0; tt < kRT && t0 + tt < n_t; ++tt) {
          float rx = 0.f, ry = 0.f, rz = 0.f;
          if (act) {
            const size_t o = ((size_t)w * n_t + t0 + tt) * 3;
            if (F16) {
              const __half* tp = reinterpret_cast<const __half*>(traj);
              rx = __half2float(tp[o]);
              ry = __half2float(tp[o + 1]);
              rz = __half2float(tp[o + 2]);
            } else {
              const float* tp = reinterpret_cast<const float*>(traj);
              rx = tp[o];
              ry = tp[o + 1];
              rz = tp[o + 2];
            }
          }
          rx *= gamma_dt;
          ry *= gamma_dt;
          rz *= gamma_dt;
#pragma unroll
          for (int j = 0; j < kRM; ++j) {
            const float* gg = Gs + (tt * kRM + j) * 3;
            const float d = fmaf(gg[2], rz, fmaf(gg[1], ry, gg[0] * rx));
            const float yk = d - kc[j];
            const float tk = phi[j] + yk;
            kc[j] = (tk - phi[j]) - yk;
            phi[j] = tk;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < kRM; ++j) {
        const int m = mt * kRM + j;
        float sn, cs;
        sincosf(phi[j], &sn, &cs);
        const float c1 = warp_sum(wgt * cs), c2 = warp_sum(wgt * sn),
                    c3 = warp_sum((wgt * cs) * (wgt * cs));
        if (lane == 0) {
          red[warp][3 * j] = c1;
          red[warp][3 * j + 1] = c2;
          red[warp][3 * j + 2] = c3;
        }
        if (act && phi_out && m < M) phi_out[(size_t)w * M + m] = phi[j];
      }
      __syncthreads();
      for (int i = tid; i < kRM * 3; i += kRB) {
        const int m = mt * kRM + i / 3;
        if (m >= M) continue;
        double acc = 0.0;
        for (int ww = 0; ww < kRB / 32; ++ww) acc += (double)red[ww][i];
        part[(size_t)blockIdx.x * M * 3 + (size_t)m * 3 + i % 3] += acc;
      }
    }
  }
}

__global__ void k_zero(double* p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = 0.0;
}

// ---- known-answer kernel: one sub-step of the device step functions per input triple ---------
// The loop is uniform across the block (every lane runs every iteration, lanes past the end on
// the last input's data without writing), so the mesh step's warp-cooperative searches see all
// 32 lanes.
template <int GEOM, int WALL>
__global__ void k_step_kat(const GeoK g, const MeshK mk, int64_t n, const float* __restrict__ rin,
                           const float* __restrict__ st, const float* __restrict__ uin,
                           const uint32_t* __restrict__ cs, const float4* __restrict__ cand,
                           float* __restrict__ rout, float* __restrict__ dlog) {
  extern __shared__ __align__(16) uint8_t kat_smem[];
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const bool live = base + threadIdx.x < n;
    const int64_t i = live ? base + threadIdx.x : n - 1;
    float x = rin[3 * i], y = rin[3 * i + 1], z = rin[3 * i + 2];
    const float sx = st[3 * i], sy = st[3 * i + 1], sz = st[3 * i + 2];
    const float u = uin ? uin[i] : 0.f;
    Tally tl;
    float dl = 0.f;
    int ix = 0, iy = 0, iz = 0;
    if constexpr (GEOM == DMSIM_GEOM_PACKED_CYLINDERS || GEOM == DMSIM_GEOM_PACKED_SPHERES) {
      ix = (int)floorf(x / g.L + 0.5f);
      x -= g.L * ix;
      iy = (int)floorf(y / g.L + 0.5f);
      y -= g.L * iy;
      if (GEOM == DMSIM_GEOM_PACKED_SPHERES) {
        iz = (int)floorf(z / g.L + 0.5f);
        z -= g.L * iz;
      }
    }
    if constexpr (GEOM == DMSIM_GEOM_FREE) {
      x += sx; y += sy; z += sz;
    } else if constexpr (GEOM == DMSIM_GEOM_CYLINDER) {
      dl = cylinder_step<WALL>(x, y, sx, sy, u, g, tl);
      z += sz;
    } else if constexpr (GEOM == DMSIM_GEOM_SPHERE) {
      dl = sphere_step<WALL>(x, y, z, sx, sy, sz, u, g, tl);
    } else if constexpr (GEOM == DMSIM_GEOM_PACKED_CYLINDERS) {
      dl = packed_cyl_step<WALL>(x, y, ix, iy, sx, sy, u, g, cs, cand, tl);
      z += sz;
    } else if constexpr (GEOM == DMSIM_GEOM_PACKED_SPHERES) {
      dl = packed_sph_step<WALL>(x, y, z, ix, iy, iz, sx, sy, sz, u, g, cs, cand, tl);
    } else if constexpr (GEOM == DMSIM_GEOM_ELLIPSOID) {
      dl = ellipsoid_step<WALL>(x, y, z, sx, sy, sz, u, g, tl);
    } else if constexpr (GEOM == DMSIM_GEOM_BOX1D) {
      dl = box1d_step<WALL == 2 ? 0 : WALL>(x, y, z, sx, sy, sz, g);
    } else if constexpr (GEOM == DMSIM_GEOM_SLAB) {
      dl = slab_step<WALL>(x, y, z, sx, sy, sz, u, g, tl);
    } else if constexpr (GEOM == DMSIM_GEOM_SHELL) {
      dl = shell_step<WALL>(x, y, z, sx, sy, sz, u, g, tl);
    } else {
      if (mk.per[0]) { ix = (int)floorf((x - mk.vmin[0]) / mk.box[0]); x -= mk.box[0] * ix; }
      if (mk.per[1]) { iy = (int)floorf((y - mk.vmin[1]) / mk.box[1]); y -= mk.box[1] * iy; }
      if (mk.per[2]) { iz = (int)floorf((z - mk.vmin[2]) / mk.box[2]); z -= mk.box[2] * iz; }
      int cls = 1, pop = 0;
      if (mk.reject && WALL != kPermeate) cls = mesh_classify(mk, x, y, z, pop);
      uint32_t nb = 0, ne = 0;
      dl = mesh_step<WALL>(x, y, z, ix, iy, iz, cls, pop, sx, sy, sz, u, mk, tl, nb, ne,
                           reinterpret_cast<MeshScratch*>(kat_smem) + (threadIdx.x >> 5));
    }
    const float Lx = GEOM == DMSIM_GEOM_MESH ? mk.box[0] : g.L;
    const float Ly = GEOM == DMSIM_GEOM_MESH ? mk.box[1] : g.L;
    const float Lz = GEOM == DMSIM_GEOM_MESH ? mk.box[2] : g.L;
    if (!live) continue;
    rout[3 * i] = x + Lx * (float)ix;
    rout[3 * i + 1] = y + Ly * (float)iy;
    rout[3 * i + 2] = z + Lz * (float)iz;
    dlog[i] = dl;
  }
}

using KatFn = void (*)(GeoK, MeshK, int64_t, const float*, const float*, const float*,
                       const uint32_t*, const float4*, float*, float*);

template <int GEOM>
KatFn kat_fn(int wall) {
  if constexpr (GEOM == DMSIM_GEOM_FREE) {
    return k_step_kat<GEOM, 0>;
  } else {
    if (wall == 0) return k_step_kat<GEOM, 0>;
    if (wall == 1) return k_step_kat<GEOM, 1>;
    return k_step_kat<GEOM, 2>;
  }
}

MeshK make_meshk(const dmsim_geometry* g) {
  MeshK m;
  memset(&m, 0, sizeof(m));
  if (g->kind != DMSIM_GEOM_MESH) return m;
  for (int a = 0; a < 3; ++a) {
    m.gmin[a] = g->grid_min[a];
    m.dims[a] = g->mesh_dims[a];
    m.per[a] = g->periodic[a] ? 1 : 0;
    m.vmin[a] = g->vmin[a];
    m.box[a] = g->box[a];
  }
  m.cs = g->mesh_cell;
  m.eps = g->mesh_eps;
  m.nudge = g->mesh_nudge;
  m.graze = g->mesh_graze;
  m.maxb = g->max_bounces;
  m.rmi = g->rho_mult_intra;
  m.rme = g->rho_mult_extra;
  m.kmo = g->kappa_mult_out;
  m.kmi = g->kappa_mult_in;
  m.kod = g->kappa_over_D;
  m.reject = g->reject_escape ? 1 : 0;
  m.seed_parity = g->seed_parity ? 1 : 0;
  m.seed_inside = g->seed_inside ? 1 : 0;
  m.tri = reinterpret_cast<const float4*>(g->tri);
  m.vn = reinterpret_cast<const float4*>(g->tri_vn);
  m.bs = reinterpret_cast<const float4*>(g->tri_bs);
  m.cstart = g->mesh_cell_start;
  m.ctri = g->mesh_cell_tri;
  m.nbstart = g->mesh_nb_start;
  m.nbtri = g->mesh_nb_tri;
  m.nbc = g->mesh_nb_start ? reinterpret_cast<const float4*>(g->mesh_nb_cent) : nullptr;
  if (g->mesh_nb_start && g->mesh_hit_start && g->mesh_hit_tri && g->mesh_hit_reach > 0.f) {
    m.hstart = g->mesh_hit_start;
    m.htri = g->mesh_hit_tri;
    m.hbs = g->tri_bs ? reinterpret_cast<const float4*>(g->mesh_hit_bs) : nullptr;
    m.hreach = g->mesh_hit_reach;
  }
  return m;
}

__global__ void k_mesh_nb(const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ct,
                          int d0, int d1, int d2, const uint32_t* __restrict__ start,
                          uint32_t* __restrict__ out) {
  const int dims[3] = {d0, d1, d2};
  const int64_t n = (int64_t)d0 * d1 * d2;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (start)
      mesh_neighbourhood(cs, ct, dims, c, out + start[c]);
    else
      out[c] = mesh_neighbourhood(cs, ct, dims, c, nullptr);
  }
}

__global__ void k_mesh_hit(const uint32_t* __restrict__ nbs, const uint32_t* __restrict__ nbt,
                           const float* __restrict__ tri, int d0, int d1, int d2, float g0,
                           float g1, float g2, float cs, float reach,
                           const uint32_t* __restrict__ start, uint32_t* __restrict__ out,
                           const float4* __restrict__ bs, float4* __restrict__ out_bs) {
  const int dims[3] = {d0, d1, d2};
  const float gmin[3] = {g0, g1, g2};
  const int64_t n = (int64_t)d0 * d1 * d2;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (start)
      mesh_hit_list(nbs, nbt, tri, dims, gmin, cs, reach, c, out + start[c], bs,
                    out_bs ? out_bs + start[c] : nullptr);
    else
      out[c] = mesh_hit_list(nbs, nbt, tri, dims, gmin, cs, reach, c, nullptr, nullptr, nullptr);
  }
}

MyelinK make_myelk(const dmsim_geometry* g) {
  MyelinK m;
  memset(&m, 0, sizeof(m));
  if (g->kind != DMSIM_GEOM_MYELIN) return m;
  m.r_in = g->radius;
  m.r_out = g->myelin_r_out;
  m.nudge = g->nudge;
  for (int c = 0; c < 3; ++c) {
    m.sl[c] = g->myelin_step[c];
    m.kin[c] = g->myelin_kin_over_D[c];
    m.kout[c] = g->myelin_kout_over_D[c];
    m.t2dec[c] = g->myelin_t2dec[c];
    m.lw0[c] = g->myelin_logw0[c];
  }
  m.n0 = g->myelin_seed_n[0];
  m.n1 = g->myelin_seed_n[1];
  return m;
}

PMyelinK make_pmyk(const dmsim_geometry* g) {
  PMyelinK m;
  memset(&m, 0, sizeof(m));
  if (g->kind != DMSIM_GEOM_PMYELIN) return m;
  m.cyl = reinterpret_cast<const float4*>(g->pmy_cyl);
  m.seed = reinterpret_cast<const long long*>(g->pmy_seed);
  m.n = g->pmy_n;
  m.nmax = g->pmy_nmax;
  m.L = g->L;
  m.nudge = g->nudge;
  m.rho = g->pmy_rho_over_D;
  m.lwm = g->pmy_logw_myelin;
  for (int c = 0; c < 3; ++c) m.t2dec[c] = g->pmy_t2dec[c];
  return m;
}

GeoK make_geok(const dmsim_geometry* g) {
  GeoK gk;
  memset(&gk, 0, sizeof(gk));
  const bool packed =
      g->kind == DMSIM_GEOM_PACKED_CYLINDERS || g->kind == DMSIM_GEOM_PACKED_SPHERES;
  gk.R = g->radius;
  gk.R2 = g->radius * g->radius;
  gk.invR = g->radius > 0.f ? 1.f / g->radius : 0.f;
  gk.eps = g->eps_detect;
  gk.nudge = g->nudge;
  gk.kod = g->kappa_over_D;
  gk.L = (packed || g->kind == DMSIM_GEOM_PMYELIN) ? g->L : 0.f;
  gk.halfL = packed ? 0.5f * g->L : 0.f;
  gk.inv_h = packed ? (float)g->grid_n / g->L : 0.f;
  gk.n = packed ? g->grid_n : 1;
  gk.mi = packed ? (g->need_min_image != 0) : 0;
  gk.kmax = packed ? g->max_cell_cand : 0;
  if (g->kind == DMSIM_GEOM_BOX1D || g->kind == DMSIM_GEOM_SLAB) gk.L = g->L;
  gk.r_out = g->shell_r_out;
  gk.cyl = g->shell_cyl ? 1 : 0;
  for (int a = 0; a < 3; ++a) gk.e2[a] = g->ell_inv2[a];
  gk.h = packed ? g->cell_h : 0.f;
  gk.reach = packed ? g->reach : 0.f;
  return gk;
}

int replay_grid(int64_t n_walkers) {
  int dev = 0, n_sm = 0, nb = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k_replay<true>, kRB, 0);
  int64_t grid = (int64_t)(nb > 0 ? nb : 1) * (n_sm > 0 ? n_sm : 1);
  const int64_t n_tiles = (n_walkers + kRB - 1) / kRB;
  if (grid > n_tiles) grid = n_tiles;
  return (int)(grid < 1 ? 1 : grid);
}


int check_outputs(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_walk_outputs* o) {
  if (!o || !o->sums || !o->status) return fail(DMSIM_EINVAL, "outputs need sums and status");
  const bool packed =
      g->kind == DMSIM_GEOM_PACKED_CYLINDERS || g->kind == DMSIM_GEOM_PACKED_SPHERES;
  if ((o->comp0 || o->comp_end || o->comp_occ) && packed && !g->cand_obj)
    return fail(DMSIM_EINVAL, "classification of packed objects needs cand_obj");
  (void)p;
  return DMSIM_OK;
}

// Kernel arguments of one walk; the per-pass fields (pass, Gp, active) and the partial buffer
// are set by the caller.
void fill_kargs(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_walk_outputs* o,
                const Plan& pl, KArgs* a) {
  memset(a, 0, sizeof(*a));
  a->n_walkers = p->n_walkers;
  a->walker_offset = p->walker_offset;
  a->seed = p->seed;
  a->n_t = p->n_t;
  a->n_chunks = pl.n_chunks;
  a->S = p->sub_steps;
  a->phase_sub = p->phase_per_substep ? 1 : 0;
  a->has_weight = p->has_weight ? 1 : 0;
  a->n_echo = p->n_echo;
  a->Mp = pl.pm == 1 ? p->n_meas : pl.n_pass * pl.mt;
  a->M = p->n_meas;
  a->step_l = p->step_length;
  a->gamma_dt = p->gamma_dt;
  a->t2dec = p->t2_decay;
  a->t1dec = p->t1_decay;
  a->rho = g->rho_over_D;
  a->g = make_geok(g);
  a->mk = make_meshk(g);
  a->my = make_myelk(g);
  a->pm = make_pmyk(g);
  a->tab_cs_bytes = (uint32_t)pl.tab_cs;
  a->tab_cand_bytes = (uint32_t)pl.tab_cand;
  a->cs = g->cell_start;
  a->cand = reinterpret_cast<const float4*>(g->cand);
  a->cand_obj = g->cand_obj;
  a->chi = p->chi;
  a->r0 = p->r0;
  a->status = o->status;
  a->final_pos = o->final_pos;
  a->log_w = o->log_w;
  a->phi_out = o->phi;
  a->comp0 = o->comp0;
  a->comp_end = o->comp_end;
  a->traj = o->traj;
  a->traj_f16 = o->traj_f16;
  a->dlog_unit = o->dlog_unit;
  a->comp_occ = o->comp_occ;
  for (int e = 0; e < p->n_echo; ++e) a->echo[e] = p->echo_idx[e];
}

// One walk on its own launches: waveform re-layout, one walk launch per pass, reduction.
int launch_single(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_walk_outputs* o,
                  const Plan& pl, uint8_t* ws, cudaStream_t st,
                  const dmsim_bloch_params* bl = nullptr) {
  int rc = check_outputs(p, g, o);
  if (rc != DMSIM_OK) return rc;
  if (p->n_walkers == 0) {
    cudaMemsetAsync(o->sums, 0, sizeof(double) * p->n_echo * p->n_meas * 3, st);
    return DMSIM_OK;
  }
  float* Gp = reinterpret_cast<float*>(ws + pl.off_gp);
  uint8_t* act = ws + pl.off_act;
  double* part = reinterpret_cast<double*>(ws + pl.off_part);
  float* Cp = reinterpret_cast<float*>(ws + pl.off_cp);
  const int t_pad = pl.n_chunks * kTC;
  if (pl.pm == 1)
    k_prep_basis<<<64, 256, 0, st>>>(p->basis_V, p->basis_C, p->n_t, p->n_meas, p->basis_rank,
                                     pl.width, t_pad, Gp, act, Cp);
  else
    k_prep<<<64, 256, 0, st>>>(p->G, p->n_t, p->n_meas, pl.mt, pl.n_pass, t_pad, Gp, act);
  KArgs a;
  fill_kargs(p, g, o, pl, &a);
  a.Cp = Cp;
  a.part = part;
  if (bl) {
    a.rf_flip = bl->rf_flip;
    a.rf_axis = bl->rf_axis;
    a.carrier = bl->carrier;
    a.crush = bl->crush;
    a.m0 = bl->m0;
    a.t1_sample = bl->t1_sample;
    a.fkind = bl->field_kind;
    a.fn = bl->field_n;
    a.ftab = bl->field_tab;
    for (int k = 0; k < 9; ++k) a.frot[k] = bl->field_rot[k];
    for (int k = 0; k < 8; ++k) a.fpar[k] = bl->field_par[k];
    for (int k = 0; k < 3; ++k) a.fdims[k] = bl->field_dims[k];
    a.fgdt = bl->field_gamma_dt;
  }
  BatchCtl none;
  memset(&none, 0, sizeof(none));
  const bool wide = pl.wide != nullptr && bl == nullptr && o->traj == nullptr &&
                    o->dlog_unit == nullptr && o->comp_occ == nullptr;
  const bool ff = wide && pl.ff != nullptr;
  // partial slices to reduce: one per warp (free flight), else one per block
  const int grid = ff ? pl.grid_ff * (pl.nt_ff / 32) : wide ? pl.grid_wide : pl.grid;
  for (int k = 0; k < 3; ++k) a.ff_quorum[k] = ff_tuning().q[k];
  a.ff_skip = p->schedule == DMSIM_SCHED_FREE_FLIGHT ? 1 : 0;
  for (int pass = 0; pass < pl.n_pass; ++pass) {
    a.pass = pass;
    a.Gp = Gp + (size_t)pass * t_pad * pl.row;
    a.active = act + (size_t)pass * p->n_t;
    if (ff)
      pl.ff<<<pl.grid_ff, pl.nt_ff, pl.smem_ff, st>>>(a);
    else if (wide)
      pl.wide<<<grid, pl.nt_wide, pl.smem_wide, st>>>(a);
    else
      pl.fn<<<grid, kBlock, pl.smem, st>>>(a, none);
  }
  const int nred = p->n_echo * p->n_meas * 3;
  k_reduce<<<(nred + 255) / 256, 256, 0, st>>>(part, grid, p->n_echo, a.Mp, p->n_meas,
                                               o->sums);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(DMSIM_ECUDA, "launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

// ---- magnetisation-transfer walk --------------------------------------------------------------
struct MtPlan {
  MtFn fn = nullptr;
  int width = 0, n_pass = 0, grid = 0;
  size_t total = 0;
};

int mt_plan(const dmsim_mt_params* p, const dmsim_geometry* g, MtPlan* pl) {
  if (!p || !g) return fail(DMSIM_EINVAL, "null MT params or geometry");
  if (p->n_walkers < 0 || p->n_t < 1 || p->n_sub < 1 || p->n_meas < 1)
    return fail(DMSIM_EINVAL, "MT walk needs n_walkers >= 0, n_t, n_sub, n_meas >= 1");
  if (p->n_walkers > 0 && !p->r0) return fail(DMSIM_EINVAL, "MT walk needs start positions");
  if (p->spin) {
    if (p->n_echo < 1 || p->n_echo > kMtMaxEcho)
      return fail(DMSIM_ETOOBIG, "n_echo must be in [1, %d]", kMtMaxEcho);
    if (!p->echo_idx || !p->G || !p->rot || !p->sums)
      return fail(DMSIM_EINVAL, "MT spin walk needs echo_idx, G, rot and sums");
    for (int e = 0; e < p->n_echo; ++e) {
      if (p->echo_idx[e] < 0 || p->echo_idx[e] >= p->n_t)
        return fail(DMSIM_EINVAL, "echo index %d out of range", p->echo_idx[e]);
      if (e > 0 && p->echo_idx[e] <= p->echo_idx[e - 1])
        return fail(DMSIM_EINVAL, "echo indices must be strictly ascending");
    }
  }
  if (!p->status) return fail(DMSIM_EINVAL, "MT walk needs the status words");
  if (!(p->dwell_substeps > 0.f)) return fail(DMSIM_EINVAL, "dwell must be > 0");
  const bool packed =
      g->kind == DMSIM_GEOM_PACKED_CYLINDERS || g->kind == DMSIM_GEOM_PACKED_SPHERES;
  if (packed) {
    if (!g->cell_start || !g->cand || g->grid_n < 1 || !(g->L > 0.f))
      return fail(DMSIM_EINVAL, "packed geometry needs a cell list");
    if (!(g->reach >= p->step_length))
      return fail(DMSIM_EINVAL, "cell list reach %g is shorter than the step %g", g->reach,
                  p->step_length);
  }
  if ((g->kind == DMSIM_GEOM_BOX1D || g->kind == DMSIM_GEOM_SLAB) && !(g->L > 0.f))
    return fail(DMSIM_EINVAL, "slab geometry needs its length L > 0");
  if (g->kind == DMSIM_GEOM_ELLIPSOID &&
      !(g->radius > 0.f && g->ell_inv2[0] > 0.f && g->ell_inv2[1] > 0.f && g->ell_inv2[2] > 0.f))
    return fail(DMSIM_EINVAL, "ellipsoid needs positive semi-axes");
  pl->width = p->n_meas <= 1 ? 1 : 4;
  pl->fn = mt_fn(g->kind, pl->width);
  if (!pl->fn)
    return fail(DMSIM_EINVAL, "no MT walk for geometry kind %d (its walls have no log-weight "
                              "rule)", g->kind);
  pl->n_pass = (p->n_meas + pl->width - 1) / pl->width;
  int dev = 0, n_sm = 0, nb = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(DMSIM_ECUDA, "cudaGetDevice failed");
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return fail(DMSIM_ECUDA, "cudaDeviceGetAttribute failed");
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)pl->fn, kMtBlock, 0) !=
          cudaSuccess ||
      nb < 1)
    return fail(DMSIM_ECUDA, "MT kernel does not fit on an SM");
  const int64_t n_tiles = (p->n_walkers + kMtBlock - 1) / kMtBlock;
  int64_t grid = (int64_t)nb * n_sm;
  if (grid > n_tiles) grid = n_tiles;
  pl->grid = (int)(grid < 1 ? 1 : grid);
  pl->total = align256((size_t)pl->grid * (p->spin ? p->n_echo : 1) * pl->width * 3 * 8);
  return DMSIM_OK;
}

// Fixed-order sum of the per-block partials of one pass into its measurements' sums.
__global__ void k_mt_reduce(const double* __restrict__ part, int grid, int n_echo, int W, int M,
                            int m_off, double* __restrict__ sums) {
  const int n = n_echo * W * 3;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int e = i / (W * 3), r = i % (W * 3), m = m_off + r / 3;
    if (m >= M) continue;
    double acc = 0.0;
    for (int b = 0; b < grid; ++b) acc += part[((size_t)b * n_echo + e) * W * 3 + r];
    sums[((size_t)e * M + m) * 3 + r % 3] = acc;
  }
}

}  // namespace

namespace dmsim {
// Records an error for dmsim_last_error() on behalf of entry points in other translation units.
int set_error(int code, const char* msg) { return fail(code, "%s", msg); }
}  // namespace dmsim

extern "C" {

int dmsim_version(void) { return DMSIM_ABI_VERSION; }

const char* dmsim_last_error(void) { return g_err; }

size_t dmsim_walk_workspace_bytes(const dmsim_walk_params* p, const dmsim_geometry* g) {
  Plan pl;
  if (make_plan(p, g, &pl) != DMSIM_OK) return 0;
  return pl.total;
}

int dmsim_walk(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_walk_outputs* o,
               void* workspace, size_t workspace_bytes, void* stream) {
  Plan pl;
  int rc = make_plan(p, g, &pl);
  if (rc != DMSIM_OK) return rc;
  rc = check_outputs(p, g, o);
  if (rc != DMSIM_OK) return rc;
  if (!workspace || workspace_bytes < pl.total)
    return fail(DMSIM_EWORKSPACE, "workspace %zu B < required %zu B", workspace_bytes, pl.total);
  if (((uintptr_t)workspace & 255) != 0) return fail(DMSIM_EINVAL, "workspace must be 256-B aligned");
  return launch_single(p, g, o, pl, static_cast<uint8_t*>(workspace), (cudaStream_t)stream);
}

size_t dmsim_bloch_mt_workspace_bytes(const dmsim_mt_params* p, const dmsim_geometry* g) {
  MtPlan pl;
  if (mt_plan(p, g, &pl) != DMSIM_OK) return 0;
  return pl.total;
}

int dmsim_bloch_mt(const dmsim_mt_params* p, const dmsim_geometry* g, void* workspace,
                   size_t workspace_bytes, void* stream) {
  MtPlan pl;
  int rc = mt_plan(p, g, &pl);
  if (rc != DMSIM_OK) return rc;
  if (!workspace || workspace_bytes < pl.total)
    return fail(DMSIM_EWORKSPACE, "workspace %zu B < required %zu B", workspace_bytes, pl.total);
  if (((uintptr_t)workspace & 255) != 0) return fail(DMSIM_EINVAL, "workspace must be 256-B aligned");
  cudaStream_t st = (cudaStream_t)stream;
  if (p->n_walkers == 0) {
    if (p->spin) cudaMemsetAsync(p->sums, 0, sizeof(double) * p->n_echo * p->n_meas * 3, st);
    return DMSIM_OK;
  }
  MtArgs a;
  memset(&a, 0, sizeof(a));
  a.n_walkers = p->n_walkers;
  a.seed = p->seed;
  a.s0 = p->substep_offset;
  a.n_t = p->n_t;
  a.n_sub = p->n_sub;
  a.M = p->n_meas;
  a.n_echo = p->spin ? p->n_echo : 0;
  a.spin = p->spin ? 1 : 0;
  a.step_l = p->step_length;
  a.kod_mt = p->kappa_mt_over_D;
  a.dwell = p->dwell_substeps;
  a.rho = p->rho_over_D;
  a.gamma_dt = p->gamma_dt;
  a.m0 = p->m0;
  for (int k = 0; k < 2; ++k) {
    a.e2h[k] = p->e2h[k];
    a.e1h[k] = p->e1h[k];
  }
  a.g = make_geok(g);
  a.cs = g->cell_start;
  a.cand = reinterpret_cast<const float4*>(g->cand);
  a.G = p->G;
  a.rot = p->rot;
  a.crush = p->crush;
  a.r0 = p->r0;
  a.brem_in = p->brem_in;
  a.brem_out = p->brem_out;
  a.r_end = p->r_end;
  a.occ = p->occ;
  a.occ_total = p->occ_total;
  a.part = reinterpret_cast<double*>(workspace);
  a.status = p->status;
  a.traj = p->traj;
  a.traj_f16 = p->traj_f16;
  a.dlog_free = p->dlog_free;
  for (int e = 0; e < a.n_echo; ++e) a.echo[e] = p->echo_idx[e];
  const int passes = p->spin ? pl.n_pass : 1;
  for (int pass = 0; pass < passes; ++pass) {
    a.pass = pass;
    a.m_off = pass * pl.width;
    pl.fn<<<pl.grid, kMtBlock, 0, st>>>(a);
    if (p->spin) {
      const int nred = a.n_echo * pl.width * 3;
      k_mt_reduce<<<(nred + 255) / 256, 256, 0, st>>>(a.part, pl.grid, a.n_echo, pl.width,
                                                      p->n_meas, a.m_off, p->sums);
    }
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(DMSIM_ECUDA, "launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

size_t dmsim_bloch_workspace_bytes(const dmsim_walk_params* p, const dmsim_geometry* g) {
  Plan pl;
  if (make_plan(p, g, &pl, kTabSmemBudget, true) != DMSIM_OK) return 0;
  return pl.total;
}

int dmsim_bloch(const dmsim_walk_params* p, const dmsim_geometry* g, const dmsim_bloch_params* b,
                const dmsim_walk_outputs* o, void* workspace, size_t workspace_bytes,
                void* stream) {
  if (!b || !b->rf_flip || !b->rf_axis)
    return fail(DMSIM_EINVAL, "Bloch parameters need the per-sample flip and axis");
  if (!(b->t1_sample >= 0.f)) return fail(DMSIM_EINVAL, "t1_sample must be >= 0");
  if (b->field_kind < 0 || b->field_kind > 3)
    return fail(DMSIM_EINVAL, "unknown susceptibility field kind %d", b->field_kind);
  if (b->field_kind && !b->field_tab)
    return fail(DMSIM_EINVAL, "susceptibility field needs its table");
  if ((b->field_kind == 1 || b->field_kind == 2) && b->field_n < 0)
    return fail(DMSIM_EINVAL, "negative susceptibility source count");
  if (b->field_kind == 3 && (b->field_dims[0] < 1 || b->field_dims[1] < 1 ||
                             b->field_dims[2] < 1 || !(b->field_par[3] > 0.f) ||
                             !(b->field_par[4] > 0.f) || !(b->field_par[5] > 0.f)))
    return fail(DMSIM_EINVAL, "susceptibility grid needs positive dims and voxel sizes");
  if (o && o->phi) return fail(DMSIM_EINVAL, "the Bloch walk has no per-walker phase output");
  Plan pl;
  int rc = make_plan(p, g, &pl, kTabSmemBudget, true);
  if (rc != DMSIM_OK) return rc;
  rc = check_outputs(p, g, o);
  if (rc != DMSIM_OK) return rc;
  if (!workspace || workspace_bytes < pl.total)
    return fail(DMSIM_EWORKSPACE, "workspace %zu B < required %zu B", workspace_bytes, pl.total);
  if (((uintptr_t)workspace & 255) != 0) return fail(DMSIM_EINVAL, "workspace must be 256-B aligned");
  return launch_single(p, g, o, pl, static_cast<uint8_t*>(workspace), (cudaStream_t)stream, b);
}

int dmsim_step_kat(const dmsim_geometry* g, int64_t n, const float* r_in, const float* steps,
                   const float* u, float* r_out, float* dlog_unit, void* stream) {
  if (!g || n < 0 || (n > 0 && (!r_in || !steps || !r_out || !dlog_unit)))
    return fail(DMSIM_EINVAL, "step_kat: bad arguments");
  if (g->wall_mode == DMSIM_WALL_PERMEATE && n > 0 && !u)
    return fail(DMSIM_EINVAL, "step_kat: permeate needs the uniforms");
  const bool packed =
      g->kind == DMSIM_GEOM_PACKED_CYLINDERS || g->kind == DMSIM_GEOM_PACKED_SPHERES;
  if (packed && (!g->cell_start || !g->cand || g->grid_n < 1))
    return fail(DMSIM_EINVAL, "step_kat: packed geometry needs a cell list");
  if (g->kind == DMSIM_GEOM_MESH && (!g->tri || !g->tri_vn || !g->mesh_cell_start ||
                                     !g->mesh_cell_tri || g->max_bounces < 1))
    return fail(DMSIM_EINVAL, "step_kat: mesh geometry needs its tables");
  KatFn fn = nullptr;
  switch (g->kind) {
    case DMSIM_GEOM_FREE: fn = kat_fn<DMSIM_GEOM_FREE>(g->wall_mode); break;
    case DMSIM_GEOM_CYLINDER: fn = kat_fn<DMSIM_GEOM_CYLINDER>(g->wall_mode); break;
    case DMSIM_GEOM_SPHERE: fn = kat_fn<DMSIM_GEOM_SPHERE>(g->wall_mode); break;
    case DMSIM_GEOM_PACKED_CYLINDERS: fn = kat_fn<DMSIM_GEOM_PACKED_CYLINDERS>(g->wall_mode); break;
    case DMSIM_GEOM_PACKED_SPHERES: fn = kat_fn<DMSIM_GEOM_PACKED_SPHERES>(g->wall_mode); break;
    case DMSIM_GEOM_MESH: fn = kat_fn<DMSIM_GEOM_MESH>(g->wall_mode); break;
    case DMSIM_GEOM_BOX1D: fn = kat_fn<DMSIM_GEOM_BOX1D>(g->wall_mode); break;
    case DMSIM_GEOM_SLAB: fn = kat_fn<DMSIM_GEOM_SLAB>(g->wall_mode); break;
    case DMSIM_GEOM_SHELL: fn = kat_fn<DMSIM_GEOM_SHELL>(g->wall_mode); break;
    case DMSIM_GEOM_ELLIPSOID: fn = kat_fn<DMSIM_GEOM_ELLIPSOID>(g->wall_mode); break;
    default: return fail(DMSIM_EINVAL, "step_kat: unsupported geometry kind %d", g->kind);
  }
  if (n == 0) return DMSIM_OK;
  const int blocks = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
  fn<<<blocks, 256, 8 * kMeshScratchBytes, (cudaStream_t)stream>>>(make_geok(g), make_meshk(g), n, r_in, steps, u,
                                                 g->cell_start,
                                                 reinterpret_cast<const float4*>(g->cand), r_out,
                                                 dlog_unit);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(DMSIM_ECUDA, "step_kat launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

int dmsim_mesh_neighbourhoods(const dmsim_geometry* g, uint32_t* nb_start, uint32_t* nb_tri,
                              void* stream) {
  if (!g || !nb_start || !g->mesh_cell_start || !g->mesh_cell_tri || g->mesh_dims[0] < 1 ||
      g->mesh_dims[1] < 1 || g->mesh_dims[2] < 1)
    return fail(DMSIM_EINVAL, "mesh_neighbourhoods: bad arguments");
  const int64_t n = (int64_t)g->mesh_dims[0] * g->mesh_dims[1] * g->mesh_dims[2];
  const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  k_mesh_nb<<<blocks, 256, 0, (cudaStream_t)stream>>>(
      g->mesh_cell_start, g->mesh_cell_tri, g->mesh_dims[0], g->mesh_dims[1], g->mesh_dims[2],
      nb_tri ? nb_start : nullptr, nb_tri ? nb_tri : nb_start);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess)
    return fail(DMSIM_ECUDA, "mesh_neighbourhoods launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

int dmsim_mesh_hit_lists(const dmsim_geometry* g, float reach, uint32_t* hit_start,
                         uint32_t* hit_tri, float* hit_bs, void* stream) {
  if (hit_bs && (!hit_tri || !g || !g->tri_bs))
    return fail(DMSIM_EINVAL, "mesh_hit_lists: hit_bs needs hit_tri and g->tri_bs");
  if (!g || !hit_start || !g->tri || !g->mesh_nb_start || !g->mesh_nb_tri ||
      g->mesh_dims[0] < 1 || g->mesh_dims[1] < 1 || g->mesh_dims[2] < 1 ||
      !(g->mesh_cell > 0.f) || !(reach > 0.f) || !isfinite(reach))
    return fail(DMSIM_EINVAL, "mesh_hit_lists: bad arguments");
  const int64_t n = (int64_t)g->mesh_dims[0] * g->mesh_dims[1] * g->mesh_dims[2];
  const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  k_mesh_hit<<<blocks, 256, 0, (cudaStream_t)stream>>>(
      g->mesh_nb_start, g->mesh_nb_tri, g->tri, g->mesh_dims[0], g->mesh_dims[1],
      g->mesh_dims[2], g->grid_min[0], g->grid_min[1], g->grid_min[2], g->mesh_cell, reach,
      hit_tri ? hit_start : nullptr, hit_tri ? hit_tri : hit_start,
      reinterpret_cast<const float4*>(g->tri_bs), reinterpret_cast<float4*>(hit_bs));
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess)
    return fail(DMSIM_ECUDA, "mesh_hit_lists launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

size_t dmsim_replay_workspace_bytes(int64_t n_walkers, int32_t n_t, int32_t n_meas) {
  (void)n_t;
  if (n_walkers <= 0 || n_meas <= 0) return 256;
  return align256((size_t)replay_grid(n_walkers) * n_meas * 3 * 8);
}

int dmsim_replay(const void* traj, int32_t traj_f16, int64_t n_walkers, int32_t n_t,
                 const float* G, int32_t n_meas, float gamma_dt, const float* log_w, double* sums,
                 float* phi_out, void* workspace, size_t workspace_bytes, void* stream) {
  if (!traj || !G || !sums || n_walkers < 1 || n_t < 1 || n_meas < 1)
    return fail(DMSIM_EINVAL, "replay: bad arguments");
  const int grid = replay_grid(n_walkers);
  const size_t need = align256((size_t)grid * n_meas * 3 * 8);
  if (!workspace || workspace_bytes < need)
    return fail(DMSIM_EWORKSPACE, "replay workspace %zu B < required %zu B", workspace_bytes, need);
  cudaStream_t st = (cudaStream_t)stream;
  double* part = static_cast<double*>(workspace);
  k_zero<<<64, 256, 0, st>>>(part, (size_t)grid * n_meas * 3);
  if (traj_f16)
    k_replay<true><<<grid, kRB, 0, st>>>(traj, n_walkers, n_t, G, n_meas, gamma_dt, log_w, part,
                                         phi_out);
  else
    k_replay<false><<<grid, kRB, 0, st>>>(traj, n_walkers, n_t, G, n_meas, gamma_dt, log_w, part,
                                          phi_out);
  const int nred = n_meas * 3;
  k_reduce<<<(nred + 255) / 256, 256, 0, st>>>(part, grid, 1, n_meas, n_meas, sums);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return fail(DMSIM_ECUDA, "replay launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

int dmsim_project_modes(const void* x, int32_t x_f16, int64_t n_walkers, int32_t n_t, int32_t n_ch,
                        const float* basis, int32_t K, const float* ramp, float* endpoint,
                        float* out, void* stream) {
  if (!x || !basis || !out || n_walkers < 1 || n_t < 1 || K < 1)
    return fail(DMSIM_EINVAL, "project_modes: bad arguments");
  if (n_ch != 1 && n_ch != 3) return fail(DMSIM_EINVAL, "project_modes: n_ch must be 1 or 3");
  if (ramp && (n_ch != 1 || !endpoint))
    return fail(DMSIM_EINVAL, "project_modes: the cumulative form needs n_ch == 1 and endpoint");
  const cudaError_t err = launch_project_modes(x, x_f16 != 0, n_walkers, n_t, n_ch, basis, K, ramp,
                                               endpoint, out, (cudaStream_t)stream);
  if (err != cudaSuccess)
    return fail(DMSIM_ECUDA, "project_modes launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

}  // extern "C"

// ================================================================================================
// Batched walks
// ================================================================================================
namespace {

struct PrepItem {  // waveform re-layout of one batched instance
  const float* V;
  const float* C;
  float* Vp;
  uint8_t* act;
  float* Cp;
  int n_t, M, r, rt, t_pad, pad;
};

struct RedItem {  // reduction of one batched instance's work-item partials
  const double* part;
  double* sums;
  int64_t n_items;
  int n, pad;
};

__global__ void k_prep_basis_batch(const PrepItem* __restrict__ items) {
  const PrepItem it = items[blockIdx.y];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t i = i0; i < it.t_pad; i += stride) {
    const int t = (int)i;
    bool any = false;
    for (int j = 0; j < it.rt; ++j) {
      const float v = (t < it.n_t && j < it.r) ? it.V[(size_t)t * it.r + j] : 0.f;
      it.Vp[(size_t)t * it.rt + j] = v;
      any |= (v != 0.f);
    }
    if (t < it.n_t) it.act[t] = any ? 1 : 0;
  }
  for (int64_t i = i0; i < (int64_t)it.M * 3 * it.rt; i += stride) {
    const int j = (int)(i % it.rt);
    it.Cp[i] = j < it.r ? it.C[(i / it.rt) * it.r + j] : 0.f;
  }
}

// Fixed-order sum of every instance's work-item partials (instance = blockIdx.y).
__global__ void k_reduce_batch(const RedItem* __restrict__ items) {
  const RedItem it = items[blockIdx.y];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < it.n; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int64_t b = 0; b < it.n_items; ++b) acc += it.part[(size_t)b * it.n + i];
    it.sums[i] = acc;
  }
}

WalkFn batch_fn(const dmsim_geometry* g, int width, bool tsm) {
  switch (g->kind) {
    case DMSIM_GEOM_FREE: return walk_batch_fn_free(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_CYLINDER: return walk_batch_fn_cyl(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_SPHERE: return walk_batch_fn_sph(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_PACKED_CYLINDERS: return walk_batch_fn_pcyl(g->wall_mode, 1, width, tsm);
    case DMSIM_GEOM_PACKED_SPHERES: return walk_batch_fn_psph(g->wall_mode, 1, width, tsm);
    case DMSIM_GEOM_MESH: return walk_batch_fn_mesh(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_BOX1D: return walk_batch_fn_box1d(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_SLAB: return walk_batch_fn_slab(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_SHELL: return walk_batch_fn_shell(g->wall_mode, 1, width, false);
    case DMSIM_GEOM_ELLIPSOID: return walk_batch_fn_ellipsoid(g->wall_mode, 1, width, false);
  }
  return nullptr;
}

struct BatchInst {
  dmsim_walk_params p;
  dmsim_geometry g;
  dmsim_walk_outputs o;
  std::vector<int32_t> echo;
  Plan pl;
  bool batched = false;
  int group = -1;
  int64_t n_items = 0;
  size_t off_gp = 0, off_act = 0, off_cp = 0, off_part = 0;  // batched: own slices
  size_t off_ws = 0;                                         // plain: its dmsim_walk workspace
};

struct BatchGroup {
  WalkFn fn = nullptr;
  int grid = 0, max_m = 0;
  size_t smem = 0, max_tab = 0;
  std::vector<int> members;  // instance indices in work-queue order
  int64_t n_items = 0;
  size_t off_items = 0;      // (members + 1) int64 prefix sums of work items
  size_t off_kargs = 0;      // members x KArgs
};

}  // namespace

struct dmsim_batch {
  int device = 0;
  dmsim_batch_tuning tune{};
  std::vector<BatchInst> inst;
  std::vector<BatchGroup> groups;
  std::vector<int> batched;  // instance indices with a batched walk (prep / reduce order)
  size_t off_prep = 0, off_red = 0, off_ctr = 0, off_tables = 0, total = 0;
  std::vector<uint8_t> blob;  // host image of [off_tables, off_ctr)
  uint8_t* ws = nullptr;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> ev;  // [0] fork, [1 + i] join of side stream i
};

namespace {

int batch_plan(dmsim_batch* b) {
  int n_sm = 0;
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess)
    return fail(DMSIM_ECUDA, "cudaDeviceGetAttribute failed");
  const size_t budget = b->tune.tab_smem_bytes > 0 ? (size_t)b->tune.tab_smem_bytes : kTabSmemBudget;
  const int tpi = b->tune.tiles_per_item > 0 ? b->tune.tiles_per_item : 1;
  std::map<std::tuple<int, int, int, bool>, int> key2group;
  size_t off = 0;
  for (size_t i = 0; i < b->inst.size(); ++i) {
    BatchInst& I = b->inst[i];
    I.p.echo_idx = I.echo.data();
    int rc = make_plan(&I.p, &I.g, &I.pl, budget);
    if (rc != DMSIM_OK) return rc;
    rc = check_outputs(&I.p, &I.g, &I.o);
    if (rc != DMSIM_OK) return rc;
    // a myelinated cylinder has no batched kernel: its instances run as plain walks
    I.batched = I.pl.pm == 1 && I.g.kind != DMSIM_GEOM_MYELIN && I.g.kind != DMSIM_GEOM_PMYELIN;
    if (!I.batched) {
      I.off_ws = off;
      off = align256(off + I.pl.total);
      continue;
    }
    const int64_t n_tiles = (I.p.n_walkers + kBlock - 1) / kBlock;
    I.n_items = (n_tiles + tpi - 1) / tpi;
    const int t_pad = I.pl.n_chunks * kTC;
    I.off_gp = off;
    off = align256(off + (size_t)t_pad * I.pl.width * 4);
    I.off_act = off;
    off = align256(off + (size_t)I.p.n_t);
    I.off_cp = off;
    off = align256(off + (size_t)I.p.n_meas * 3 * I.pl.width * 4);
    I.off_part = off;
    off = align256(off + (size_t)I.n_items * I.p.n_echo * I.p.n_meas * 3 * 8);
    const auto key = std::make_tuple((int)I.g.kind, (int)I.g.wall_mode, I.pl.width, I.pl.tsm);
    auto itg = key2group.find(key);
    if (itg == key2group.end()) {
      itg = key2group.emplace(key, (int)b->groups.size()).first;
      b->groups.emplace_back();
      b->groups.back().fn = batch_fn(&I.g, I.pl.width, I.pl.tsm);
      if (!b->groups.back().fn) return fail(DMSIM_EINVAL, "no batched kernel for instance %zu", i);
    }
    I.group = itg->second;
    BatchGroup& G = b->groups[I.group];
    G.members.push_back((int)i);
    G.max_m = std::max(G.max_m, I.p.n_meas);
    if (I.pl.tsm) G.max_tab = std::max(G.max_tab, I.pl.tab_cs + I.pl.tab_cand);
    b->batched.push_back((int)i);
  }
  // work-queue order inside a group: costliest tile first (longest-processing-time rule)
  for (BatchGroup& G : b->groups) {
    if (b->tune.order == 1)
      std::stable_sort(G.members.begin(), G.members.end(), [&](int x, int y) {
        const BatchInst &X = b->inst[x], &Y = b->inst[y];
        return (double)X.p.n_t * X.p.sub_steps > (double)Y.p.n_t * Y.p.sub_steps;
      });
    G.n_items = 0;
    for (int m : G.members) G.n_items += b->inst[m].n_items;
    G.smem = walk_smem_layout(1, b->inst[G.members[0]].pl.width, G.max_m).off_tab + G.max_tab +
             (b->inst[G.members[0]].g.kind == DMSIM_GEOM_MESH ? kWarps * kMeshScratchBytes : 0);
    if (cudaFuncSetAttribute((const void*)G.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)G.smem) != cudaSuccess)
      return fail(DMSIM_ECUDA, "cudaFuncSetAttribute(%zu B shared) failed", G.smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)G.fn, kBlock, G.smem) !=
            cudaSuccess ||
        nb < 1)
      return fail(DMSIM_ECUDA, "batched kernel does not fit on an SM (%zu B shared)", G.smem);
    if (b->tune.blocks_per_sm > 0) nb = std::min(nb, (int)b->tune.blocks_per_sm);
    int64_t grid = (int64_t)nb * n_sm;
    grid = std::min<int64_t>(grid, std::max<int64_t>(G.n_items, 1));
    G.grid = (int)grid;
  }
  // tables: per group the item prefix sums and the KArgs, then prep / reduce items, counters
  b->off_tables = off;
  for (BatchGroup& G : b->groups) {
    G.off_items = off;
    off = align256(off + (G.members.size() + 1) * sizeof(int64_t));
    G.off_kargs = off;
    off = align256(off + G.members.size() * sizeof(KArgs));
  }
  b->off_prep = off;
  off = align256(off + b->batched.size() * sizeof(PrepItem));
  b->off_red = off;
  off = align256(off + b->batched.size() * sizeof(RedItem));
  b->off_ctr = off;
  off = align256(off + std::max<size_t>(b->groups.size(), 1) * 8);
  b->total = off;
  return DMSIM_OK;
}

}  // namespace

extern "C" {

int dmsim_batch_create(int32_t n, const dmsim_walk_params* p, const dmsim_geometry* g,
                       const dmsim_walk_outputs* o, const dmsim_batch_tuning* tuning,
                       dmsim_batch** out, size_t* workspace_bytes) {
  if (!out) return fail(DMSIM_EINVAL, "batch_create: out is null");
  *out = nullptr;
  if (n < 0 || (n > 0 && (!p || !g || !o))) return fail(DMSIM_EINVAL, "batch_create: bad arguments");
  if (tuning && (tuning->blocks_per_sm < 0 || tuning->tiles_per_item < 0 || tuning->order < 0 ||
                 tuning->order > 1 || tuning->tab_smem_bytes < 0 ||
                 tuning->tab_smem_bytes > 200 * 1024))
    return fail(DMSIM_EINVAL, "batch_create: bad tuning");
  dmsim_batch* b = new dmsim_batch();
  if (tuning) b->tune = *tuning;
  else b->tune.concurrent_groups = 1;
  if (cudaGetDevice(&b->device) != cudaSuccess) {
    delete b;
    return fail(DMSIM_ECUDA, "cudaGetDevice failed");
  }
  b->inst.resize(n);
  for (int i = 0; i < n; ++i) {
    BatchInst& I = b->inst[i];
    I.p = p[i];
    I.g = g[i];
    I.o = o[i];
    if (p[i].n_echo < 1 || p[i].n_echo > kMaxEcho || !p[i].echo_idx) {
      delete b;
      return fail(DMSIM_EINVAL, "batch instance %d: n_echo must be in [1, %d] with echo_idx", i,
                  kMaxEcho);
    }
    I.echo.assign(p[i].echo_idx, p[i].echo_idx + p[i].n_echo);
  }
  const int rc = batch_plan(b);
  if (rc != DMSIM_OK) {
    delete b;
    return rc;
  }
  if (b->tune.concurrent_groups && b->groups.size() > 1) {
    const size_t n_side = std::min<size_t>(b->groups.size(), 4);
    b->ev.resize(1 + n_side, nullptr);
    bool ok = true;
    for (auto& e : b->ev) ok &= cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    b->side.resize(n_side, nullptr);
    for (auto& s : b->side) ok &= cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
      dmsim_batch_destroy(b);
      return fail(DMSIM_ECUDA, "batch_create: stream/event creation failed");
    }
  }
  if (workspace_bytes) *workspace_bytes = b->total;
  *out = b;
  return DMSIM_OK;
}

int dmsim_batch_bind(dmsim_batch* b, void* workspace, size_t workspace_bytes, void* stream) {
  if (!b) return fail(DMSIM_EINVAL, "batch_bind: null plan");
  if (!workspace || workspace_bytes < b->total)
    return fail(DMSIM_EWORKSPACE, "batch workspace %zu B < required %zu B", workspace_bytes,
                b->total);
  if (((uintptr_t)workspace & 255) != 0)
    return fail(DMSIM_EINVAL, "workspace must be 256-B aligned");
  uint8_t* ws = static_cast<uint8_t*>(workspace);
  b->blob.assign(b->off_ctr - b->off_tables, 0);
  auto at = [&](size_t off) { return b->blob.data() + (off - b->off_tables); };
  for (BatchGroup& G : b->groups) {
    int64_t* starts = reinterpret_cast<int64_t*>(at(G.off_items));
    KArgs* ka = reinterpret_cast<KArgs*>(at(G.off_kargs));
    int64_t acc = 0;
    for (size_t k = 0; k < G.members.size(); ++k) {
      const BatchInst& I = b->inst[G.members[k]];
      starts[k] = acc;
      acc += I.n_items;
      KArgs a;
      fill_kargs(&I.p, &I.g, &I.o, I.pl, &a);
      a.Cp = reinterpret_cast<const float*>(ws + I.off_cp);
      a.Gp = reinterpret_cast<const float*>(ws + I.off_gp);
      a.active = ws + I.off_act;
      a.part = reinterpret_cast<double*>(ws + I.off_part);
      a.pass = 0;
      memcpy(&ka[k], &a, sizeof(KArgs));
    }
    starts[G.members.size()] = acc;
  }
  PrepItem* prep = reinterpret_cast<PrepItem*>(at(b->off_prep));
  RedItem* red = reinterpret_cast<RedItem*>(at(b->off_red));
  for (size_t k = 0; k < b->batched.size(); ++k) {
    const BatchInst& I = b->inst[b->batched[k]];
    PrepItem& P = prep[k];
    P.V = I.p.basis_V;
    P.C = I.p.basis_C;
    P.Vp = reinterpret_cast<float*>(ws + I.off_gp);
    P.act = ws + I.off_act;
    P.Cp = reinterpret_cast<float*>(ws + I.off_cp);
    P.n_t = I.p.n_t;
    P.M = I.p.n_meas;
    P.r = I.p.basis_rank;
    P.rt = I.pl.width;
    P.t_pad = I.pl.n_chunks * kTC;
    RedItem& R = red[k];
    R.part = reinterpret_cast<const double*>(ws + I.off_part);
    R.sums = I.o.sums;
    R.n_items = I.n_items;
    R.n = I.p.n_echo * I.p.n_meas * 3;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (!b->blob.empty() &&
      cudaMemcpyAsync(ws + b->off_tables, b->blob.data(), b->blob.size(), cudaMemcpyHostToDevice,
                      st) != cudaSuccess)
    return fail(DMSIM_ECUDA, "batch_bind: table upload failed");
  if (cudaStreamSynchronize(st) != cudaSuccess)
    return fail(DMSIM_ECUDA, "batch_bind: %s", cudaGetErrorString(cudaGetLastError()));
  b->ws = ws;
  return DMSIM_OK;
}

int dmsim_batch_launch(const dmsim_batch* b, void* stream) {
  if (!b || !b->ws) return fail(DMSIM_EINVAL, "batch_launch: plan is null or not bound");
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* ws = b->ws;
  const int nb = (int)b->batched.size();
  if (nb > 0) {
    if (cudaMemsetAsync(ws + b->off_ctr, 0, b->groups.size() * 8, st) != cudaSuccess)
      return fail(DMSIM_ECUDA, "batch_launch: counter reset failed");
    k_prep_basis_batch<<<dim3(8, nb), 256, 0, st>>>(
        reinterpret_cast<const PrepItem*>(ws + b->off_prep));
  }
  const bool fork = !b->side.empty();
  if (fork && cudaEventRecord(b->ev[0], st) != cudaSuccess)
    return fail(DMSIM_ECUDA, "batch_launch: event record failed");
  for (size_t s = 0; fork && s < b->side.size(); ++s)
    if (cudaStreamWaitEvent(b->side[s], b->ev[0], 0) != cudaSuccess)
      return fail(DMSIM_ECUDA, "batch_launch: stream wait failed");
  KArgs none;
  memset(&none, 0, sizeof(none));
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    const BatchGroup& G = b->groups[gi];
    BatchCtl bc;
    memset(&bc, 0, sizeof(bc));
    bc.inst = reinterpret_cast<const KArgs*>(ws + G.off_kargs);
    bc.item_start = reinterpret_cast<const int64_t*>(ws + G.off_items);
    bc.n_inst = (int)G.members.size();
    bc.max_m = G.max_m;
    bc.tiles_per_item = b->tune.tiles_per_item > 0 ? b->tune.tiles_per_item : 1;
    bc.total = G.n_items;
    bc.counter = reinterpret_cast<unsigned long long*>(ws + b->off_ctr + 8 * gi);
    cudaStream_t gs = fork ? b->side[gi % b->side.size()] : st;
    G.fn<<<G.grid, kBlock, G.smem, gs>>>(none, bc);
  }
  for (const BatchInst& I : b->inst) {
    if (I.batched) continue;
    const int rc = launch_single(&I.p, &I.g, &I.o, I.pl, ws + I.off_ws, st);
    if (rc != DMSIM_OK) return rc;
  }
  for (size_t s = 0; fork && s < b->side.size(); ++s) {
    if (cudaEventRecord(b->ev[1 + s], b->side[s]) != cudaSuccess ||
        cudaStreamWaitEvent(st, b->ev[1 + s], 0) != cudaSuccess)
      return fail(DMSIM_ECUDA, "batch_launch: stream join failed");
  }
  if (nb > 0) {
    int max_n = 1;
    for (int k : b->batched) max_n = std::max(max_n, b->inst[k].p.n_echo * b->inst[k].p.n_meas * 3);
    const int gx = std::min(64, (max_n + 255) / 256);
    k_reduce_batch<<<dim3(gx, nb), 256, 0, st>>>(reinterpret_cast<const RedItem*>(ws + b->off_red));
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess)
    return fail(DMSIM_ECUDA, "batch launch failed: %s", cudaGetErrorString(err));
  return DMSIM_OK;
}

int dmsim_batch_info(const dmsim_batch* b, int32_t* n_groups, int32_t* n_single, int64_t* n_items,
                     int32_t* n_kernels) {
  if (!b) return fail(DMSIM_EINVAL, "batch_info: null plan");
  int singles = 0, kern = 0;
  int64_t items = 0;
  for (const BatchInst& I : b->inst) {
    if (I.batched) continue;
    ++singles;
    if (I.p.n_walkers > 0) kern += 2 + I.pl.n_pass;
  }
  for (const BatchGroup& G : b->groups) items += G.n_items;
  if (!b->batched.empty()) kern += 2 + (int)b->groups.size();
  if (n_groups) *n_groups = (int32_t)b->groups.size();
  if (n_single) *n_single = singles;
  if (n_items) *n_items = items;
  if (n_kernels) *n_kernels = kern;
  return DMSIM_OK;
}

void dmsim_batch_destroy(dmsim_batch* b) {
  if (!b) return;
  for (auto& s : b->side)
    if (s) cudaStreamDestroy(s);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  delete b;
}

}  // extern "C"
