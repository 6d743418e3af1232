// The persistent walk kernel: one walker per thread, walker state in registers.
//
// Replaces the vmap(lax.scan(step_fn)) of dmipy-sim (core.py:700-727, physics.py:191-417) and the
// producer walk of simulate_trajectories (core.py:1137-1155, 1246-1307).  Per block:
//   * the packed-object cell list is staged into shared memory once with a bulk async copy
//     (cp.async.bulk + mbarrier), when it fits;
//   * the gradient waveform streams through shared memory in chunks of kTC samples, double
//     buffered with bulk async copies, so every walker of the block reads each G(t) as a
//     broadcast;
//   * each thread walks its walker for all n_t samples x S sub-steps, drawing from a Philox
//     stream keyed by (seed, global walker index);
//   * the phase is accumulated in FP32 registers with Kahan compensation, from R(t), the sample's
//     last position (walk-once + replay, trajectories.py:550-552) or the sum of its S sub-step
//     positions (fused engine: G is constant over the sub-steps of a sample, physics.py:293-317,
//     so sum_s g.r_s = g . sum_s r_s), in one of two forms:
//       direct (PM = 0): phi_m += gamma_dt * g_m(t) . R(t) for MT measurements per pass;
//       basis  (PM = 1): when the measurement set is built from RT waveform shapes,
//         G[t, m, k] = sum_j C[m, k, j] V[t, j], the kernel accumulates only
//         Q[j, k] += gamma_dt * V[t, j] R_k(t) (3 RT registers, 3 RT FMAs per sample) and forms
//         phi_m = sum_jk C[m, k, j] Q[j, k] at the echo samples;
//       vector Bloch (PM = 2, bloch.py:44-57, 109-131, 180-198): each walker carries the
//         magnetisation M_m = (Mx, My, Mz) of every measurement through RF rotations, free
//         precession and relaxation.  Between RF events precession, T2 and the wall weight act on
//         Mxy alone and commute, so the kernel keeps M_m as of the last RF event plus the phase
//         (gradient, Kahan; carriers), log-weight and T1 time accrued since, and forms M_m only
//         at an RF sample (before the rotation) and at an echo;
//   * at every echo sample the block reduces w*cos(phi), w*sin(phi) and (w*cos(phi))^2 (Bloch:
//     Mx, My, Mz) with warp shuffles and adds them, in FP64 and in a fixed order, into the
//     block's own partial slice.
// Blocks loop over walker tiles (grid = SMs x resident blocks), so the partial buffer is
// independent of n_walkers.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "dmsim.h"
#include "geometry.cuh"
#include "mesh.cuh"
#include "philox.cuh"

namespace dmsim {

constexpr int kBlock = 320;  // walkers per tile (10 warps share one staged cell list)
constexpr int kWarps = kBlock / 32;
constexpr int kTC = 16;  // samples per staged waveform chunk
constexpr int kMaxEcho = 512;

struct KArgs {
  int64_t n_walkers, walker_offset;
  uint64_t seed;
  int n_t, n_chunks, S, phase_sub, has_weight, n_echo, Mp, pass, M;
  float step_l, gamma_dt, t2dec, t1dec, rho;
  GeoK g;
  MeshK mk;  // GEOM_MESH only
  MyelinK my;  // GEOM_MYELIN only
  PMyelinK pm;  // GEOM_PMYELIN only
  uint32_t tab_cs_bytes, tab_cand_bytes;  // shared-memory staging sizes (multiples of 16 B)
  const float* Cp;                        // basis mode: (M, 3, RT) coefficients
  const uint32_t* cs;
  const float4* cand;
  const int32_t* cand_obj;
  const float* Gp;          // this pass: direct (n_chunks*kTC, MT, 3); basis (n_chunks*kTC, RT)
  const uint8_t* active;    // this pass, (n_t): 1 where some g_m(t) != 0
  const float* chi;         // (n_t) or null
  const float* r0;          // (n_walkers, 3) or null
  double* part;             // single: [gridDim.x][n_echo][Mp][3]; batched: [item][n_echo][M][3]
  uint32_t* status;
  float* final_pos;
  float* log_w;
  float* phi_out;
  int32_t* comp0;
  int32_t* comp_end;
  void* traj;
  int traj_f16;
  float* dlog_unit;
  float* comp_occ;
  // vector-Bloch form: per-sample RF flip and B1 axis (rad; flip 0 = no pulse), extra precession
  // per sample (rad: off-resonance + pulse carrier), crusher rate per sample (rad per unit of the
  // walker's crusher coordinate), equilibrium M0 and dt/T1 per sample
  const float* rf_flip;
  const float* rf_axis;
  const float* carrier;
  const float* crush;
  float m0, t1_sample;
  // susceptibility field of the Bloch form: kind (0 none, 1 spheres, 2 myelin cylinders, 3 grid),
  // table or grid, rotation into the field frame, parameters, grid dims, gamma * dt
  int fkind, fn;
  const float* ftab;
  float frot[9], fpar[8];
  int fdims[3];
  float fgdt;
  // free-flight kernel: lanes waiting for a wall scan, a hit resolution and a sample update
  // before the warp runs that stage
  int ff_quorum[3];
  int ff_skip;  // 1: free flight inside the wall-free disc; 0: a scan on every sub-step
  int echo[kMaxEcho];
};

// dBz (T) of the susceptibility field at a walk-frame position (susceptibility.py:78-205,
// 348-365): superposed magnetised spheres (distance clamped to the radius inside), periodic
// hollow myelin cylinders, or a trilinearly sampled grid.
static __device__ __noinline__ float field_dbz(const KArgs& a, float rx, float ry, float rz) {
  const float* R = a.frot;
  const float x = R[0] * rx + R[1] * ry + R[2] * rz;
  const float y = R[3] * rx + R[4] * ry + R[5] * rz;
  const float z = R[6] * rx + R[7] * ry + R[8] * rz;
  if (a.fkind == 1) {
    float sum = 0.f;
    for (int k = 0; k < a.fn; ++k) {
      const float* t = a.ftab + 5 * k;
      const float dx = x - __ldg(t), dy = y - __ldg(t + 1), dz = z - __ldg(t + 2);
      const float q = fmaxf(dx * dx + dy * dy + dz * dz, __ldg(t + 4));
      sum += __ldg(t + 3) * (3.f * (dz * dz) / q - 1.f) / (q * sqrtf(q));
    }
    return sum;
  }
  if (a.fkind == 2) {
    const float L = a.fpar[0];
    float px = x, py = y;
    if (a.fpar[5] != 0.f) {
      px += 0.5f * L;
      px -= L * floorf(px / L);
      px -= 0.5f * L;
      py += 0.5f * L;
      py -= L * floorf(py / L);
      py -= 0.5f * L;
    }
    const int ni = (int)a.fpar[4];
    float p0 = 0.f, pc = 0.f, ps = 0.f;
    for (int k = 0; k < a.fn; ++k) {
      const float* t = a.ftab + 8 * k;
      const float cx = __ldg(t), cy = __ldg(t + 1), a2 = __ldg(t + 2), b2 = __ldg(t + 3);
      const float a4 = __ldg(t + 4), lba = __ldg(t + 5);
      for (int jy = -ni; jy <= ni; ++jy)
        for (int jx = -ni; jx <= ni; ++jx) {
          const float dx = px - (cx + (float)jx * L), dy = py - (cy + (float)jy * L);
          const float r2 = dx * dx + dy * dy, r4 = r2 * r2;
          float f = 0.f;
          if (r2 > b2) {
            f = (b2 - a2) / r4;
          } else if (r2 > a2) {
            f = (r4 - a4) / (r4 * (b2 + a2));
            p0 += -0.5f * logf(r2 / b2);
          } else if (r2 < a2) {
            p0 += lba;
          }
          pc += f * (dx * dx - dy * dy);
          ps += f * 2.f * dx * dy;
        }
    }
    return a.fpar[1] * p0 + a.fpar[1] * (a.fpar[2] * pc + a.fpar[3] * ps);
  }
  // grid: voxel (0, 0, 0) centred at origin + voxel / 2
  const int per = a.fpar[6] != 0.f;
  float f[3] = {(x - a.fpar[0]) / a.fpar[3] - 0.5f, (y - a.fpar[1]) / a.fpar[4] - 0.5f,
                (z - a.fpar[2]) / a.fpar[5] - 0.5f};
  int i0[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float n = (float)a.fdims[d];
    if (per) f[d] -= n * floorf(f[d] / n);
    const float fl = floorf(f[d]);
    i0[d] = (int)fl;
    f[d] -= fl;
  }
  float acc = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float w = 1.f;
    int ii[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int bit = (c >> d) & 1;
      int j = i0[d] + bit;
      w *= bit ? f[d] : 1.f - f[d];
      const int n = a.fdims[d];
      j = per ? ((j % n) + n) % n : min(max(j, 0), n - 1);
      ii[d] = j;
    }
    acc += w * __ldg(a.ftab + ((size_t)ii[0] * a.fdims[1] + ii[1]) * a.fdims[2] + ii[2]);
  }
  return acc;
}

// Batched launch: a table of instances (one KArgs each, in global memory) walked by persistent
// blocks that pull work items from a global counter.  A work item is up to `tiles_per_item`
// consecutive walker tiles of one instance; item i belongs to the last instance whose
// item_start <= i.  Each item owns one partial slice [n_echo][M][3] of its instance, so the
// per-instance reduction runs in a fixed order whatever the schedule.
struct BatchCtl {
  const KArgs* inst;          // n_inst entries
  const int64_t* item_start;  // n_inst + 1 prefix sums of work items per instance
  int n_inst;
  int max_m;                  // largest M of the batch (shared-memory layout)
  int tiles_per_item;
  int pad0;
  int64_t total;              // total work items
  unsigned long long* counter;
};

// ---- shared-memory async-copy helpers (bulk copy + mbarrier), bounded waits -------------------
__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(saddr(dst)),
      "l"(src), "r"(bytes), "r"(saddr(b))
      : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Gives up after a bounded number of polls (well under a second) instead of spinning forever.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
  for (uint32_t i = 0; i < (1u << 22); ++i)
    if (mbar_try(b, parity)) return true;
  return false;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Floats per sample of the staged waveform: 3 per measurement (direct, Bloch) or 1 per shape
// (basis).
__host__ __device__ constexpr int walk_row(int pm, int w) { return pm == 1 ? w : 3 * w; }

__host__ __device__ inline size_t pad16z(size_t v) { return (v + 15) & ~(size_t)15; }

// Shared-memory layout: [waveform chunk ring (2 x kTC x row)] [3 mbarriers + abort flag, 64 B]
// [basis coefficients C (M x 3 x RT)] [warp reduction scratch (warps x M_red x 3)] [cell list
// (packed substrates) or one MeshScratch per warp (meshes)].
struct SmemLayout {
  size_t off_bar, off_cs, off_red, off_tab;
};
__host__ __device__ inline SmemLayout walk_smem_layout(int pm, int w, int M) {
  SmemLayout L;
  L.off_bar = (size_t)2 * kTC * walk_row(pm, w) * 4;
  L.off_cs = L.off_bar + 64;
  L.off_red = L.off_cs + (pm == 1 ? pad16z((size_t)M * 3 * w * 4) : 0);
  L.off_tab = L.off_red + pad16z((size_t)kWarps * (pm == 1 ? M : w) * 3 * 4);
  return L;
}

// Resident blocks per SM the batched variants are compiled for (the register cap follows).
#ifndef DMSIM_BATCH_MIN_BLOCKS
#define DMSIM_BATCH_MIN_BLOCKS 2
#endif
#ifndef DMSIM_SINGLE_MIN_BLOCKS
#define DMSIM_SINGLE_MIN_BLOCKS 0
#endif
__host__ __device__ constexpr int batch_min_blocks(int pm, int w) {
  return (pm == 0 ? w <= 16 : w <= 4) ? DMSIM_BATCH_MIN_BLOCKS : 1;
}

template <int GEOM>
__device__ __forceinline__ int classify(float x, float y, float z, const GeoK& g,
                                        const uint32_t* cs, const float4* cand,
                                        const int32_t* cobj) {
  if constexpr (GEOM == DMSIM_GEOM_CYLINDER) {
    return (x * x + y * y < g.R2) ? 0 : 1;  // geometries.py:803-813
  } else if constexpr (GEOM == DMSIM_GEOM_SPHERE) {
    return (x * x + y * y + z * z < g.R2) ? 0 : 1;  // geometries.py:161-165
  } else if constexpr (GEOM == DMSIM_GEOM_ELLIPSOID) {  // geometries.py:1396-1403
    return (x * g.e2[0] * x + y * g.e2[1] * y + z * g.e2[2] * z) < 1.f ? 0 : 1;
  } else if constexpr (GEOM == DMSIM_GEOM_SLAB) {
    return x < g.R ? 0 : 1;  // geometries.py:3262-3263
  } else if constexpr (GEOM == DMSIM_GEOM_SHELL) {
    return sqrtf(x * x + y * y + (g.cyl ? 0.f : z * z)) < g.R ? 0 : 1;  // geometries.py:3362-3364
  } else if constexpr (GEOM == DMSIM_GEOM_PACKED_CYLINDERS || GEOM == DMSIM_GEOM_PACKED_SPHERES) {
    // 0 = extra, k+1 = inside object k; the largest id wins (geometries.py:2185-2214)
    constexpr bool P3 = GEOM == DMSIM_GEOM_PACKED_SPHERES;
    int c = cell_of(y, g) * g.n + cell_of(x, g);
    if (P3) c = cell_of(z, g) * g.n * g.n + c;
    int id = 0;
    for (uint32_t k = cs[c]; k < cs[c + 1]; ++k) {
      const float4 C = cand[k];
      const float qx = x - C.x, qy = y - C.y, qz = P3 ? z - C.z : 0.f;
      if (!(min_image(qx, g) && min_image(qy, g) && (!P3 || min_image(qz, g)))) continue;
      if (qx * qx + qy * qy + qz * qz < C.w * C.w) id = max(id, cobj[k] + 1);
    }
    return id;
  } else {
    return 0;
  }
}

__device__ __forceinline__ int classify_mesh(float x, float y, float z, const MeshK& m) {
  int pop;
  return mesh_classify(m, x, y, z, pop);
}

template <int GEOM, int WALL, int PM, int W, bool TSM, bool BATCH>
__global__ void __launch_bounds__(kBlock, BATCH ? batch_min_blocks(PM, W) : DMSIM_SINGLE_MIN_BLOCKS) k_walk(const __grid_constant__ KArgs a0,
                                                 const __grid_constant__ BatchCtl bc) {
  extern __shared__ __align__(128) uint8_t smem[];
  constexpr int ROW = walk_row(PM, W);
  constexpr int GCH = kTC * ROW;  // floats per waveform chunk
  constexpr int MT = PM == 1 ? 1 : W;  // measurements held per thread (direct, Bloch)
  constexpr bool BLOCH = PM == 2;
  float* Gs = reinterpret_cast<float*>(smem);
  const SmemLayout lay = walk_smem_layout(PM, W, BATCH ? bc.max_m : a0.M);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.off_bar);
  volatile int* s_abort = reinterpret_cast<volatile int*>(smem + lay.off_bar + 32);
  float* Cs = reinterpret_cast<float*>(smem + lay.off_cs);
  float* red = reinterpret_cast<float*>(smem + lay.off_red);
  uint8_t* tab = smem + lay.off_tab;
  volatile long long* s_item = reinterpret_cast<volatile long long*>(smem + lay.off_bar + 40);

  constexpr bool PACKED = GEOM == DMSIM_GEOM_PACKED_CYLINDERS || GEOM == DMSIM_GEOM_PACKED_SPHERES;
  constexpr bool P3 = GEOM == DMSIM_GEOM_PACKED_SPHERES;
  constexpr bool MESH = GEOM == DMSIM_GEOM_MESH;
  constexpr bool MYEL = GEOM == DMSIM_GEOM_MYELIN;
  constexpr bool PMYEL = GEOM == DMSIM_GEOM_PMYELIN;
  // compartment ids reported by a packed myelin walk: 0 intra, 1 myelin, 2 extra (core.py:548-550)
  auto to3 = [&](int c, int nmax) { return c == 0 ? 2 : (c > nmax ? 1 : 0); };
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // single-instance launches walk a static share of tiles; batched ones pull work items
  const int64_t n_tiles0 = (a0.n_walkers + kBlock - 1) / kBlock;
  const int my_tiles = BATCH ? 0 : (int)((n_tiles0 - blockIdx.x + gridDim.x - 1) / gridDim.x);
  const int64_t total_chunks = (int64_t)my_tiles * a0.n_chunks;
  const uint32_t chunk_bytes = (uint32_t)GCH * 4u;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    *s_abort = 0;
    fence_async_smem();
  }
  if constexpr (!BATCH) {
    // zero this block's partial slice for this pass
    for (int e = 0; e < a0.n_echo; ++e)
      for (int j = tid; j < (PM == 1 ? a0.M : W) * 3; j += kBlock)
        a0.part[((size_t)(blockIdx.x * a0.n_echo + e) * a0.Mp + a0.pass * MT) * 3 + j] = 0.0;
  }
  __syncthreads();
  if (!BATCH && tid == 0 && total_chunks > 0) {
    mbar_expect(&bar[0], chunk_bytes);
    bulk_g2s(Gs, a0.Gp, chunk_bytes, &bar[0]);
  }

  Tally tl, tl_idle;  // tallies of real walkers / of the idle threads of the last tile
  uint32_t n_nonfinite = 0, n_initfail = 0, n_budget = 0, n_escape = 0, n_idle = 0;
  int64_t q = 0;      // running chunk counter of this block (parity of the chunk barriers)
  uint32_t tabq = 0;  // staged cell lists so far (parity of the table barrier)
  int cur_inst = -1;

  int64_t tile = -1, tile_end = 0, item_local = 0;  // batched: current item's tile range
  for (int it = 0;; ++it) {
    // ---- next tile: the next of this work item, or the first of a new one ---------------------
    int inst = 0;
    bool fresh = false;
    if constexpr (BATCH) {
      inst = cur_inst < 0 ? 0 : cur_inst;
      if (++tile >= tile_end) {
        __syncthreads();
        if (tid == 0) *s_item = (long long)atomicAdd(bc.counter, 1ull);
        __syncthreads();
        const int64_t item = *s_item;
        if (item >= bc.total) break;
        int lo = 0, hi = bc.n_inst;  // last instance whose first item <= item
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (bc.item_start[mid] <= item) lo = mid; else hi = mid;
        }
        inst = lo;
        item_local = item - bc.item_start[inst];
        const int64_t nt = (bc.inst[inst].n_walkers + kBlock - 1) / kBlock;
        tile = item_local * bc.tiles_per_item;
        tile_end = min(tile + (int64_t)bc.tiles_per_item, nt);
        fresh = true;
      }
    } else {
      if (it >= my_tiles) break;
      tile = blockIdx.x + (int64_t)it * gridDim.x;
    }
    const KArgs* __restrict__ ap = BATCH ? bc.inst + inst : &a0;
    const KArgs& a = *ap;
    const GeoK g = a.g;
    // per-axis period used to unfold positions (packed: the cell side; mesh: the periodic box)
    const float Lx = MESH ? a.mk.box[0] : g.L, Ly = MESH ? a.mk.box[1] : g.L,
                Lz = MESH ? a.mk.box[2] : g.L;
    const int MR = PM == 1 ? a.M : W;  // measurements reduced per emission
    const uint32_t* cs = a.cs;
    const float4* cand = a.cand;
    if constexpr (PACKED && TSM) {
      cs = reinterpret_cast<const uint32_t*>(tab);
      cand = reinterpret_cast<const float4*>(tab + a.tab_cs_bytes);
    }
    if (inst != cur_inst) {
      // stage this instance's basis coefficients and cell list
      if constexpr (PM == 1)
        for (int j = tid; j < a.M * 3 * W; j += kBlock) Cs[j] = a.Cp[j];
      if constexpr (PACKED && TSM) {
        if (tid == 0) {
          fence_async_smem();
          mbar_expect(&bar[2], a.tab_cs_bytes + a.tab_cand_bytes);
          bulk_g2s(tab, a.cs, a.tab_cs_bytes, &bar[2]);
          if (a.tab_cand_bytes)
            bulk_g2s(tab + a.tab_cs_bytes, a.cand, a.tab_cand_bytes, &bar[2]);
        }
        if (!mbar_wait(&bar[2], tabq & 1u)) *s_abort = 1;
        ++tabq;
      }
      __syncthreads();
      if (*s_abort) {
        if (tid == 0) {
          atomicAdd(&a.status[DMSIM_STATUS_WAIT_TIMEOUT], 1u);
          if (!BATCH && total_chunks > 0) mbar_wait(&bar[0], 0);
        }
        return;
      }
      cur_inst = inst;
    }
    if constexpr (BATCH) {
      if (fresh) {
        // a work item zeroes its partial slice and starts its own waveform pipeline
        double* pp = a.part + (size_t)item_local * a.n_echo * a.M * 3;
        for (int j = tid; j < a.n_echo * a.M * 3; j += kBlock) pp[j] = 0.0;
        if (tid == 0) {
          fence_async_smem();
          mbar_expect(&bar[q & 1], chunk_bytes);
          bulk_g2s(Gs + (q & 1) * GCH, a.Gp, chunk_bytes, &bar[q & 1]);
        }
      }
    }
    const int64_t w = tile * kBlock + tid;
    const bool act = w < a.n_walkers;
    const uint64_t gw = (uint64_t)(a.walker_offset + w);
    Tally& tw = act ? tl : tl_idle;

    // ---- initial position -----------------------------------------------------------------
    float x = 0.f, y = 0.f, z = 0.f;
    int ix = 0, iy = 0, iz = 0;
    int mcls = 1, mpop = 0;  // mesh: class and gather population of the current position
    int mcomp = 0;           // myelinated cylinder: the walker's compartment
    if (a.r0 != nullptr) {
      if (act) {
        x = a.r0[3 * w];
        y = a.r0[3 * w + 1];
        z = a.r0[3 * w + 2];
      }
      if constexpr (PACKED) {
        ix = (int)floorf(x / g.L + 0.5f);
        x -= g.L * ix;
        iy = (int)floorf(y / g.L + 0.5f);
        y -= g.L * iy;
        if (P3) {
          iz = (int)floorf(z / g.L + 0.5f);
          z -= g.L * iz;
        }
      }
      if constexpr (MYEL) {  // compartment of a given start position (geometries.py:1018-1029)
        const float q = x * x + y * y;
        mcomp = q < a.my.r_in * a.my.r_in ? 0 : (q < a.my.r_out * a.my.r_out ? 1 : 2);
      }
      if constexpr (PMYEL) {  // intra of the first axon holding it, else myelin, else extra
        const PMyelinK& m = a.pm;
        int ci = -1, cm = -1;
        for (int j = m.n - 1; j >= 0; --j) {
          const float4 Cj = m.cyl[4 * j];
          const float fx = pm_mi(x - Cj.x, m.L), fy = pm_mi(y - Cj.y, m.L);
          const float d2 = fx * fx + fy * fy;
          if (d2 < Cj.z * Cj.z) ci = j;
          if (d2 < Cj.w * Cj.w) cm = j;
        }
        mcomp = ci >= 0 ? ci + 1 : (cm >= 0 ? m.nmax + cm + 1 : 0);
      }
      if constexpr (MESH) {
        const MeshK& m = a.mk;
        if (m.per[0]) { ix = (int)floorf((x - m.vmin[0]) / m.box[0]); x -= m.box[0] * ix; }
        if (m.per[1]) { iy = (int)floorf((y - m.vmin[1]) / m.box[1]); y -= m.box[1] * iy; }
        if (m.per[2]) { iz = (int)floorf((z - m.vmin[2]) / m.box[2]); z -= m.box[2] * iz; }
      }
    } else if constexpr (GEOM != DMSIM_GEOM_FREE) {
      // Uniform seeding by rejection, as the reference's host samplers (geometries.py:186-195,
      // 477-491, 1717-1744, 2421-2443), on the seeding stream.  A myelinated cylinder takes its
      // compartment from the walker's index range (volume-proportional counts, intra first,
      // geometries.py:928-1006) and a uniform point of that disc or annulus (extra: out to
      // 2 R_out).
      if constexpr (MYEL) {
        const long long gi = (long long)gw;
        mcomp = gi < a.my.n0 ? 0 : (gi < a.my.n1 ? 1 : 2);
      }
      // packed myelin: the seeding segment of this walker (intra of axon 0..n-1, then myelin of
      // axon 0..n-1, then extra-axonal; geometries.py:3127-3208), its axon and compartment
      int pm_seg = 0;
      if constexpr (PMYEL) {
        const long long gi = (long long)gw;
        int lo = 0, hi = 2 * a.pm.n;  // first segment whose end exceeds gi
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (a.pm.seed[mid] > gi) hi = mid; else lo = mid + 1;
        }
        pm_seg = lo;
        mcomp = pm_seg < a.pm.n ? pm_seg + 1
                                : (pm_seg < 2 * a.pm.n ? a.pm.nmax + (pm_seg - a.pm.n) + 1 : 0);
      }
      const float s_lo = MYEL ? (mcomp == 0 ? 0.f : (mcomp == 1 ? a.my.r_in : a.my.r_out)) : 0.f;
      const float s_hi = MYEL ? (mcomp == 0 ? a.my.r_in : (mcomp == 1 ? a.my.r_out
                                                                       : 2.f * a.my.r_out))
                              : 0.f;
      bool ok = false;
#pragma unroll 1
      for (uint32_t j = 0; j < 256u && !ok; ++j) {
        const u32x4 r = draw(a.seed, gw, 1u, j);
        const float u0 = u01(r.x), u1 = u01(r.y), u2 = u01(r.z), u3 = u01(r.w);
        if constexpr (GEOM == DMSIM_GEOM_ELLIPSOID) {
          // uniform in the unit ball, scaled by the semi-axes (geometries.py:1167-1182)
          const float px = 2.f * u0 - 1.f, py = 2.f * u1 - 1.f, pz = 2.f * u2 - 1.f;
          if (px * px + py * py + pz * pz < 1.f) {
            x = px * rsqrtf(g.e2[0]);
            y = py * rsqrtf(g.e2[1]);
            z = pz * rsqrtf(g.e2[2]);
            ok = true;
          }
        } else if constexpr (GEOM == DMSIM_GEOM_BOX1D || GEOM == DMSIM_GEOM_SLAB) {
          // x uniform over the slab (Box1D) or its first half (the permeable slab starts every
          // walker in compartment A), y = z = 0 (geometries.py:84-88, 3257-3261)
          x = (GEOM == DMSIM_GEOM_BOX1D ? g.L : g.R) * u0;
          ok = true;
        } else if constexpr (GEOM == DMSIM_GEOM_SHELL) {
          // uniform in compartment A (r < R_in); a cylindrical shell also spreads z over
          // [0, R_in) (geometries.py:3343-3358)
          const float px = g.R * (2.f * u0 - 1.f), py = g.R * (2.f * u1 - 1.f);
          const float pz = g.R * (2.f * u2 - 1.f);
          const float q = px * px + py * py + (g.cyl ? 0.f : pz * pz);
          if (q < g.R2) {
            x = px;
            y = py;
            z = g.cyl ? g.R * u3 : pz;
            ok = true;
          }
        } else if constexpr (PMYEL) {
          const PMyelinK& m = a.pm;
          for (int h = 0; h < 2 && !ok; ++h) {
            const float v0 = h ? u2 : u0, v1 = h ? u3 : u1;
            if (pm_seg < 2 * m.n) {  // inner disc or sheath of one axon, around its centre
              const float4 Cj = m.cyl[4 * (pm_seg % m.n)];
              const float lo = pm_seg < m.n ? 0.f : Cj.z, hi = pm_seg < m.n ? Cj.z : Cj.w;
              const float px = hi * (2.f * v0 - 1.f), py = hi * (2.f * v1 - 1.f);
              const float q = px * px + py * py;
              if (q >= lo * lo && q < hi * hi) { x = Cj.x + px; y = Cj.y + py; ok = true; }
            } else {  // extra-axonal: uniform in the cell outside every sheath
              const float px = m.L * (v0 - 0.5f), py = m.L * (v1 - 0.5f);
              bool out = true;
              for (int j = 0; j < m.n && out; ++j) {
                const float4 Cj = m.cyl[4 * j];
                const float fx = px - Cj.x - m.L * rintf((px - Cj.x) / m.L);
                const float fy = py - Cj.y - m.L * rintf((py - Cj.y) / m.L);
                if (!(fx * fx + fy * fy > Cj.w * Cj.w)) out = false;
              }
              if (out) { x = px; y = py; ok = true; }
            }
          }
        } else if constexpr (MYEL) {
          for (int h = 0; h < 2 && !ok; ++h) {
            const float px = s_hi * (2.f * (h ? u2 : u0) - 1.f);
            const float py = s_hi * (2.f * (h ? u3 : u1) - 1.f);
            const float q = px * px + py * py;
            if (q >= s_lo * s_lo && q < s_hi * s_hi) { x = px; y = py; ok = true; }
          }
        } else if constexpr (GEOM == DMSIM_GEOM_CYLINDER) {
          float px = g.R * (2.f * u0 - 1.f), py = g.R * (2.f * u1 - 1.f);
          if (px * px + py * py < g.R2) {
            x = px; y = py; ok = true;
          } else {
            px = g.R * (2.f * u2 - 1.f);
            py = g.R * (2.f * u3 - 1.f);
            if (px * px + py * py < g.R2) { x = px; y = py; ok = true; }
          }
        } else if constexpr (GEOM == DMSIM_GEOM_SPHERE) {
          const float px = g.R * (2.f * u0 - 1.f), py = g.R * (2.f * u1 - 1.f),
                      pz = g.R * (2.f * u2 - 1.f);
          if (px * px + py * py + pz * pz < g.R2) { x = px; y = py; z = pz; ok = true; }
        } else if constexpr (GEOM == DMSIM_GEOM_PACKED_CYLINDERS) {
          for (int h = 0; h < 2 && !ok; ++h) {
            const float px = g.L * ((h ? u2 : u0) - 0.5f), py = g.L * ((h ? u3 : u1) - 0.5f);
            const int c = cell_of(py, g) * g.n + cell_of(px, g);
            bool out = true;
            for (uint32_t k = cs[c]; k < cs[c + 1]; ++k) {
              const float4 C = cand[k];
              const float qx = px - C.x, qy = py - C.y;
              if (qx * qx + qy * qy <= C.w * C.w) out = false;
            }
            if (out) { x = px; y = py; ok = true; }
          }
        } else if constexpr (MESH) {
          // uniform in the box; keep points on the requested side of the closed surface (ray
          // parity), or by the nearest-centroid classifier for an open surface
          // (mesh.py:746-807)
          const MeshK& m = a.mk;
          const float px = m.vmin[0] + m.box[0] * u0, py = m.vmin[1] + m.box[1] * u1,
                      pz = m.vmin[2] + m.box[2] * u2;
          int side;
          if (m.seed_parity) {
            side = mesh_parity(m, px, py, pz);
          } else {
            int pop;
            side = mesh_classify(m, px, py, pz, pop) == 0 ? 1 : 0;
          }
          if (side == m.seed_inside) { x = px; y = py; z = pz; ok = true; }
        } else if constexpr (GEOM == DMSIM_GEOM_PACKED_SPHERES) {
          const float px = g.L * (u0 - 0.5f), py = g.L * (u1 - 0.5f), pz = g.L * (u2 - 0.5f);
          const int c = (cell_of(pz, g) * g.n + cell_of(py, g)) * g.n + cell_of(px, g);
          bool out = true;
          for (uint32_t k = cs[c]; k < cs[c + 1]; ++k) {
            const float4 C = cand[k];
            const float qx = px - C.x, qy = py - C.y, qz = pz - C.z;
            if (qx * qx + qy * qy + qz * qz <= C.w * C.w) out = false;
          }
          if (out) { x = px; y = py; z = pz; ok = true; }
        }
      }
      if (!ok && act) ++n_initfail;
    }
    if constexpr (MESH) {
      if (a.mk.reject && WALL != kPermeate) mcls = mesh_classify(a.mk, x, y, z, mpop);
    }
    if (act && a.comp0 != nullptr && a.pass == 0)
      a.comp0[w] = PMYEL ? to3(mcomp, a.pm.nmax) : MYEL ? mcomp
                        : (MESH ? classify_mesh(x, y, z, a.mk)
                                : classify<GEOM>(x, y, z, g, cs, cand, a.cand_obj));

    // phase accumulators: direct form phi[m] (+ Kahan), basis form Q[j][k] (+ Kahan)
    constexpr int NACC = PM == 1 ? 3 * W : W;
    float acc[NACC], kc[NACC];
#pragma unroll
    for (int i = 0; i < NACC; ++i) acc[i] = kc[i] = 0.f;
    // Bloch form: M as of the last RF event, the carrier phase (Kahan) and the T1 samples since,
    // the log-weight at that event and the walker's crusher coordinate (its own Philox stream)
    constexpr int NB = BLOCH ? W : 1;
    float bx[NB], by[NB], bz[NB];
    float psi = 0.f, psik = 0.f, lw_rf = 0.f, uc = 0.f;
    int k1 = 0;
    if constexpr (BLOCH) {
#pragma unroll
      for (int m = 0; m < W; ++m) {
        bx[m] = by[m] = 0.f;
        bz[m] = a.m0;
      }
      if (a.crush) uc = u01(draw(a.seed, gw, 2u, 0u).x);
    }
    // a myelinated cylinder's walkers start with the log of their compartment's spin weight
    const float logw0 =
        MYEL ? (mcomp == 0 ? a.my.lw0[0] : (mcomp == 1 ? a.my.lw0[1] : a.my.lw0[2]))
             : (PMYEL ? (mcomp > a.pm.nmax ? a.pm.lwm : 0.f) : 0.f);
    float logw = logw0;
    lw_rf = logw0;
    uint32_t s = 0;   // global sub-step counter of this walker
    u32x4 rr{0, 0, 0, 0};
    int e = 0;        // next echo ordinal
    int t = 0;

    for (int ch = 0; ch < a.n_chunks; ++ch, ++q) {
      // ---- waveform chunk pipeline: prefetch q+1, wait for q ----------------------------------
      __syncthreads();
      // prefetch the next chunk: of this tile, or (single instance) the next tile's first
      const bool has_next =
          (ch + 1 < a.n_chunks) || (BATCH ? tile + 1 < tile_end : q + 1 < total_chunks);
      if (tid == 0 && has_next) {
        const int64_t qn = q + 1;
        const int src_chunk = ch + 1 < a.n_chunks ? ch + 1 : 0;
        fence_async_smem();
        mbar_expect(&bar[qn & 1], chunk_bytes);
        bulk_g2s(Gs + (qn & 1) * GCH, a.Gp + (size_t)src_chunk * GCH, chunk_bytes, &bar[qn & 1]);
      }
      if (!mbar_wait(&bar[q & 1], (uint32_t)((q >> 1) & 1))) *s_abort = 1;
      __syncthreads();
      if (*s_abort) {
        if (tid == 0) {
          atomicAdd(&a.status[DMSIM_STATUS_WAIT_TIMEOUT], 1u);
          if (has_next) mbar_wait(&bar[(q + 1) & 1], (uint32_t)(((q + 1) >> 1) & 1));
        }
        return;
      }
      const float* Gc = Gs + (q & 1) * GCH;

      const int t_end = min(a.n_t, (ch + 1) * kTC);
#pragma unroll 1
      for (; t < t_end; ++t) {
        const float chi = a.chi ? __ldg(a.chi + t) : 1.f;
        const float rc = a.rho * chi;
        const float dec = a.t2dec * chi + a.t1dec * (1.f - chi);
        const float logw_t0 = logw;  // Bloch: the weight through sample t - 1
        float Rx = 0.f, Ry = 0.f, Rz = 0.f, dls = 0.f, occ = 0.f;
#pragma unroll 1
        for (int sub = 0; sub < a.S; ++sub, ++s) {
          float ua, ub, up = 0.f, up2 = 0.f;
          if constexpr (WALL == kPermeate) {
            rr = draw(a.seed, gw, 0u, s);
            ua = u01(rr.x);
            ub = u01(rr.y);
            up = u01(rr.z);
            if constexpr (MYEL || PMYEL) up2 = u01(rr.w);  // the outer wall's own uniform
          } else {
            if ((s & 1u) == 0u) {
              rr = draw(a.seed, gw, 0u, s >> 1);
              ua = u01(rr.x);
              ub = u01(rr.y);
            } else {
              ua = u01(rr.z);
              ub = u01(rr.w);
            }
          }
          // isotropic direction from two uniforms: cos(theta) = 1 - 2 ua, azimuth = pi (2 ub - 1)
          const float cz = 1.f - 2.f * ua;
          const float sz = sqrtf(fmaxf(0.f, 1.f - cz * cz));
          float sn, cs_;
          __sincosf(3.14159265358979f * (2.f * ub - 1.f), &sn, &cs_);
          const float stx = a.step_l * sz * cs_, sty = a.step_l * sz * sn, stz = a.step_l * cz;

          float dl = 0.f;
          if constexpr (GEOM == DMSIM_GEOM_FREE) {
            x += stx;
            y += sty;
            z += stz;
          } else if constexpr (GEOM == DMSIM_GEOM_CYLINDER) {
            dl = cylinder_step<WALL>(x, y, stx, sty, up, g, tw);
            z += stz;
          } else if constexpr (GEOM == DMSIM_GEOM_SPHERE) {
            dl = sphere_step<WALL>(x, y, z, stx, sty, stz, up, g, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_PACKED_CYLINDERS) {
            dl = packed_cyl_step<WALL>(x, y, ix, iy, stx, sty, up, g, cs, cand, tw);
            z += stz;
          } else if constexpr (GEOM == DMSIM_GEOM_PACKED_SPHERES) {
            dl = packed_sph_step<WALL>(x, y, z, ix, iy, iz, stx, sty, stz, up, g, cs, cand, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_ELLIPSOID) {
            dl = ellipsoid_step<WALL>(x, y, z, stx, sty, stz, up, g, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_BOX1D) {
            dl = box1d_step<WALL == kPermeate ? kReflect : WALL>(x, y, z, stx, sty, stz, g);
          } else if constexpr (GEOM == DMSIM_GEOM_SLAB) {
            dl = slab_step<WALL>(x, y, z, stx, sty, stz, up, g, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_SHELL) {
            dl = shell_step<WALL>(x, y, z, stx, sty, stz, up, g, tw);
          } else if constexpr (MYEL) {
            dl = myelin_step<WALL>(x, y, z, mcomp, stx, sty, stz, up, up2, a.my, tw);
          } else if constexpr (PMYEL) {
            // the phase reads the unwrapped position: the image counters take up the minimum-
            // image displacement of the in-cell step (physics.py:1038-1042)
            const float xo = x, yo = y;
            dl = pmyelin_step<WALL>(x, y, z, mcomp, stx, sty, stz, up, up2, a.pm, tw);
            ix -= (int)rintf((x - xo) / a.pm.L);
            iy -= (int)rintf((y - yo) / a.pm.L);
          } else if constexpr (MESH) {
            dl = mesh_step<WALL>(x, y, z, ix, iy, iz, mcls, mpop, stx, sty, stz, up, a.mk, tw,
                                 act ? n_budget : n_idle, act ? n_escape : n_idle,
                                 reinterpret_cast<MeshScratch*>(tab) + warp);
          }
          if (a.has_weight) logw += rc * dl - dec;
          if (a.phase_sub) {
            Rx += x + Lx * (float)ix;
            Ry += y + Ly * (float)iy;
            Rz += z + Lz * (float)iz;
          }
          if (a.dlog_unit) dls += dl;
          if (a.comp_occ)
            occ += (float)(PMYEL ? to3(mcomp, a.pm.nmax) : MYEL ? mcomp
                                : (MESH ? classify_mesh(x, y, z, a.mk)
                                        : classify<GEOM>(x, y, z, g, cs, cand, a.cand_obj)));
        }
        const float ux = x + Lx * (float)ix, uy = y + Ly * (float)iy, uz = z + Lz * (float)iz;
        if (!a.phase_sub) {
          Rx = ux;
          Ry = uy;
          Rz = uz;
        }
        // ---- Bloch: an RF pulse at this sample rotates M, formed through sample t - 1, about the
        // in-plane axis (cos ax, sin ax, 0) before this sample's precession (bloch.py:44-57,
        // 125).  The flip is the same for every walker: a block-uniform branch.
        if constexpr (BLOCH) {
          const float flip = __ldg(a.rf_flip + t);
          if (flip != 0.f) {
            float ux, uy, sf, cf;
            sincosf(__ldg(a.rf_axis + t), &uy, &ux);
            sincosf(flip, &sf, &cf);
            const float omc = 1.f - cf;
            const float amp = a.has_weight ? expf(logw_t0 - lw_rf) : 1.f;
            const float e1 = expf(-(float)k1 * a.t1_sample);
#pragma unroll
            for (int m = 0; m < W; ++m) {
              float sn, cs_;
              sincosf(acc[m] + psi, &sn, &cs_);
              const float mx = amp * (cs_ * bx[m] - sn * by[m]);
              const float my = amp * (sn * bx[m] + cs_ * by[m]);
              const float mz = a.m0 + (bz[m] - a.m0) * e1;
              bx[m] = (cf + ux * ux * omc) * mx + (ux * uy * omc) * my + (uy * sf) * mz;
              by[m] = (ux * uy * omc) * mx + (cf + uy * uy * omc) * my - (ux * sf) * mz;
              bz[m] = -(uy * sf) * mx + (ux * sf) * my + cf * mz;
              acc[m] = kc[m] = 0.f;
            }
            psi = psik = 0.f;
            lw_rf = logw_t0;
            k1 = 0;
          }
        }
        // ---- phase, Kahan-compensated ------------------------------------------------------
        if (__ldg(a.active + t)) {
          const float px = a.gamma_dt * Rx, py = a.gamma_dt * Ry, pz = a.gamma_dt * Rz;
          const float* gt = Gc + (t - ch * kTC) * ROW;
          if constexpr (PM != 1) {
            // direct: phi_m += g_m(t) . R
            const float4* g4 = reinterpret_cast<const float4*>(gt);
            float d = 0.f;
#pragma unroll
            for (int j = 0; j < W * 3 / 4; ++j) {
              const float4 v = g4[j];
              const float gv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
              for (int h = 0; h < 4; ++h) {
                const int el = 4 * j + h, m = el / 3, k = el % 3;
                const float pk = k == 0 ? px : (k == 1 ? py : pz);
                d = (k == 0) ? gv[h] * pk : fmaf(gv[h], pk, d);
                if (k == 2) {
                  const float yk = d - kc[m];
                  const float tk = acc[m] + yk;
                  kc[m] = (tk - acc[m]) - yk;
                  acc[m] = tk;
                }
              }
            }
          } else {
            // basis: Q[j][k] += V_j(t) * R_k
#pragma unroll
            for (int j = 0; j < W; ++j) {
              const float v = gt[j];
              const float pv[3] = {v * px, v * py, v * pz};
#pragma unroll
              for (int k = 0; k < 3; ++k) {
                const int i = 3 * j + k;
                const float yk = pv[k] - kc[i];
                const float tk = acc[i] + yk;
                kc[i] = (tk - acc[i]) - yk;
                acc[i] = tk;
              }
            }
          }
        }
        if constexpr (BLOCH) {
          // carriers of this sample: off-resonance + pulse carrier + crusher (bloch.py:126)
          float dpsi = (a.carrier ? __ldg(a.carrier + t) : 0.f) +
                       (a.crush ? __ldg(a.crush + t) * uc : 0.f);
          if (a.fkind) dpsi += a.fgdt * field_dbz(a, ux, uy, uz);
          const float yk = dpsi - psik;
          const float tk = psi + yk;
          psik = (tk - psi) - yk;
          psi = tk;
          ++k1;
        }
        if (act) {
          if (a.traj != nullptr && a.pass == 0) {
            const size_t o = ((size_t)w * a.n_t + t) * 3;
            if (a.traj_f16) {
              __half* tp = reinterpret_cast<__half*>(a.traj);
              tp[o] = __float2half_rn(ux);
              tp[o + 1] = __float2half_rn(uy);
              tp[o + 2] = __float2half_rn(uz);
            } else {
              float* tp = reinterpret_cast<float*>(a.traj);
              tp[o] = ux;
              tp[o + 1] = uy;
              tp[o + 2] = uz;
            }
          }
          if (a.dlog_unit != nullptr && a.pass == 0) a.dlog_unit[(size_t)w * a.n_t + t] = dls;
          if (a.comp_occ != nullptr && a.pass == 0)
            a.comp_occ[(size_t)w * a.n_t + t] = occ / (float)a.S;
        }
        // ---- ensemble sums at an echo sample (block-uniform branch) --------------------------
        if (e < a.n_echo && t == a.echo[e]) {
          const float wgt = act ? (a.has_weight ? expf(logw) : 1.f) : 0.f;
          auto emit = [&](int m, float ph) {
            float sn, cs_;
            sincosf(ph, &sn, &cs_);
            const float c1 = warp_sum(wgt * cs_);
            const float c2 = warp_sum(wgt * sn);
            const float c3 = warp_sum((wgt * cs_) * (wgt * cs_));
            if (lane == 0) {
              red[(warp * MR + m) * 3] = c1;
              red[(warp * MR + m) * 3 + 1] = c2;
              red[(warp * MR + m) * 3 + 2] = c3;
            }
          };
          if constexpr (PM == 0) {
#pragma unroll
            for (int m = 0; m < W; ++m) emit(m, acc[m]);
          } else if constexpr (BLOCH) {
            // walker's (Mx, My, Mz) at this sample (bloch.py:127-131)
            const float amp = act ? (a.has_weight ? expf(logw - lw_rf) : 1.f) : 0.f;
            const float e1 = expf(-(float)k1 * a.t1_sample);
#pragma unroll
            for (int m = 0; m < W; ++m) {
              float sn, cs_;
              sincosf(acc[m] + psi, &sn, &cs_);
              const float c1 = warp_sum(amp * (cs_ * bx[m] - sn * by[m]));
              const float c2 = warp_sum(amp * (sn * bx[m] + cs_ * by[m]));
              const float c3 = warp_sum(act ? a.m0 + (bz[m] - a.m0) * e1 : 0.f);
              if (lane == 0) {
                red[(warp * MR + m) * 3] = c1;
                red[(warp * MR + m) * 3 + 1] = c2;
                red[(warp * MR + m) * 3 + 2] = c3;
              }
            }
          } else {
#pragma unroll 1
            for (int m = 0; m < MR; ++m) {
              const float* c = Cs + (size_t)m * 3 * W;
              float ph = 0.f;
#pragma unroll
              for (int j = 0; j < W; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) ph = fmaf(c[k * W + j], acc[3 * j + k], ph);
              emit(m, ph);
            }
          }
          __syncthreads();
          for (int j = tid; j < MR * 3; j += kBlock) {
            double sacc = 0.0;
#pragma unroll
            for (int ww = 0; ww < kWarps; ++ww) sacc += (double)red[ww * MR * 3 + j];
            if constexpr (BATCH)
              a.part[((size_t)item_local * a.n_echo + e) * a.M * 3 + j] += sacc;
            else
              a.part[((size_t)(blockIdx.x * a.n_echo + e) * a.Mp + a.pass * MT) * 3 + j] += sacc;
          }
          __syncthreads();
          ++e;
        }
      }
    }

    // ---- per-walker outputs --------------------------------------------------------------------
    const float ux = x + Lx * (float)ix, uy = y + Ly * (float)iy, uz = z + Lz * (float)iz;
    if (act) {
      if (!(isfinite(ux) && isfinite(uy) && isfinite(uz))) ++n_nonfinite;
      if (a.pass == 0) {
        if (a.final_pos) {  // a packed myelin walk reports the in-cell position (core.py:560-566)
          a.final_pos[3 * w] = PMYEL ? x : ux;
          a.final_pos[3 * w + 1] = PMYEL ? y : uy;
          a.final_pos[3 * w + 2] = uz;
        }
        if (a.log_w) a.log_w[w] = logw - logw0;  // the walk's own log-weight, without spin weight
        if (a.comp_end)
          a.comp_end[w] = PMYEL ? to3(mcomp, a.pm.nmax) : MYEL ? mcomp
                               : (MESH ? classify_mesh(x, y, z, a.mk)
                                       : classify<GEOM>(x, y, z, g, cs, cand, a.cand_obj));
      }
      if (a.phi_out && !BLOCH) {
        if constexpr (PM == 0) {
#pragma unroll
          for (int m = 0; m < W; ++m)
            if (a.pass * W + m < a.M) a.phi_out[(size_t)w * a.M + a.pass * W + m] = acc[m];
        } else if constexpr (PM == 1) {
          for (int m = 0; m < a.M; ++m) {
            const float* c = Cs + (size_t)m * 3 * W;
            float ph = 0.f;
#pragma unroll
            for (int j = 0; j < W; ++j)
#pragma unroll
              for (int k = 0; k < 3; ++k) ph = fmaf(c[k * W + j], acc[3 * j + k], ph);
            a.phi_out[(size_t)w * a.M + m] = ph;
          }
        }
      }
    }

    if constexpr (BATCH) {
      // flush the tallies into this instance's status words after each work item
      const uint32_t b0 = __reduce_add_sync(0xffffffffu, n_nonfinite);
      const uint32_t b1 = __reduce_add_sync(0xffffffffu, tl.clamp);
      const uint32_t b2 = __reduce_add_sync(0xffffffffu, n_initfail);
      const uint32_t b3 = __reduce_add_sync(0xffffffffu, tl.transmit);
      const uint32_t b4 = __reduce_add_sync(0xffffffffu, n_budget);
      const uint32_t b5 = __reduce_add_sync(0xffffffffu, n_escape);
      const uint32_t b6 = __reduce_add_sync(0xffffffffu, tl.graze);
      if (lane == 0 && a.pass == 0) {
        if (b6) atomicAdd(&a.status[DMSIM_STATUS_GRAZE_FP64], b6);
        if (b0) atomicAdd(&a.status[DMSIM_STATUS_NONFINITE], b0);
        if (b1) atomicAdd(&a.status[DMSIM_STATUS_CLAMPED], b1);
        if (b2) atomicAdd(&a.status[DMSIM_STATUS_INIT_FAIL], b2);
        if (b3) atomicAdd(&a.status[DMSIM_STATUS_TRANSMIT], b3);
        if (b4) atomicAdd(&a.status[DMSIM_STATUS_BOUNCE_BUDGET], b4);
        if (b5) atomicAdd(&a.status[DMSIM_STATUS_ESCAPE_REJECT], b5);
      }
      n_nonfinite = n_initfail = n_budget = n_escape = 0;
      tl.clamp = tl.transmit = tl.graze = 0;
    }
  }
  if constexpr (BATCH) return;

  // ---- anomaly tallies ------------------------------------------------------------------------
  const KArgs& a = a0;
  const uint32_t v0 = __reduce_add_sync(0xffffffffu, n_nonfinite);
  const uint32_t v1 = __reduce_add_sync(0xffffffffu, tl.clamp);
  const uint32_t v2 = __reduce_add_sync(0xffffffffu, n_initfail);
  const uint32_t v3 = __reduce_add_sync(0xffffffffu, tl.graze);
  const uint32_t v4 = __reduce_add_sync(0xffffffffu, tl.transmit);
  const uint32_t v5 = __reduce_add_sync(0xffffffffu, n_budget);
  const uint32_t v6 = __reduce_add_sync(0xffffffffu, n_escape);
  if (lane == 0 && a.pass == 0) {
    if (v0) atomicAdd(&a.status[DMSIM_STATUS_NONFINITE], v0);
    if (v1) atomicAdd(&a.status[DMSIM_STATUS_CLAMPED], v1);
    if (v2) atomicAdd(&a.status[DMSIM_STATUS_INIT_FAIL], v2);
    if (v3) atomicAdd(&a.status[DMSIM_STATUS_GRAZE_FP64], v3);
    if (v4) atomicAdd(&a.status[DMSIM_STATUS_TRANSMIT], v4);
    if (v5) atomicAdd(&a.status[DMSIM_STATUS_BOUNCE_BUDGET], v5);
    if (v6) atomicAdd(&a.status[DMSIM_STATUS_ESCAPE_REJECT], v6);
  }
}

using WalkFn = void (*)(KArgs, BatchCtl);

}  // namespace dmsim
