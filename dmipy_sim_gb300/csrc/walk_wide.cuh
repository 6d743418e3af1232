// The wide-block walk kernel of packed cylinders.
//
// The single-instance walk of dmipy-sim's PackedCylinders (geometries.py:1604-2242) through
// make_step_fn's reflect / surface-relaxivity / permeable branches (physics.py:276-415) and the
// producer walk of simulate_trajectories (core.py:1137-1155), in the basis phase form.  It walks
// what k_walk<DMSIM_GEOM_PACKED_CYLINDERS, ...> walks -- the same Philox stream, the same
// packed_cyl_step, waveform pipeline and reduction order -- with a different occupancy plan.
//
// The packed walk is bound by instruction latency (dependent ALU and MUFU chains, shared-memory
// loads of the candidates), so it runs faster the more warps an SM keeps resident.  k_walk holds
// two 320-thread blocks per SM, each with its own copy of the cell list (up to 96 KB) and the
// walker's phase accumulators in registers.  This kernel runs one block of NT threads (1024 = 32
// warps) per SM around a single copy of the cell list, with the walk's Kahan phase accumulators
// (3 RT sums and their compensations per walker, touched once per waveform sample) in shared
// memory, thread-strided so that they cost no bank conflicts; the registers left hold the step.
// Every run-time choice k_walk makes per sub-step (replay or fused phase, exports, Bloch
// carriers, batched work items) is fixed at compile time or excluded, and the sub-step loop takes
// the two directions of one Philox draw in turn.
#pragma once
#include "walk_kernel.cuh"

namespace dmsim {

constexpr int kWideEmit = 32;  // measurements reduced per emission chunk

// Shared-memory layout: [waveform chunk ring (2 x kTC x RT)] [3 mbarriers + abort flag, 64 B]
// [basis coefficients (M x 3 x RT)] [warp reduction scratch (warps x kWideEmit x 3)]
// [phase sums and compensations (6 RT x NT floats)] [cell list].
struct WideLayout {
  size_t off_bar, off_cs, off_red, off_acc, off_tab, total;
};
__host__ __device__ inline WideLayout wide_layout(int nt, int rt, int M, size_t tab_bytes) {
  WideLayout L;
  L.off_bar = (size_t)2 * kTC * rt * 4;
  L.off_cs = L.off_bar + 64;
  L.off_red = L.off_cs + pad16z((size_t)M * 3 * rt * 4);
  L.off_acc = L.off_red + pad16z((size_t)(nt / 32) * kWideEmit * 3 * 4);
  L.off_tab = L.off_acc + (size_t)6 * rt * nt * 4;
  L.total = L.off_tab + pad16z(tab_bytes);
  return L;
}

template <int WALL, int RT, bool PSUB, int NT>
__global__ void __launch_bounds__(NT, 1) k_pcyl_wide(const __grid_constant__ KArgs a) {
  extern __shared__ __align__(128) uint8_t smem[];
  constexpr int GCH = kTC * RT;
  constexpr int NACC = 3 * RT;
  constexpr int NW = NT / 32;
  float* Gs = reinterpret_cast<float*>(smem);
  const WideLayout lay = wide_layout(NT, RT, a.M, (size_t)a.tab_cs_bytes + a.tab_cand_bytes);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + lay.off_bar);
  volatile int* s_abort = reinterpret_cast<volatile int*>(smem + lay.off_bar + 32);
  float* Cs = reinterpret_cast<float*>(smem + lay.off_cs);
  float* red = reinterpret_cast<float*>(smem + lay.off_red);
  float* accs = reinterpret_cast<float*>(smem + lay.off_acc) + threadIdx.x;  // [i * NT]
  float* kcs = accs + (size_t)NACC * NT;
  const uint32_t* cs = reinterpret_cast<const uint32_t*>(smem + lay.off_tab);
  const float4* cand = reinterpret_cast<const float4*>(smem + lay.off_tab + a.tab_cs_bytes);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const GeoK g = a.g;

  const int64_t n_tiles = (a.n_walkers + NT - 1) / NT;
  const int my_tiles = (int)((n_tiles - blockIdx.x + gridDim.x - 1) / gridDim.x);
  const int64_t total_chunks = (int64_t)my_tiles * a.n_chunks;
  const uint32_t chunk_bytes = (uint32_t)GCH * 4u;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    *s_abort = 0;
    fence_async_smem();
  }
  for (int e = 0; e < a.n_echo; ++e)
    for (int j = tid; j < a.M * 3; j += NT)
      a.part[((size_t)(blockIdx.x * a.n_echo + e) * a.Mp) * 3 + j] = 0.0;
  for (int j = tid; j < a.M * 3 * RT; j += NT) Cs[j] = a.Cp[j];
  __syncthreads();
  if (my_tiles <= 0) return;
  if (tid == 0) {
    fence_async_smem();
    mbar_expect(&bar[2], a.tab_cs_bytes + a.tab_cand_bytes);
    bulk_g2s(smem + lay.off_tab, a.cs, a.tab_cs_bytes, &bar[2]);
    if (a.tab_cand_bytes)
      bulk_g2s(smem + lay.off_tab + a.tab_cs_bytes, a.cand, a.tab_cand_bytes, &bar[2]);
    mbar_expect(&bar[0], chunk_bytes);
    bulk_g2s(Gs, a.Gp, chunk_bytes, &bar[0]);
  }
  if (!mbar_wait(&bar[2], 0u)) *s_abort = 1;
  __syncthreads();
  if (*s_abort) {
    if (tid == 0) {
      atomicAdd(&a.status[DMSIM_STATUS_WAIT_TIMEOUT], 1u);
      mbar_wait(&bar[0], 0u);
    }
    return;
  }

  Tally tl;
  uint32_t n_nonfinite = 0, n_initfail = 0;
  int64_t q = 0;  // running chunk counter of this block (parity of the chunk barriers)
  const bool weighted = a.has_weight != 0;

  for (int it = 0; it < my_tiles; ++it) {
    const int64_t tile = blockIdx.x + (int64_t)it * gridDim.x;
    const int64_t w = tile * NT + tid;
    const bool act = w < a.n_walkers;
    const uint64_t gw = (uint64_t)(a.walker_offset + w);
    Tally tt;  // this tile's tallies (the idle threads of the last tile do not count)

    // ---- initial position (geometries.py:1717-1744: uniform outside every cylinder) ---------
    float x = 0.f, y = 0.f, z = 0.f;
    int ix = 0, iy = 0;
    if (a.r0 != nullptr) {
      if (act) {
        x = a.r0[3 * w];
        y = a.r0[3 * w + 1];
        z = a.r0[3 * w + 2];
      }
      ix = (int)floorf(x / g.L + 0.5f);
      x -= g.L * ix;
      iy = (int)floorf(y / g.L + 0.5f);
      y -= g.L * iy;
    } else {
      bool ok = false;
#pragma unroll 1
      for (uint32_t j = 0; j < 256u && !ok; ++j) {
        const u32x4 r = draw(a.seed, gw, 1u, j);
        const float u0 = u01(r.x), u1 = u01(r.y), u2 = u01(r.z), u3 = u01(r.w);
        for (int h = 0; h < 2 && !ok; ++h) {
          const float px = g.L * ((h ? u2 : u0) - 0.5f), py = g.L * ((h ? u3 : u1) - 0.5f);
          const int c = cell_of(py, g) * g.n + cell_of(px, g);
          bool out = true;
          for (uint32_t k = cs[c]; k < cs[c + 1]; ++k) {
            const float4 C = cand[k];
            const float qx = px - C.x, qy = py - C.y;
            if (qx * qx + qy * qy <= C.w * C.w) out = false;
          }
          if (out) {
            x = px;
            y = py;
            ok = true;
          }
        }
      }
      if (!ok && act) ++n_initfail;
    }
    if (act && a.comp0 != nullptr && a.pass == 0)
      a.comp0[w] = classify<DMSIM_GEOM_PACKED_CYLINDERS>(x, y, z, g, cs, cand, a.cand_obj);

#pragma unroll
    for (int i = 0; i < NACC; ++i) accs[i * NT] = kcs[i * NT] = 0.f;
    float logw = 0.f;
    uint32_t s = 0;  // global sub-step counter of this walker
    u32x4 rr{0, 0, 0, 0};
    int e = 0, t = 0;

    for (int ch = 0; ch < a.n_chunks; ++ch, ++q) {
      __syncthreads();
      const bool has_next = (ch + 1 < a.n_chunks) || (q + 1 < total_chunks);
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
        float rc = 0.f, dec = 0.f;
        if (weighted) {
          const float chi = a.chi ? __ldg(a.chi + t) : 1.f;
          rc = a.rho * chi;
          dec = a.t2dec * chi + a.t1dec * (1.f - chi);
        }
        float Rx = 0.f, Ry = 0.f, Rz = 0.f;
        auto sub_step = [&](float ua, float ub, float up) {
          // isotropic direction from two uniforms: cos(theta) = 1 - 2 ua, azimuth pi (2 ub - 1)
          const float cz = 1.f - 2.f * ua;
          const float st = sqrtf(fmaxf(0.f, 1.f - cz * cz));
          float sn, cs_;
          __sincosf(3.14159265358979f * (2.f * ub - 1.f), &sn, &cs_);
          const float stx = a.step_l * st * cs_, sty = a.step_l * st * sn, stz = a.step_l * cz;
          const float dl = packed_cyl_step<WALL>(x, y, ix, iy, stx, sty, up, g, cs, cand, tt);
          z += stz;
          if (weighted) logw += rc * dl - dec;
          if constexpr (PSUB) {
            Rx += x + g.L * (float)ix;
            Ry += y + g.L * (float)iy;
            Rz += z;
          }
        };
        int sub = 0;
        if constexpr (WALL == kPermeate) {
#pragma unroll 1
          for (; sub < a.S; ++sub, ++s) {
            rr = draw(a.seed, gw, 0u, s);
            sub_step(u01(rr.x), u01(rr.y), u01(rr.z));
          }
        } else {
          // two sub-steps per Philox draw; the draw of an even counter serves s and s + 1
          if ((s & 1u) && sub < a.S) {
            sub_step(u01(rr.z), u01(rr.w), 0.f);
            ++sub;
            ++s;
          }
#pragma unroll 1
          for (; sub + 1 < a.S; sub += 2, s += 2) {
            rr = draw(a.seed, gw, 0u, s >> 1);
            sub_step(u01(rr.x), u01(rr.y), 0.f);
            sub_step(u01(rr.z), u01(rr.w), 0.f);
          }
          if (sub < a.S) {
            rr = draw(a.seed, gw, 0u, s >> 1);
            sub_step(u01(rr.x), u01(rr.y), 0.f);
            ++s;
          }
        }
        const float ux = x + g.L * (float)ix, uy = y + g.L * (float)iy, uz = z;
        if constexpr (!PSUB) {
          Rx = ux;
          Ry = uy;
          Rz = uz;
        }
        // ---- phase, Kahan-compensated: Q[j][k] += V_j(t) R_k ----------------------------------
        if (__ldg(a.active + t)) {
          const float px = a.gamma_dt * Rx, py = a.gamma_dt * Ry, pz = a.gamma_dt * Rz;
          const float* gt = Gc + (t - ch * kTC) * RT;
#pragma unroll
          for (int j = 0; j < RT; ++j) {
            const float v = gt[j];
            const float pv[3] = {v * px, v * py, v * pz};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              const int i = 3 * j + k;
              const float acc = accs[i * NT], kc = kcs[i * NT];
              const float yk = pv[k] - kc;
              const float tk = acc + yk;
              kcs[i * NT] = (tk - acc) - yk;
              accs[i * NT] = tk;
            }
          }
        }
        // ---- ensemble sums at an echo sample (block-uniform branch), kWideEmit at a time -------
        if (e < a.n_echo && t == a.echo[e]) {
          const float wgt = act ? (weighted ? expf(logw) : 1.f) : 0.f;
          float qv[NACC];
#pragma unroll
          for (int i = 0; i < NACC; ++i) qv[i] = accs[i * NT];
#pragma unroll 1
          for (int m0 = 0; m0 < a.M; m0 += kWideEmit) {
            const int mn = min(kWideEmit, a.M - m0);
#pragma unroll 1
            for (int mm = 0; mm < mn; ++mm) {
              const float* cc = Cs + (size_t)(m0 + mm) * 3 * RT;
              float ph = 0.f;
#pragma unroll
              for (int j = 0; j < RT; ++j)
#pragma unroll
                for (int k = 0; k < 3; ++k) ph = fmaf(cc[k * RT + j], qv[3 * j + k], ph);
              float sn, cs_;
              sincosf(ph, &sn, &cs_);
              const float c1 = warp_sum(wgt * cs_);
              const float c2 = warp_sum(wgt * sn);
              const float c3 = warp_sum((wgt * cs_) * (wgt * cs_));
              if (lane == 0) {
                red[(warp * kWideEmit + mm) * 3] = c1;
                red[(warp * kWideEmit + mm) * 3 + 1] = c2;
                red[(warp * kWideEmit + mm) * 3 + 2] = c3;
              }
            }
            __syncthreads();
            for (int j = tid; j < mn * 3; j += NT) {
              double sacc = 0.0;
#pragma unroll
              for (int ww = 0; ww < NW; ++ww) sacc += (double)red[ww * kWideEmit * 3 + j];
              a.part[((size_t)(blockIdx.x * a.n_echo + e) * a.Mp + m0) * 3 + j] += sacc;
            }
            __syncthreads();
          }
          ++e;
        }
      }
    }

    // ---- per-walker outputs ----------------------------------------------------------------------
    const float ux = x + g.L * (float)ix, uy = y + g.L * (float)iy, uz = z;
    if (act) {
      tl.clamp += tt.clamp;
      tl.graze += tt.graze;
      tl.transmit += tt.transmit;
      if (!(isfinite(ux) && isfinite(uy) && isfinite(uz))) ++n_nonfinite;
      if (a.pass == 0) {
        if (a.final_pos) {
          a.final_pos[3 * w] = ux;
          a.final_pos[3 * w + 1] = uy;
          a.final_pos[3 * w + 2] = uz;
        }
        if (a.log_w) a.log_w[w] = logw;
        if (a.comp_end)
          a.comp_end[w] = classify<DMSIM_GEOM_PACKED_CYLINDERS>(x, y, z, g, cs, cand, a.cand_obj);
      }
      if (a.phi_out) {
        float qv[NACC];
#pragma unroll
        for (int i = 0; i < NACC; ++i) qv[i] = accs[i * NT];
        for (int m = 0; m < a.M; ++m) {
          const float* cc = Cs + (size_t)m * 3 * RT;
          float ph = 0.f;
#pragma unroll
          for (int j = 0; j < RT; ++j)
#pragma unroll
            for (int k = 0; k < 3; ++k) ph = fmaf(cc[k * RT + j], qv[3 * j + k], ph);
          a.phi_out[(size_t)w * a.M + m] = ph;
        }
      }
    }
  }

  // ---- anomaly tallies --------------------------------------------------------------------------
  const uint32_t v0 = __reduce_add_sync(0xffffffffu, n_nonfinite);
  const uint32_t v1 = __reduce_add_sync(0xffffffffu, tl.clamp);
  const uint32_t v2 = __reduce_add_sync(0xffffffffu, n_initfail);
  const uint32_t v3 = __reduce_add_sync(0xffffffffu, tl.graze);
  const uint32_t v4 = __reduce_add_sync(0xffffffffu, tl.transmit);
  if (lane == 0 && a.pass == 0) {
    if (v0) atomicAdd(&a.status[DMSIM_STATUS_NONFINITE], v0);
    if (v1) atomicAdd(&a.status[DMSIM_STATUS_CLAMPED], v1);
    if (v2) atomicAdd(&a.status[DMSIM_STATUS_INIT_FAIL], v2);
    if (v3) atomicAdd(&a.status[DMSIM_STATUS_GRAZE_FP64], v3);
    if (v4) atomicAdd(&a.status[DMSIM_STATUS_TRANSMIT], v4);
  }
}

using WideFn = void (*)(KArgs);

}  // namespace dmsim
