// The magnetisation-transfer Bloch walk kernel (bloch.py:468-553 per sample and sub-step).
//
// Per walker and sub-step: one Philox draw (x, y: the direction; z: the binding test; w: the
// dwell); a free walker steps through the geometry's reflecting-with-log-weight rule and sticks
// with p = min(1, kappa_MT/D * 2 sum d_perp); a bound walker stays put and counts its dwell down.
// With spin on, the FP64 magnetisation of each measurement takes a Strang split with the
// walker's current pool -- half relaxation, the sample's per-sub-step rotation for that pool
// (precomputed on the host: RF nutation and off-resonance, two 3x3 matrices per sample, the same
// for every walker in that pool), half relaxation and the free-contact surface weight -- and
// after the sample's sub-steps the gradient (and crusher) phase rotates Mxy.  Echo samples are
// reduced per block in FP64 in a fixed order.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "mt_kernel.cuh"
#include "philox.cuh"

namespace dmsim {

namespace {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int GEOM, int W>
__global__ void __launch_bounds__(kMtBlock) k_bloch_mt(const __grid_constant__ MtArgs a) {
  __shared__ double red[kMtWarps][W * 3];
  constexpr bool PACKED =
      GEOM == DMSIM_GEOM_PACKED_CYLINDERS || GEOM == DMSIM_GEOM_PACKED_SPHERES;
  constexpr bool P3 = GEOM == DMSIM_GEOM_PACKED_SPHERES;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const GeoK g = a.g;
  if (a.spin)
    for (int j = tid; j < a.n_echo * W * 3; j += kMtBlock)
      a.part[(size_t)blockIdx.x * a.n_echo * W * 3 + j] = 0.0;
  __syncthreads();

  Tally tl, tl_idle;
  uint32_t n_nonfinite = 0;
  const int64_t n_tiles = (a.n_walkers + kMtBlock - 1) / kMtBlock;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t w = tile * kMtBlock + tid;
    const bool act = w < a.n_walkers;
    const uint64_t gw = (uint64_t)w;
    Tally& tw = act ? tl : tl_idle;
    float x = 0.f, y = 0.f, z = 0.f;
    int ix = 0, iy = 0, iz = 0;
    float brem = 0.f;
    if (act) {
      x = a.r0[3 * w];
      y = a.r0[3 * w + 1];
      z = a.r0[3 * w + 2];
      if (a.brem_in) brem = a.brem_in[w];
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
    const float uc = a.crush ? u01(draw(a.seed, gw, 2u, 0u).x) : 0.f;
    double Mx[W], My[W], Mz[W];
#pragma unroll
    for (int m = 0; m < W; ++m) {
      Mx[m] = My[m] = 0.0;
      Mz[m] = a.m0;
    }
    float occ_sum = 0.f;
    uint32_t s = a.s0;
    int e = 0;
#pragma unroll 1
    for (int t = 0; t < a.n_t; ++t) {
      // the sample's rotations for the free (f) and the bound (b) pool
      double f[9], b[9];
      if (a.spin) {
        const double* rt = a.rot + (size_t)t * 18;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          f[k] = __ldg(rt + k);
          b[k] = __ldg(rt + 9 + k);
        }
      }
      int n_bound = 0;
      float dl_free = 0.f;  // the sample's boundary log-weight over free, non-binding sub-steps
#pragma unroll 1
      for (int sub = 0; sub < a.n_sub; ++sub, ++s) {
        const u32x4 rr = draw(a.seed, gw, 0u, s);
        const bool bound = brem > 0.f;
        float dl = 0.f;
        if (!bound) {
          const float cz = 1.f - 2.f * u01(rr.x);
          const float sz = sqrtf(fmaxf(0.f, 1.f - cz * cz));
          float sn, cs_;
          __sincosf(3.14159265358979f * (2.f * u01(rr.y) - 1.f), &sn, &cs_);
          const float stx = a.step_l * sz * cs_, sty = a.step_l * sz * sn, stz = a.step_l * cz;
          if constexpr (GEOM == DMSIM_GEOM_CYLINDER) {
            dl = cylinder_step<kRelax>(x, y, stx, sty, 0.f, g, tw);
            z += stz;
          } else if constexpr (GEOM == DMSIM_GEOM_SPHERE) {
            dl = sphere_step<kRelax>(x, y, z, stx, sty, stz, 0.f, g, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_ELLIPSOID) {
            dl = ellipsoid_step<kRelax>(x, y, z, stx, sty, stz, 0.f, g, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_BOX1D) {
            dl = box1d_step<kRelax>(x, y, z, stx, sty, stz, g);
          } else if constexpr (GEOM == DMSIM_GEOM_SLAB) {
            dl = slab_step<kRelax>(x, y, z, stx, sty, stz, 0.f, g, tw);
          } else if constexpr (GEOM == DMSIM_GEOM_PACKED_CYLINDERS) {
            dl = packed_cyl_step<kRelax>(x, y, ix, iy, stx, sty, 0.f, g, a.cs, a.cand, tw);
            z += stz;
          } else if constexpr (GEOM == DMSIM_GEOM_PACKED_SPHERES) {
            dl = packed_sph_step<kRelax>(x, y, z, ix, iy, iz, stx, sty, stz, 0.f, g, a.cs,
                                         a.cand, tw);
          }
        }
        // binding: the boundary local time of this step is -dl (bloch.py:480-484)
        const bool newly = !bound && u01(rr.z) < fminf(1.f, a.kod_mt * (-dl));
        const float dwell = -logf(fmaxf(u01(rr.w), 1e-20f)) * a.dwell;
        brem = bound ? brem - 1.f : (newly ? dwell : 0.f);
        n_bound += bound ? 1 : 0;
        if (!(bound || newly)) dl_free += dl;
        if (a.spin) {
          // Strang split with the pool of this sub-step (bloch.py:488-538)
          const double e2h = bound ? a.e2h[1] : a.e2h[0];
          const double e1h = bound ? a.e1h[1] : a.e1h[0];
          const double surf =
              (bound || newly || dl == 0.f || a.rho == 0.f) ? 1.0 : exp((double)a.rho * (double)dl);
          double r[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) r[k] = bound ? b[k] : f[k];
#pragma unroll
          for (int m = 0; m < W; ++m) {
            const double mx = Mx[m] * e2h, my = My[m] * e2h;
            const double mz = a.m0 + (Mz[m] - a.m0) * e1h;
            const double rx = r[0] * mx + r[1] * my + r[2] * mz;
            const double ry = r[3] * mx + r[4] * my + r[5] * mz;
            const double rz = r[6] * mx + r[7] * my + r[8] * mz;
            Mx[m] = rx * e2h * surf;
            My[m] = ry * e2h * surf;
            Mz[m] = a.m0 + (rz - a.m0) * e1h;
          }
        }
      }
      const float bf = (float)n_bound / (float)a.n_sub;
      occ_sum += bf;
      if (act && a.pass == 0) {
        if (a.occ) a.occ[(size_t)w * a.n_t + t] = bf;
        if (a.dlog_free) a.dlog_free[(size_t)w * a.n_t + t] = dl_free;
        if (a.traj) {
          const size_t o = ((size_t)w * a.n_t + t) * 3;
          const float px = x + g.L * (float)ix, py = y + g.L * (float)iy, pz = z + g.L * (float)iz;
          if (a.traj_f16) {
            __half* tp = reinterpret_cast<__half*>(a.traj);
            tp[o] = __float2half_rn(px);
            tp[o + 1] = __float2half_rn(py);
            tp[o + 2] = __float2half_rn(pz);
          } else {
            float* tp = reinterpret_cast<float*>(a.traj);
            tp[o] = px;
            tp[o + 1] = py;
            tp[o + 2] = pz;
          }
        }
      }
      if (a.spin) {
        // the sample's gradient and crusher phase at the walker's position (bloch.py:544-548)
        const float ux = x + g.L * (float)ix, uy = y + g.L * (float)iy, uz = z + g.L * (float)iz;
        const float cr = a.crush ? __ldg(a.crush + t) * uc : 0.f;
#pragma unroll
        for (int m = 0; m < W; ++m) {
          if (a.m_off + m >= a.M) break;
          const float* gt = a.G + ((size_t)t * a.M + a.m_off + m) * 3;
          const float dot = __ldg(gt) * ux + __ldg(gt + 1) * uy + __ldg(gt + 2) * uz;
          const double ph = a.gamma_dt * (double)dot + (double)cr;
          if (ph != 0.0) {
            double sn, cs_;
            sincos(ph, &sn, &cs_);
            const double mx = cs_ * Mx[m] - sn * My[m];
            My[m] = sn * Mx[m] + cs_ * My[m];
            Mx[m] = mx;
          }
        }
        // echo sample: block sums of Mx, My, Mz (block-uniform branch)
        if (e < a.n_echo && t == a.echo[e]) {
#pragma unroll
          for (int m = 0; m < W; ++m) {
            const double c1 = warp_sum_d(act ? Mx[m] : 0.0);
            const double c2 = warp_sum_d(act ? My[m] : 0.0);
            const double c3 = warp_sum_d(act ? Mz[m] : 0.0);
            if (lane == 0) {
              red[warp][3 * m] = c1;
              red[warp][3 * m + 1] = c2;
              red[warp][3 * m + 2] = c3;
            }
          }
          __syncthreads();
          for (int j = tid; j < W * 3; j += kMtBlock) {
            double acc = 0.0;
#pragma unroll
            for (int ww = 0; ww < kMtWarps; ++ww) acc += red[ww][j];
            a.part[((size_t)blockIdx.x * a.n_echo + e) * W * 3 + j] += acc;
          }
          __syncthreads();
          ++e;
        }
      }
    }
    if (act && a.pass == 0) {
      const float ux = x + g.L * (float)ix, uy = y + g.L * (float)iy, uz = z + g.L * (float)iz;
      if (!(isfinite(ux) && isfinite(uy) && isfinite(uz))) ++n_nonfinite;
      if (a.r_end) {
        a.r_end[3 * w] = ux;
        a.r_end[3 * w + 1] = uy;
        a.r_end[3 * w + 2] = uz;
      }
      if (a.brem_out) a.brem_out[w] = brem;
      if (a.occ_total) a.occ_total[w] = occ_sum;
    }
  }
  const uint32_t v0 = __reduce_add_sync(0xffffffffu, n_nonfinite);
  const uint32_t v1 = __reduce_add_sync(0xffffffffu, tl.clamp);
  const uint32_t v2 = __reduce_add_sync(0xffffffffu, tl.graze);
  if (lane == 0 && a.pass == 0) {
    if (v0) atomicAdd(&a.status[DMSIM_STATUS_NONFINITE], v0);
    if (v1) atomicAdd(&a.status[DMSIM_STATUS_CLAMPED], v1);
    if (v2) atomicAdd(&a.status[DMSIM_STATUS_GRAZE_FP64], v2);
  }
}

template <int W>
MtFn pick(int kind) {
  switch (kind) {
    case DMSIM_GEOM_CYLINDER: return k_bloch_mt<DMSIM_GEOM_CYLINDER, W>;
    case DMSIM_GEOM_SPHERE: return k_bloch_mt<DMSIM_GEOM_SPHERE, W>;
    case DMSIM_GEOM_ELLIPSOID: return k_bloch_mt<DMSIM_GEOM_ELLIPSOID, W>;
    case DMSIM_GEOM_BOX1D: return k_bloch_mt<DMSIM_GEOM_BOX1D, W>;
    case DMSIM_GEOM_SLAB: return k_bloch_mt<DMSIM_GEOM_SLAB, W>;
    case DMSIM_GEOM_PACKED_CYLINDERS: return k_bloch_mt<DMSIM_GEOM_PACKED_CYLINDERS, W>;
    case DMSIM_GEOM_PACKED_SPHERES: return k_bloch_mt<DMSIM_GEOM_PACKED_SPHERES, W>;
    default: return nullptr;
  }
}

}  // namespace

MtFn mt_fn(int kind, int width) {
  if (width == 1) return pick<1>(kind);
  if (width == 4) return pick<4>(kind);
  return nullptr;
}

}  // namespace dmsim
