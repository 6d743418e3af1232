// Vector-Bloch replay of a stored walk (trajectories.py:734-949): every walker's magnetisation
// M_m = (Mx, My, Mz) (FP64, W measurements per pass in registers) is carried through the
// sequence on the saved positions, sample by sample in the reference's order: the RF
// increments of the sample (Rodrigues about (cos ax, sin ax, 0), the flip scaled by the
// walker's B1+ factor), precession by gamma dt G(t).r(t) plus the extra phases of the sample
// (per-walker phase, bound-pool offset, pulse carrier, slice select while a pulse is on),
// the wall attenuation exp(rho/D dlog), then Mxy *= E2 and Mz *= E1 with the walker's rates
// (per compartment, blended toward the bound pool by the walker's occupancy).  At each echo
// sample the block sums w Mx and w My in FP64 in a fixed order; per-walker echoes and the
// final magnetisation are written on request.  Positions stream from HBM (float16 or float32),
// each sample's G row is a broadcast read.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "dmsim.h"

namespace dmsim {
int set_error(int code, const char* msg);
}

namespace {

constexpr int kRbBlock = 256;
constexpr int kRbWarps = kRbBlock / 32;
constexpr int kRbW = 4;

__device__ __forceinline__ double warp_sum_rb(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct RbArgs {
  dmsim_replay_bloch_params p;
  int m_off, pass;
};

__global__ void __launch_bounds__(kRbBlock) k_replay_bloch(const __grid_constant__ RbArgs A,
                                                           double* __restrict__ part) {
  const dmsim_replay_bloch_params& p = A.p;
  __shared__ double red[kRbWarps][kRbW * 2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int j = tid; j < p.n_echo * kRbW * 2; j += kRbBlock)
    part[(size_t)blockIdx.x * p.n_echo * kRbW * 2 + j] = 0.0;
  __syncthreads();
  const int nm = min(kRbW, p.n_meas - A.m_off);
  const int64_t n_tiles = (p.n_walkers + kRbBlock - 1) / kRbBlock;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t w = tile * kRbBlock + tid;
    const bool act = w < p.n_walkers;
    const int64_t wi = act ? w : 0;
    const double wt = act ? (p.weights ? p.weights[wi] : 1.0) : 0.0;
    const double b1 = p.b1_scale ? p.b1_scale[wi] : 1.0;
    const double sl = p.slice_dphi ? p.slice_dphi[wi] : 0.0;
    double Mx[kRbW], My[kRbW], Mz[kRbW];
#pragma unroll
    for (int m = 0; m < kRbW; ++m) {
      Mx[m] = My[m] = 0.0;
      Mz[m] = 1.0;
    }
    int e = 0;
#pragma unroll 1
    for (int t = 0; t < p.n_t; ++t) {
      // RF increments of this sample (trajectories.py:922-924)
      for (int k = p.rf_start[t]; k < p.rf_start[t + 1]; ++k) {
        const double flip = p.rf_flip[k] * b1;
        double uy, ux, s, c;
        sincos(p.rf_axis[k], &uy, &ux);
        sincos(flip, &s, &c);
        const double omc = 1.0 - c;
#pragma unroll
        for (int m = 0; m < kRbW; ++m) {
          const double x = Mx[m], y = My[m], z = Mz[m];
          Mx[m] = (c + ux * ux * omc) * x + (ux * uy * omc) * y + (uy * s) * z;
          My[m] = (ux * uy * omc) * x + (c + uy * uy * omc) * y + (-ux * s) * z;
          Mz[m] = (-uy * s) * x + (ux * s) * y + c * z;
        }
      }
      const size_t o = (size_t)wi * p.n_t + t;
      double rx, ry, rz;
      if (p.traj_f16) {
        const __half* tp = reinterpret_cast<const __half*>(p.traj) + o * 3;
        rx = (double)__half2float(tp[0]);
        ry = (double)__half2float(tp[1]);
        rz = (double)__half2float(tp[2]);
      } else {
        const float* tp = reinterpret_cast<const float*>(p.traj) + o * 3;
        rx = (double)tp[0];
        ry = (double)tp[1];
        rz = (double)tp[2];
      }
      const double bf = p.bound_frac ? (double)p.bound_frac[o] : 0.0;
      // extra phases in the reference's order of addition (trajectories.py:928-935)
      const double xph = p.extra_phase ? p.extra_phase[o] : 0.0;
      const double dbound = (p.bound_frac && p.dphi_bound != 0.0) ? bf * p.dphi_bound : 0.0;
      const double roff = p.rf_offset ? p.rf_offset[t] : 0.0;
      const bool slice_on = p.slice_dphi && p.rf_active[t];
      double e2 = p.e2, e1 = p.e1;
      if (p.comp || p.bound_frac) {
        double i2 = p.inv_t2, i1 = p.inv_t1;
        if (p.comp) {
          const int c = p.comp[o];
          i2 = p.inv_t2_comp[c];
          i1 = p.inv_t1_comp[c];
        }
        if (p.bound_frac) {
          i2 = (1.0 - bf) * i2 + bf * p.inv_t2_bound;
          i1 = (1.0 - bf) * i1 + bf * p.inv_t1_bound;
        }
        e2 = exp(-p.dt_traj * i2);
        e1 = exp(-p.dt_traj * i1);
      }
      const double sf = p.dlog ? exp(p.rho_over_D * (double)p.dlog[o]) : 1.0;
#pragma unroll
      for (int m = 0; m < kRbW; ++m) {
        if (m >= nm) continue;
        const double* g = p.G + ((size_t)t * p.n_meas + A.m_off + m) * 3;
        double dphi = p.gamma_dt * (rx * __ldg(g) + ry * __ldg(g + 1) + rz * __ldg(g + 2));
        if (p.extra_phase) dphi = dphi + xph;
        if (p.bound_frac && p.dphi_bound != 0.0) dphi = dphi + dbound;
        if (p.rf_offset) dphi = dphi + roff;
        if (slice_on) dphi = dphi + sl;
        double s, c;
        sincos(dphi, &s, &c);
        const double x = c * Mx[m] - s * My[m];
        const double y = s * Mx[m] + c * My[m];
        Mx[m] = x * sf * e2;
        My[m] = y * sf * e2;
        Mz[m] = Mz[m] * e1;
      }
      // echo sample (block-uniform branch)
      if (e < p.n_echo && t == p.echo_idx[e]) {
        if (act && p.echo_walker) {
#pragma unroll
          for (int m = 0; m < kRbW; ++m)
            if (m < nm) {
              double* ew = p.echo_walker +
                           (((size_t)(A.m_off + m) * p.n_echo + e) * p.n_walkers + w) * 2;
              ew[0] = Mx[m];
              ew[1] = My[m];
            }
        }
#pragma unroll
        for (int m = 0; m < kRbW; ++m) {
          const double c1 = warp_sum_rb(wt * Mx[m]);
          const double c2 = warp_sum_rb(wt * My[m]);
          if (lane == 0) {
            red[warp][2 * m] = c1;
            red[warp][2 * m + 1] = c2;
          }
        }
        __syncthreads();
        for (int j = tid; j < kRbW * 2; j += kRbBlock) {
          double acc = 0.0;
#pragma unroll
          for (int ww = 0; ww < kRbWarps; ++ww) acc += red[ww][j];
          part[((size_t)blockIdx.x * p.n_echo + e) * kRbW * 2 + j] += acc;
        }
        __syncthreads();
        ++e;
      }
    }
    if (act && p.m_last && A.m_off + nm == p.n_meas) {
#pragma unroll
      for (int m = 0; m < kRbW; ++m)
        if (m == nm - 1) {
          p.m_last[w] = Mx[m];
          p.m_last[p.n_walkers + w] = My[m];
          p.m_last[2 * p.n_walkers + w] = Mz[m];
        }
    }
  }
}

__global__ void k_rb_reduce(const double* __restrict__ part, int grid, int n_echo, int n_meas,
                            int m_off, double* __restrict__ sums) {
  const int n = n_echo * kRbW * 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int e = i / (kRbW * 2), r = i % (kRbW * 2), m = m_off + r / 2;
    if (m >= n_meas) continue;
    double acc = 0.0;
    for (int b = 0; b < grid; ++b) acc += part[((size_t)b * n_echo + e) * kRbW * 2 + r];
    sums[((size_t)m * n_echo + e) * 2 + r % 2] = acc;
  }
}

int rb_grid(int64_t n_walkers) {
  int dev = 0, n_sm = 0, nb = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k_replay_bloch, kRbBlock, 0);
  int64_t grid = (int64_t)(nb > 0 ? nb : 1) * (n_sm > 0 ? n_sm : 1);
  const int64_t n_tiles = (n_walkers + kRbBlock - 1) / kRbBlock;
  if (grid > n_tiles) grid = n_tiles;
  return (int)(grid < 1 ? 1 : grid);
}

int rb_check(const dmsim_replay_bloch_params* p) {
  if (!p) return dmsim::set_error(DMSIM_EINVAL, "replay_bloch: null parameters");
  if (p->n_walkers < 0 || p->n_t < 1 || p->n_meas < 1 || p->n_echo < 1)
    return dmsim::set_error(DMSIM_EINVAL, "replay_bloch: need n_walkers >= 0, n_t, n_meas, "
                                          "n_echo >= 1");
  if (!p->traj || !p->G || !p->rf_start || !p->echo_idx || !p->sums || !p->rf_active)
    return dmsim::set_error(DMSIM_EINVAL, "replay_bloch: missing traj, G, RF table, echo "
                                          "samples, activity flags or sums");
  if (p->comp && (!p->inv_t2_comp || !p->inv_t1_comp))
    return dmsim::set_error(DMSIM_EINVAL, "replay_bloch: compartments need their rates");
  return DMSIM_OK;
}

}  // namespace

extern "C" {

size_t dmsim_replay_bloch_workspace_bytes(const dmsim_replay_bloch_params* p) {
  if (rb_check(p) != DMSIM_OK) return 0;
  const int grid = rb_grid(p->n_walkers);
  if (grid < 1) return 0;
  return (((size_t)grid * p->n_echo * kRbW * 2 * 8) + 255) & ~(size_t)255;
}

int dmsim_replay_bloch(const dmsim_replay_bloch_params* p, void* workspace,
                       size_t workspace_bytes, void* stream) {
  const int rc = rb_check(p);
  if (rc != DMSIM_OK) return rc;
  const size_t need = dmsim_replay_bloch_workspace_bytes(p);
  if (!workspace || workspace_bytes < need)
    return dmsim::set_error(DMSIM_EWORKSPACE, "replay_bloch: workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  if (p->n_walkers == 0) {
    cudaMemsetAsync(p->sums, 0, sizeof(double) * p->n_meas * p->n_echo * 2, st);
    return DMSIM_OK;
  }
  const int grid = rb_grid(p->n_walkers);
  RbArgs a;
  memset(&a, 0, sizeof(a));
  a.p = *p;
  double* part = reinterpret_cast<double*>(workspace);
  for (int m0 = 0, pass = 0; m0 < p->n_meas; m0 += kRbW, ++pass) {
    a.m_off = m0;
    a.pass = pass;
    k_replay_bloch<<<grid, kRbBlock, 0, st>>>(a, part);
    const int nred = p->n_echo * kRbW * 2;
    k_rb_reduce<<<(nred + 255) / 256, 256, 0, st>>>(part, grid, p->n_echo, p->n_meas, m0,
                                                    p->sums);
  }
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return dmsim::set_error(DMSIM_ECUDA, cudaGetErrorString(err));
  return DMSIM_OK;
}

}  // extern "C"
