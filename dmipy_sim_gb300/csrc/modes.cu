// Temporal-mode projection of saved per-walker series: the orthonormal DCT-II bands that the
// compressed trajectory export and the replay packs store instead of the series itself.
//
//   out[w, k, c] = sum_t basis[k, t] * x[w, t, c]
//
// x is (n_walkers, n_t, n_ch) float16 or float32, basis (K, n_t) float32 (rows = the first K
// DCT-II basis vectors), out (n_walkers, K, n_ch) float32.  With `ramp` (n_ch == 1) the channel is
// first replaced by its detrended running sum: B_t = sum_{s<=t} x_s, endpoint = B_{n_t-1},
// r_t = B_t - endpoint * ramp_t, and r is projected (the cumulative boundary-local-time codec);
// the endpoint is written to endpoint[w].
//
// Layout: one thread per walker, kPB walkers per block, kPK modes held per thread (all channels),
// basis rows staged through shared memory kPT samples at a time.  Sums are Kahan-compensated FP32,
// so the coefficients agree with an FP64 projection to FP32 rounding.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace dmsim {

namespace {

constexpr int kPB = 128;  // walkers per block
constexpr int kPT = 16;   // samples per staged chunk
constexpr int kPK = 8;    // modes per register tile

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

template <bool F16>
__device__ __forceinline__ float load_x(const void* x, size_t o) {
  if constexpr (F16) return __half2float(reinterpret_cast<const __half*>(x)[o]);
  else return reinterpret_cast<const float*>(x)[o];
}

template <bool F16, int NCH, bool CUM>
__global__ void __launch_bounds__(kPB) k_project_modes(const void* __restrict__ x,
                                                       int64_t n_walkers, int n_t,
                                                       const float* __restrict__ basis, int K,
                                                       const float* __restrict__ ramp,
                                                       float* __restrict__ endpoint,
                                                       float* __restrict__ out) {
  __shared__ float bs[kPK * kPT];
  __shared__ float rs[kPT];
  const int tid = threadIdx.x;
  const int n_kt = (K + kPK - 1) / kPK;
  const int64_t n_tiles = (n_walkers + kPB - 1) / kPB;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t w = tile * kPB + tid;
    const bool act = w < n_walkers;
    const size_t row = (size_t)(act ? w : 0) * n_t * NCH;
    float ep = 0.f;
    if constexpr (CUM) {  // endpoint B(T) = sum of the whole series
      Kahan e;
      if (act)
        for (int t = 0; t < n_t; ++t) e.add(load_x<F16>(x, row + t));
      ep = e.s;
      if (act) endpoint[w] = ep;
    }
    for (int kt = 0; kt < n_kt; ++kt) {
      Kahan acc[kPK][NCH];
      Kahan run;  // running sum B_t (CUM)
      for (int t0 = 0; t0 < n_t; t0 += kPT) {
        __syncthreads();
        for (int i = tid; i < kPK * kPT; i += kPB) {
          const int k = kt * kPK + i / kPT, t = t0 + i % kPT;
          bs[i] = (k < K && t < n_t) ? basis[(size_t)k * n_t + t] : 0.f;
        }
        if (CUM && tid < kPT) rs[tid] = (t0 + tid < n_t) ? ramp[t0 + tid] : 0.f;
        __syncthreads();
        if (!act) continue;
        const int tn = min(kPT, n_t - t0);
        for (int tt = 0; tt < tn; ++tt) {
          float v[NCH];
#pragma unroll
          for (int c = 0; c < NCH; ++c) v[c] = load_x<F16>(x, row + (size_t)(t0 + tt) * NCH + c);
          if constexpr (CUM) {
            run.add(v[0]);
            v[0] = run.s - ep * rs[tt];
          }
#pragma unroll
          for (int j = 0; j < kPK; ++j) {
            const float b = bs[j * kPT + tt];
#pragma unroll
            for (int c = 0; c < NCH; ++c) acc[j][c].add(b * v[c]);
          }
        }
      }
      if (act) {
#pragma unroll
        for (int j = 0; j < kPK; ++j) {
          const int k = kt * kPK + j;
          if (k < K)
#pragma unroll
            for (int c = 0; c < NCH; ++c) out[((size_t)w * K + k) * NCH + c] = acc[j][c].s;
        }
      }
    }
  }
}

template <bool F16, int NCH, bool CUM>
cudaError_t launch(const void* x, int64_t n_walkers, int n_t, const float* basis, int K,
                   const float* ramp, float* endpoint, float* out, cudaStream_t st) {
  int dev = 0, n_sm = 0, nb = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k_project_modes<F16, NCH, CUM>,
                                                kPB, 0);
  int64_t grid = (int64_t)(nb > 0 ? nb : 1) * (n_sm > 0 ? n_sm : 1);
  const int64_t n_tiles = (n_walkers + kPB - 1) / kPB;
  if (grid > n_tiles) grid = n_tiles;
  k_project_modes<F16, NCH, CUM><<<(int)grid, kPB, 0, st>>>(x, n_walkers, n_t, basis, K, ramp,
                                                            endpoint, out);
  return cudaGetLastError();
}

}  // namespace

// Arguments are checked by the C entry point (dmsim_project_modes in capi.cu).
cudaError_t launch_project_modes(const void* x, bool f16, int64_t n_walkers, int n_t, int n_ch,
                                 const float* basis, int K, const float* ramp, float* endpoint,
                                 float* out, cudaStream_t st) {
  if (ramp) {
    return f16 ? launch<true, 1, true>(x, n_walkers, n_t, basis, K, ramp, endpoint, out, st)
               : launch<false, 1, true>(x, n_walkers, n_t, basis, K, ramp, endpoint, out, st);
  }
  if (n_ch == 1)
    return f16 ? launch<true, 1, false>(x, n_walkers, n_t, basis, K, nullptr, nullptr, out, st)
               : launch<false, 1, false>(x, n_walkers, n_t, basis, K, nullptr, nullptr, out, st);
  return f16 ? launch<true, 3, false>(x, n_walkers, n_t, basis, K, nullptr, nullptr, out, st)
             : launch<false, 3, false>(x, n_walkers, n_t, basis, K, nullptr, nullptr, out, st);
}

}  // namespace dmsim
