// dmsim_fp32_fma_peak: the FP32 fused-multiply-add rate of this GPU, measured.
//
// The walk kernels are bound by FP32/INT issue, and their roofline fraction is quoted against
// this measured rate rather than a nominal one.  Each thread runs 8 independent FMA chains (one
// FMA of each chain issues every cycle the pipe allows, hiding its latency), iters times; the
// chains' sum is stored so that nothing is optimised away.  FLOPs per launch = blocks * threads *
// iters * 8 * 2.  No counterpart in the reference (a measurement helper of this library).
#include <cuda_runtime.h>

#include "dmsim.h"

namespace dmsim {
int set_error(int code, const char* msg);

__global__ void __launch_bounds__(256) k_fma_peak(int iters, float b, float c, float* sink) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-6f, a2 = a0 + 2e-6f, a3 = a0 + 3e-6f;
  float a4 = a0 + 4e-6f, a5 = a0 + 5e-6f, a6 = a0 + 6e-6f, a7 = a0 + 7e-6f;
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, b, c);
      a1 = fmaf(a1, b, c);
      a2 = fmaf(a2, b, c);
      a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c);
      a5 = fmaf(a5, b, c);
      a6 = fmaf(a6, b, c);
      a7 = fmaf(a7, b, c);
    }
  }
  const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  // every thread's chains stay live: the store is conditional on their value (sink holds 1 float)
  if (s == 12345.678f || (threadIdx.x == 0 && blockIdx.x == 0)) sink[0] = s;
}

}  // namespace dmsim

extern "C" int dmsim_fp32_fma_peak(int blocks, int threads, int iters, float* sink,
                                   void* stream) {
  if (blocks < 1 || threads < 32 || threads > 256 || (threads & 31) || iters < 1 || !sink)
    return dmsim::set_error(DMSIM_EINVAL, "fp32_fma_peak: need blocks >= 1, threads a multiple "
                                          "of 32 in [32, 256], iters >= 1 and a sink");
  dmsim::k_fma_peak<<<blocks, threads, 0, (cudaStream_t)stream>>>(iters, 0.999999f, 1e-7f, sink);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmsim::set_error(DMSIM_ECUDA, "fp32_fma_peak: launch failed");
  return DMSIM_OK;
}
