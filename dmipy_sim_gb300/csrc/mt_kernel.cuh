// The magnetisation-transfer Bloch walk (bloch.py:343-671): kernel arguments and the table of
// instantiations.  One walker per thread; blocks loop over walker tiles (grid = SMs x resident
// blocks); the magnetisation of up to W measurements per pass lives in FP64 registers.
#pragma once
#include <stdint.h>

#include "dmsim.h"
#include "geometry.cuh"

namespace dmsim {

constexpr int kMtBlock = 256;
constexpr int kMtWarps = kMtBlock / 32;
constexpr int kMtMaxEcho = 512;

struct MtArgs {
  int64_t n_walkers;
  uint64_t seed;
  uint32_t s0;  // Philox counter of the first sub-step
  int n_t, n_sub, M, m_off, n_echo, spin, pass;
  float step_l, kod_mt, dwell, rho;
  double gamma_dt, m0, e2h[2], e1h[2];
  GeoK g;
  const uint32_t* cs;
  const float4* cand;
  const float* G;
  const double* rot;
  const float* crush;
  const float* r0;
  const float* brem_in;
  float* brem_out;
  float* r_end;
  float* occ;
  float* occ_total;
  double* part;  // [gridDim.x][n_echo][W][3]
  uint32_t* status;
  void* traj;
  int traj_f16;
  float* dlog_free;
  int echo[kMtMaxEcho];
};

using MtFn = void (*)(MtArgs);
// The kernel for a geometry kind and a measurement width (1 or 4), or null.
MtFn mt_fn(int kind, int width);

}  // namespace dmsim
