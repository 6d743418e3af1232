// Counter-based random stream for the walk.
//
// Philox4x32 with 10 rounds, the counter-based generator of Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3" (SC'11), written from the published round
// function: two 32x32->64 multiplications by the round multipliers, a swap-xor with the key, and a
// Weyl-sequence key schedule.  It replaces JAX's threefry keys of the reference
// (core.py:445-447 split per walker, physics.py:298-300 split per sub-step).
//
// Stream contract (shared by the CUDA kernels and the CPU oracle, so the two walk the same
// walkers step for step):
//   key     = (seed & 0xffffffff, seed >> 32)
//   counter = (call index j, walker & 0xffffffff, walker >> 32, stream)
//   stream 0: the walk; stream 1: seeding (init positions), one call per rejection attempt.
//   uniform = (word >> 8) * 2^-24, a float in [0, 1) with 24 random bits.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define DMSIM_HD __host__ __device__ __forceinline__
#else
#define DMSIM_HD static inline
#endif

namespace dmsim {

struct u32x4 {
  uint32_t x, y, z, w;
};

DMSIM_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

DMSIM_HD u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi0 = mulhi32(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z);
    c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

DMSIM_HD float u01(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

DMSIM_HD u32x4 draw(uint64_t seed, uint64_t walker, uint32_t stream, uint32_t j) {
  return philox4x32_10(u32x4{j, (uint32_t)walker, (uint32_t)(walker >> 32), stream},
                       (uint32_t)seed, (uint32_t)(seed >> 32));
}

}  // namespace dmsim
