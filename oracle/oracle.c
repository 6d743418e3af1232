/* CPU oracle of the dmipy-sim Monte-Carlo walk — TEST INFRASTRUCTURE ONLY (see oracle.h).
 * Build: oracle/build.sh (gcc -O2 -fopenmp -ffp-contract=off), output oracle/_build/liboracle.so. */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Philox4x32-10 (Salmon et al., SC'11): the stream contract of the walk (philox.cuh). */
void or_philox(uint64_t seed, uint64_t walker, uint32_t stream, uint32_t j, uint32_t out[4]) {
  uint32_t c0 = j, c1 = (uint32_t)walker, c2 = (uint32_t)(walker >> 32), c3 = stream;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* float -> IEEE half (round to nearest even, subnormals kept) -> double: the float16 storage of
   simulate_trajectories (core.py:1426-1449). */
static double round_half(float f) {
  if (!isfinite(f)) return (double)f;
  double a = fabs((double)f);
  if (a >= 65520.0) return f > 0 ? INFINITY : -INFINITY;
  int e;
  frexp(a, &e);                 /* a = m * 2^e, m in [0.5, 1) */
  int ex = e - 1;               /* a in [2^ex, 2^(ex+1)) */
  if (ex < -14) ex = -14;       /* subnormal range: fixed quantum 2^-24 */
  double q = ldexp(1.0, ex - 10);
  double v = nearbyint(a / q) * q;   /* default rounding mode: nearest even */
  return f < 0 ? -v : v;
}

#define REAL float
#define SUF _f32
#define SQRT sqrtf
#define FLOOR floorf
#define FMOD fmodf
#define FABS fabsf
#define NEARBYINT nearbyintf
#define SIN sinf
#define COS cosf
#define EXP expf
#define LOG logf
#define MAX(a, b) fmaxf((a), (b))
#define MIN(a, b) fminf((a), (b))
#include "oracle_impl.inc"
#undef REAL
#undef SUF
#undef SQRT
#undef FLOOR
#undef FMOD
#undef FABS
#undef NEARBYINT
#undef SIN
#undef COS
#undef EXP
#undef LOG
#undef MAX
#undef MIN

#define REAL double
#define SUF _f64
#define SQRT sqrt
#define FLOOR floor
#define FMOD fmod
#define FABS fabs
#define NEARBYINT nearbyint
#define SIN sin
#define COS cos
#define EXP exp
#define LOG log
#define MAX(a, b) fmax((a), (b))
#define MIN(a, b) fmin((a), (b))
#include "oracle_impl.inc"
