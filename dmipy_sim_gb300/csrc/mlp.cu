// Surrogate MLP kernels: a BF16 tensor-core GEMM (tcgen05.mma, accumulator in tensor memory,
// operands staged by TMA) with fused epilogues, plus the small kernels around it (input packing,
// the linear head with the squared-error seed gradient, row reductions, AdamW).
//
// GEMM: C[M, N] = A[M, K] . B[N, K]^T, A and B row-major bf16 (K contiguous, "K-major" for the
// tensor core).  One CTA computes a 128 x BN tile (BN = 128 or 256 accumulator columns of tensor
// memory) over its share of K:
//   warp 0      TMA producer: 64-wide K slices of A and B into a ring of shared-memory stages
//               (128-byte swizzle), one mbarrier per stage;
//   warp 1      allocates the tensor memory, and one lane issues tcgen05.mma (K = 16 per
//               instruction, 4 per stage); tcgen05.commit frees each stage and finally signals
//               the accumulator;
//   warps 2..5  epilogue: tcgen05.ld of 32 accumulator columns at a time (each warp owns the 32
//               tensor-memory lanes = tile rows its warp index selects), fused bias / GELU /
//               GELU-derivative, and stores of the row-major result and, optionally, its
//               transpose (a warp writes 32 consecutive rows of one column: 64 contiguous bytes).
// Every mbarrier wait is bounded; a wait that gives up sets an error word and the CTA drains,
// frees its tensor memory and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "dmsim.h"

namespace dmsim {
int set_error(int code, const char* msg);
}

namespace {

constexpr int BM = 128;      // tile rows (tensor-memory lanes)
constexpr int BK = 64;       // K slice per stage: 64 bf16 = 128 bytes = one swizzle row
constexpr int kEpiWarps = 8;
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kWaitPolls = 1u << 24;

// ---- PTX helpers --------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t s_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_addr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_expect(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(s_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitPolls; ++i)
    if (bar_try(b, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(s_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(s_addr(b))
      : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   s_addr(b))
               : "memory");
}
// Shared-memory matrix descriptor of a K-major, 128-byte-swizzled tile whose rows are 128 bytes
// apart and whose 8-row groups are 1024 bytes apart (the layout a TMA box of 64 bf16 columns with
// CU_TENSOR_MAP_SWIZZLE_128B writes).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                       // leading byte offset (unused when swizzled)
  d |= (uint64_t)(1024 >> 4) << 32;             // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                       // descriptor version
  d |= (uint64_t)2 << 61;                       // 128-byte swizzle
  return d;
}
// Instruction descriptor of kind::f16: bf16 A and B, fp32 accumulator, both K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4)                    // accumulator format: f32
         | (1u << 7)                  // A format: bf16
         | (1u << 10)                 // B format: bf16
         | ((uint32_t)(N >> 3) << 17)  // N / 8
         | ((uint32_t)(M >> 4) << 24); // M / 16
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))) (Hendrycks and Gimpel,
// "Gaussian Error Linear Units", 2016), with the tensor-core-era MUFU tanh (PTX tanh.approx.f32,
// relative error about 2^-11, far below the bf16 rounding of the stored activations), and its
// derivative 0.5 (1 + t) + 0.5 x (1 - t^2) sqrt(2/pi) (1 + 3 * 0.044715 x^2).
__device__ __forceinline__ float tanh_mufu(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kGeluC0 = 0.7978845608028654f;  // sqrt(2 / pi)
constexpr float kGeluC1 = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
  const float x2 = x * x;
  const float t = tanh_mufu(kGeluC0 * x * fmaf(kGeluC1, x2, 1.f));
  const float hx = 0.5f * x;
  return fmaf(hx, t, hx);
}
// Two fp32 lanes in one 64-bit register and Blackwell's packed add / mul / fma on them: each
// lane is an IEEE round-to-nearest fp32 operation, so a packed sequence gives exactly the
// scalar sequence's results with half the instructions.
__device__ __forceinline__ uint64_t pk2(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void up2(uint64_t r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
// gelu(a + ba), gelu(b + bb) by the same operations as gelu() on each lane
__device__ __forceinline__ void gelu2_bias(float a, float b, float ba, float bb, float& ya,
                                           float& yb) {
  const uint64_t x = add2(pk2(a, b), pk2(ba, bb));
  const uint64_t x2 = mul2(x, x);
  const uint64_t p = fma2(pk2(kGeluC1, kGeluC1), x2, pk2(1.f, 1.f));
  const uint64_t arg = mul2(mul2(pk2(kGeluC0, kGeluC0), x), p);
  float a0, a1;
  up2(arg, a0, a1);
  const uint64_t t = pk2(tanh_mufu(a0), tanh_mufu(a1));
  const uint64_t hx = mul2(pk2(0.5f, 0.5f), x);
  up2(fma2(hx, t, hx), ya, yb);
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float x2 = x * x;
  const float t = tanh_mufu(kGeluC0 * x * fmaf(kGeluC1, x2, 1.f));
  const float du = kGeluC0 * fmaf(3.f * kGeluC1, x2, 1.f);
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * du;
}

struct GemmArgs {
  int64_t M;
  int N, K, k_per_split, epi, splits;
  float* C;
  const float* bias;
  float* P;
  __nv_bfloat16* H;
  __nv_bfloat16* HT;
  int64_t ldht;
  unsigned int* err;
};

template <int BN, int STAGES>
struct GemmSmem {
  static constexpr uint32_t kA = BM * BK * 2;
  static constexpr uint32_t kB = BN * BK * 2;
  static constexpr uint32_t kStage = kA + kB;
  static constexpr uint32_t kBars = 1024;  // barriers + tensor-memory address, then 1 KB align
  static constexpr uint32_t kEpi = kEpiWarps * 32 * 33 * 4;  // per-warp 32 x 33 staging tiles
  static constexpr uint32_t kTotal = STAGES * kStage + kBars + kEpi + 1024;
};

__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_addr(b)) : "memory");
}

// One tile's epilogue for one warp: tensor-memory lanes 32*q .. +31 (tile rows), accumulator
// columns [c_lo, c_hi) of the tile.  A lane holds one row's 32 consecutive values per chunk, so
// row-major stores from registers would send the 32 lanes to 32 different rows.  The warp
// instead stages each 32 x 32 chunk in its shared-memory tile `st` (padded to 33 columns) and
// writes it back row by row, two rows per instruction (lanes 0-15 and 16-31, two values each):
// every store covers whole 64- or 128-byte row segments.  The transposed copy (HT) is already
// contiguous from registers (lane = row).
__device__ __forceinline__ void gemm_epilogue(const GemmArgs& g, uint32_t tacc, int q, int lane,
                                              int64_t m0, int n0, int split, int c_lo, int c_hi,
                                              float* st) {
  const int64_t row0 = m0 + q * 32;
  const int64_t row = row0 + lane;
  const bool in = row < g.M;
  const int half = lane >> 4, pair = lane & 15;  // write-back: row parity, column pair
  for (int c0 = c_lo; c0 < c_hi; c0 += 32) {
    float v[32];
    tmem_ld32(tacc + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
    const int col0 = n0 + c0;
    if (g.epi == DMSIM_EPI_STORE_F32) {
#pragma unroll
      for (int i = 0; i < 32; ++i) st[lane * 33 + i] = v[i];
      __syncwarp();
      for (int r = half; r < 32; r += 2) {
        if (row0 + r < g.M) {
          float* dst = g.C + ((size_t)split * g.M + row0 + r) * g.N + col0;
          *reinterpret_cast<float2*>(dst + 2 * pair) =
              make_float2(st[r * 33 + 2 * pair], st[r * 33 + 2 * pair + 1]);
        }
      }
      __syncwarp();
      continue;
    }
    if (g.epi == DMSIM_EPI_BIAS_GELU) {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] += __ldg(g.bias + col0 + i);
      if (g.P) {  // pre-activations for the backward pass, staged like the outputs
#pragma unroll
        for (int i = 0; i < 32; ++i) st[lane * 33 + i] = v[i];
        __syncwarp();
        for (int r = half; r < 32; r += 2) {
          if (row0 + r < g.M)
            *reinterpret_cast<float2*>(g.P + (size_t)(row0 + r) * g.N + col0 + 2 * pair) =
                make_float2(st[r * 33 + 2 * pair], st[r * 33 + 2 * pair + 1]);
        }
        __syncwarp();
      }
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = gelu(v[i]);
    } else {  // DMSIM_EPI_GELU_BWD: the pre-activations arrive through the same staging
      for (int r = half; r < 32; r += 2) {
        float2 p = make_float2(0.f, 0.f);
        if (row0 + r < g.M)
          p = *reinterpret_cast<const float2*>(g.P + (size_t)(row0 + r) * g.N + col0 + 2 * pair);
        st[r * 33 + 2 * pair] = p.x;
        st[r * 33 + 2 * pair + 1] = p.y;
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = in ? v[i] * gelu_grad(st[lane * 33 + i]) : 0.f;
      __syncwarp();
    }
    if (g.HT && in) {
#pragma unroll
      for (int i = 0; i < 32; ++i)
        g.HT[(size_t)(col0 + i) * g.ldht + row] = __float2bfloat16_rn(v[i]);
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) st[lane * 33 + i] = v[i];
    __syncwarp();
    for (int r = half; r < 32; r += 2) {
      if (row0 + r < g.M)
        *reinterpret_cast<__nv_bfloat162*>(g.H + (size_t)(row0 + r) * g.N + col0 + 2 * pair) =
            __floats2bfloat162_rn(st[r * 33 + 2 * pair], st[r * 33 + 2 * pair + 1]);
    }
    __syncwarp();
  }
}

// Persistent GEMM: each CTA walks the tiles blockIdx.x, +gridDim.x, ... (m fastest, then n, then
// the K split).  Two accumulators of BN columns in tensor memory let the epilogue of one tile run
// while the next tile's MMAs fill the other: the MMA issuer waits on acc_empty (released by the 8
// epilogue warps after their last tcgen05.ld of that accumulator), the epilogue waits on acc_full
// (committed after the tile's last MMA).
template <int BN, int STAGES>
__global__ void __launch_bounds__(kThreads, 1)
    k_gemm(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
           const GemmArgs g) {
  using L = GemmSmem<BN, STAGES>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * L::kStage);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;   // [2]
  uint64_t* acc_empty = acc_full + 2;    // [2]
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(acc_empty + 2);
  volatile uint32_t* abort_flag = tmem_slot + 1;
  volatile int* consumed = reinterpret_cast<volatile int*>(tmem_slot + 2);
  volatile int* committed = reinterpret_cast<volatile int*>(tmem_slot + 3);
  float* epi_tiles = reinterpret_cast<float*>(smem + STAGES * L::kStage + L::kBars);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_m = (int)((g.M + BM - 1) / BM), n_n = g.N / BN;
  const int n_tiles = n_m * n_n * g.splits;
  const int n_k = g.k_per_split / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      bar_init(&full[s], 1);
      bar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      bar_init(&acc_full[a], 1);
      bar_init(&acc_empty[a], kEpiWarps);
    }
    *abort_flag = 0;
    *consumed = 0;
    *committed = -1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     s_addr((const void*)tmem_slot)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int issued = 0;  // warp 0 lane 0: k-steps whose loads were issued
  if (warp == 0) {
    if (lane == 0) {
      int qk = 0;
      for (int tile = blockIdx.x; tile < n_tiles && !*abort_flag; tile += gridDim.x) {
        const int mt = tile % n_m, rest = tile / n_m;
        const int64_t m0 = (int64_t)mt * BM;
        const int n0 = (rest % n_n) * BN, kb = (rest / n_n) * g.k_per_split;
        for (int k = 0; k < n_k; ++k, ++qk) {
          const int s = qk % STAGES;
          if (!bar_wait(&empty[s], ((qk / STAGES) & 1) ^ 1)) {
            *abort_flag = 1;
            break;
          }
          uint8_t* sa = smem + s * L::kStage;
          bar_expect(&full[s], L::kStage);
          tma_load_2d(sa, &map_a, kb + k * BK, (int)m0, &full[s]);
          tma_load_2d(sa + L::kA, &map_b, kb + k * BK, n0, &full[s]);
          issued = qk + 1;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = instr_desc(BM, BN);
      int qk = 0, it = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x, ++it) {
        const int acc = it & 1;
        if (!bar_wait(&acc_empty[acc], ((it >> 1) & 1) ^ 1)) {
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t tacc = tmem + (uint32_t)(acc * BN);
        for (int k = 0; k < n_k; ++k, ++qk) {
          const int s = qk % STAGES;
          if (!bar_wait(&full[s], (qk / STAGES) & 1)) {
            *abort_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = s_addr(smem + s * L::kStage);
          const uint32_t b0 = a0 + L::kA;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16(tacc, smem_desc(a0 + kk * 32), smem_desc(b0 + kk * 32), idesc,
                     (k > 0 || kk > 0) ? 1u : 0u);
          tc_commit(&empty[s]);
          *consumed = qk + 1;
        }
        tc_commit(&acc_full[acc]);  // also after an abort: fires when the issued MMAs finish
        *committed = it;
      }
    }
  } else {
    // epilogue warps 2..9: lane quarter warp % 4, column half (warp - 2) / 4
    const int q = warp & 3, half = (warp - 2) >> 2;
    int it = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++it) {
      const int acc = it & 1;
      const bool ok = bar_wait(&acc_full[acc], (it >> 1) & 1);
      tc_fence_after();
      if (!ok || *abort_flag) {
        *abort_flag = 1;
        break;
      }
      const int mt = tile % n_m, rest = tile / n_m;
      gemm_epilogue(g, tmem + (uint32_t)(acc * BN), q, lane, (int64_t)mt * BM,
                    (rest % n_n) * BN, rest / n_n, half * (BN / 2), (half + 1) * (BN / 2),
                    epi_tiles + (warp - 2) * 32 * 33);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(&acc_empty[acc]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (*abort_flag) {
    // drain before leaving: the loads still in flight, then the last committed MMAs (bounded)
    if (threadIdx.x == 0) {
      atomicAdd(g.err, 1u);
      for (int k = *consumed; k < issued; ++k) bar_wait(&full[k % STAGES], (k / STAGES) & 1);
    }
    if (warp == 1 && lane == 0 && *committed >= 0) {
      const int it = *committed;
      bar_wait(&acc_full[it & 1], (it >> 1) & 1);
    }
    __syncthreads();
  }
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * BN)
                 : "memory");
  }
}

// ---- fused forward pass -------------------------------------------------------------------------
// The whole network on one 128-row tile of queries per step, on chip: the packed inputs and every
// hidden layer's activations live in shared memory in the K-major, 128-byte-swizzled layout the
// tensor core reads (the layout a TMA box of 64 bf16 columns writes: the 16-byte chunk c of row r
// of a 64-column K slice sits at r * 128 + ((c ^ (r & 7)) * 16), 8-row groups 1024 bytes apart),
// the accumulator of the current layer lives in tensor memory, and the weights stream from L2 by
// TMA in 16 KB slices (128 output rows x 64 K columns).  Only the fp32 inputs are read from and
// the fp32 outputs written to global memory.
//   warp 0      TMA producer of the weight slices (a ring of kFwdStages), in the order the
//               tensor core consumes them: per tile, per layer, per 64-wide K slice, both
//               128-row halves of the output;
//   warp 1      allocates 256 tensor-memory columns; one lane issues tcgen05.mma (M = 128,
//               N = 128, K = 16) into the two 128-column halves of the accumulator, commits each
//               weight slot back to the producer and each finished layer to the epilogue;
//   warps 2..9  pack each tile's inputs ((x - shift) * scale as bf16), and after each layer read
//               the accumulator (warp w owns tensor-memory lanes 32 (w % 4) .. + 31 = those tile
//               rows, and one 128-column half), add the bias, apply GELU and write the next
//               layer's operand back into shared memory; after the last layer they form the head
//               y = H w + b (bf16-rounded activations, fp32 sums) and store y.
// Two CTAs fit on an SM (about 103 KB of shared memory, 256 tensor-memory columns each), so one
// CTA's epilogue overlaps the other's tensor-core work.  Every wait is bounded.
constexpr int kFwdWidth = 256;
constexpr int kFwdKp = 128;
constexpr int kFwdMaxDepth = 8;
constexpr int kFwdStages = 2;
constexpr uint32_t kFwdSlice = 128 * BK * 2;       // 16 KB
constexpr uint32_t kFwdAct = BM * kFwdWidth * 2;   // 64 KB: 4 K slices of 16 KB
constexpr uint32_t kFwdBars = 256;  // mbarriers and flags, after the ring
// then the parameters the epilogue reads as broadcasts: shift and scale (kFwdKp each), the head
// weights (kFwdWidth) and each layer's bias (kFwdWidth)
__host__ __device__ constexpr uint32_t fwd_smem(int depth) {
  return kFwdAct + kFwdStages * kFwdSlice + kFwdBars + (2 * kFwdKp + kFwdWidth) * 4 +
         (uint32_t)depth * kFwdWidth * 4;
}
constexpr int kFwdEpiWarps = 8;
constexpr int kFwdThreads = 64 + 32 * kFwdEpiWarps;

struct FwdArgs {
  int64_t rows;
  int n_in, depth;
  const float* x;
  const float* shift;
  const float* scale;
  const float* bias[kFwdMaxDepth];
  const float* w_head;
  const float* b_head;
  float* y;
  unsigned int* err;
};
struct FwdMaps {
  CUtensorMap w[kFwdMaxDepth];
};

__device__ __forceinline__ uint32_t swz128(int r, int c16) {
  return (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u + (uint32_t)((c16 ^ (r & 7)) * 16);
}
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__global__ void __launch_bounds__(kFwdThreads, 2)
    k_mlp_forward(const __grid_constant__ FwdMaps maps, const __grid_constant__ FwdArgs g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* act = smem;
  uint8_t* ring = smem + kFwdAct;
  uint64_t* w_full = reinterpret_cast<uint64_t*>(ring + kFwdStages * kFwdSlice);
  uint64_t* w_empty = w_full + kFwdStages;
  uint64_t& acc_full = w_empty[kFwdStages];
  uint64_t& act_ready = w_empty[kFwdStages + 1];
  uint64_t& head_ready = w_empty[kFwdStages + 2];
  uint32_t* flags = reinterpret_cast<uint32_t*>(&w_empty[kFwdStages + 3]);
  uint32_t& tmem_slot = flags[0];
  uint32_t& abort_flag = flags[1];
  int& issued_s = reinterpret_cast<int&>(flags[2]);
  int& consumed_s = reinterpret_cast<int&>(flags[3]);
  int& committed_s = reinterpret_cast<int&>(flags[4]);
  // the second column half's head partials (K slice 3 of the operand is free from the last
  // layer's epilogue until the next tile's first epilogue)
  float* head_part = reinterpret_cast<float*>(act + 3 * (BM * BK * 2));
  float* s_shift = reinterpret_cast<float*>(ring + kFwdStages * kFwdSlice + kFwdBars);
  float* s_scale = s_shift + kFwdKp;
  float* s_whead = s_scale + kFwdKp;
  float* s_bias = s_whead + kFwdWidth;  // [depth][kFwdWidth]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n_tiles = (g.rows + BM - 1) / BM;

  if ((s_addr(smem) & 1023u) != 0u) {  // the swizzled layout needs 1024-byte alignment
    if (threadIdx.x == 0) atomicAdd(g.err, 1u);
    return;
  }
  for (int i = threadIdx.x; i < kFwdKp; i += blockDim.x) {
    s_shift[i] = (g.shift && i < g.n_in) ? __ldg(g.shift + i) : 0.f;
    s_scale[i] = (g.scale && i < g.n_in) ? __ldg(g.scale + i) : 1.f;
  }
  for (int i = threadIdx.x; i < kFwdWidth; i += blockDim.x) s_whead[i] = __ldg(g.w_head + i);
  for (int l = 0; l < g.depth; ++l)
    for (int i = threadIdx.x; i < kFwdWidth; i += blockDim.x)
      s_bias[l * kFwdWidth + i] = __ldg(g.bias[l] + i);
  if (threadIdx.x == 0) {
    for (int s = 0; s < kFwdStages; ++s) {
      bar_init(&w_full[s], 1);
      bar_init(&w_empty[s], 1);
    }
    bar_init(&acc_full, 1);
    bar_init(&act_ready, kFwdEpiWarps);
    bar_init(&head_ready, kFwdEpiWarps / 2);
    abort_flag = 0;
    issued_s = consumed_s = 0;
    committed_s = -1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     s_addr(&tmem_slot)),
                 "r"(kFwdWidth)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  volatile uint32_t* abort_v = &abort_flag;

  if (warp == 0) {
    if (lane == 0) {
      int q = 0;
      for (int64_t tile = blockIdx.x; tile < n_tiles && !*abort_v; tile += gridDim.x) {
        for (int l = 0; l < g.depth && !*abort_v; ++l) {
          const int nk = (l == 0 ? kFwdKp : kFwdWidth) / BK;
          for (int ks = 0; ks < nk; ++ks)
            for (int nh = 0; nh < 2; ++nh, ++q) {
              const int st = q % kFwdStages;
              if (!bar_wait(&w_empty[st], ((q / kFwdStages) & 1) ^ 1)) {
                *abort_v = 1;
                goto producer_done;
              }
              bar_expect(&w_full[st], kFwdSlice);
              tma_load_2d(ring + st * kFwdSlice, &maps.w[l], ks * BK, nh * 128, &w_full[st]);
              issued_s = q + 1;
            }
        }
      }
    producer_done:;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = instr_desc(BM, 128);
      int q = 0, layer_it = 0;
      for (int64_t tile = blockIdx.x; tile < n_tiles && !*abort_v; tile += gridDim.x) {
        for (int l = 0; l < g.depth; ++l, ++layer_it) {
          if (!bar_wait(&act_ready, layer_it & 1)) {
            *abort_v = 1;
            goto mma_done;
          }
          tc_fence_after();
          const int nk = (l == 0 ? kFwdKp : kFwdWidth) / BK;
          for (int ks = 0; ks < nk; ++ks)
            for (int nh = 0; nh < 2; ++nh, ++q) {
              const int st = q % kFwdStages;
              if (!bar_wait(&w_full[st], (q / kFwdStages) & 1)) {
                *abort_v = 1;
                tc_commit(&acc_full);
                committed_s = layer_it;
                goto mma_done;
              }
              tc_fence_after();
              const uint32_t a0 = s_addr(act + ks * (BM * BK * 2));
              const uint32_t b0 = s_addr(ring + st * kFwdSlice);
#pragma unroll
              for (int kk = 0; kk < BK / 16; ++kk)
                mma_bf16(tmem + (uint32_t)(nh * 128), smem_desc(a0 + kk * 32),
                         smem_desc(b0 + kk * 32), idesc, (ks > 0 || kk > 0) ? 1u : 0u);
              tc_commit(&w_empty[st]);
              consumed_s = q + 1;
            }
          tc_commit(&acc_full);
          committed_s = layer_it;
        }
      }
    mma_done:;
    }
  } else {
    // epilogue warps: tile rows 32 * (warp % 4) + lane, accumulator / operand columns
    // [128 * half, 128 * half + 128)
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    const int r = quarter * 32 + lane;
    const uint32_t t_row = tmem + ((uint32_t)(quarter * 32) << 16);
    int layer_it = 0, tile_it = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x, ++tile_it) {
      const int64_t row = tile * BM + r;
      // ---- pack the inputs: the two warps of each lane quarter take 16 of its 32 rows each;
      // lane l owns columns l, l + 32, l + 64, l + 96, so every load reads 32 consecutive floats
      // of one row and every store lands in one 128-byte row of the operand; columns from n_in
      // to 127 and rows past the end are written as zeros
      {
        const int64_t row_base = tile * BM + quarter * 32 + half * 16;
        float sh[4], sc[4];
#pragma unroll
        for (int gq = 0; gq < 4; ++gq) {
          const int c = 32 * gq + lane;
          sh[gq] = s_shift[c];
          sc[gq] = s_scale[c];
        }
#pragma unroll 1
        for (int r0 = 0; r0 < 16; r0 += 8) {
          float v[8][4];
#pragma unroll
          for (int rr = 0; rr < 8; ++rr) {
            const int64_t row = row_base + r0 + rr;
#pragma unroll
            for (int gq = 0; gq < 4; ++gq) {
              const int c = 32 * gq + lane;
              v[rr][gq] = (row < g.rows && c < g.n_in) ? __ldg(g.x + (size_t)row * g.n_in + c)
                                                        : 0.f;
            }
          }
#pragma unroll
          for (int rr = 0; rr < 8; ++rr) {
            const int64_t row = row_base + r0 + rr;
            const int rt = quarter * 32 + half * 16 + r0 + rr;
#pragma unroll
            for (int gq = 0; gq < 4; ++gq) {
              const int c = 32 * gq + lane;
              const float val = (row < g.rows && c < g.n_in) ? (v[rr][gq] - sh[gq]) * sc[gq] : 0.f;
              *reinterpret_cast<__nv_bfloat16*>(act + (c >> 6) * (BM * BK * 2) +
                                                swz128(rt, (c & 63) >> 3) + (c & 7) * 2) =
                  __float2bfloat16_rn(val);
            }
          }
        }
      }
      fence_async_shared();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(&act_ready);
      uint64_t head2 = pk2(0.f, 0.f);
      for (int l = 0; l < g.depth; ++l, ++layer_it) {
        if (!bar_wait(&acc_full, layer_it & 1) || *abort_v) {
          *abort_v = 1;
          ok = false;
          break;
        }
        tc_fence_after();
        const bool last = l == g.depth - 1;
        const float* bl = s_bias + l * kFwdWidth;
        if (last) {
          // this CTA's next tile's inputs (one contiguous block): into L2 while the head runs
          const int64_t nt = tile + gridDim.x;
          if (nt < n_tiles) {
            const int64_t e0 = nt * BM * g.n_in;
            const int64_t e1 = min((nt + 1) * BM, g.rows) * g.n_in;
            for (int64_t e = e0 + (int64_t)(threadIdx.x - 64) * 32; e < e1;
                 e += (int64_t)32 * kFwdEpiWarps * 32)
              asm volatile("prefetch.global.L2 [%0];" ::"l"(g.x + e));
          }
        }
        // two 32-column loads in flight per wait; the second chunk is processed from registers
        // while nothing is pending
        uint32_t u[2][32];
#pragma unroll 1
        for (int cc = half * 128; cc < half * 128 + 128; cc += 64) {
          tmem_ld32_nowait(t_row + (uint32_t)cc, u[0]);
          tmem_ld32_nowait(t_row + (uint32_t)(cc + 32), u[1]);
          tmem_wait_ld();
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
          const int c0 = cc + 32 * hh;
          float v[32];
#pragma unroll
          for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(u[hh][i]);
#pragma unroll
          for (int i = 0; i < 32; i += 4) {
            const float4 b4 = *reinterpret_cast<const float4*>(bl + c0 + i);
            gelu2_bias(v[i], v[i + 1], b4.x, b4.y, v[i], v[i + 1]);
            gelu2_bias(v[i + 2], v[i + 3], b4.z, b4.w, v[i + 2], v[i + 3]);
          }
          if (last) {
            // the head on the bf16 activations: even and odd columns in the two lanes
#pragma unroll
            for (int i = 0; i < 32; i += 4) {
              const float4 w4 = *reinterpret_cast<const float4*>(s_whead + c0 + i);
              const float2 a01 = __bfloat1622float2(__floats2bfloat162_rn(v[i], v[i + 1]));
              const float2 a23 = __bfloat1622float2(__floats2bfloat162_rn(v[i + 2], v[i + 3]));
              head2 = fma2(pk2(a01.x, a01.y), pk2(w4.x, w4.y), head2);
              head2 = fma2(pk2(a23.x, a23.y), pk2(w4.z, w4.w), head2);
            }
          } else {
            uint8_t* base = act + (c0 >> 6) * (BM * BK * 2);
            const int cs = (c0 & 63) >> 3;  // first 16-byte chunk of these 32 columns
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              uint32_t pk[4];
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const __nv_bfloat162 b = __floats2bfloat162_rn(v[8 * k + 2 * j], v[8 * k + 2 * j + 1]);
                pk[j] = *reinterpret_cast<const uint32_t*>(&b);
              }
              *reinterpret_cast<uint4*>(base + swz128(r, cs + k)) =
                  make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
          }
          }
        }
        if (!last) {
          // the next layer's operand is in place and this layer's accumulator is read out
          fence_async_shared();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) bar_arrive(&act_ready);
        }
      }
      if (!ok) break;
      float head0, head1;
      up2(head2, head0, head1);
      const float head = head0 + head1;
      // ---- head: the second half's partial sums reach the first half through shared memory
      if (half == 1) {
        head_part[r] = head;
        __syncwarp();
        if (lane == 0) bar_arrive(&head_ready);
      } else {
        if (!bar_wait(&head_ready, tile_it & 1)) {
          *abort_v = 1;
          break;
        }
        if (row < g.rows) g.y[row] = (head + head_part[r]) + __ldg(g.b_head);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (*abort_v) {
    // drain before leaving: the weight loads still in flight, then the last committed MMAs
    if (threadIdx.x == 0) {
      atomicAdd(g.err, 1u);
      for (int k = consumed_s; k < issued_s; ++k)
        bar_wait(&w_full[k % kFwdStages], (k / kFwdStages) & 1);
    }
    if (warp == 1 && lane == 0 && committed_s >= 0) bar_wait(&acc_full, committed_s & 1);
    __syncthreads();
  }
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kFwdWidth)
                 : "memory");
  }
}

// ---- small kernels ------------------------------------------------------------------------------
// Inputs (rows, F) fp32 -> (x - shift) * scale as bf16 (rows, Kp), zero padded; optional
// transpose (Kp, ldt).
__global__ void k_pack(const float* __restrict__ x, int64_t rows, int F, int Kp,
                       const float* __restrict__ shift, const float* __restrict__ scale,
                       __nv_bfloat16* __restrict__ out, __nv_bfloat16* __restrict__ outT,
                       int64_t ldt) {
  const int64_t n = rows * Kp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / Kp;
    const int c = (int)(i % Kp);
    float v = 0.f;
    if (c < F) v = (x[r * F + c] - (shift ? shift[c] : 0.f)) * (scale ? scale[c] : 1.f);
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    out[i] = b;
    if (outT) outT[(size_t)c * ldt + r] = b;
  }
}

// Linear head y = H w + b (one warp per row; fp32 accumulation in a fixed lane order).  With a
// target: dy = 2 (y - t) / rows, the row's squared error in sqerr, and the seed gradient of the
// last hidden layer dP = dy * w * gelu'(P) as bf16 (rows, N) and transposed (N, ldt).
__global__ void k_head(const __nv_bfloat16* __restrict__ H, int64_t rows, int N,
                       const float* __restrict__ w, const float* __restrict__ b,
                       float* __restrict__ y, const float* __restrict__ target,
                       float* __restrict__ dy, float* __restrict__ sqerr,
                       const float* __restrict__ P, __nv_bfloat16* __restrict__ dP,
                       __nv_bfloat16* __restrict__ dPT, int64_t ldt) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); r < rows;
       r += warps) {
    float acc = 0.f;
    for (int c = lane; c < N; c += 32) acc = fmaf(__bfloat162float(H[r * N + c]), w[c], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    const float yr = acc + b[0];
    if (lane == 0 && y) y[r] = yr;
    if (!target) continue;
    const float e = yr - target[r];
    const float g = 2.f * e / (float)rows;
    if (lane == 0) {
      if (dy) dy[r] = g;
      if (sqerr) sqerr[r] = e * e;
    }
    for (int c = lane; c < N; c += 32) {
      const __nv_bfloat16 v = __float2bfloat16_rn(g * w[c] * gelu_grad(P[r * N + c]));
      dP[r * N + c] = v;
      if (dPT) dPT[(size_t)c * ldt + r] = v;
    }
  }
}

// out[i] = sum_j X[i, j] * (v ? v[j] : 1) over a bf16 row-major (rows, cols) matrix: one block
// per row, fixed-order tree reduction.
__global__ void k_rowdot(const __nv_bfloat16* __restrict__ X, int64_t rows, int64_t cols,
                         int64_t ld, const float* __restrict__ v, float* __restrict__ out) {
  __shared__ float red[32];
  for (int64_t r = blockIdx.x; r < rows; r += gridDim.x) {
    float acc = 0.f;
    for (int64_t c = threadIdx.x; c < cols; c += blockDim.x)
      acc = fmaf(__bfloat162float(X[r * ld + c]), v ? v[c] : 1.f, acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
      float s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) out[r] = s;
    }
    __syncthreads();
  }
}

// AdamW on fp32 master weights; the gradient is the sum of `splits` partial buffers of n values.
// Refreshes the bf16 copies W (rows, cols) and, if given, WT (cols, rows).
// Hyper-parameters come from device memory hp = [lr, beta1, beta2, eps, weight_decay, step], so
// a captured training step needs no host update (k_adam_advance bumps the step).
__global__ void k_adamw(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                        const float* __restrict__ grad, int splits, int64_t n, int cols,
                        const float* __restrict__ hp, __nv_bfloat16* __restrict__ W,
                        __nv_bfloat16* __restrict__ WT, int rows) {
  const float lr = hp[0], b1 = hp[1], b2 = hp[2], eps = hp[3], wd = hp[4], step = hp[5];
  const float bc1 = 1.f - powf(b1, step), bc2 = 1.f - powf(b2, step);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float gsum = 0.f;
    for (int s = 0; s < splits; ++s) gsum += grad[(size_t)s * n + i];
    const float mi = b1 * m[i] + (1.f - b1) * gsum;
    const float vi = b2 * v[i] + (1.f - b2) * gsum * gsum;
    m[i] = mi;
    v[i] = vi;
    const float upd = (mi / bc1) / (sqrtf(vi / bc2) + eps);
    const float pi = p[i] * (1.f - lr * wd) - lr * upd;
    p[i] = pi;
    if (W) {
      const __nv_bfloat16 bv = __float2bfloat16_rn(pi);
      W[i] = bv;
      if (WT) {
        const int64_t r = i / cols, c = i % cols;
        WT[c * rows + r] = bv;
      }
    }
  }
}

__global__ void k_adam_advance(float* hp) { hp[5] += 1.f; }

// Fixed-order sum of n fp32 values (one block).
__global__ void k_sum(const float* __restrict__ x, int64_t n, float* __restrict__ out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += (double)x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = (float)s;
  }
}

// ---- host side ----------------------------------------------------------------------------------
thread_local char g_msg[256];

int err(int code, const char* what) {
  snprintf(g_msg, sizeof(g_msg), "%s", what);
  return dmsim::set_error(code, g_msg);
}

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                              const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                              const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

// 2-D bf16 tensor map over a row-major (rows, cols) matrix with row stride ld elements; box of
// 64 columns x box_rows rows, 128-byte swizzle, zero fill out of bounds.
bool make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld,
              int box_rows) {
  EncodeFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int STAGES>
int launch_gemm(const CUtensorMap& ma, const CUtensorMap& mb, const GemmArgs& a, int64_t M, int N,
                int splits, cudaStream_t st) {
  using L = GemmSmem<BN, STAGES>;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute((const void*)k_gemm<BN, STAGES>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kTotal) !=
        cudaSuccess)
      return err(DMSIM_ECUDA, "gemm: cudaFuncSetAttribute failed");
    attr = true;
  }
  static int n_sm = 0;
  if (n_sm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (n_sm < 1) n_sm = 1;
  }
  const int64_t tiles = ((M + BM - 1) / BM) * (N / BN) * splits;
  const int grid = (int)(tiles < n_sm ? tiles : n_sm);
  k_gemm<BN, STAGES><<<grid, kThreads, L::kTotal, st>>>(ma, mb, a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return err(DMSIM_ECUDA, cudaGetErrorString(e));
  return DMSIM_OK;
}

}  // namespace

extern "C" {

int dmsim_gemm_bf16(const dmsim_gemm* g, void* stream) {
  if (!g || !g->A || !g->B || !g->err) return err(DMSIM_EINVAL, "gemm: null argument");
  if (g->M < 1 || g->N < 128 || g->N % 128 || g->K < BK || g->K % BK)
    return err(DMSIM_EINVAL, "gemm: need M >= 1, N a multiple of 128, K a multiple of 64");
  if (g->lda < g->K || g->ldb < g->K || g->lda % 8 || g->ldb % 8)
    return err(DMSIM_EINVAL, "gemm: row strides must be >= K and multiples of 8 elements");
  if (((uintptr_t)g->A & 15) || ((uintptr_t)g->B & 15))
    return err(DMSIM_EINVAL, "gemm: A and B must be 16-byte aligned");
  const int splits = g->splits > 0 ? g->splits : 1;
  if ((g->K / BK) % splits) return err(DMSIM_EINVAL, "gemm: K / 64 must divide by splits");
  if (g->epilogue == DMSIM_EPI_STORE_F32) {
    if (!g->C) return err(DMSIM_EINVAL, "gemm: STORE_F32 needs C");
  } else if (g->epilogue == DMSIM_EPI_BIAS_GELU || g->epilogue == DMSIM_EPI_GELU_BWD) {
    if (splits != 1) return err(DMSIM_EINVAL, "gemm: only STORE_F32 splits K");
    if (!g->H || ((uintptr_t)g->H & 15)) return err(DMSIM_EINVAL, "gemm: H missing or unaligned");
    if (g->epilogue == DMSIM_EPI_BIAS_GELU && !g->bias) return err(DMSIM_EINVAL, "gemm: no bias");
    if (g->epilogue == DMSIM_EPI_GELU_BWD && !g->P) return err(DMSIM_EINVAL, "gemm: no P");
    if (g->HT && g->ldht < g->M) return err(DMSIM_EINVAL, "gemm: ldht < M");
  } else {
    return err(DMSIM_EINVAL, "gemm: unknown epilogue");
  }
  const int BN = (g->N % 256 == 0) ? 256 : 128;
  CUtensorMap ma, mb;
  if (!make_map(&ma, g->A, g->M, g->K, g->lda, BM) || !make_map(&mb, g->B, g->N, g->K, g->ldb, BN))
    return err(DMSIM_ECUDA, "gemm: tensor map encoding failed");
  GemmArgs a;
  a.M = g->M;
  a.N = g->N;
  a.K = g->K;
  a.k_per_split = g->K / splits;
  a.splits = splits;
  a.epi = g->epilogue;
  a.C = g->C;
  a.bias = g->bias;
  a.P = g->P;
  a.H = static_cast<__nv_bfloat16*>(g->H);
  a.HT = static_cast<__nv_bfloat16*>(g->HT);
  a.ldht = g->ldht;
  a.err = g->err;
  cudaStream_t st = (cudaStream_t)stream;
  return BN == 256 ? launch_gemm<256, 3>(ma, mb, a, g->M, g->N, splits, st)
                   : launch_gemm<128, 5>(ma, mb, a, g->M, g->N, splits, st);
}

int dmsim_mlp_forward(const dmsim_mlp_fwd* f, void* stream) {
  if (!f || !f->x || !f->y || !f->w_head || !f->b_head || !f->err || f->rows < 0)
    return err(DMSIM_EINVAL, "mlp_forward: null argument");
  if (f->depth < 1 || f->depth > kFwdMaxDepth || f->n_in < 1 || f->n_in > kFwdKp)
    return err(DMSIM_EINVAL, "mlp_forward: need 1 <= depth <= 8 and 1 <= n_in <= 128");
  if ((uintptr_t)f->w_head & 15) return err(DMSIM_EINVAL, "mlp_forward: w_head not 16-byte aligned");
  for (int l = 0; l < f->depth; ++l)
    if (!f->W[l] || !f->bias[l] || ((uintptr_t)f->W[l] & 15) || ((uintptr_t)f->bias[l] & 15))
      return err(DMSIM_EINVAL, "mlp_forward: missing or unaligned layer weights / bias");
  if (f->rows == 0) return DMSIM_OK;
  FwdMaps maps;
  memset(&maps, 0, sizeof(maps));
  for (int l = 0; l < f->depth; ++l) {
    const int K = l == 0 ? kFwdKp : kFwdWidth;
    if (!make_map(&maps.w[l], f->W[l], kFwdWidth, K, K, 128))
      return err(DMSIM_ECUDA, "mlp_forward: tensor map encoding failed");
  }
  FwdArgs a;
  memset(&a, 0, sizeof(a));
  a.rows = f->rows;
  a.n_in = f->n_in;
  a.depth = f->depth;
  a.x = f->x;
  a.shift = f->shift;
  a.scale = f->scale;
  for (int l = 0; l < f->depth; ++l) a.bias[l] = f->bias[l];
  a.w_head = f->w_head;
  a.b_head = f->b_head;
  a.y = f->y;
  a.err = f->err;
  const uint32_t smem = fwd_smem(f->depth);
  static bool attr = false;
  static int n_sm = 0;
  if (!attr) {
    if (cudaFuncSetAttribute((const void*)k_mlp_forward,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)fwd_smem(kFwdMaxDepth)) != cudaSuccess ||
        cudaFuncSetAttribute((const void*)k_mlp_forward,
                             cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess)
      return err(DMSIM_ECUDA, "mlp_forward: cudaFuncSetAttribute failed");
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (n_sm < 1) n_sm = 1;
    attr = true;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_mlp_forward,
                                                    kFwdThreads, smem) != cudaSuccess ||
      per_sm < 1)
    return err(DMSIM_ECUDA, "mlp_forward: the kernel does not fit on an SM");
  // the kernel is sized for two resident CTAs per SM (registers, shared and tensor memory); the
  // occupancy query may count one under the default shared-memory carveout
  const int64_t tiles = (f->rows + BM - 1) / BM;
  const int64_t slots = (int64_t)2 * n_sm;
  const int grid = (int)(tiles < slots ? tiles : slots);
  k_mlp_forward<<<grid, kFwdThreads, smem, (cudaStream_t)stream>>>(maps, a);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, cudaGetErrorString(e));
}

int dmsim_mlp_pack(const float* x, int64_t rows, int32_t features, int32_t kp, const float* shift,
                   const float* scale, void* out, void* out_t, int64_t ldt, void* stream) {
  if (!x || !out || rows < 0 || features < 1 || kp < features || (out_t && ldt < rows))
    return err(DMSIM_EINVAL, "mlp_pack: bad arguments");
  if (rows == 0) return DMSIM_OK;
  k_pack<<<1024, 256, 0, (cudaStream_t)stream>>>(x, rows, features, kp, shift, scale,
                                                  static_cast<__nv_bfloat16*>(out),
                                                  static_cast<__nv_bfloat16*>(out_t), ldt);
  return cudaGetLastError() == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, "mlp_pack launch");
}

int dmsim_mlp_head(const void* H, int64_t rows, int32_t n, const float* w, const float* b,
                   float* y, const float* target, float* dy, float* sqerr, const float* P,
                   void* dP, void* dP_t, int64_t ldt, void* stream) {
  if (!H || !w || !b || rows < 0 || n < 1 || (target && (!P || !dP)) || (dP_t && ldt < rows))
    return err(DMSIM_EINVAL, "mlp_head: bad arguments");
  if (rows == 0) return DMSIM_OK;
  int blocks = (int)((rows + 7) / 8);
  if (blocks > 4096) blocks = 4096;
  k_head<<<blocks, 256, 0, (cudaStream_t)stream>>>(
      static_cast<const __nv_bfloat16*>(H), rows, n, w, b, y, target, dy, sqerr, P,
      static_cast<__nv_bfloat16*>(dP), static_cast<__nv_bfloat16*>(dP_t), ldt);
  return cudaGetLastError() == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, "mlp_head launch");
}

int dmsim_rowdot_bf16(const void* X, int64_t rows, int64_t cols, int64_t ld, const float* v,
                      float* out, void* stream) {
  if (!X || !out || rows < 0 || cols < 0 || ld < cols)
    return err(DMSIM_EINVAL, "rowdot: bad arguments");
  if (rows == 0) return DMSIM_OK;
  const int blocks = (int)(rows < 65535 ? rows : 65535);
  k_rowdot<<<blocks, 256, 0, (cudaStream_t)stream>>>(static_cast<const __nv_bfloat16*>(X), rows,
                                                      cols, ld, v, out);
  return cudaGetLastError() == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, "rowdot launch");
}

int dmsim_adamw(float* p, float* m, float* v, const float* grad, int32_t splits, int64_t n,
                int32_t cols, const float* hp, void* W, void* WT, int32_t rows, void* stream) {
  if (!p || !m || !v || !grad || !hp || n < 0 || splits < 1 || cols < 1 ||
      (W && (int64_t)rows * cols != n))
    return err(DMSIM_EINVAL, "adamw: bad arguments");
  if (n == 0) return DMSIM_OK;
  k_adamw<<<512, 256, 0, (cudaStream_t)stream>>>(p, m, v, grad, splits, n, cols, hp,
                                                  static_cast<__nv_bfloat16*>(W),
                                                  static_cast<__nv_bfloat16*>(WT), rows);
  return cudaGetLastError() == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, "adamw launch");
}

int dmsim_adam_advance(float* hp, void* stream) {
  if (!hp) return err(DMSIM_EINVAL, "adam_advance: null");
  k_adam_advance<<<1, 1, 0, (cudaStream_t)stream>>>(hp);
  return cudaGetLastError() == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, "adam_advance launch");
}

int dmsim_sum_f32(const float* x, int64_t n, float* out, void* stream) {
  if (!x || !out || n < 0) return err(DMSIM_EINVAL, "sum_f32: bad arguments");
  k_sum<<<1, 1024, 0, (cudaStream_t)stream>>>(x, n, out);
  return cudaGetLastError() == cudaSuccess ? DMSIM_OK : err(DMSIM_ECUDA, "sum_f32 launch");
}

}  // extern "C"
