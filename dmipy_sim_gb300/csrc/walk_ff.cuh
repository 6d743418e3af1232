// The free-flight packed-cylinder walk kernel.
//
// The same walk as k_pcyl_wide / k_walk<DMSIM_GEOM_PACKED_CYLINDERS> (dmipy-sim's PackedCylinders,
// geometries.py:1604-2242, through make_step_fn's reflect / surface-relaxivity / permeable
// branches, physics.py:276-415, and the producer walk of simulate_trajectories,
// core.py:1137-1155), walker for walker and bit for bit, in the basis phase form.  What changes is
// the work schedule:
//
// Free flight.  A wall scan of sub-step k (packed_cyl_step: cell lookup, every candidate's root
// and end-point containment) that meets no wall also yields a wall-free disc around the step's
// end point, where the walker now is: its radius is the end point's distance to the nearest wall
// of the start cell's candidates, bounded by the start point's distance to the cell's edge plus
// the reach the cell list was built for, less the step (an object that is not listed lies
// farther than the reach from every point of the cell), less a tolerance of 16 nudges that covers
// the FP32 rounding of the roots.  While the walker's displacement since that scan stays inside
// the disc, every step starts and ends inside it, so no step can meet a wall: a scan would find
// no root and no contained end point, and packed_cyl_step would return x + step, which is what
// the free step computes.  So walks are bit-identical with the scan on every sub-step.  Among
// the extra-axonal gaps of a dense packing about 70 % of sub-steps are free.
//
// Measured on GB300 (dense lattice, f = 0.6): about 57 % of sub-steps fly free, but the lanes'
// independence costs more than the skipped scans save -- 49 % of lanes active per instruction and
// 14.5 warp instructions per walker-step against the lock-step kernel's 11.4 -- so the lock-step
// kernel stays the default and this schedule is opt-in (DMSIM_SCHED_FREE_FLIGHT).
//
// Independent lanes.  A free step is cheap but a scan is not, and in lock-step SIMT a warp pays
// for the scan whenever any of its 32 walkers needs one (nearly always).  Here each lane walks its
// own walker at its own pace through a small state machine -- free stepping, waiting for a scan,
// waiting for a wall hit's resolution, waiting for the sample's phase update -- and every
// iteration the warp votes: free steps run for every free lane, while scans, hit resolutions and
// sample updates run only once enough lanes wait for them (or nothing else can run).  The rare,
// long hit path (reflection, FP64 grazing re-solve, fold-first clamp) then runs for several lanes
// at once instead of for one lane at a time.
//
// Per-lane time: each lane reads its own sample's waveform row (global, cached) and accumulates
// its own Kahan phase moments (shared memory, thread-strided).  At an echo sample the warp adds
// that walker's w cos(phi_m), w sin(phi_m), (w cos(phi_m))^2 for all measurements, lane m taking
// measurement m, in FP64 into the warp's own partial slice; slices are summed in a fixed order by
// k_reduce.  Walkers are assigned to lanes statically (lane l of the grid walks walkers
// l, l + lanes, ...), so results do not depend on scheduling.
#pragma once
#include "walk_kernel.cuh"

namespace dmsim {

enum : int { kFfFree = 0, kFfScan = 1, kFfHit = 2, kFfSample = 3, kFfDone = 4 };

// Shared-memory layout: [mbarrier, abort flag, 5 anomaly tallies: 64 B] [basis coefficients (M x 3 x RT)]
// [phase moments and compensations (6 RT x NT floats)] [cell list].
struct FfLayout {
  size_t off_cs, off_acc, off_tab, total;
};
__host__ __device__ inline FfLayout ff_layout(int nt, int rt, int M, size_t tab_bytes) {
  FfLayout L;
  L.off_cs = 64;
  L.off_acc = L.off_cs + pad16z((size_t)M * 3 * rt * 4);
  L.off_tab = L.off_acc + (size_t)6 * rt * nt * 4;
  L.total = L.off_tab + pad16z(tab_bytes);
  return L;
}

// Tolerance of the wall-free disc, in nudges (1e-4 R_min): the FP32 roots and containment tests
// of a scan err by ~1e-7 of the coordinates, some 1e3 times less.
constexpr float kFfTolNudges = 16.f;

template <int WALL, int RT, bool PSUB, int NT>
__global__ void __launch_bounds__(NT, 1) k_pcyl_ff(const __grid_constant__ KArgs a) {
  extern __shared__ __align__(128) uint8_t smem[];
  constexpr int NACC = 3 * RT;
  constexpr int NW = NT / 32;
  constexpr unsigned FULL = 0xffffffffu;
  const FfLayout lay = ff_layout(NT, RT, a.M, (size_t)a.tab_cs_bytes + a.tab_cand_bytes);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  volatile int* s_abort = reinterpret_cast<volatile int*>(smem + 32);
  // block tallies of rare events (kept out of the lanes' registers)
  uint32_t* s_tally = reinterpret_cast<uint32_t*>(smem + 36);  // nonfinite, clamp, initfail,
                                                               // graze, transmit
  float* Cs = reinterpret_cast<float*>(smem + lay.off_cs);
  float* acc_base = reinterpret_cast<float*>(smem + lay.off_acc);
  float* accs = acc_base + threadIdx.x;  // [i * NT]: moments, then compensations
  float* kcs = accs + (size_t)NACC * NT;
  const uint32_t* cs = reinterpret_cast<const uint32_t*>(smem + lay.off_tab);
  const float4* cand = reinterpret_cast<const float4*>(smem + lay.off_tab + a.tab_cs_bytes);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const GeoK g = a.g;
  const size_t slice = (size_t)a.n_echo * a.Mp * 3;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    *s_abort = 0;
    for (int k = 0; k < 5; ++k) s_tally[k] = 0u;
    fence_async_smem();
  }
  {
    double* part = a.part + ((size_t)blockIdx.x * NW + warp) * slice;
    for (size_t j = lane; j < slice; j += 32) part[j] = 0.0;
  }
  for (int j = tid; j < a.M * 3 * RT; j += NT) Cs[j] = a.Cp[j];
  __syncthreads();
  if (tid == 0) {
    fence_async_smem();
    mbar_expect(&bar[0], a.tab_cs_bytes + a.tab_cand_bytes);
    bulk_g2s(smem + lay.off_tab, a.cs, a.tab_cs_bytes, &bar[0]);
    if (a.tab_cand_bytes)
      bulk_g2s(smem + lay.off_tab + a.tab_cs_bytes, a.cand, a.tab_cand_bytes, &bar[0]);
  }
  if (!mbar_wait(&bar[0], 0u)) *s_abort = 1;
  __syncthreads();
  if (*s_abort) {
    if (tid == 0) atomicAdd(&a.status[DMSIM_STATUS_WAIT_TIMEOUT], 1u);
    return;
  }

  const bool weighted = a.has_weight != 0;
  const float tol = kFfTolNudges * g.nudge;
  const int qb = a.ff_quorum[0], qh = a.ff_quorum[1], qc = a.ff_quorum[2];

  Tally tl;  // counted into s_tally as the events happen (pcyl_* take a Tally)
  // ---- lane state ---------------------------------------------------------------------------
  int64_t w = (int64_t)blockIdx.x * NT + tid;  // this lane's walker (static assignment)
  int mode = kFfDone;
  float x = 0.f, y = 0.f, z = 0.f, logw = 0.f;
  int ix = 0, iy = 0;
  uint32_t s = 0;   // sub-step counter of the walker (Philox call index)
  int t = 0, e = 0;  // sample, next echo
  u32x4 rr{0, 0, 0, 0};
  float adx = 0.f, ady = 0.f, br2 = -1.f;  // displacement since the last scan; disc radius^2
  float sx = 0.f, sy = 0.f, sz = 0.f;      // the step a scan / hit waits on
  float tb = INFINITY, dh = 0.f;           // its nearest root and discriminant
  int kw = 0;  // winning candidate (bits 0-27, -1 none) | hit_in << 28 | end_in << 29
  float rc = 0.f, dec = 0.f;               // this sample's weight rates
  float Rx = 0.f, Ry = 0.f, Rz = 0.f;      // fused form: the sample's summed positions

  auto sample_rates = [&]() {
    if (weighted) {
      const float chi = a.chi ? __ldg(a.chi + t) : 1.f;
      rc = a.rho * chi;
      dec = a.t2dec * chi + a.t1dec * (1.f - chi);
    }
  };
  // Start walker w (geometries.py:1717-1744: uniform outside every cylinder), or retire the lane.
  auto begin = [&]() {
    if (w >= a.n_walkers) {
      mode = kFfDone;
      return;
    }
    const uint64_t gw = (uint64_t)(a.walker_offset + w);
    x = y = z = 0.f;
    ix = iy = 0;
    if (a.r0 != nullptr) {
      x = a.r0[3 * w];
      y = a.r0[3 * w + 1];
      z = a.r0[3 * w + 2];
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
      if (!ok) atomicAdd(&s_tally[2], 1u);
    }
    if (a.comp0 != nullptr && a.pass == 0)
      a.comp0[w] = classify<DMSIM_GEOM_PACKED_CYLINDERS>(x, y, z, g, cs, cand, a.cand_obj);
#pragma unroll
    for (int i = 0; i < NACC; ++i) accs[i * NT] = kcs[i * NT] = 0.f;
    logw = 0.f;
    s = 0;
    t = 0;
    e = 0;
    adx = ady = 0.f;
    br2 = -1.f;
    Rx = Ry = Rz = 0.f;
    mode = kFfFree;
    sample_rates();
  };
  // The walker's outputs once its last sample is done.
  auto finish = [&]() {
    const float ux = x + g.L * (float)ix, uy = y + g.L * (float)iy, uz = z;
    if (!(isfinite(ux) && isfinite(uy) && isfinite(uz))) atomicAdd(&s_tally[0], 1u);
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
  };
  // A completed sub-step: z, the weight, the fused form's position sum, the counters.  The
  // position adds are written as __fadd_rn, which the compiler never fuses with the step's own
  // product: a free step and a scanned one then round alike (an FMA would not).
  auto advance = [&](float dl) {
    z = __fadd_rn(z, sz);
    if (weighted) logw += rc * dl - dec;
    if constexpr (PSUB) {
      Rx += __fmaf_rn(g.L, (float)ix, x);
      Ry += __fmaf_rn(g.L, (float)iy, y);
      Rz += z;
    }
    ++s;
    mode = s == (uint32_t)(t + 1) * (uint32_t)a.S ? kFfSample : kFfFree;
  };
  // One free-flight attempt of sub-step s from the uniforms (ua, ub): the isotropic direction
  // cos(theta) = 1 - 2 ua, azimuth pi (2 ub - 1), as in every walk kernel.
  auto attempt = [&](float ua, float ub) {
    const float cz = 1.f - 2.f * ua;
    const float st = sqrtf(fmaxf(0.f, 1.f - cz * cz));
    float sn, cs_;
    __sincosf(3.14159265358979f * (2.f * ub - 1.f), &sn, &cs_);
    sx = a.step_l * st * cs_;
    sy = a.step_l * st * sn;
    sz = a.step_l * cz;
    const float nx = adx + sx, ny = ady + sy;
    if (nx * nx + ny * ny < br2) {
      // inside the wall-free disc: packed_cyl_step's no-wall outcome
      x = __fadd_rn(x, sx);
      y = __fadd_rn(y, sy);
      fold(x, ix, g);
      fold(y, iy, g);
      adx = nx;
      ady = ny;
      advance(0.f);
    } else {
      mode = kFfScan;
    }
  };

  begin();

  for (;;) {
    const unsigned live = __ballot_sync(FULL, mode != kFfDone);
    if (live == 0u) break;

    // ---- free steps: up to two per lane (the two halves of one Philox draw) -------------------
    if (mode == kFfFree) {
      const uint64_t gw = (uint64_t)(a.walker_offset + w);
      if constexpr (WALL == kPermeate) {
        rr = draw(a.seed, gw, 0u, s);
        attempt(u01(rr.x), u01(rr.y));
        if (mode == kFfFree) {
          rr = draw(a.seed, gw, 0u, s);
          attempt(u01(rr.x), u01(rr.y));
        }
      } else {
        if ((s & 1u) == 0u) {
          rr = draw(a.seed, gw, 0u, s >> 1);
          attempt(u01(rr.x), u01(rr.y));
        } else {
          attempt(u01(rr.z), u01(rr.w));
        }
        if (mode == kFfFree && (s & 1u)) attempt(u01(rr.z), u01(rr.w));
      }
    }

    // ---- wall scans ------------------------------------------------------------------------
    {
      const unsigned m_scan = __ballot_sync(FULL, mode == kFfScan);
      const unsigned m_free = __ballot_sync(FULL, mode == kFfFree);
      if (m_scan != 0u && (__popc(m_scan) >= qb || m_free == 0u)) {
        if (mode == kFfScan) {
          float lxy, dx, dy;
          pcyl_dir(sx, sy, lxy, dx, dy);
          const int cxi = cell_of(x, g), cyi = cell_of(y, g);
          const int c = cyi * g.n + cxi;
          const uint32_t kb = cs[c], ke = cs[c + 1];
          float tbest = INFINITY, disc_hit = 0.f, dmin = INFINITY;
          int kwin = -1;
          bool hit_in = false, end_in = false, inside = false;
          const float ex = __fadd_rn(x, sx), ey = __fadd_rn(y, sy);
          auto visit = [&](const float4 C, int k) {
            const PcylRoot r = pcyl_test<WALL>(C, x, y, ex, ey, dx, dy, lxy, g);
            end_in |= r.end_in;
            if (r.valid && r.t < tbest) {
              tbest = r.t;
              disc_hit = r.disc;
              kwin = k;
              hit_in = r.ins;
            }
            // the end point's distance to this candidate's wall
            const float fx = ex - C.x, fy = ey - C.y;
            const float f2 = fx * fx + fy * fy;
            inside |= f2 < C.w * C.w;
            dmin = fminf(dmin, fabsf(sqrtf(f2) - C.w));
          };
          if (g.kmax == 2) {
#pragma unroll
            for (uint32_t j = 0; j < 2u; ++j)
              visit(kb + j < ke ? cand[kb + j] : make_float4(kFarAway, kFarAway, kFarAway, 0.f),
                    (int)(kb + j));
          } else {
#pragma unroll 1
            for (uint32_t k = kb; k < ke; ++k) visit(cand[k], (int)k);
          }
          if (tbest == INFINITY && !end_in) {
            // no wall within the step: the disc about its end point
            const float xlo = -g.halfL + (float)cxi * g.h, ylo = -g.halfL + (float)cyi * g.h;
            const float dbox = fminf(fminf(x - xlo, xlo + g.h - x), fminf(y - ylo, ylo + g.h - y));
            const float rs = fminf(dmin, dbox + g.reach - lxy) - tol;
            // a reflecting walker that ends inside an object (a clamp case) never flies free
            br2 = (a.ff_skip && rs > 0.f && (WALL == kPermeate || !inside)) ? rs * rs : -1.f;
            adx = 0.f;
            ady = 0.f;
            x = ex;
            y = ey;
            fold(x, ix, g);
            fold(y, iy, g);
            advance(0.f);
          } else {
            tb = tbest;
            dh = disc_hit;
            kw = (kwin & 0x0fffffff) | (hit_in ? 1 << 28 : 0) | (end_in ? 1 << 29 : 0);
            if (kwin < 0) kw |= 0x0fffffff;
            br2 = -1.f;
            mode = kFfHit;
          }
        }
      }
    }

    // ---- wall hits: graze re-solve, the wall's action, the clamp, the fold -----------------
    {
      const unsigned m_hit = __ballot_sync(FULL, mode == kFfHit);
      const unsigned m_run = __ballot_sync(FULL, mode == kFfFree || mode == kFfScan);
      if (m_hit != 0u && (__popc(m_hit) >= qh || m_run == 0u)) {
        if (mode == kFfHit) {
          float lxy, dx, dy;
          pcyl_dir(sx, sy, lxy, dx, dy);
          const int c = cell_of(y, g) * g.n + cell_of(x, g);
          const uint32_t kb = cs[c], ke = cs[c + 1];
          float tbest = tb, disc_hit = dh, hcx = 0.f, hcy = 0.f, hR = 1.f;
          const bool hit_in = (kw >> 28) & 1, end_in = (kw >> 29) & 1;
          const int kwin = kw & 0x0fffffff;
          if (kwin != 0x0fffffff) {
            const float4 C = cand[kwin];
            hcx = C.x;
            hcy = C.y;
            hR = C.w;
          }
          if (tbest < INFINITY && disc_hit < kGrazeTol * hR * hR)
            pcyl_graze(x, y, dx, dy, lxy, hcx, hcy, hR, hit_in, g, tbest, disc_hit, tl);
          const float u = WALL == kPermeate ? u01(rr.z) : 0.f;
          float nxp = __fadd_rn(x, sx), nyp = __fadd_rn(y, sy), dlog = 0.f;
          if (tbest < INFINITY)
            pcyl_hit<WALL>(x, y, sx, sy, dx, dy, lxy, u, tbest, disc_hit, hcx, hcy, hR, hit_in, g,
                           tl, nxp, nyp, dlog);
          if constexpr (WALL != kPermeate)
            if (tbest < INFINITY || end_in) pcyl_clamp(nxp, nyp, kb, ke, g, cand, tl);
          x = nxp;
          y = nyp;
          fold(x, ix, g);
          fold(y, iy, g);
          advance(dlog);
          if (tl.clamp) atomicAdd(&s_tally[1], tl.clamp);
          if (tl.graze) atomicAdd(&s_tally[3], tl.graze);
          if (tl.transmit) atomicAdd(&s_tally[4], tl.transmit);
          tl = Tally();
        }
      }
    }

    // ---- sample ends: phase moments, echo emission, the next sample or walker --------------
    {
      const unsigned m_smp = __ballot_sync(FULL, mode == kFfSample);
      const unsigned m_run = __ballot_sync(FULL, mode == kFfFree || mode == kFfScan || mode == kFfHit);
      if (m_smp != 0u && (__popc(m_smp) >= qc || m_run == 0u)) {
        bool emit = false;
        float wgt = 0.f;
        if (mode == kFfSample) {
          float Qx, Qy, Qz;
          if constexpr (PSUB) {
            Qx = Rx;
            Qy = Ry;
            Qz = Rz;
          } else {
            Qx = x + g.L * (float)ix;
            Qy = y + g.L * (float)iy;
            Qz = z;
          }
          // Kahan-compensated Q[j][k] += V_j(t) R_k (the same operations as the other kernels)
          if (__ldg(a.active + t)) {
            const float px = a.gamma_dt * Qx, py = a.gamma_dt * Qy, pz = a.gamma_dt * Qz;
            const float* gt = a.Gp + (size_t)t * RT;
#pragma unroll
            for (int j = 0; j < RT; ++j) {
              const float v = __ldg(gt + j);
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
          emit = e < a.n_echo && t == a.echo[e];
          wgt = weighted ? expf(logw) : 1.f;
        }
        __syncwarp();
        unsigned m_emit = __ballot_sync(FULL, emit);
        while (m_emit) {
          const int src = __ffs(m_emit) - 1;
          m_emit &= m_emit - 1u;
          const float ws = __shfl_sync(FULL, wgt, src);
          const int es = __shfl_sync(FULL, e, src);
          const float* qs = acc_base + (warp * 32 + src);
          float qv[NACC];
#pragma unroll
          for (int i = 0; i < NACC; ++i) qv[i] = qs[i * NT];
          for (int m = lane; m < a.M; m += 32) {
            const float* cc = Cs + (size_t)m * 3 * RT;
            float ph = 0.f;
#pragma unroll
            for (int j = 0; j < RT; ++j)
#pragma unroll
              for (int k = 0; k < 3; ++k) ph = fmaf(cc[k * RT + j], qv[3 * j + k], ph);
            float sn, cs_;
            sincosf(ph, &sn, &cs_);
            double* pp = a.part + ((size_t)blockIdx.x * NW + warp) * slice +
                         ((size_t)es * a.Mp + m) * 3;
            const float wc = ws * cs_;
            pp[0] += (double)wc;
            pp[1] += (double)(ws * sn);
            pp[2] += (double)(wc * wc);
          }
        }
        if (mode == kFfSample) {
          if (emit) ++e;
          ++t;
          if constexpr (PSUB) Rx = Ry = Rz = 0.f;
          if (t == a.n_t) {
            finish();
            w += (int64_t)gridDim.x * NT;
            begin();
          } else {
            mode = kFfFree;
            sample_rates();
          }
        }
      }
    }
  }

  // ---- anomaly tallies --------------------------------------------------------------------------
  __syncthreads();
  if (tid == 0 && a.pass == 0) {
    const int words[5] = {DMSIM_STATUS_NONFINITE, DMSIM_STATUS_CLAMPED, DMSIM_STATUS_INIT_FAIL,
                          DMSIM_STATUS_GRAZE_FP64, DMSIM_STATUS_TRANSMIT};
    for (int k = 0; k < 5; ++k)
      if (s_tally[k]) atomicAdd(&a.status[words[k]], s_tally[k]);
  }
}

using FfFn = void (*)(KArgs);

}  // namespace dmsim
