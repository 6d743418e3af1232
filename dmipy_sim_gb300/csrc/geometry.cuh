// Device-side geometry step functions of the walk.
//
// Each function advances one walker by one physics sub-step against one geometry and returns the
// unit boundary log-weight (-2 * sum of perpendicular overshoots d_perp, i.e. the reference's
// dlog_w at rho/D = 1; the kernel scales it by rho/D and by the transverse mask).  The arithmetic
// follows the reference's per-walker JAX functions statement by statement (same epsilons, nudges,
// clamps, root choices and argmin rules) so that the walk is the same random process:
//   Cylinder.reflect / reflect_with_log_weight / permeate   geometries.py:493-563, 565-653, 655-801
//   Sphere.reflect / reflect_with_log_weight / permeate     geometries.py:197-264, 266-318, 320-424
//   PackedCylinders.reflect / reflect_with_log_weight / permeate   geometries.py:1746-1884,
//                                                           1886-2016, 2018-2183
//   PackedSpheres.reflect / reflect_with_log_weight / permeate     geometries.py:2445-2537,
//                                                           2539-2631, 2633-2756
// What differs is the data layout, not the process:
//   * Cylinders walk in their own frame (axis = z): an isotropic step is isotropic in any frame, so
//     the per-step frame rotation of the reference (geometries.py:510-515) is folded into the
//     gradient once on the host.
//   * Packed substrates keep the position folded into the periodic cell plus integer image
//     counters (the reference keeps an unfolded FP32 position and min-images every object,
//     geometries.py:1782-1783).  The unfolded position for the phase is x + L*image.
//   * Packed substrates test only the objects listed for the walker's cell of a uniform cell list
//     (every object within reach of the cell), instead of all K objects; a candidate counts only if
//     it is the minimum image of its object, which is exactly the reference's min-image rule.
//   * A wall root whose discriminant is within 1e-4*R^2 of grazing is re-solved in FP64.
#pragma once
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "dmsim.h"

namespace dmsim {

enum { kReflect = DMSIM_WALL_REFLECT, kRelax = DMSIM_WALL_RELAX, kPermeate = DMSIM_WALL_PERMEATE };

constexpr float kGrazeTol = 1e-4f;
// Centre of the zero-radius dummy object that pads a cell's candidate slots (its squared
// distances stay finite in FP32 and no wall test can select it).
constexpr float kFarAway = 1e18f;

struct Tally {
  uint32_t clamp = 0, graze = 0, transmit = 0;
};

// Geometry constants in registers/param space (a trimmed copy of dmsim_geometry).
struct GeoK {
  float R, R2, invR, eps, nudge, kod;  // single objects: R; packed: eps/nudge from R_min
  float L, halfL, inv_h;
  int n;   // cells per axis
  int mi;  // 1 when some cell lists two images of one object: candidates need the min-image test
  int kmax;  // most candidates any cell lists (0: unknown); 2 selects the two-slot scan
  float r_out;  // shell: the reflecting outer wall
  int cyl;      // shell: radii from the z axis (1) or the origin (0)
  float e2[3];  // ellipsoid: 1 / semi-axis^2
  float h, reach;  // packed: cell side; the reach (step + margin) the cell lists cover
};

// Myelinated cylinder: two concentric walls (axis z) around three compartments.
struct MyelinK {
  float r_in, r_out, nudge;
  float sl[3];     // step length of each compartment
  float kin[3];    // kappa_inner / max(D_c, 1e-30) of the compartment left
  float kout[3];   // kappa_outer / max(D_c, 1e-30)
  float t2dec[3];  // dt / T2_c
  float lw0[3];    // log water proton density of each compartment
  long long n0, n1;  // seeding ranges of the global walker index (intra, myelin, extra)
};

// One step of make_myelin_step_fn (physics.py:506-677): the walker moves by its compartment's
// step along the unit direction (ux, uy, uz); a crossing of the inner (intra <-> myelin) or outer
// (myelin <-> extra) wall -- decided on the end point's radius, at most one per step -- transmits
// with the Powles probability min(1, 2 kappa/D_left |r - R|) on its own uniform (u1 inner, u2
// outer), else the end point is mirrored across the wall; then the walker is clamped onto its
// compartment's side of each wall (1e-4 R_in inside).  Returns the per-compartment T2 decrement
// (-dt/T2 of the new compartment), which the kernel gates by the coherence flag.
template <int WALL>
__device__ __forceinline__ float myelin_step(float& x, float& y, float& z, int& comp, float ux,
                                             float uy, float uz, float u1, float u2,
                                             const MyelinK& m, Tally& tl) {
  const float sl = comp == 0 ? m.sl[0] : (comp == 1 ? m.sl[1] : m.sl[2]);
  float nx = x + ux * sl, ny = y + uy * sl;
  const float nz = z + uz * sl;
  const float rn = sqrtf(nx * nx + ny * ny);
  const bool cio = comp == 0 && rn >= m.r_in, cii = comp == 1 && rn < m.r_in;
  const bool coo = comp == 1 && rn >= m.r_out, coi = comp == 2 && rn < m.r_out;
  const bool ci = cio || cii, co = coo || coi;
  bool ti = false, to = false;
  if constexpr (WALL == kPermeate) {
    const float kin = comp == 0 ? m.kin[0] : (comp == 1 ? m.kin[1] : m.kin[2]);
    const float kout = comp == 0 ? m.kout[0] : (comp == 1 ? m.kout[1] : m.kout[2]);
    const float p_in = fminf(1.f, 2.f * kin * fabsf(rn - m.r_in));
    const float p_out = fminf(1.f, 2.f * kout * fabsf(rn - m.r_out));
    ti = ci && (u1 < p_in);
    to = co && (u2 < p_out);
  }
  int nc = comp;
  if (ci && !ti) {  // mirror across the inner wall
    const float s = (2.f * m.r_in - rn) / fmaxf(rn, 1e-20f);
    nx *= s;
    ny *= s;
  }
  if (ti) nc = cio ? 1 : 0;
  if (co && !to) {  // mirror across the outer wall
    const float r2 = sqrtf(nx * nx + ny * ny);
    const float s = (2.f * m.r_out - r2) / fmaxf(r2, 1e-20f);
    nx *= s;
    ny *= s;
  }
  if (to) nc = coo ? 2 : 1;
  // safety clamps onto the compartment's side of each wall (physics.py:633-664)
  float rc = sqrtf(nx * nx + ny * ny);
  auto put = [&](float target) {
    const float s = target / fmaxf(rc, 1e-20f);
    nx *= s;
    ny *= s;
    rc = sqrtf(nx * nx + ny * ny);
    ++tl.clamp;
  };
  if (nc == 0 && rc >= m.r_in) put(m.r_in - m.nudge);
  if (nc == 1 && rc < m.r_in) put(m.r_in + m.nudge);
  if (nc == 1 && rc >= m.r_out) put(m.r_out - m.nudge);
  if (nc == 2 && rc < m.r_out) put(m.r_out + m.nudge);
  if (ti || to) ++tl.transmit;
  x = nx;
  y = ny;
  z = nz;
  comp = nc;
  return -(nc == 0 ? m.t2dec[0] : (nc == 1 ? m.t2dec[1] : m.t2dec[2]));
}

// Packed myelinated cylinders: N axons in a periodic square cell.
struct PMyelinK {
  const float4* cyl;  // 4 float4 per axon: (cx, cy, R_in, R_out), (sl_i, sl_m, sl_e, kin_i),
                      // (kin_m, kin_e, kout_i, kout_m), (kout_e, -, -, -)
  const long long* seed;  // 2n + 1 range ends of the seeding
  int n, nmax;
  float L, nudge, rho, lwm;
  float t2dec[3];
};

__device__ __forceinline__ float pm_mi(float q, float L) { return q - L * floorf(q / L + 0.5f); }

// One sub-step of make_packed_myelin_traj_step_fn + the fused weight (physics.py:742-930,
// 1034-1056).  (x, y) is the in-cell position (wrapped into [-L/2, L/2) where the reference
// wraps it), z free; comp the encoded compartment.  The walker's axon k (axon 0 for an
// extra-axonal walker, as in the reference) supplies the walls it can cross and the step length;
// an extra-axonal walker that ends inside any sheath is mirrored out of the deepest one.  Returns
// the step's log-weight without the coherence gate's T1 part: (rho/D * unit boundary log-weight
// - dt/T2 of the new compartment); the kernel multiplies it by chi.
template <int WALL>
__device__ __forceinline__ float pmyelin_step(float& x, float& y, float& z, int& comp, float ux,
                                              float uy, float uz, float u1, float u2,
                                              const PMyelinK& m, Tally& tl) {
  const bool ext = comp == 0, intra = comp >= 1 && comp <= m.nmax, myel = comp > m.nmax;
  int k = intra ? comp - 1 : (myel ? comp - m.nmax - 1 : 0);
  k = max(k, 0);
  const float4 A = m.cyl[4 * k], B = m.cyl[4 * k + 1], C4 = m.cyl[4 * k + 2],
               D4 = m.cyl[4 * k + 3];
  const float cx = A.x, cy = A.y, rin = A.z, rout = A.w;
  const float sl = intra ? B.x : (myel ? B.y : B.z);
  const float stx = ux * sl, sty = uy * sl, stz = uz * sl;
  float qx = pm_mi(x + stx - cx, m.L), qy = pm_mi(y + sty - cy, m.L);
  const float rn = sqrtf(qx * qx + qy * qy);
  const bool cio = intra && rn >= rin, cii = myel && rn < rin;
  const bool coo = myel && rn >= rout, coi = ext && rn < rout;
  const bool ci = cio || cii, co = coo || coi;
  const float dpi = fabsf(rn - rin), dpo = fabsf(rn - rout);
  bool ti = false, to = false;
  if constexpr (WALL == kPermeate) {
    const float kin = intra ? B.w : (myel ? C4.x : C4.y);
    const float kout = intra ? C4.z : (myel ? C4.w : D4.x);
    ti = ci && (u1 < fminf(1.f, 2.f * kin * dpi));
    to = co && (u2 < fminf(1.f, 2.f * kout * dpo));
  }
  int nc = comp;
  float dlog = 0.f;
  if (ci && !ti) {  // mirror across the inner wall
    const float s = (2.f * rin - rn) / fmaxf(rn, 1e-20f);
    qx *= s;
    qy *= s;
    dlog += -2.f * dpi;
  }
  if (ti) nc = cio ? m.nmax + k + 1 : k + 1;
  if (co && !to) {  // mirror across the outer wall
    const float r2 = sqrtf(qx * qx + qy * qy);
    const float s = (2.f * rout - r2) / fmaxf(r2, 1e-20f);
    qx *= s;
    qy *= s;
    dlog += -2.f * dpo;
  }
  if (to) nc = coo ? 0 : m.nmax + k + 1;
  float nx = pm_mi(qx + cx, m.L), ny = pm_mi(qy + cy, m.L);
  if (ext) {
    // an extra-axonal end point inside any sheath: mirror out of the one it penetrates deepest
    // (relative to R_out^2; first of equals), recording its outer-wall contact
    float pmin = 1.f;
    int kc = 0;
#pragma unroll 1
    for (int j = 0; j < m.n; ++j) {
      const float4 Cj = m.cyl[4 * j];
      const float fx = pm_mi(nx - Cj.x, m.L), fy = pm_mi(ny - Cj.y, m.L);
      const float d2 = fx * fx + fy * fy, R2 = Cj.w * Cj.w;
      const float pen = (Cj.w > 0.f && d2 < R2) ? d2 / (R2 + 1e-30f) : 1.f;
      if (pen < pmin) {
        pmin = pen;
        kc = j;
      }
    }
    if (pmin < 1.f) {
      const float4 Cc = m.cyl[4 * kc];
      const float qcx = pm_mi(nx - Cc.x, m.L), qcy = pm_mi(ny - Cc.y, m.L);
      const float dcl = sqrtf(qcx * qcx + qcy * qcy);
      const float s = (2.f * Cc.w - dcl) / fmaxf(dcl, m.nudge);
      nx = (nx - qcx) + qcx * s;
      ny = (ny - qcy) + qcy * s;
      dlog += -2.f * fmaxf(Cc.w - dcl, 0.f);
      ++tl.clamp;
    }
  } else if (nc == comp) {
    // clamps of a walker that stayed in its axon's intra space or sheath
    auto put = [&](float target) {
      const float ex = pm_mi(nx - cx, m.L), ey = pm_mi(ny - cy, m.L);
      const float d = sqrtf(ex * ex + ey * ey);
      const float s = target / fmaxf(d, 1e-20f);
      nx = cx + ex * s;
      ny = cy + ey * s;
      ++tl.clamp;
    };
    auto dist = [&]() {
      const float ex = pm_mi(nx - cx, m.L), ey = pm_mi(ny - cy, m.L);
      return sqrtf(ex * ex + ey * ey);
    };
    if (intra && dist() >= rin) put(rin - m.nudge);
    if (myel && dist() < rin) put(rin + m.nudge);
    if (myel && dist() >= rout) put(rout - m.nudge);
  }
  // reclassification of an intra / myelin walker against its own axon
  if (!ext) {
    const float ex = pm_mi(nx - cx, m.L), ey = pm_mi(ny - cy, m.L);
    const float d2 = ex * ex + ey * ey;
    if (d2 < rin * rin) nc = k + 1;
    else if (d2 < rout * rout) nc = m.nmax + k + 1;
  }
  if (ti || to) ++tl.transmit;
  x = nx;
  y = ny;
  z = z + stz;
  comp = nc;
  const float t2 = nc == 0 ? m.t2dec[2] : (nc > m.nmax ? m.t2dec[1] : m.t2dec[0]);
  return m.rho * dlog - t2;
}

// ------------------------------------------------------------------------------------------------
// Validation slabs and shell (geometries.py:48-140, 3221-3431).
// ------------------------------------------------------------------------------------------------
// x mirrored into [0, L]: the floored modulo 2L, then the upper half folded back.
__device__ __forceinline__ float fold_slab(float x, float L) {
  const float L2 = 2.f * L;
  float xf = fmodf(x, L2);
  if (xf < 0.f) xf += L2;
  return xf > L ? L2 - xf : xf;
}

// Box1D.reflect / reflect_with_log_weight (geometries.py:90-140): walls at x = 0 and L.
template <int WALL>
__device__ __forceinline__ float box1d_step(float& x, float& y, float& z, float sx, float sy,
                                            float sz, const GeoK& g) {
  const float xr = x + sx;
  float dl = 0.f;
  if constexpr (WALL == kRelax) {
    const float dp = fmaxf(xr - g.L, 0.f) + fmaxf(-xr, 0.f);
    dl = dp > 0.f ? -2.f * dp : 0.f;
  }
  x = fold_slab(xr, g.L);
  y += sy;
  z += sz;
  return dl;
}

// PermeableSlab1D (geometries.py:3268-3300): membrane at x = L/2 (g.R), outer walls folded.
template <int WALL>
__device__ __forceinline__ float slab_step(float& x, float& y, float& z, float sx, float sy,
                                           float sz, float u, const GeoK& g, Tally& tl) {
  const float xm = g.R, xn = x + sx;
  const bool crossed = (x - xm) * (xn - xm) < 0.f;
  const float dp = crossed ? fabsf(xn - xm) : 0.f;
  bool refl = crossed;
  if constexpr (WALL == kPermeate) {
    const bool transmit = crossed && (u < fminf(1.f, 2.f * g.kod * dp));
    refl = crossed && !transmit;
    if (transmit) ++tl.transmit;
  }
  x = fold_slab(refl ? 2.f * xm - xn : xn, g.L);
  y += sy;
  z += sz;
  if constexpr (WALL == kRelax) return -2.f * dp;
  return refl ? -2.f * dp : 0.f;
}

// PermeableShell._permeate_impl (geometries.py:3366-3425): the first crossing of the permeable
// membrane R_in (g.R) or the reflecting wall R_out along the step, radii measured from the origin
// (sphere) or the z axis (cylinder); a membrane hit transmits with p = min(1, 2 kappa/D d_perp),
// d_perp = remaining * |d . n|; a reflection nudges the hit point onto its own side and flies
// the rest along the mirrored direction; a walker past R_out is mirrored back.
template <int WALL>
__device__ __forceinline__ float shell_step(float& x, float& y, float& z, float sx, float sy,
                                            float sz, float u, const GeoK& g, Tally& tl) {
  const float r_out = g.r_out;
  const int cyl = g.cyl;
  const float Rin = g.R, EPS = g.eps, BIG = 1e30f;
  const float sl = sqrtf(sx * sx + sy * sy + sz * sz);
  const float inv = 1.f / fmaxf(sl, EPS);
  const float dx = sx * inv, dy = sy * inv, dz = sz * inv;
  const float cz = cyl ? 0.f : 1.f;  // radial subspace: drop z for a cylindrical shell
  const float b = dx * x + dy * y + cz * dz * z;
  const float r2 = x * x + y * y + cz * z * z;
  const float dd2 = fmaxf(dx * dx + dy * dy + cz * dz * dz, EPS);
  auto first_t = [&](float Rk) {
    const float c = r2 - Rk * Rk;
    const float disc = b * b - dd2 * c;
    const float s = sqrtf(fmaxf(disc, 0.f));
    float t1 = (-b - s) / dd2, t2 = (-b + s) / dd2;
    t1 = (disc > 0.f && t1 > EPS && t1 < sl) ? t1 : BIG;
    t2 = (disc > 0.f && t2 > EPS && t2 < sl) ? t2 : BIG;
    return fminf(t1, t2);
  };
  const float t_in = first_t(Rin), t_out = first_t(r_out);
  const bool hit_in = t_in < t_out;
  const float t = fminf(t_in, t_out);
  const bool any = t < 1e29f;
  float dl = 0.f;
  if (any) {
    const float hx = x + t * dx, hy = y + t * dy, hz = z + t * dz;
    const float nrm = sqrtf(hx * hx + hy * hy + cz * hz * hz);
    const float ni = 1.f / fmaxf(nrm, EPS);
    const float nx = hx * ni, ny = hy * ni, nz = cz * hz * ni;
    const float rem = sl - t;
    const float dn = dx * nx + dy * ny + dz * nz;
    const float dperp = rem * fabsf(dn);
    bool transmit = false;
    if constexpr (WALL == kPermeate) transmit = hit_in && (u < fminf(1.f, 2.f * g.kod * dperp));
    if (transmit) {
      ++tl.transmit;
      x += sx;
      y += sy;
      z += sz;
    } else {
      const float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny, rz = dz - 2.f * dn * nz;
      const float Rk = hit_in ? Rin : r_out;
      const float side = sqrtf(r2) < Rk ? -1.f : 1.f;
      const float f = fmaxf(rem - g.nudge, 0.f);
      x = hx + side * g.nudge * nx + rx * f;
      y = hy + side * g.nudge * ny + ry * f;
      z = hz + side * g.nudge * nz + rz * f;
      if (hit_in) dl = -2.f * dperp;
    }
  } else {
    x += sx;
    y += sy;
    z += sz;
  }
  const float ro = sqrtf(x * x + y * y + cz * z * z);
  const float over = ro - r_out;
  if (over > 0.f) {  // never outside the reflecting wall
    const float s = 2.f * over / fmaxf(ro, EPS);
    x -= s * x;
    y -= s * y;
    z -= s * cz * z;
    ++tl.clamp;
  }
  return dl;
}

// ------------------------------------------------------------------------------------------------
// Axis-aligned ellipsoid at the origin (geometries.py:1137-1427): reflect /
// reflect_with_log_weight with up to 10 specular bounces on the quadratic
// A t^2 + 2 B t + C = 0 (A = d.D.d, B = r.D.d, C = r.D.r - 1, D = diag(1/a^2, 1/b^2, 1/c^2)), the
// outward normal along D r, the nudge inwards, and the clamp to the scaled surface; permeate with
// one Powles decision on the inside or outside root.  g.R = the smallest semi-axis.
// ------------------------------------------------------------------------------------------------
template <int WALL>
__device__ __forceinline__ float ellipsoid_step(float& x, float& y, float& z, float sx, float sy,
                                                float sz, float u, const GeoK& g, Tally& tl) {
  const float ea = g.e2[0], eb = g.e2[1], ec = g.e2[2];
  const float l = sqrtf(sx * sx + sy * sy + sz * sz);
  float dx = sx / l, dy = sy / l, dz = sz / l;
  if constexpr (WALL != kPermeate) {
    float rx = x, ry = y, rz = z, rem = l, dsum = 0.f;
#pragma unroll 1
    for (int it = 0; it < 10; ++it) {
      const float A = dx * ea * dx + dy * eb * dy + dz * ec * dz;
      const float B = rx * ea * dx + ry * eb * dy + rz * ec * dz;
      const float C = (rx * ea * rx + ry * eb * ry + rz * ec * rz) - 1.f;
      const float disc = fmaxf(B * B - A * C, 0.f);
      const float d = (-B + sqrtf(disc)) / A;
      if (!(d > g.eps && d < rem)) break;
      const float hx = rx + d * dx, hy = ry + d * dy, hz = rz + d * dz;
      float nx = hx * ea, ny = hy * eb, nz = hz * ec;
      const float nn = sqrtf(nx * nx + ny * ny + nz * nz);
      nx /= nn;
      ny /= nn;
      nz /= nn;
      const float dn = dx * nx + dy * ny + dz * nz;
      float qx = dx - 2.f * dn * nx, qy = dy - 2.f * dn * ny, qz = dz - 2.f * dn * nz;
      const float qn = sqrtf(qx * qx + qy * qy + qz * qz);
      if constexpr (WALL == kRelax) dsum += (rem - d) * dn;
      rx = hx - g.nudge * nx;
      ry = hy - g.nudge * ny;
      rz = hz - g.nudge * nz;
      dx = qx / qn;
      dy = qy / qn;
      dz = qz / qn;
      rem = rem - d - g.nudge;
    }
    const float f = fmaxf(rem, 0.f);
    x = rx + dx * f;
    y = ry + dy * f;
    z = rz + dz * f;
    const float q = sqrtf(x * x * ea + y * y * eb + z * z * ec);
    if (q >= 1.f) {
      const float s = (1.f - g.nudge / g.R) / q;
      x *= s;
      y *= s;
      z *= s;
      ++tl.clamp;
    }
    return -2.f * dsum;
  } else {
    const float A = dx * ea * dx + dy * eb * dy + dz * ec * dz;
    const float B = x * ea * dx + y * eb * dy + z * ec * dz;
    const float C = (x * ea * x + y * eb * y + z * ec * z) - 1.f;
    const float draw_ = B * B - A * C;
    const float sq = sqrtf(fmaxf(draw_, 0.f));
    const bool inside = C < 0.f;
    const float t = inside ? (-B + sq) / A : (-B - sq) / A;
    const bool hit = (draw_ > 0.f) && (t > g.eps) && (t < l) && (l > 0.f);
    if (!hit) {
      x += sx;
      y += sy;
      z += sz;
      return 0.f;
    }
    const float hx = x + t * dx, hy = y + t * dy, hz = z + t * dz;
    float nx = hx * ea, ny = hy * eb, nz = hz * ec;
    const float nn = sqrtf(nx * nx + ny * ny + nz * nz);
    nx /= nn;
    ny /= nn;
    nz /= nn;
    const float rem = l - t;
    const float dn = dx * nx + dy * ny + dz * nz;
    const float dperp = rem * fabsf(dn);
    if (u < fminf(1.f, 2.f * g.kod * dperp)) {
      ++tl.transmit;
      x += sx;
      y += sy;
      z += sz;
      return 0.f;
    }
    float qx = dx - 2.f * dn * nx, qy = dy - 2.f * dn * ny, qz = dz - 2.f * dn * nz;
    const float qn = sqrtf(qx * qx + qy * qy + qz * qz);
    const float sg = inside ? -1.f : 1.f;
    const float f = fmaxf(rem - g.nudge, 0.f);
    x = hx + g.nudge * sg * nx + qx / qn * f;
    y = hy + g.nudge * sg * ny + qy / qn * f;
    z = hz + g.nudge * sg * nz + qz / qn * f;
    return -2.f * dperp;
  }
}

// ------------------------------------------------------------------------------------------------
// Single cylinder, axis z, centred at the origin.
// ------------------------------------------------------------------------------------------------
template <int WALL>
__device__ __forceinline__ float cylinder_step(float& x, float& y, float sx, float sy, float u,
                                               const GeoK& g, Tally& tl) {
  const float lxy = sqrtf(sx * sx + sy * sy);
  float dx = 0.f, dy = 0.f;
  if (lxy > 0.f) {
    dx = sx / lxy;
    dy = sy / lxy;
  }
  float dsum = 0.f;  // sum of d_perp
  if constexpr (WALL != kPermeate) {
    // Up to 10 specular bounces (geometries.py:523-559).  An iteration without a crossing leaves
    // the state unchanged, so the loop stops at the first one.
    float rem = lxy;
    if (lxy > 0.f) {
#pragma unroll 1
      for (int it = 0; it < 10; ++it) {
        const float dp = dx * x + dy * y;
        float disc = fmaxf(dp * dp - ((x * x + y * y) - g.R2), 0.f);
        float d = -dp + sqrtf(disc);
        if (disc < kGrazeTol * g.R2) {
          const double dpd = (double)dx * x + (double)dy * y;
          const double dd = fmax(dpd * dpd - (((double)x * x + (double)y * y) - (double)g.R * g.R), 0.0);
          disc = (float)dd;
          d = (float)(-dpd + sqrt(dd));
          ++tl.graze;
        }
        if (!(d > g.eps && d < rem)) break;
        const float hx = x + d * dx, hy = y + d * dy;
        const float nx = hx / g.R, ny = hy / g.R;
        const float dn = dx * nx + dy * ny;
        float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny;
        const float rn = sqrtf(rx * rx + ry * ry);
        rx /= rn;
        ry /= rn;
        if constexpr (WALL == kRelax) dsum += (rem - d) * (sqrtf(disc) / g.R);
        x = hx - g.nudge * nx;
        y = hy - g.nudge * ny;
        dx = rx;
        dy = ry;
        rem = rem - d - g.nudge;
      }
    }
    const float f = fmaxf(rem, 0.f);
    x += dx * f;
    y += dy * f;
    const float rr = sqrtf(x * x + y * y);
    if (rr >= g.R) {  // safety clamp, geometries.py:555-559
      const float s = (g.R - g.nudge) / rr;
      x *= s;
      y *= s;
      ++tl.clamp;
    }
    return -2.f * dsum;
  } else {
    // Powles crossing, one decision per sub-step (geometries.py:705-801).
    const float dp = dx * x + dy * y;
    const float q2 = x * x + y * y;
    float disc = dp * dp - (q2 - g.R2);
    const bool inside = q2 < g.R2;
    float sq = sqrtf(fmaxf(disc, 0.f));
    float t = inside ? -dp + sq : -dp - sq;
    if (fabsf(disc) < kGrazeTol * g.R2) {
      const double dpd = (double)dx * x + (double)dy * y;
      const double dd = dpd * dpd - (((double)x * x + (double)y * y) - (double)g.R * g.R);
      const double sd = sqrt(fmax(dd, 0.0));
      disc = (float)dd;
      sq = (float)sd;
      t = (float)(inside ? -dpd + sd : -dpd - sd);
      ++tl.graze;
    }
    const bool hit = (disc > 0.f) && (t > g.eps) && (t < lxy) && (lxy > 0.f);
    if (!hit) {
      x += sx;
      y += sy;
      return 0.f;
    }
    const float hrx = x + t * dx, hry = y + t * dy;
    const float hl = fmaxf(sqrtf(hrx * hrx + hry * hry), 1e-30f);
    const float nx = hrx / hl, ny = hry / hl;
    const float hx = g.R * nx, hy = g.R * ny;  // snapped to the wall
    const float rem = lxy - t;
    const float dperp = rem * (sq / g.R);
    const float p = fminf(1.f, 2.f * g.kod * dperp);
    if (u < p) {
      x += sx;
      y += sy;
      ++tl.transmit;
      return 0.f;
    }
    const float dn = dx * nx + dy * ny;
    float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny;
    const float rn = sqrtf(rx * rx + ry * ry);
    rx /= rn;
    ry /= rn;
    const float sgn = inside ? -1.f : 1.f;
    const float f = fmaxf(rem - g.nudge, 0.f);
    float ox = hx + g.nudge * sgn * nx + rx * f;
    float oy = hy + g.nudge * sgn * ny + ry * f;
    const float on = sqrtf(ox * ox + oy * oy);
    const bool wrong = inside ? (on >= g.R) : (on <= g.R);
    if (wrong) {
      const float s = (inside ? g.R - g.nudge : g.R + g.nudge) / fmaxf(on, 1e-30f);
      ox *= s;
      oy *= s;
      ++tl.clamp;
    }
    x = ox;
    y = oy;
    return -2.f * dperp;
  }
}

// ------------------------------------------------------------------------------------------------
// Single sphere centred at the origin.
// ------------------------------------------------------------------------------------------------
template <int WALL>
__device__ __forceinline__ float sphere_step(float& x, float& y, float& z, float sx, float sy,
                                             float sz, float u, const GeoK& g, Tally& tl) {
  const float l = sqrtf(sx * sx + sy * sy + sz * sz);
  float dx = sx / l, dy = sy / l, dz = sz / l;
  if constexpr (WALL != kPermeate) {
    // geometries.py:236-264
    float rem = l;
    float dsum = 0.f;
#pragma unroll 1
    for (int it = 0; it < 10; ++it) {
      const float dp = dx * x + dy * y + dz * z;
      float disc = fmaxf(dp * dp - ((x * x + y * y + z * z) - g.R2), 0.f);
      float d = -dp + sqrtf(disc);
      if (disc < kGrazeTol * g.R2) {
        const double dpd = (double)dx * x + (double)dy * y + (double)dz * z;
        const double dd = fmax(dpd * dpd - (((double)x * x + (double)y * y + (double)z * z) -
                                            (double)g.R * g.R), 0.0);
        disc = (float)dd;
        d = (float)(-dpd + sqrt(dd));
        ++tl.graze;
      }
      if (!(d > g.eps && d < rem)) break;
      const float hx = x + d * dx, hy = y + d * dy, hz = z + d * dz;
      const float nx = hx / g.R, ny = hy / g.R, nz = hz / g.R;
      const float dn = dx * nx + dy * ny + dz * nz;
      float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny, rz = dz - 2.f * dn * nz;
      const float rn = sqrtf(rx * rx + ry * ry + rz * rz);
      rx /= rn;
      ry /= rn;
      rz /= rn;
      if constexpr (WALL == kRelax) dsum += (rem - d) * (sqrtf(disc) / g.R);
      x = hx - g.nudge * nx;
      y = hy - g.nudge * ny;
      z = hz - g.nudge * nz;
      dx = rx;
      dy = ry;
      dz = rz;
      rem = rem - d - g.nudge;
    }
    const float f = fmaxf(rem, 0.f);
    x += dx * f;
    y += dy * f;
    z += dz * f;
    const float rr = sqrtf(x * x + y * y + z * z);
    if (rr >= g.R) {  // geometries.py:260-263
      const float s = (g.R - g.nudge) / rr;
      x *= s;
      y *= s;
      z *= s;
      ++tl.clamp;
    }
    return -2.f * dsum;
  } else {
    // geometries.py:367-424 (no snapping and no side clamp, unlike the cylinder)
    const float dp = dx * x + dy * y + dz * z;
    const float q2 = x * x + y * y + z * z;
    float disc = dp * dp - (q2 - g.R2);
    const bool inside = q2 < g.R2;
    float sq = sqrtf(fmaxf(disc, 0.f));
    float t = inside ? -dp + sq : -dp - sq;
    if (fabsf(disc) < kGrazeTol * g.R2) {
      const double dpd = (double)dx * x + (double)dy * y + (double)dz * z;
      const double dd = dpd * dpd - (((double)x * x + (double)y * y + (double)z * z) - (double)g.R * g.R);
      const double sd = sqrt(fmax(dd, 0.0));
      disc = (float)dd;
      sq = (float)sd;
      t = (float)(inside ? -dpd + sd : -dpd - sd);
      ++tl.graze;
    }
    const bool hit = (disc > 0.f) && (t > g.eps) && (t < l) && (l > 0.f);
    if (!hit) {
      x += sx;
      y += sy;
      z += sz;
      return 0.f;
    }
    const float hx = x + t * dx, hy = y + t * dy, hz = z + t * dz;
    const float nx = hx / g.R, ny = hy / g.R, nz = hz / g.R;
    const float rem = l - t;
    const float dperp = rem * (sq / g.R);
    const float p = fminf(1.f, 2.f * g.kod * dperp);
    if (u < p) {
      x += sx;
      y += sy;
      z += sz;
      ++tl.transmit;
      return 0.f;
    }
    const float dn = dx * nx + dy * ny + dz * nz;
    float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny, rz = dz - 2.f * dn * nz;
    const float rn = sqrtf(rx * rx + ry * ry + rz * rz);
    rx /= rn;
    ry /= rn;
    rz /= rn;
    const float sgn = inside ? -1.f : 1.f;
    const float f = fmaxf(rem - g.nudge, 0.f);
    x = hx + g.nudge * sgn * nx + rx * f;
    y = hy + g.nudge * sgn * ny + ry * f;
    z = hz + g.nudge * sgn * nz + rz * f;
    return -2.f * dperp;
  }
}

// ------------------------------------------------------------------------------------------------
// Packed objects: cell lookup of the walker's candidate list.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ int cell_of(float v, const GeoK& g) {
  int i = (int)floorf((v + g.halfL) * g.inv_h);
  return min(max(i, 0), g.n - 1);
}

__device__ __forceinline__ bool min_image(float q, const GeoK& g) {
  return q >= -g.halfL && q < g.halfL;
}

__device__ __forceinline__ void fold(float& v, int& img, const GeoK& g) {
  if (v >= g.halfL) {
    v -= g.L;
    ++img;
  } else if (v < -g.halfL) {
    v += g.L;
    --img;
  }
}

// Packed cylinders (2-D cross-section; z is free).  The step is assembled from the pieces below
// (shared with the free-flight kernel of walk_ff.cuh, which runs them in separate stages):
//   pcyl_dir     step length and unit direction in the cross-section;
//   pcyl_test    one candidate's entry root and straight-end containment (geometries.py:1777-1805
//                / 2054-2081 for the root, 1851-1877 for the containment);
//   pcyl_graze   the FP64 re-solve of a grazing winning root;
//   pcyl_hit     the wall's action on the winner: specular reflection (+ boundary weight) or the
//                Powles decision with its snapped, side-clamped reflection (geometries.py:1810-1842,
//                1943-1967, 2083-2165);
//   pcyl_clamp   the fold-first safety clamp over a cell's candidates (geometries.py:1851-1877).

// Crossing of one candidate by the segment from (x, y) along (dx, dy) of length lxy.
struct PcylRoot {
  float t, disc;  // entry (or, from inside, exit) distance; discriminant of the root
  bool valid;     // a forward crossing within the step
  bool ins;       // the walker starts inside the candidate (permeable walls only)
  bool end_in;    // the straight end point (ex, ey) lies inside (reflecting walls only)
};

__device__ __forceinline__ void pcyl_dir(float sx, float sy, float& lxy, float& dx, float& dy) {
  lxy = sqrtf(sx * sx + sy * sy);
  dx = 0.f;
  dy = 0.f;
  if (lxy > 0.f) {
    const float inv = 1.f / lxy;
    dx = sx * inv;
    dy = sy * inv;
  }
}

// MI = false compiles the test for cell lists that never list two images of one object
// (g.mi == 0), where the minimum-image test always passes.
template <int WALL, bool MI = true>
__device__ __forceinline__ PcylRoot pcyl_test(const float4 C, float x, float y, float ex, float ey,
                                              float dx, float dy, float lxy, const GeoK& g) {
  PcylRoot r;
  const float R2 = C.w * C.w;
  r.end_in = false;
  if constexpr (WALL != kPermeate) {
    const float fx = ex - C.x, fy = ey - C.y;
    const float d2 = fx * fx + fy * fy;
    r.end_in = d2 < R2 && (!(MI && g.mi) || (min_image(fx, g) && min_image(fy, g)));
  }
  const float qx = x - C.x, qy = y - C.y;
  const bool mi_ok = !(MI && g.mi) || (min_image(qx, g) && min_image(qy, g));
  const float dp = dx * qx + dy * qy;
  const float q2 = qx * qx + qy * qy;
  r.disc = dp * dp - (q2 - R2);
  r.ins = (WALL == kPermeate) && (q2 < R2);
  const float sq = sqrtf(fmaxf(r.disc, 0.f));
  r.t = r.ins ? -dp + sq : -dp - sq;
  // an entry root with dp >= 0 is -dp - sqrt(disc) <= 0: no forward crossing
  r.valid = mi_ok && (r.ins || dp < 0.f) && (r.disc > 0.f) && (r.t > g.eps) && (r.t < lxy) &&
            (lxy > 0.f);
  return r;
}

// A winning root whose discriminant is within kGrazeTol R^2 of grazing, re-solved in FP64; the
// hit may vanish (tbest = INFINITY).
__device__ __forceinline__ void pcyl_graze(float x, float y, float dx, float dy, float lxy,
                                           float hcx, float hcy, float hR, bool hit_in,
                                           const GeoK& g, float& tbest, float& disc_hit,
                                           Tally& tl) {
  const double qxd = (double)(x - hcx), qyd = (double)(y - hcy);
  const double dpd = (double)dx * qxd + (double)dy * qyd;
  const double dd = dpd * dpd - ((qxd * qxd + qyd * qyd) - (double)hR * hR);
  const double sd = sqrt(fmax(dd, 0.0));
  const float t = (float)(hit_in ? -dpd + sd : -dpd - sd);
  disc_hit = (float)dd;
  tbest = ((dd > 0.0) && (t > g.eps) && (t < lxy)) ? t : INFINITY;
  ++tl.graze;
}

// The wall's action on a hit at distance tbest of candidate (hcx, hcy, hR): the new position in
// the start cell's frame and the boundary log-weight at rho/D = 1.
template <int WALL>
__device__ __forceinline__ void pcyl_hit(float x, float y, float sx, float sy, float dx, float dy,
                                         float lxy, float u, float tbest, float disc_hit,
                                         float hcx, float hcy, float hR, bool hit_in,
                                         const GeoK& g, Tally& tl, float& nxp, float& nyp,
                                         float& dlog) {
  dlog = 0.f;
  const float qcx = x - hcx, qcy = y - hcy;
  if constexpr (WALL != kPermeate) {
    // geometries.py:1810-1842 / 1943-1967
    const float nx = (qcx + tbest * dx) / hR, ny = (qcy + tbest * dy) / hR;
    const float dn = dx * nx + dy * ny;
    float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny;
    const float rn = sqrtf(rx * rx + ry * ry);
    if (rn > 0.f) {
      rx /= fmaxf(rn, 1e-30f);
      ry /= fmaxf(rn, 1e-30f);
    } else {
      rx = 0.f;
      ry = 0.f;
    }
    const float remr = lxy - tbest;
    const float f = fmaxf(remr - g.nudge, 0.f);
    nxp = (x + tbest * dx) + g.nudge * nx + rx * f;
    nyp = (y + tbest * dy) + g.nudge * ny + ry * f;
    if constexpr (WALL == kRelax) dlog = -2.f * (remr * (sqrtf(fmaxf(disc_hit, 0.f)) / hR));
  } else {
    // geometries.py:2083-2165
    const float hrx = qcx + tbest * dx, hry = qcy + tbest * dy;
    const float hl = fmaxf(sqrtf(hrx * hrx + hry * hry), 1e-30f);
    const float nx = hrx / hl, ny = hry / hl;
    const float rem = lxy - tbest;
    const float dperp = rem * (sqrtf(fmaxf(disc_hit, 0.f)) / hR);
    const float p = fminf(1.f, 2.f * g.kod * dperp);
    if (u < p) {
      nxp = x + sx;
      nyp = y + sy;
      ++tl.transmit;
    } else {
      const float dn = dx * nx + dy * ny;
      float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny;
      const float rn = sqrtf(rx * rx + ry * ry);
      if (rn > 0.f) {
        rx /= fmaxf(rn, 1e-30f);
        ry /= fmaxf(rn, 1e-30f);
      } else {
        rx = 0.f;
        ry = 0.f;
      }
      const float sgn = hit_in ? -1.f : 1.f;
      const float f = fmaxf(rem - g.nudge, 0.f);
      float ox = hR * nx + g.nudge * sgn * nx + rx * f;
      float oy = hR * ny + g.nudge * sgn * ny + ry * f;
      const float on = sqrtf(ox * ox + oy * oy);
      const bool wrong = hit_in ? (on >= hR) : (on <= hR);
      if (wrong) {
        const float s = (hit_in ? hR - g.nudge : hR + g.nudge) / fmaxf(on, 1e-30f);
        ox *= s;
        oy *= s;
        ++tl.clamp;
      }
      nxp = x + (ox - qcx);
      nyp = y + (oy - qcy);
      dlog = -2.f * dperp;
    }
  }
}

// Fold-first safety clamp (geometries.py:1851-1877): push (nxp, nyp) out of the candidate it
// penetrates most deeply (relative to R^2).  The start cell's list covers every object within
// reach of the end point.
template <bool MI = true>
__device__ __forceinline__ void pcyl_clamp(float& nxp, float& nyp, uint32_t kb, uint32_t ke,
                                           const GeoK& g, const float4* __restrict__ cand,
                                           Tally& tl) {
  float pe = 1.f, pqx = 0.f, pqy = 0.f, pR = 1.f;
  auto pen_of = [&](const float4 C) {
    const float qx = nxp - C.x, qy = nyp - C.y;
    const float d2 = qx * qx + qy * qy, R2 = C.w * C.w;
    if (d2 < R2 && (!(MI && g.mi) || (min_image(qx, g) && min_image(qy, g)))) {
      const float pen = d2 / R2;
      if (pen < pe) {
        pe = pen;
        pqx = qx;
        pqy = qy;
        pR = C.w;
      }
    }
  };
  if (g.kmax == 2) {
#pragma unroll
    for (uint32_t j = 0; j < 2u; ++j)
      pen_of(kb + j < ke ? cand[kb + j] : make_float4(kFarAway, kFarAway, kFarAway, 0.f));
  } else {
#pragma unroll 1
    for (uint32_t k = kb; k < ke; ++k) pen_of(cand[k]);
  }
  if (pe < 1.f) {
    const float dcl = sqrtf(pqx * pqx + pqy * pqy);
    const float s = (pR + g.nudge) / fmaxf(dcl, g.nudge);
    nxp += pqx * (s - 1.f);
    nyp += pqy * (s - 1.f);
    ++tl.clamp;
  }
}

// One sub-step of a walker: the nearest crossing over the cell's candidates (branch free; the
// straight end point's containment is noted in the same pass, so the clamp scan runs only after a
// reflection or when that end point lies inside a candidate), the grazing re-solve, the wall's
// action, the clamp, and the fold back into the periodic cell.  cs/cand point at the cell list
// (shared or global memory).
template <int WALL>
__device__ __forceinline__ float packed_cyl_step(float& x, float& y, int& ix, int& iy, float sx,
                                                 float sy, float u, const GeoK& g,
                                                 const uint32_t* __restrict__ cs,
                                                 const float4* __restrict__ cand, Tally& tl) {
  float lxy, dx, dy;
  pcyl_dir(sx, sy, lxy, dx, dy);
  const int c = cell_of(y, g) * g.n + cell_of(x, g);
  const uint32_t kb = cs[c], ke = cs[c + 1];
  float tbest = INFINITY, disc_hit = 0.f, hcx = 0.f, hcy = 0.f, hR = 1.f;
  bool hit_in = false, end_in = false;
  const float ex = x + sx, ey = y + sy;
  auto visit = [&](const float4 C, auto mi) {
    const PcylRoot r = pcyl_test<WALL, decltype(mi)::value>(C, x, y, ex, ey, dx, dy, lxy, g);
    end_in |= r.end_in;
    if (r.valid && r.t < tbest) {
      tbest = r.t;
      disc_hit = r.disc;
      hcx = C.x;
      hcy = C.y;
      hR = C.w;
      hit_in = r.ins;
    }
  };
  // every cell lists at most two candidates and no two images of one object: two slots for every
  // lane, no divergent trip count and no minimum-image tests; the slot past a shorter list holds
  // a zero-radius object far outside the cell, which no test can select
  const bool two = g.kmax == 2 && !g.mi;
  if (two) {
#pragma unroll
    for (uint32_t j = 0; j < 2u; ++j)
      visit(kb + j < ke ? cand[kb + j] : make_float4(kFarAway, kFarAway, kFarAway, 0.f),
            std::false_type());
  } else {
#pragma unroll 1
    for (uint32_t k = kb; k < ke; ++k) visit(cand[k], std::true_type());
  }
  if (tbest < INFINITY && disc_hit < kGrazeTol * hR * hR)
    pcyl_graze(x, y, dx, dy, lxy, hcx, hcy, hR, hit_in, g, tbest, disc_hit, tl);

  float nxp = x + sx, nyp = y + sy, dlog = 0.f;  // new position in the start cell's frame
  if (tbest < INFINITY)
    pcyl_hit<WALL>(x, y, sx, sy, dx, dy, lxy, u, tbest, disc_hit, hcx, hcy, hR, hit_in, g, tl,
                   nxp, nyp, dlog);
  if constexpr (WALL != kPermeate)
    if (tbest < INFINITY || end_in) {
      if (two)
        pcyl_clamp<false>(nxp, nyp, kb, ke, g, cand, tl);
      else
        pcyl_clamp<true>(nxp, nyp, kb, ke, g, cand, tl);
    }
  x = nxp;
  y = nyp;
  fold(x, ix, g);
  fold(y, iy, g);
  return dlog;
}

// Packed spheres (3-D periodic cell).
template <int WALL>
__device__ __forceinline__ float packed_sph_step(float& x, float& y, float& z, int& ix, int& iy,
                                                 int& iz, float sx, float sy, float sz, float u,
                                                 const GeoK& g, const uint32_t* __restrict__ cs,
                                                 const float4* __restrict__ cand, Tally& tl) {
  const float l = sqrtf(sx * sx + sy * sy + sz * sz);
  float dx = 0.f, dy = 0.f, dz = 0.f;
  if (l > 0.f) {
    dx = sx / l;
    dy = sy / l;
    dz = sz / l;
  }
  const int c = (cell_of(z, g) * g.n + cell_of(y, g)) * g.n + cell_of(x, g);
  const uint32_t kb = cs[c], ke = cs[c + 1];

  float tbest = INFINITY, disc_hit = 0.f, hcx = 0.f, hcy = 0.f, hcz = 0.f, hR = 1.f;
  bool hit_in = false;
  const float ex = x + sx, ey = y + sy, ez = z + sz;
  float pe = 1.f, pqx = 0.f, pqy = 0.f, pqz = 0.f, pR = 1.f;
  // the candidate scan, compiled twice: with the minimum-image tests, and without them for cell
  // lists that never list two images of one object (g.mi == 0, where the tests always pass)
  auto scan = [&](auto mi_c) {
    constexpr bool MI = decltype(mi_c)::value;
#pragma unroll 1
    for (uint32_t k = kb; k < ke; ++k) {
      const float4 C = cand[k];
      const float R2 = C.w * C.w;
      if constexpr (WALL != kPermeate) {
        const float fx = ex - C.x, fy = ey - C.y, fz = ez - C.z;
        const float d2 = fx * fx + fy * fy + fz * fz;
        if (d2 < R2 && (!MI || (min_image(fx, g) && min_image(fy, g) && min_image(fz, g)))) {
          const float pen = d2 / R2;
          if (pen < pe) {
            pe = pen;
            pqx = fx;
            pqy = fy;
            pqz = fz;
            pR = C.w;
          }
        }
      }
      const float qx = x - C.x, qy = y - C.y, qz = z - C.z;
      if (MI && !(min_image(qx, g) && min_image(qy, g) && min_image(qz, g))) continue;
      const float dp = dx * qx + dy * qy + dz * qz;
      const float q2 = qx * qx + qy * qy + qz * qz;
      float disc = dp * dp - (q2 - R2);
      const bool ins = (WALL == kPermeate) && (q2 < R2);
      if (!ins && dp >= 0.f) continue;
      const float sq = sqrtf(fmaxf(disc, 0.f));
      const float t = ins ? -dp + sq : -dp - sq;
      const bool valid = (disc > 0.f) && (t > g.eps) && (t < l) && (l > 0.f);
      if (valid && t < tbest) {
        tbest = t;
        disc_hit = disc;
        hcx = C.x;
        hcy = C.y;
        hcz = C.z;
        hR = C.w;
        hit_in = ins;
      }
    }
  };
  if (g.mi)
    scan(std::true_type());
  else
    scan(std::false_type());
  if (tbest < INFINITY && disc_hit < kGrazeTol * hR * hR) {
    const double qxd = (double)(x - hcx), qyd = (double)(y - hcy), qzd = (double)(z - hcz);
    const double dpd = (double)dx * qxd + (double)dy * qyd + (double)dz * qzd;
    const double dd = dpd * dpd - ((qxd * qxd + qyd * qyd + qzd * qzd) - (double)hR * hR);
    const double sd = sqrt(fmax(dd, 0.0));
    const float t = (float)(hit_in ? -dpd + sd : -dpd - sd);
    disc_hit = (float)dd;
    tbest = ((dd > 0.0) && (t > g.eps) && (t < l)) ? t : INFINITY;
    ++tl.graze;
  }

  float nxp, nyp, nzp;
  float dlog = 0.f;
  if (tbest < INFINITY) {
    const float qcx = x - hcx, qcy = y - hcy, qcz = z - hcz;
    if constexpr (WALL != kPermeate) {
      // geometries.py:2490-2515 / 2584-2604
      const float nx = (qcx + tbest * dx) / hR, ny = (qcy + tbest * dy) / hR,
                  nz = (qcz + tbest * dz) / hR;
      const float dn = dx * nx + dy * ny + dz * nz;
      float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny, rz = dz - 2.f * dn * nz;
      const float rn = sqrtf(rx * rx + ry * ry + rz * rz);
      if (rn > 0.f) {
        const float inv = 1.f / fmaxf(rn, 1e-30f);
        rx *= inv;
        ry *= inv;
        rz *= inv;
      } else {
        rx = ry = rz = 0.f;
      }
      const float remr = l - tbest;
      const float f = fmaxf(remr - g.nudge, 0.f);
      nxp = (x + tbest * dx) + g.nudge * nx + rx * f;
      nyp = (y + tbest * dy) + g.nudge * ny + ry * f;
      nzp = (z + tbest * dz) + g.nudge * nz + rz * f;
      if constexpr (WALL == kRelax) dlog = -2.f * (remr * (sqrtf(fmaxf(disc_hit, 0.f)) / hR));
    } else {
      // geometries.py:2690-2745
      const float hrx = qcx + tbest * dx, hry = qcy + tbest * dy, hrz = qcz + tbest * dz;
      const float hl = fmaxf(sqrtf(hrx * hrx + hry * hry + hrz * hrz), 1e-30f);
      const float nx = hrx / hl, ny = hry / hl, nz = hrz / hl;
      const float rem = l - tbest;
      const float dperp = rem * (sqrtf(fmaxf(disc_hit, 0.f)) / hR);
      const float p = fminf(1.f, 2.f * g.kod * dperp);
      if (u < p) {
        nxp = x + sx;
        nyp = y + sy;
        nzp = z + sz;
        ++tl.transmit;
      } else {
        const float dn = dx * nx + dy * ny + dz * nz;
        float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny, rz = dz - 2.f * dn * nz;
        const float rn = sqrtf(rx * rx + ry * ry + rz * rz);
        if (rn > 0.f) {
          const float inv = 1.f / fmaxf(rn, 1e-30f);
          rx *= inv;
          ry *= inv;
          rz *= inv;
        } else {
          rx = ry = rz = 0.f;
        }
        const float sgn = hit_in ? -1.f : 1.f;
        const float f = fmaxf(rem - g.nudge, 0.f);
        float ox = hR * nx + g.nudge * sgn * nx + rx * f;
        float oy = hR * ny + g.nudge * sgn * ny + ry * f;
        float oz = hR * nz + g.nudge * sgn * nz + rz * f;
        const float on = sqrtf(ox * ox + oy * oy + oz * oz);
        const bool wrong = hit_in ? (on >= hR) : (on <= hR);
        if (wrong) {
          const float s = (hit_in ? hR - g.nudge : hR + g.nudge) / fmaxf(on, 1e-30f);
          ox *= s;
          oy *= s;
          oz *= s;
          ++tl.clamp;
        }
        nxp = x + (ox - qcx);
        nyp = y + (oy - qcy);
        nzp = z + (oz - qcz);
        dlog = -2.f * dperp;
      }
    }
  } else {
    nxp = x + sx;
    nyp = y + sy;
    nzp = z + sz;
  }

  if constexpr (WALL != kPermeate) {
    if (tbest < INFINITY) {  // geometries.py:2520-2535, after a reflection
      pe = 1.f;
#pragma unroll 1
      for (uint32_t k = kb; k < ke; ++k) {
        const float4 C = cand[k];
        const float qx = nxp - C.x, qy = nyp - C.y, qz = nzp - C.z;
        const float d2 = qx * qx + qy * qy + qz * qz, R2 = C.w * C.w;
        if (d2 < R2 &&
            (!g.mi || (min_image(qx, g) && min_image(qy, g) && min_image(qz, g)))) {
          const float pen = d2 / R2;
          if (pen < pe) {
            pe = pen;
            pqx = qx;
            pqy = qy;
            pqz = qz;
            pR = C.w;
          }
        }
      }
    }
    if (pe < 1.f) {
      const float dcl = sqrtf(pqx * pqx + pqy * pqy + pqz * pqz);
      const float s = (pR + g.nudge) / fmaxf(dcl, g.nudge);
      nxp += pqx * (s - 1.f);
      nyp += pqy * (s - 1.f);
      nzp += pqz * (s - 1.f);
      ++tl.clamp;
    }
  }
  x = nxp;
  y = nyp;
  z = nzp;
  fold(x, ix, g);
  fold(y, iy, g);
  fold(z, iz, g);
  return dlog;
}

}  // namespace dmsim
