// Device step function of the triangle-mesh substrate.
//
// Follows dmipy-sim's mesh.py statement by statement:
//   27-cell candidate gather around the step's start (mesh.py:208-215), gathered once per step
//   and reused for every bounce; Moller-Trumbore segment test (561-569); smooth-normal reflection
//   lifted above the geometric plane by the graze margin, nudge along the geometric normal
//   (607-635); at most max_bounces bounces, and when the budget runs out with a hit the leftover
//   path is not flown (662-668); reflect (637-671), reflect_with_log_weight (673-705) with the
//   side-dependent relaxivity multiplier; permeate (707-743) with one Powles decision at the first
//   hit and direction-dependent permeability; nearest-centroid classification (227-254) and the
//   leak guard that rejects a step whose decidable start and end classify differently (578-597).
// Periodic axes keep the position folded into the box plus an integer image count (the
// reference wraps an unfolded position each step, mesh.py:200-206).  The class and gather
// population of the current position are carried from the previous step instead of recomputed.
#pragma once
#include <math.h>
#include <stdint.h>

#include "geometry.cuh"

namespace dmsim {

struct MeshK {
  float gmin[3];
  float cs;          // grid cell size
  int dims[3];
  int per[3];
  float vmin[3], box[3];
  float eps, nudge, graze;
  int maxb;
  float rmi, rme, kmo, kmi;  // side multipliers of rho (intra/extra) and kappa (out/in)
  float kod;
  int reject;
  int seed_parity, seed_inside;
  const float4* tri;  // 4 x float4 per triangle: A, E1, E2, geometric normal, centroid, 1=original
  const float4* vn;   // 3 x float4 per triangle: smooth normals at the three vertices
  const float4* bs;   // optional bounding sphere per triangle (centre, radius)
  const uint32_t* cstart;
  const uint32_t* ctri;
  const uint32_t* nbstart;  // optional neighbourhood lists (see mesh_neighbourhood): one list
  const uint32_t* nbtri;    // per cell with the distinct triangles of its 27-cell gather
  const uint32_t* hstart;   // optional hit lists (see mesh_hit_list): the neighbourhood list's
  const uint32_t* htri;     // triangles within hreach of the cell, for the nearest-hit search
  const float4* hbs;        // optional: the hit-list entries' bounding spheres, in list order
  const float4* nbc;        // optional: the neighbourhood-list entries' centroids, in list order
  float hreach;
};

struct Tri {
  float ax, ay, az, e1x, e1y, e1z, e2x, e2y, e2z, nx, ny, nz;
};

// Per-warp shared-memory scratch of the cooperative candidate searches: each lane's list range,
// ray (or point), the inclusive prefix of the warp's list lengths, and the best key found.
struct MeshScratch {
  uint32_t incl[32];
  uint32_t ls[32];
  float rx[32], ry[32], rz[32], dx[32], dy[32], dz[32], rem[32];
  unsigned long long best[32];
};
constexpr size_t kMeshScratchBytes = sizeof(MeshScratch);

__device__ __forceinline__ Tri load_tri(const MeshK& m, uint32_t k) {
  const float4 a = m.tri[4 * k], b = m.tri[4 * k + 1], c = m.tri[4 * k + 2];
  return Tri{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
}

__device__ __forceinline__ int mesh_cell(float p, int a, const MeshK& m) {
  const int c = (int)floorf((p - m.gmin[a]) / m.cs);
  return min(max(c, 0), m.dims[a] - 1);
}

// The neighbourhood list of grid cell `cid`: the triangles of its 27 neighbour cells (indices
// clamped to the grid, neighbours in x-major order, each cell's triangles in increasing order)
// with every repeat after the first dropped.  A triangle larger than a cell is listed in several
// cells; a repeat is recognised by a binary search of the earlier neighbours' (sorted) lists.
// Writes the list to `out` when given; returns its length.
__device__ __forceinline__ uint32_t mesh_neighbourhood(const uint32_t* __restrict__ cs,
                                                       const uint32_t* __restrict__ ct,
                                                       const int* dims, int64_t cid,
                                                       uint32_t* __restrict__ out) {
  const int cz = (int)(cid % dims[2]);
  const int cy = (int)((cid / dims[2]) % dims[1]);
  const int cx = (int)(cid / ((int64_t)dims[1] * dims[2]));
  int nb[27];
#pragma unroll
  for (int d = 0; d < 27; ++d) {
    const int nx = min(max(cx + d / 9 - 1, 0), dims[0] - 1);
    const int ny = min(max(cy + (d / 3) % 3 - 1, 0), dims[1] - 1);
    const int nz = min(max(cz + d % 3 - 1, 0), dims[2] - 1);
    nb[d] = (nx * dims[1] + ny) * dims[2] + nz;
  }
  uint32_t n = 0;
#pragma unroll 1
  for (int d = 0; d < 27; ++d) {
    bool same_cell = false;
    for (int e = 0; e < d; ++e) same_cell |= nb[e] == nb[d];
    if (same_cell) continue;  // a clamped neighbour already visited whole
    const uint32_t kb = cs[nb[d]], ke = cs[nb[d] + 1];
#pragma unroll 1
    for (uint32_t k = kb; k < ke; ++k) {
      const uint32_t t = ct[k];
      bool seen = false;
#pragma unroll 1
      for (int e = 0; e < d && !seen; ++e) {
        uint32_t lo = cs[nb[e]], hi = cs[nb[e] + 1];  // lower bound of t in a sorted list
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (ct[mid] < t) lo = mid + 1; else hi = mid;
        }
        seen = lo < cs[nb[e] + 1] && ct[lo] == t;
      }
      if (seen) continue;
      if (out) out[n] = t;
      ++n;
    }
  }
  return n;
}

// Separating-axis test of a triangle (vertices relative to the box centre) against the box of
// half-extents h: false when a face axis of the box, the triangle's normal or one of the nine
// edge x box-axis cross products separates them.  A zero axis (degenerate triangle) separates
// nothing, so the test only errs towards overlap.
__device__ __forceinline__ bool tri_box_overlap(const double (&v)[3][3], const double (&h)[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double lo = fmin(v[0][a], fmin(v[1][a], v[2][a]));
    const double hi = fmax(v[0][a], fmax(v[1][a], v[2][a]));
    if (lo > h[a] || hi < -h[a]) return false;
  }
  double e[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int a = 0; a < 3; ++a) e[i][a] = v[(i + 1) % 3][a] - v[i][a];
  {
    // the triangle's plane: normal e0 x (v2 - v0) = -(e0 x e2)
    const double nx = e[2][1] * e[0][2] - e[2][2] * e[0][1];
    const double ny = e[2][2] * e[0][0] - e[2][0] * e[0][2];
    const double nz = e[2][0] * e[0][1] - e[2][1] * e[0][0];
    const double d = nx * v[0][0] + ny * v[0][1] + nz * v[0][2];
    const double r = fabs(nx) * h[0] + fabs(ny) * h[1] + fabs(nz) * h[2];
    if (fabs(d) > r) return false;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      // axis = e_i x unit_a
      double ax[3];
      ax[a] = 0.0;
      ax[(a + 1) % 3] = e[i][(a + 2) % 3];
      ax[(a + 2) % 3] = -e[i][(a + 1) % 3];
      const double p0 = ax[0] * v[0][0] + ax[1] * v[0][1] + ax[2] * v[0][2];
      const double p1 = ax[0] * v[1][0] + ax[1] * v[1][1] + ax[2] * v[1][2];
      const double p2 = ax[0] * v[2][0] + ax[1] * v[2][1] + ax[2] * v[2][2];
      const double r = fabs(ax[0]) * h[0] + fabs(ax[1]) * h[1] + fabs(ax[2]) * h[2];
      if (fmin(p0, fmin(p1, p2)) > r || fmax(p0, fmax(p1, p2)) < -r) return false;
    }
  }
  return true;
}

// The hit list of grid cell `cid` for steps no longer than `reach`: the entries of its
// neighbourhood list whose triangle overlaps the cell widened by reach + margin on every side.
// A step starting in the cell keeps its path (every bounce and nudge included) within its length
// of the start, so a triangle it can hit overlaps that box; the list keeps the neighbourhood
// order, so the first of equal hits is the same triangle.  The cells on the grid's faces also hold
// the positions clamped into the grid and keep their whole list.  Writes to `out` when given;
// returns the length.
__device__ __forceinline__ uint32_t mesh_hit_list(const uint32_t* __restrict__ nbs,
                                                  const uint32_t* __restrict__ nbt,
                                                  const float* __restrict__ tri, const int* dims,
                                                  const float* gmin, float cs, float reach,
                                                  int64_t cid, uint32_t* __restrict__ out,
                                                  const float4* __restrict__ bs,
                                                  float4* __restrict__ out_bs) {
  const int c[3] = {(int)(cid / ((int64_t)dims[1] * dims[2])), (int)((cid / dims[2]) % dims[1]),
                    (int)(cid % dims[2])};
  const uint32_t kb = nbs[cid], ke = nbs[cid + 1];
  bool face = false;
#pragma unroll
  for (int a = 0; a < 3; ++a) face |= c[a] == 0 || c[a] == dims[a] - 1;
  // widening: the reach, a relative allowance for the length of a float32 step, and an absolute
  // one far above the rounding of float32 positions, cell indices and hit points
  const double w = (double)reach * 1.001 + 4e-9 + 1e-5 * (double)cs;
  double ctr[3], h[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ctr[a] = (double)gmin[a] + ((double)c[a] + 0.5) * (double)cs;
    h[a] = 0.5 * (double)cs + w;
  }
  uint32_t n = 0;
#pragma unroll 1
  for (uint32_t k = kb; k < ke; ++k) {
    const uint32_t t = nbt[k];
    bool keep = face;
    if (!keep) {
      const float* r = tri + 16 * (size_t)t;
      double v[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double A = (double)r[a];
        v[0][a] = A - ctr[a];
        v[1][a] = A + (double)r[3 + a] - ctr[a];
        v[2][a] = A + (double)r[6 + a] - ctr[a];
      }
      keep = tri_box_overlap(v, h);
    }
    if (!keep) continue;
    if (out) out[n] = t;
    if (out_bs) out_bs[n] = bs[t];
    ++n;
  }
  return n;
}

// Visit every candidate of the 27-cell gather around p in the reference's order.  With the
// neighbourhood lists each distinct triangle is visited once, at its first position in that
// order; every use of the gather keeps the first of equal candidates (strict comparisons), so
// the result is the same as visiting the repeats.
template <typename Fn>
__device__ __forceinline__ void mesh_gather(const MeshK& m, float px, float py, float pz, Fn&& fn) {
  const int cx = mesh_cell(px, 0, m), cy = mesh_cell(py, 1, m), cz = mesh_cell(pz, 2, m);
  if (m.nbstart != nullptr) {
    const int cid = (cx * m.dims[1] + cy) * m.dims[2] + cz;
    const uint32_t e = m.nbstart[cid + 1];
#pragma unroll 1
    for (uint32_t k = m.nbstart[cid]; k < e; ++k) fn(m.nbtri[k]);
    return;
  }
#pragma unroll 1
  for (int dx = -1; dx <= 1; ++dx) {
    const int nx = min(max(cx + dx, 0), m.dims[0] - 1);
#pragma unroll 1
    for (int dy = -1; dy <= 1; ++dy) {
      const int ny = min(max(cy + dy, 0), m.dims[1] - 1);
#pragma unroll 1
      for (int dz = -1; dz <= 1; ++dz) {
        const int nz = min(max(cz + dz, 0), m.dims[2] - 1);
        const int cid = (nx * m.dims[1] + ny) * m.dims[2] + nz;
        const uint32_t e = m.cstart[cid + 1];
#pragma unroll 1
        for (uint32_t k = m.cstart[cid]; k < e; ++k) fn(m.ctri[k]);
      }
    }
  }
}

// Moller-Trumbore: ray r0 + t d against the triangle; returns t (INFINITY when the barycentric
// test fails) and the barycentric u, v.
__device__ __forceinline__ float mt_hit(const Tri& T, float r0x, float r0y, float r0z, float dx,
                                        float dy, float dz, float& u, float& v) {
  const float px = dy * T.e2z - dz * T.e2y, py = dz * T.e2x - dx * T.e2z,
              pz = dx * T.e2y - dy * T.e2x;
  const float det = px * T.e1x + py * T.e1y + pz * T.e1z;
  const float tx = r0x - T.ax, ty = r0y - T.ay, tz = r0z - T.az;
  const float qx = ty * T.e1z - tz * T.e1y, qy = tz * T.e1x - tx * T.e1z,
              qz = tx * T.e1y - ty * T.e1x;
  const float t = (qx * T.e2x + qy * T.e2y + qz * T.e2z) / det;
  u = (px * tx + py * ty + pz * tz) / det;
  v = (qx * dx + qy * dy + qz * dz) / det;
  const bool ok = (u >= 0.f) && (u <= 1.f) && (v >= 0.f) && (u + v <= 1.f);
  return ok ? t : INFINITY;
}

// Outgoing direction for a hit (mesh.py:599-635): reflect off the interpolated normal, then lift
// the ray above the triangle's own plane by the graze margin.  Also returns the oriented smooth
// normal n (for the relaxivity path length) and the oriented geometric normal nf (for the nudge).
__device__ __forceinline__ void mesh_bounce(const MeshK& m, uint32_t k, const Tri& T, float u,
                                            float v, float& dx, float& dy, float& dz, float& nx,
                                            float& ny, float& nz, float& fx, float& fy,
                                            float& fz) {
  const float4 a = m.vn[3 * k], b = m.vn[3 * k + 1], c = m.vn[3 * k + 2];
  const float w = 1.f - u - v;
  float sx = w * a.x + u * a.w + v * b.z;
  float sy = w * a.y + u * b.x + v * b.w;
  float sz = w * a.z + u * b.y + v * c.x;
  const float sl = sqrtf(sx * sx + sy * sy + sz * sz);
  sx /= sl;
  sy /= sl;
  sz /= sl;
  const bool flip = (dx * T.nx + dy * T.ny + dz * T.nz) > 0.f;
  nx = flip ? -sx : sx;
  ny = flip ? -sy : sy;
  nz = flip ? -sz : sz;
  fx = flip ? -T.nx : T.nx;
  fy = flip ? -T.ny : T.ny;
  fz = flip ? -T.nz : T.nz;
  const float dn = dx * nx + dy * ny + dz * nz;
  float rx = dx - 2.f * dn * nx, ry = dy - 2.f * dn * ny, rz = dz - 2.f * dn * nz;
  float rl = sqrtf(rx * rx + ry * ry + rz * rz);
  rx /= rl;
  ry /= rl;
  rz /= rl;
  const float cf = rx * fx + ry * fy + rz * fz;
  if (cf < m.graze) {
    rx += (m.graze - cf) * fx;
    ry += (m.graze - cf) * fy;
    rz += (m.graze - cf) * fz;
    rl = sqrtf(rx * rx + ry * ry + rz * rz);
    rx /= rl;
    ry /= rl;
    rz /= rl;
  }
  dx = rx;
  dy = ry;
  dz = rz;
}

// Nearest hit of the gathered candidates (first index on ties, like argmin).
struct MeshHit {
  float t, u, v;
  uint32_t k;
};

__device__ __forceinline__ MeshHit mesh_nearest(const MeshK& m, float gx, float gy, float gz,
                                                float r0x, float r0y, float r0z, float dx,
                                                float dy, float dz, float rem) {
  MeshHit h{INFINITY, 0.f, 0.f, 0u};
  mesh_gather(m, gx, gy, gz, [&](uint32_t k) {
    if (m.bs != nullptr) {
      // a triangle whose bounding sphere misses the segment r0 + s d, s in [0, rem], cannot
      // be hit within the step (the sphere covers the float32 triangle with a margin)
      const float4 b = __ldg(m.bs + k);
      const float cx = b.x - r0x, cy = b.y - r0y, cz = b.z - r0z;
      const float s = fminf(fmaxf(cx * dx + cy * dy + cz * dz, 0.f), rem);
      const float ex = cx - s * dx, ey = cy - s * dy, ez = cz - s * dz;
      if (ex * ex + ey * ey + ez * ez > b.w * b.w) return;
    }
    const Tri T = load_tri(m, k);
    float u, v;
    const float t = mt_hit(T, r0x, r0y, r0z, dx, dy, dz, u, v);
    if (t > m.eps && t < rem && t < h.t) {
      h.t = t;
      h.u = u;
      h.v = v;
      h.k = k;
    }
  });
  return h;
}

// Class of a point (0 interior, 1 exterior) and whether its gather holds any triangle.
__device__ __forceinline__ int mesh_classify(const MeshK& m, float px, float py, float pz,
                                             int& populated) {
  float best = INFINITY;
  uint32_t kb = 0;
  int any = 0;
  mesh_gather(m, px, py, pz, [&](uint32_t k) {
    const float4 c = m.tri[4 * k + 3];
    const float ddx = px - c.x, ddy = py - c.y, ddz = pz - c.z;
    const float d = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
    any = 1;
    if (d < best) {
      best = d;
      kb = k;
    }
  });
  populated = any;
  if (!any) return 1;
  const float4 c = m.tri[4 * kb + 3];
  const float4 nn = m.tri[4 * kb + 2];
  const float side = (px - c.x) * nn.y + (py - c.y) * nn.z + (pz - c.z) * nn.w;
  return side < 0.f ? 0 : 1;
}

// Inside-ness by the parity of crossings of a ray along +x through the grid row of p (original
// triangles only; each crossing counted in the cell that holds its hit point).
__device__ __forceinline__ int mesh_parity(const MeshK& m, float px, float py, float pz) {
  const int cy = mesh_cell(py, 1, m), cz = mesh_cell(pz, 2, m);
  int parity = 0;
#pragma unroll 1
  for (int cx = mesh_cell(px, 0, m); cx < m.dims[0]; ++cx) {
    const int cid = (cx * m.dims[1] + cy) * m.dims[2] + cz;
    const uint32_t e = m.cstart[cid + 1];
#pragma unroll 1
    for (uint32_t i = m.cstart[cid]; i < e; ++i) {
      const uint32_t k = m.ctri[i];
      if (m.tri[4 * k + 3].w == 0.f) continue;  // periodic ghost
      const Tri T = load_tri(m, k);
      float u, v;
      const float t = mt_hit(T, px, py, pz, 1.f, 0.f, 0.f, u, v);
      if (t > 0.f && t < INFINITY && mesh_cell(px + t, 0, m) == cx) parity ^= 1;
    }
  }
  return parity;
}

__device__ __forceinline__ void mesh_fold(float& v, int& img, int a, const MeshK& m) {
  if (!m.per[a]) return;
  const float hi = m.vmin[a] + m.box[a];
  if (v >= hi) {
    v -= m.box[a];
    ++img;
  } else if (v < m.vmin[a]) {
    v += m.box[a];
    --img;
  }
}

// One sub-step.  (x, y, z) is the folded position; cls / pop carry the class and gather
// population of the current position (the leak guard's start state).  Returns -2 * sum d_perp
// including the side multipliers (rho/D = 1).
// ---- warp-cooperative candidate searches -----------------------------------------------------
// Every lane of the warp calls these together (the walk keeps all 32 lanes in step).  A lane's
// neighbourhood list can hold from none to dozens of triangles, so a lane-per-walker scan runs as
// long as the warp's longest list while most lanes idle.  Here the warp lays the (walker,
// candidate) pairs of all its lanes end to end and tests 32 pairs per round; each pair's result
// goes to its walker's slot as a 64-bit key (distance bits, list position), so the minimum is the
// nearest candidate and, among equal distances, the first in list order -- exactly what the
// sequential scan with strict comparisons returns.
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

__device__ __forceinline__ int scratch_owner(const MeshScratch* w, uint32_t j) {
  int lo = 0, hi = 31;  // first lane whose inclusive prefix exceeds j
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (w->incl[mid] > j) hi = mid; else lo = mid + 1;
  }
  return lo;
}

__device__ __forceinline__ MeshHit mesh_nearest_coop(const MeshK& m, MeshScratch* w, bool need,
                                                     bool hit_lists, float gx, float gy,
                                                     float gz, float r0x, float r0y, float r0z,
                                                     float dx, float dy, float dz, float rem) {
  const int lane = threadIdx.x & 31;
  const uint32_t* __restrict__ lst = hit_lists ? m.hstart : m.nbstart;
  const uint32_t* __restrict__ ltri = hit_lists ? m.htri : m.nbtri;
  const float4* __restrict__ lbs = hit_lists ? m.hbs : nullptr;  // spheres in list order
  uint32_t ls = 0, cnt = 0;
  if (need) {
    const int cid = (mesh_cell(gx, 0, m) * m.dims[1] + mesh_cell(gy, 1, m)) * m.dims[2] +
                    mesh_cell(gz, 2, m);
    ls = lst[cid];
    cnt = lst[cid + 1] - ls;
  }
  const uint32_t incl = warp_incl_scan(cnt, lane);
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  MeshHit h{INFINITY, 0.f, 0.f, 0u};
  if (total == 0) return h;
  w->incl[lane] = incl;
  w->ls[lane] = ls;
  w->rx[lane] = r0x; w->ry[lane] = r0y; w->rz[lane] = r0z;
  w->dx[lane] = dx; w->dy[lane] = dy; w->dz[lane] = dz;
  w->rem[lane] = rem;
  w->best[lane] = ~0ull;
  __syncwarp();
#pragma unroll 1
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t j = base + lane;
    if (j < total) {
      const int L = scratch_owner(w, j);
      const uint32_t pos = j - (L ? w->incl[L - 1] : 0u);
      const uint32_t li = w->ls[L] + pos;
      const uint32_t k = ltri[li];
      const float ox = w->rx[L], oy = w->ry[L], oz = w->rz[L];
      const float ux = w->dx[L], uy = w->dy[L], uz = w->dz[L], rm = w->rem[L];
      bool test = true;
      if (m.bs != nullptr) {
        const float4 b = lbs != nullptr ? __ldg(lbs + li) : __ldg(m.bs + k);
        const float cx = b.x - ox, cy = b.y - oy, cz = b.z - oz;
        const float s = fminf(fmaxf(cx * ux + cy * uy + cz * uz, 0.f), rm);
        const float ex = cx - s * ux, ey = cy - s * uy, ez = cz - s * uz;
        test = ex * ex + ey * ey + ez * ez <= b.w * b.w;
      }
      if (test) {
        const Tri T = load_tri(m, k);
        float u, v;
        const float t = mt_hit(T, ox, oy, oz, ux, uy, uz, u, v);
        if (t > m.eps && t < rm)
          atomicMin(&w->best[L], ((unsigned long long)__float_as_uint(t) << 32) | pos);
      }
    }
  }
  __syncwarp();
  const unsigned long long b = w->best[lane];
  __syncwarp();
  if (need && b != ~0ull) {
    const uint32_t k = ltri[ls + (uint32_t)(b & 0xffffffffull)];
    const Tri T = load_tri(m, k);
    float u, v;
    h.t = mt_hit(T, r0x, r0y, r0z, dx, dy, dz, u, v);
    h.u = u;
    h.v = v;
    h.k = k;
  }
  return h;
}

__device__ __forceinline__ int mesh_classify_coop(const MeshK& m, MeshScratch* w, float px,
                                                  float py, float pz, int& populated) {
  const int lane = threadIdx.x & 31;
  const int cid = (mesh_cell(px, 0, m) * m.dims[1] + mesh_cell(py, 1, m)) * m.dims[2] +
                  mesh_cell(pz, 2, m);
  const uint32_t ls = m.nbstart[cid];
  const uint32_t cnt = m.nbstart[cid + 1] - ls;
  const uint32_t incl = warp_incl_scan(cnt, lane);
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  populated = cnt > 0;
  if (total == 0) return 1;
  w->incl[lane] = incl;
  w->ls[lane] = ls;
  w->rx[lane] = px; w->ry[lane] = py; w->rz[lane] = pz;
  w->best[lane] = ~0ull;
  __syncwarp();
#pragma unroll 1
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t j = base + lane;
    if (j < total) {
      const int L = scratch_owner(w, j);
      const uint32_t pos = j - (L ? w->incl[L - 1] : 0u);
      const uint32_t li = w->ls[L] + pos;
      const float4 c = m.nbc != nullptr ? __ldg(m.nbc + li) : m.tri[4 * m.nbtri[li] + 3];
      const float ddx = w->rx[L] - c.x, ddy = w->ry[L] - c.y, ddz = w->rz[L] - c.z;
      const float d = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
      atomicMin(&w->best[L], ((unsigned long long)__float_as_uint(d) << 32) | pos);
    }
  }
  __syncwarp();
  const unsigned long long b = w->best[lane];
  __syncwarp();
  if (cnt == 0) return 1;
  const uint32_t kb = m.nbtri[ls + (uint32_t)(b & 0xffffffffull)];
  const float4 c = m.tri[4 * kb + 3];
  const float4 nn = m.tri[4 * kb + 2];
  const float side = (px - c.x) * nn.y + (py - c.y) * nn.z + (pz - c.z) * nn.w;
  return side < 0.f ? 0 : 1;
}

template <int WALL>
// All 32 lanes of a warp call mesh_step together: with neighbourhood lists the candidate searches
// are warp-cooperative (each lane's outcome is the one its own sequential search gives).
__device__ __forceinline__ float mesh_step(float& x, float& y, float& z, int& ix, int& iy,
                                           int& iz, int& cls, int& pop, float sx, float sy,
                                           float sz, float u_rand, const MeshK& m, Tally& tl,
                                           uint32_t& n_budget, uint32_t& n_escape,
                                           MeshScratch* ws) {
  const bool coop = m.nbstart != nullptr;
  const float l = sqrtf(sx * sx + sy * sy + sz * sz);
  // the hit lists serve the warp's searches when every lane's step is within their reach
  const bool hit_lists =
      coop && m.hstart != nullptr && __all_sync(0xffffffffu, l <= m.hreach);
  float dx = sx / l, dy = sy / l, dz = sz / l;
  float r0x = x, r0y = y, r0z = z, rem = l;
  float dsum = 0.f;
  bool last_reflect = false;
  bool decided = false;
  bool active = true;  // this lane is still bouncing
#pragma unroll 1
  for (int it = 0; it < m.maxb; ++it) {
    if (coop ? !__any_sync(0xffffffffu, active) : !active) break;
    const MeshHit h = coop ? mesh_nearest_coop(m, ws, active, hit_lists, x, y, z, r0x, r0y,
                                               r0z, dx, dy, dz, rem)
                           : mesh_nearest(m, x, y, z, r0x, r0y, r0z, dx, dy, dz, rem);
    if (!active) continue;
    const bool hit = h.t < INFINITY;
    if constexpr (WALL != kPermeate) {
      if (!hit) {
        last_reflect = false;
        active = false;
        continue;
      }
      const Tri T = load_tri(m, h.k);
      const bool outward = (dx * T.nx + dy * T.ny + dz * T.nz) > 0.f;
      float ndx = dx, ndy = dy, ndz = dz, nx, ny, nz, fx, fy, fz;
      mesh_bounce(m, h.k, T, h.u, h.v, ndx, ndy, ndz, nx, ny, nz, fx, fy, fz);
      if constexpr (WALL == kRelax) {
        const float cos_a = -(dx * nx + dy * ny + dz * nz);
        dsum += (outward ? m.rmi : m.rme) * (rem - h.t) * cos_a;
      }
      r0x = r0x + h.t * dx + m.nudge * fx;
      r0y = r0y + h.t * dy + m.nudge * fy;
      r0z = r0z + h.t * dz + m.nudge * fz;
      dx = ndx;
      dy = ndy;
      dz = ndz;
      rem = rem - h.t - m.nudge;
      last_reflect = true;
    } else {
      bool do_reflect = false;
      if (hit) {
        const Tri T = load_tri(m, h.k);
        const bool outward = (dx * T.nx + dy * T.ny + dz * T.nz) > 0.f;
        float ndx = dx, ndy = dy, ndz = dz, nx, ny, nz, fx, fy, fz;
        mesh_bounce(m, h.k, T, h.u, h.v, ndx, ndy, ndz, nx, ny, nz, fx, fy, fz);
        const float cos_a = -(dx * nx + dy * ny + dz * nz);
        const float dperp = (rem - h.t) * cos_a;
        const bool first = !decided;
        const float p = fminf(1.f, 2.f * m.kod * (outward ? m.kmo : m.kmi) * dperp);
        const bool transmit = first && (u_rand < p);
        do_reflect = !transmit;
        if (first && !transmit) dsum += (outward ? m.rmi : m.rme) * dperp;
        if (transmit) ++tl.transmit;
        decided = true;
        if (do_reflect) {
          r0x = r0x + h.t * dx + m.nudge * fx;
          r0y = r0y + h.t * dy + m.nudge * fy;
          r0z = r0z + h.t * dz + m.nudge * fz;
          dx = ndx;
          dy = ndy;
          dz = ndz;
          rem = rem - h.t - m.nudge;
        }
      }
      last_reflect = do_reflect;
      if (!do_reflect) {  // no hit or a transmission: fly the rest of the step straight
        r0x += rem * dx;
        r0y += rem * dy;
        r0z += rem * dz;
        rem = 0.f;
        active = false;
      }
    }
  }
  if (last_reflect) ++n_budget;  // the budget ran out with a hit: the leftover is not flown
  const float f = last_reflect ? 0.f : fmaxf(rem, 0.f);
  float nxp = r0x + dx * f, nyp = r0y + dy * f, nzp = r0z + dz * f;
  int jx = ix, jy = iy, jz = iz;
  mesh_fold(nxp, jx, 0, m);
  mesh_fold(nyp, jy, 1, m);
  mesh_fold(nzp, jz, 2, m);
  if constexpr (WALL != kPermeate) {
    if (m.reject) {
      int pop_new;
      const int cls_new = coop ? mesh_classify_coop(m, ws, nxp, nyp, nzp, pop_new)
                               : mesh_classify(m, nxp, nyp, nzp, pop_new);
      if (pop && pop_new && cls_new != cls) {
        ++n_escape;  // leak guard: a decidable class change without a crossing
        return 0.f;
      }
      cls = cls_new;
      pop = pop_new;
    }
  }
  x = nxp;
  y = nyp;
  z = nzp;
  ix = jx;
  iy = jy;
  iz = jz;
  return -2.f * dsum;
}

}  // namespace dmsim
