// Closest triangle and signed distance over a built soup tree.
//
// Reference: igl::signed_distance (include/igl/signed_distance.cpp:20-137,
// 372-440) for 3-D triangle meshes with every sign type, and the closest-point
// query it runs per point, igl::AABB::squared_distance
// (include/igl/AABB.cpp:1135-1205) with point_simplex_squared_distance
// (include/igl/point_simplex_squared_distance.cpp:40-124), and the
// PSEUDONORMAL sign: the angle-weighted pseudonormal of the closest feature
// (pseudonormal_test.cpp:16-135 over per_face_normals, per_vertex_normals
// with angle weights and per_edge_normals with uniform weights).
//
// The reference builds an AABB tree; here the closest-triangle query uses
// the soup tree that the fast winding number already has, with an FP32 box
// per node rounded outward: one thread per query searches depth-first,
// nearer child first, and prunes a subtree when its box lower bound (minus
// a slack covering the FP32 rounding of the query and the arithmetic) is at
// least the distance found so far -- the order of the reference's
// AABB::squared_distance.  Leaves are evaluated in FP64.  For a tree deeper
// than the search stack, a warp-coherent walk over the pre-order array
// (bounding-sphere pruning after a greedy descent) is used instead.
// Triangle distance: the closest point by Voronoi region (Ericson, Real-Time
// Collision Detection 5.1.5; the reference's region order and its a == b
// guard), squared distance from the closest point.  A strictly smaller
// distance replaces the current one, so in a tie the first triangle reached
// is kept (the reference's tree reaches its own first).
#include <cuda_runtime.h>

#include <cmath>
#include <limits>

#include "bh_common.cuh"
#include "gwn_common.cuh"
#include "gwn_internal.cuh"
#include "soup.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 daxpy(D3 a, double s, D3 d) {
  return {a.x + s * d.x, a.y + s * d.y, a.z + s * d.z};
}

__device__ D3 closest_on_triangle(D3 p, D3 a, D3 b, D3 c) {
  const D3 ab = dsub(b, a), ac = dsub(c, a), ap = dsub(p, a);
  const double d1 = ddot(ab, ap), d2 = ddot(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return a;
  const D3 bp = dsub(p, b);
  const double d3 = ddot(ab, bp), d4 = ddot(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return b;
  const double vc = d1 * d4 - d3 * d2;
  const bool a_is_b = a.x == b.x && a.y == b.y && a.z == b.z;
  if (!a_is_b && vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return daxpy(a, d1 / (d1 - d3), ab);
  const D3 cp = dsub(p, c);
  const double d5 = ddot(ab, cp), d6 = ddot(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return c;
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return daxpy(a, d2 / (d2 - d6), ac);
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0)
    return daxpy(b, (d4 - d3) / ((d4 - d3) + (d5 - d6)), dsub(c, b));
  const double denom = 1.0 / (va + vb + vc);
  return daxpy(daxpy(a, vb * denom, ab), vc * denom, ac);
}

struct ClosestParams {
  const SoupNodeF* nf;
  const float4* snode;
  const float4* tf;
  const double* td;
  const int32_t* tri_index;
  int nnodes;
  float cmax;
};

// Depth-first search stack entries per thread (node, lower bound); the tree's
// depth must stay below it (checked on the host, else the walk is used).
constexpr int kStack = 96;

// Best candidate so far: squared distance, slot, closest point, and an FP32
// upper bound of the distance (sqrt(d2) rounded up) for the pruning tests.
struct Best {
  double d2;
  int slot;
  D3 c;
  float bound;
};

__device__ __forceinline__ float dist_bound(double d2) {
  return __fsqrt_ru(__double2float_ru(d2));
}

// Squared distance from p to triangle (a, b, c) in FP32, same regions.
__device__ float dist2_triangle32(float px, float py, float pz, float ax, float ay, float az,
                                  float bx, float by, float bz, float cx, float cy, float cz) {
  const float abx = bx - ax, aby = by - ay, abz = bz - az;
  const float acx = cx - ax, acy = cy - ay, acz = cz - az;
  const float apx = px - ax, apy = py - ay, apz = pz - az;
  const float d1 = abx * apx + aby * apy + abz * apz, d2 = acx * apx + acy * apy + acz * apz;
  float qx, qy, qz;
  if (d1 <= 0.f && d2 <= 0.f) {
    qx = ax; qy = ay; qz = az;
  } else {
    const float bpx = px - bx, bpy = py - by, bpz = pz - bz;
    const float d3 = abx * bpx + aby * bpy + abz * bpz, d4 = acx * bpx + acy * bpy + acz * bpz;
    const float vc = d1 * d4 - d3 * d2;
    const float cpx = px - cx, cpy = py - cy, cpz = pz - cz;
    const float d5 = abx * cpx + aby * cpy + abz * cpz, d6 = acx * cpx + acy * cpy + acz * cpz;
    const float vb = d5 * d2 - d1 * d6;
    const float va = d3 * d6 - d5 * d4;
    if (d3 >= 0.f && d4 <= d3) {
      qx = bx; qy = by; qz = bz;
    } else if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) {
      const float v = d1 / (d1 - d3);
      qx = ax + v * abx; qy = ay + v * aby; qz = az + v * abz;
    } else if (d6 >= 0.f && d5 <= d6) {
      qx = cx; qy = cy; qz = cz;
    } else if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) {
      const float w = d2 / (d2 - d6);
      qx = ax + w * acx; qy = ay + w * acy; qz = az + w * acz;
    } else if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) {
      const float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
      qx = bx + w * (cx - bx); qy = by + w * (cy - by); qz = bz + w * (cz - bz);
    } else {
      const float denom = 1.f / (va + vb + vc);
      const float v = vb * denom, w = vc * denom;
      qx = ax + abx * v + acx * w; qy = ay + aby * v + acy * w; qz = az + abz * v + acz * w;
    }
  }
  const float dx = px - qx, dy = py - qy, dz = pz - qz;
  return dx * dx + dy * dy + dz * dz;
}

// FP32 screen of a leaf: true when the triangle is farther than the
// current best (its FP32 distance minus the triangle's stored slack and the
// query-rounding slack 1e-6 (S + d) is above the best's upper bound).
__device__ __forceinline__ bool screened_out(const ClosestParams& prm, int slot, float fx,
                                             float fy, float fz, float S, float bound) {
  const float4 t0 = __ldg(&prm.tf[(int64_t)slot * 3]);
  const float4 t1 = __ldg(&prm.tf[(int64_t)slot * 3 + 1]);
  const float4 t2 = __ldg(&prm.tf[(int64_t)slot * 3 + 2]);
  const float d = sqrtf(dist2_triangle32(fx, fy, fz, t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z,
                                         t1.w, t2.x));
  const float lower = d - t2.y - 1e-6f * (S + d);
  return lower > bound;
}

// FP32 bounds of the distance from q to a leaf's triangle: its FP32
// distance minus / plus the triangle's stored slack and the query-rounding
// slack 1e-6 (S + d).
__device__ __forceinline__ void leaf_bounds(const ClosestParams& prm, int slot, float fx, float fy,
                                            float fz, float S, float& lower, float& upper) {
  const float4 t0 = __ldg(&prm.tf[(int64_t)slot * 3]);
  const float4 t1 = __ldg(&prm.tf[(int64_t)slot * 3 + 1]);
  const float4 t2 = __ldg(&prm.tf[(int64_t)slot * 3 + 2]);
  const float d = sqrtf(dist2_triangle32(fx, fy, fz, t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z,
                                         t1.w, t2.x));
  const float e = t2.y + 1e-6f * (S + d);
  lower = d - e;
  upper = __fadd_ru(d, e);
}

// A candidate replaces the best when strictly closer, or equally close with
// a smaller input triangle index: with pruning only of what is strictly
// farther, every triangle at the smallest distance is evaluated, so the
// result does not depend on the visiting order.
__device__ __forceinline__ void eval_leaf(const ClosestParams& prm, int slot, D3 q, Best& b) {
  const double* t = prm.td + (int64_t)slot * 9;
  const D3 cp = closest_on_triangle(q, {t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]});
  const D3 d = dsub(q, cp);
  const double d2 = ddot(d, d);
  if (d2 < b.d2 || (d2 == b.d2 && b.slot >= 0 && prm.tri_index[slot] < prm.tri_index[b.slot])) {
    b.d2 = d2;
    b.slot = slot;
    b.c = cp;
    b.bound = dist_bound(d2);
  }
}

// FP32 lower bound of the distance from q to anything inside node r's
// sphere, lowered by a slack that covers the rounding of q and P to FP32
// (u |q|, u |P| per coordinate, u = 2^-24) and of the norm and sqrt
// (a few u of d and R): 1e-6 (S + d + R) with S = max|q| + max|P| is more
// than four times that bound.
__device__ __forceinline__ float sphere_lower_bound(const float4 a, float fx, float fy, float fz,
                                                    float S) {
  const float dx = fx - a.x, dy = fy - a.y, dz = fz - a.z;
  const float d = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
  const float R = sqrtf(a.w);
  return d - R - 1e-6f * (S + d + R);
}

__device__ __forceinline__ int node_link(const SoupNodeF* nf, int n) {
  return __float_as_int(__ldg(&nf[n].f).w);
}

template <typename QT>
__global__ void __launch_bounds__(128) closest_kernel(ClosestParams prm, const QT* __restrict__ Q,
                                                      const int32_t* __restrict__ perm,
                                                      int64_t nQ, double up_sqr_d,
                                                      double* __restrict__ sqrD,
                                                      int32_t* __restrict__ I,
                                                      double* __restrict__ C) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool valid = i < nQ;
  int64_t qi = 0;
  D3 q{0, 0, 0};
  if (valid) {
    qi = perm ? (int64_t)perm[i] : i;
    q = {(double)Q[qi * 3], (double)Q[qi * 3 + 1], (double)Q[qi * 3 + 2]};
  }
  const bool finite = isfinite(q.x) && isfinite(q.y) && isfinite(q.z);
  const bool walk = valid && finite && prm.nnodes > 0;
  const float fx = (float)q.x, fy = (float)q.y, fz = (float)q.z;
  const float S = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) + prm.cmax;
  Best b{up_sqr_d, -1, {0, 0, 0}, dist_bound(up_sqr_d)};
  // 1. greedy descent to one leaf: an initial bound
  if (walk) {
    int n = 0;
    for (int depth = 0; depth < prm.nnodes; ++depth) {
      const int link = node_link(prm.nf, n);
      if (link < 0) {
        eval_leaf(prm, ~link, q, b);
        break;
      }
      const int l = n + 1;
      const int ll = node_link(prm.nf, l);
      const int r = ll < 0 ? l + 1 : ll;
      const float lbl = sphere_lower_bound(__ldg(&prm.nf[l].a), fx, fy, fz, S);
      const float lbr = sphere_lower_bound(__ldg(&prm.nf[r].a), fx, fy, fz, S);
      n = lbl <= lbr ? l : r;
    }
  }
  // 2. the warp-coherent pruned walk (kept for trees deeper than kStack)
  int resume = walk ? 0 : 0x7fffffff;
  int node = 0;
  const unsigned full = 0xffffffffu;
  while (node < prm.nnodes) {
    const float4 a = __ldg(&prm.nf[node].a);
    const int link = node_link(prm.nf, node);
    bool open = false;
    if (node >= resume) {
      const bool leaf = link < 0;
      const float lb = sphere_lower_bound(a, fx, fy, fz, S);
      if (lb > b.bound) {
        resume = leaf ? node + 1 : link;
      } else if (leaf) {
        eval_leaf(prm, ~link, q, b);
        resume = node + 1;
      } else {
        open = true;
      }
    }
    if (__any_sync(full, open))
      node = node + 1;
    else
      node = __reduce_min_sync(full, resume);
  }
  if (!valid) return;
  sqrD[qi] = b.d2;
  I[qi] = b.slot >= 0 ? prm.tri_index[b.slot] : -1;
  C[qi * 3] = b.c.x;
  C[qi * 3 + 1] = b.c.y;
  C[qi * 3 + 2] = b.c.z;
}

// Conservative FP32 lower bound of the distance from q to a box (lo, hi):
// the box is rounded outward to FP32; the query's rounding to FP32 and the
// FP32 arithmetic move the exterior distance by at most a few u
// (|q| + |box| + d), covered by the slack 1e-6 (S + d).
__device__ __forceinline__ float box_lower_bound(const float4 lo, const float4 hi, float fx,
                                                 float fy, float fz, float S) {
  const float dx = fmaxf(fmaxf(lo.x - fx, fx - hi.x), 0.f);
  const float dy = fmaxf(fmaxf(lo.y - fy, fy - hi.y), 0.f);
  const float dz = fmaxf(fmaxf(lo.z - fz, fz - hi.z), 0.f);
  const float d = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
  return fmaxf(d - 1e-6f * (S + d), 0.f);
}

// Closest triangle by depth-first search over the search nodes, nearer
// child first, pruned by the children's box lower bounds: the order of
// igl::AABB::squared_distance (AABB.cpp:1180-1203).  One query per thread;
// one 64-byte search node per internal visit, leaves go straight to their
// triangle.  A push beyond the stack (the host picks this kernel only for
// trees shallower than kStack) is reported instead of written.
template <typename QT>
__global__ void __launch_bounds__(128) closest_dfs_kernel(ClosestParams prm,
                                                          const QT* __restrict__ Q,
                                                          const int32_t* __restrict__ perm,
                                                          int64_t nQ, double up_sqr_d,
                                                          double* __restrict__ sqrD,
                                                          int32_t* __restrict__ I,
                                                          double* __restrict__ C,
                                                          unsigned* __restrict__ status) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nQ) return;
  const int64_t qi = perm ? (int64_t)perm[i] : i;
  const D3 q{(double)Q[qi * 3], (double)Q[qi * 3 + 1], (double)Q[qi * 3 + 2]};
  Best b{up_sqr_d, -1, {0, 0, 0}, dist_bound(up_sqr_d)};
  if (isfinite(q.x) && isfinite(q.y) && isfinite(q.z) && prm.nnodes > 0) {
    const float fx = (float)q.x, fy = (float)q.y, fz = (float)q.z;
    const float S = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) + prm.cmax;
    // ub: an FP32 upper bound of the best distance (the smallest FP32 upper
    // bound of any leaf seen, or of the FP64 best).  A leaf whose FP32 lower
    // bound is within ub becomes a candidate; the FP64 closest point is
    // computed only for the candidates still within ub at the end (or when
    // the four candidate slots are full), so every triangle that can be the
    // closest, ties included, is evaluated in FP64 as before.
    float ub = b.bound;
    int cs0 = 0, cs1 = 0, cs2 = 0, cs3 = 0;
    float cl0 = 0.f, cl1 = 0.f, cl2 = 0.f, cl3 = 0.f;
    int nc = 0;
    auto flush = [&]() {
      if (nc > 0 && !(cl0 > ub)) eval_leaf(prm, cs0, q, b);
      if (nc > 1 && !(cl1 > ub)) eval_leaf(prm, cs1, q, b);
      if (nc > 2 && !(cl2 > ub)) eval_leaf(prm, cs2, q, b);
      if (nc > 3 && !(cl3 > ub)) eval_leaf(prm, cs3, q, b);
      nc = 0;
      ub = fminf(ub, b.bound);
    };
    int stk_n[kStack];
    float stk_lb[kStack];
    int sp = 0;
    stk_n[sp] = prm.nnodes > 1 ? 0 : ~0;  // root: internal node 0, or the only leaf
    stk_lb[sp] = 0.f;
    ++sp;
    while (sp > 0) {
      --sp;
      const int ref = stk_n[sp];
      const float lb = stk_lb[sp];
      if (lb > ub) continue;
      if (ref < 0) {
        float lower, upper;
        leaf_bounds(prm, ~ref, fx, fy, fz, S, lower, upper);
        if (!(lower > ub)) {
          if (nc == 4) flush();
          if (nc == 0) { cs0 = ~ref; cl0 = lower; }
          else if (nc == 1) { cs1 = ~ref; cl1 = lower; }
          else if (nc == 2) { cs2 = ~ref; cl2 = lower; }
          else { cs3 = ~ref; cl3 = lower; }
          ++nc;
          ub = fminf(ub, upper);
        }
        continue;
      }
      const float4* sn = prm.snode + 4 * (int64_t)ref;
      const float4 lo_l = __ldg(sn), hi_l = __ldg(sn + 1), lo_r = __ldg(sn + 2),
                   hi_r = __ldg(sn + 3);
      const int l = __float_as_int(lo_l.w), r = __float_as_int(hi_l.w);
      const float lbl = box_lower_bound(lo_l, hi_l, fx, fy, fz, S);
      const float lbr = box_lower_bound(lo_r, hi_r, fx, fy, fz, S);
      const bool left_first = lbl <= lbr;
      const int far_n = left_first ? r : l, near_n = left_first ? l : r;
      const float far_lb = left_first ? lbr : lbl, near_lb = left_first ? lbl : lbr;
      if (!(far_lb > ub)) {
        if (sp == kStack) {
          atomicOr(status, kStatusBadInput);
          break;
        }
        stk_n[sp] = far_n;
        stk_lb[sp] = far_lb;
        ++sp;
      }
      if (!(near_lb > ub)) {
        if (sp == kStack) {
          atomicOr(status, kStatusBadInput);
          break;
        }
        stk_n[sp] = near_n;
        stk_lb[sp] = near_lb;
        ++sp;
      }
    }
    flush();
  }
  sqrD[qi] = b.d2;
  I[qi] = b.slot >= 0 ? prm.tri_index[b.slot] : -1;
  C[qi * 3] = b.c.x;
  C[qi * 3 + 1] = b.c.y;
  C[qi * 3 + 2] = b.c.z;
}

// ------------------------------------------------------------ pseudonormal --
// The normals of SIGNED_DISTANCE_TYPE_PSEUDONORMAL (signed_distance.cpp:
// 69-76): per_face_normals, per_vertex_normals with angle weights,
// per_edge_normals with uniform weights; sums in the reference's loop order.
__device__ __forceinline__ D3 vrow(const double* V, const int32_t* F, int64_t f, int c) {
  const double* p = V + (int64_t)F[f * 3 + c] * 3;
  return {p[0], p[1], p[2]};
}
__device__ __forceinline__ double dnorm(D3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// per_face_normals.cpp:17-30: (V1-V0) x (V2-V0), normalised; zero stays zero.
__global__ void face_normals_kernel(const double* __restrict__ V, const int32_t* __restrict__ F,
                                    int64_t nF, double* __restrict__ FN) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (f >= nF) return;
  const D3 a = vrow(V, F, f, 0), v1 = dsub(vrow(V, F, f, 1), a), v2 = dsub(vrow(V, F, f, 2), a);
  D3 n{v1.y * v2.z - v1.z * v2.y, v1.z * v2.x - v1.x * v2.z, v1.x * v2.y - v1.y * v2.x};
  const double r = dnorm(n);
  if (r == 0) n = {0, 0, 0};
  else n = {n.x / r, n.y / r, n.z / r};
  FN[f * 3] = n.x;
  FN[f * 3 + 1] = n.y;
  FN[f * 3 + 2] = n.z;
}

// internal_angles.cpp:15-38: the corner angle 2 atan(|u1 - u2| / |u1 + u2|)
// of unit edge vectors; entries keyed for the per-vertex sums.
__global__ void corner_entries_kernel(const double* __restrict__ V, const int32_t* __restrict__ F,
                                      int64_t nF, double* __restrict__ angle,
                                      uint32_t* __restrict__ vkey, int32_t* __restrict__ ventry,
                                      unsigned long long* __restrict__ ekey,
                                      int32_t* __restrict__ eentry) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nF * 3) return;
  const int64_t f = e / 3;
  const int j = (int)(e % 3);
  const D3 x = vrow(V, F, f, (j + 2) % 3), y = vrow(V, F, f, j), z = vrow(V, F, f, (j + 1) % 3);
  const D3 v1 = dsub(x, y), v2 = dsub(z, y);
  const double n1 = dnorm(v1), n2 = dnorm(v2);
  const D3 u1{v1.x / n1, v1.y / n1, v1.z / n1}, u2{v2.x / n2, v2.y / n2, v2.z / n2};
  const D3 dm{u1.x - u2.x, u1.y - u2.y, u1.z - u2.z}, dp{u1.x + u2.x, u1.y + u2.y, u1.z + u2.z};
  angle[e] = 2.0 * atan(dnorm(dm) / dnorm(dp));
  vkey[e] = (uint32_t)F[f * 3 + j];
  ventry[e] = (int32_t)e;
  // edge opposite corner j (oriented_facets.cpp: (F1,F2), (F2,F0), (F0,F1))
  const uint32_t a = (uint32_t)F[f * 3 + (j + 1) % 3], b = (uint32_t)F[f * 3 + (j + 2) % 3];
  ekey[e] = ((unsigned long long)min(a, b) << 32) | (unsigned long long)max(a, b);
  eentry[e] = (int32_t)e;
}

// Segmented sums over sorted entries, in entry order within a segment.
// mode 0: vertex normals, sum of angle(e) * FN(face(e)); mode 1: edge normals,
// sum of FN(face(e)).  Each segment start writes its normalised sum to
// out[seg_id(e)] and, for edges, seg_of[entry] for every entry of the segment.
template <typename K>
__global__ void segment_normals_kernel(const K* __restrict__ key, const int32_t* __restrict__ ent,
                                       int64_t n, const double* __restrict__ angle,
                                       const double* __restrict__ FN, int mode,
                                       const uint32_t* __restrict__ seg_index,
                                       double* __restrict__ out, int32_t* __restrict__ seg_of) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n || (i > 0 && key[i - 1] == key[i])) return;
  double sx = 0, sy = 0, sz = 0;
  const int64_t slot = mode == 0 ? (int64_t)key[i] : (int64_t)seg_index[i];
  for (int64_t j = i; j < n && key[j] == key[i]; ++j) {
    const int32_t e = ent[j];
    const int64_t f = e / 3;
    const double w = mode == 0 ? angle[e] : 1.0;
    sx += w * FN[f * 3];
    sy += w * FN[f * 3 + 1];
    sz += w * FN[f * 3 + 2];
    if (seg_of) seg_of[e] = (int32_t)slot;
  }
  const double r = sqrt(sx * sx + sy * sy + sz * sz);
  if (r > 0) {
    sx /= r;
    sy /= r;
    sz /= r;
  }
  out[slot * 3] = sx;
  out[slot * 3 + 1] = sy;
  out[slot * 3 + 2] = sz;
}

__global__ void segment_start_flags_kernel(const unsigned long long* __restrict__ key, int64_t n,
                                           uint32_t* __restrict__ flag) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || key[i - 1] != key[i]) ? 1u : 0u;
}

// pseudonormal_test.cpp:16-135 at the closest point c of face f.
__device__ void pseudonormal_sign(const double* __restrict__ V, const int32_t* __restrict__ F,
                                  int64_t nF, const double* __restrict__ FN,
                                  const double* __restrict__ VN, const double* __restrict__ EN,
                                  const int32_t* __restrict__ edge_of, int64_t f, D3 q, D3 c,
                                  double& s, D3& n) {
  const D3 A = vrow(V, F, f, 0), B = vrow(V, F, f, 1), Cc = vrow(V, F, f, 2);
  auto fn = [&](int64_t x) -> D3 { return {FN[x * 3], FN[x * 3 + 1], FN[x * 3 + 2]}; };
  auto vn = [&](int64_t x) -> D3 { return {VN[x * 3], VN[x * 3 + 1], VN[x * 3 + 2]}; };
  auto en = [&](int corner) -> D3 {
    const int64_t e = edge_of[f * 3 + corner];
    return {EN[e * 3], EN[e * 3 + 1], EN[e * 3 + 2]};
  };
  // doublearea of (A, B, C): Kahan's formula on the sorted edge lengths
  double l0 = dnorm(dsub(B, Cc)), l1 = dnorm(dsub(Cc, A)), l2 = dnorm(dsub(A, B));
  if (l0 < l1) { const double t = l0; l0 = l1; l1 = t; }
  if (l1 < l2) { const double t = l1; l1 = l2; l2 = t; }
  if (l0 < l1) { const double t = l0; l0 = l1; l1 = t; }
  const double arg = (l0 + (l1 + l2)) * (l2 - (l0 - l1)) * (l2 + (l0 - l1)) * (l0 + (l1 - l2));
  const double area = 2.0 * 0.25 * sqrt(arg);
  const double kMinDoubleArea = 1e-4, kEps = 1e-12;
  bool found = false;
  if (area > kMinDoubleArea) {
    // barycentric_coordinates.cpp:57-98
    const D3 v0 = dsub(B, A), v1 = dsub(Cc, A), v2 = dsub(c, A);
    const double d00 = ddot(v0, v0), d01 = ddot(v0, v1), d11 = ddot(v1, v1);
    const double d20 = ddot(v2, v0), d21 = ddot(v2, v1);
    const double denom = d00 * d11 - d01 * d01;
    const double b1 = (d11 * d20 - d01 * d21) / denom, b2 = (d00 * d21 - d01 * d20) / denom;
    const double b[3] = {1.0 - (b1 + b2), b1, b2};
    const int type = (b[0] <= kEps) + (b[1] <= kEps) + (b[2] <= kEps);
    if (type == 2) {
      for (int x = 0; x < 3; ++x)
        if (b[x] > kEps) {
          n = vn(F[f * 3 + x]);
          found = true;
          break;
        }
    } else if (type == 1) {
      for (int x = 0; x < 3; ++x)
        if (b[x] <= kEps) {
          n = en(x);
          found = true;
          break;
        }
    }
    if (!found) n = fn(f);
    found = true;
  } else {
    for (int v = 0; v < 3 && !found; ++v)
      if (dnorm(dsub(c, vrow(V, F, f, v))) < kEps) {
        n = vn(F[f * 3 + v]);
        found = true;
      }
    for (int e = 0; e < 3 && !found; ++e) {
      // project_to_line_segment(c, s, d)
      const D3 S = vrow(V, F, f, (e + 1) % 3), Dd = vrow(V, F, f, (e + 2) % 3);
      const D3 dms = dsub(Dd, S);
      const double len2 = ddot(dms, dms);
      const D3 smp = dsub(S, c);
      double t = -(dms.x * smp.x + dms.y * smp.y + dms.z * smp.z) / len2;
      double sq;
      if (t < 0) {
        sq = ddot(dsub(c, S), dsub(c, S));
      } else if (t > 1) {
        sq = ddot(dsub(c, Dd), dsub(c, Dd));
      } else {
        const D3 pp{(1 - t) * S.x + t * Dd.x, (1 - t) * S.y + t * Dd.y, (1 - t) * S.z + t * Dd.z};
        sq = ddot(dsub(c, pp), dsub(c, pp));
      }
      if (sqrt(sq) < kEps) {
        n = en(e);
        found = true;
      }
    }
    if (!found) n = fn(f);
  }
  s = ddot(dsub(q, c), n) >= 0 ? 1.0 : -1.0;
}

__global__ void pseudonormal_kernel(const double* __restrict__ P, int64_t nP,
                                    const double* __restrict__ V, const int32_t* __restrict__ F,
                                    int64_t nF, const double* __restrict__ FN,
                                    const double* __restrict__ VN, const double* __restrict__ EN,
                                    const int32_t* __restrict__ edge_of,
                                    const double* __restrict__ sqrD, const int32_t* __restrict__ I,
                                    const double* __restrict__ C, double* __restrict__ sgn,
                                    double* __restrict__ N) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= nP) return;
  const int32_t f = I[p];
  if (f < 0 || f >= nF) {
    sgn[p] = 1.0;
    if (N) N[p * 3] = N[p * 3 + 1] = N[p * 3 + 2] = 0.0;
    return;
  }
  double s;
  D3 n;
  pseudonormal_sign(V, F, nF, FN, VN, EN, edge_of, f, {P[p * 3], P[p * 3 + 1], P[p * 3 + 2]},
                    {C[p * 3], C[p * 3 + 1], C[p * 3 + 2]}, s, n);
  sgn[p] = s;
  if (N) {
    N[p * 3] = n.x;
    N[p * 3 + 1] = n.y;
    N[p * 3 + 2] = n.z;
  }
}

// signed_distance.cpp:96-137: out-of-bounds distances give NaN, F.rows()+1
// and a zero closest point; otherwise S = s sqrt(sqrD) with s = 1 (unsigned),
// 1 - 2 W (winding number) or 1 - 2 |W| (fast winding number).
__global__ void combine_kernel(const double* __restrict__ sqrD, const double* __restrict__ W,
                               int sign_mode, double low_sqr_d, double up_sqr_d, int64_t nP,
                               int64_t nF, double* __restrict__ S, int32_t* __restrict__ I,
                               double* __restrict__ C) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= nP) return;
  const double d2 = sqrD[p];
  if (d2 >= up_sqr_d || d2 < low_sqr_d || !(d2 == d2)) {
    S[p] = __longlong_as_double(0x7ff8000000000000ll);
    I[p] = (int32_t)(nF + 1);
    C[p * 3] = C[p * 3 + 1] = C[p * 3 + 2] = 0.0;
    return;
  }
  double s = 1.0;
  if (sign_mode == 1) s = 1.0 - 2.0 * W[p];
  else if (sign_mode == 2) s = 1.0 - 2.0 * fabs(W[p]);
  else if (sign_mode == 3) s = W[p];  // pseudonormal sign
  S[p] = s * sqrt(d2);
}

__global__ void fill_empty_kernel(int64_t nP, double* __restrict__ S, int32_t* __restrict__ I,
                                  double* __restrict__ C) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= nP) return;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  S[p] = nan;
  I[p] = -1;
  C[p * 3] = C[p * 3 + 1] = C[p * 3 + 2] = nan;
}

}  // namespace

void soup_squared_distance(const gwn_soup_impl& s, const void* Q, int q_dtype, int64_t nQ,
                           double up_sqr_d, double* sqrD, int32_t* I, double* C,
                           cudaStream_t st) {
  if (nQ == 0) return;
  ClosestParams prm;
  prm.nf = s.nf.get();
  prm.snode = s.snode.get();
  prm.tf = s.tf.get();
  prm.td = s.td.get();
  prm.tri_index = s.tri_index.get();
  prm.nnodes = (int)s.nnodes;
  prm.cmax = (float)s.cmax;
  QueryOrder qo;
  {
    PhaseTimer ph("order_queries", st);
    order_queries(Q, q_dtype, nQ, s.lo, s.hi, qo, st);
  }
  const int32_t* perm = qo.active ? qo.perm.get() : nullptr;
  const unsigned grid = (unsigned)((nQ + 127) / 128);
  PhaseTimer ph("closest", st);
  // The stack holds at most one entry per level plus one (each pop pushes at
  // most two children).
  const bool dfs = s.max_depth + 2 < kStack;
  unsigned* status = sticky_status_word();
  if (q_dtype == GWN_F64) {
    if (dfs)
      launch_kernel(closest_dfs_kernel<double>, grid, 128, 0, st, prm,
                    static_cast<const double*>(Q), perm, nQ, up_sqr_d, sqrD, I, C, status);
    else
      launch_kernel(closest_kernel<double>, grid, 128, 0, st, prm,
                    static_cast<const double*>(Q), perm, nQ, up_sqr_d, sqrD, I, C);
  } else {
    if (dfs)
      launch_kernel(closest_dfs_kernel<float>, grid, 128, 0, st, prm,
                    static_cast<const float*>(Q), perm, nQ, up_sqr_d, sqrD, I, C, status);
    else
      launch_kernel(closest_kernel<float>, grid, 128, 0, st, prm, static_cast<const float*>(Q),
                    perm, nQ, up_sqr_d, sqrD, I, C);
  }
}

void pseudonormal_precompute(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                             PseudonormalData& d, cudaStream_t st) {
  const int64_t ne = nF * 3;
  auto grid = [](int64_t n) { return (unsigned)std::max<int64_t>(1, (n + 255) / 256); };
  d.FN.alloc((size_t)nF * 3, st);
  d.VN.alloc((size_t)std::max<int64_t>(nV, 1) * 3, st);
  d.EN.alloc((size_t)ne * 3, st);
  d.edge_of.alloc((size_t)ne, st);
  DevBuf<double> angle((size_t)ne, st);
  DevBuf<uint32_t> vkey((size_t)ne, st), vkey_t((size_t)ne, st), eflag((size_t)ne, st);
  DevBuf<int32_t> vent((size_t)ne, st), vent_t((size_t)ne, st), eent((size_t)ne, st),
      eent_t((size_t)ne, st);
  DevBuf<unsigned long long> ekey((size_t)ne, st), ekey_t((size_t)ne, st);
  launch_kernel(face_normals_kernel, grid(nF), 256, 0, st, V, F, nF, d.FN.get());
  launch_kernel(corner_entries_kernel, grid(ne), 256, 0, st, V, F, nF, angle.get(), vkey.get(),
                vent.get(), ekey.get(), eent.get());
  int vbits = 1;
  while (vbits < 32 && (int64_t(1) << vbits) < nV) ++vbits;
  radix_sort_pairs<uint32_t>(vkey.get(), vent.get(), vkey_t.get(), vent_t.get(), ne, 0,
                             (vbits + 7) / 8 * 8, st);
  d.VN.zero(st);
  launch_kernel(segment_normals_kernel<uint32_t>, grid(ne), 256, 0, st, (const uint32_t*)vkey.get(),
                (const int32_t*)vent.get(), ne, (const double*)angle.get(),
                (const double*)d.FN.get(), 0, (const uint32_t*)nullptr, d.VN.get(),
                (int32_t*)nullptr);
  radix_sort_pairs<unsigned long long>(ekey.get(), eent.get(), ekey_t.get(), eent_t.get(), ne, 0,
                                       64, st);
  launch_kernel(segment_start_flags_kernel, grid(ne), 256, 0, st,
                (const unsigned long long*)ekey.get(), ne, eflag.get());
  exclusive_scan_u32(eflag.get(), eflag.get(), ne, st);
  launch_kernel(segment_normals_kernel<unsigned long long>, grid(ne), 256, 0, st,
                (const unsigned long long*)ekey.get(), (const int32_t*)eent.get(), ne,
                (const double*)angle.get(), (const double*)d.FN.get(), 1,
                (const uint32_t*)eflag.get(), d.EN.get(), d.edge_of.get());
}

void pseudonormal_apply(const PseudonormalData& d, const double* P, int64_t nP, const double* V,
                        const int32_t* F, int64_t nF, const int32_t* I, const double* C,
                        const double* sqrD, double* sgn, double* N, cudaStream_t st) {
  if (nP == 0) return;
  launch_kernel(pseudonormal_kernel, (unsigned)((nP + 255) / 256), 256, 0, st, P, nP, V, F, nF,
                (const double*)d.FN.get(), (const double*)d.VN.get(), (const double*)d.EN.get(),
                (const int32_t*)d.edge_of.get(), sqrD, I, C, sgn, N);
}

void signed_distance_run(const double* P, int64_t nP, const double* V, int64_t nV,
                         const int32_t* F, int64_t nF, int sign_type, double lower_bound,
                         double upper_bound, double* S, int32_t* I, double* C, double* N,
                         int precision, cudaStream_t st) {
  if (nP == 0) return;
  const unsigned grid = (unsigned)((nP + 255) / 256);
  if (nF == 0) {  // signed_distance.cpp:395-402
    launch_kernel(fill_empty_kernel, grid, 256, 0, st, nP, S, I, C);
    return;
  }
  // bounds on squared distances, signed_distance.cpp:83-88
  const double max_abs = std::fmax(std::fabs(lower_bound), std::fabs(upper_bound));
  const double up_sqr_d = std::pow(max_abs, 2.0);
  const double low_sqr_d = std::pow(std::fmax(max_abs - (upper_bound - lower_bound), 0.0), 2.0);
  gwn_soup_impl tree;
  soup_build(tree, V, nV, F, nF, 2, true, st);
  DevBuf<double> sqrD((size_t)nP, st);
  soup_squared_distance(tree, P, GWN_F64, nP, up_sqr_d, sqrD.get(), I, C, st);
  DevBuf<double> W;
  int mode = 0;
  if (sign_type == GWN_SD_WINDING_NUMBER || sign_type == GWN_SD_DEFAULT) {
    W.alloc((size_t)nP, st);
    ExactArgs a{V, nV, 3, F, nF, P, GWN_F64, nP, W.get(), GWN_F64, precision, true};
    run_exact(a, st);
    mode = 1;
  } else if (sign_type == GWN_SD_FAST_WINDING_NUMBER) {
    W.alloc((size_t)nP, st);
    soup_eval(tree, 2.0f, P, GWN_F64, nP, W.get(), GWN_F64, precision, st);
    mode = 2;
  } else if (sign_type == GWN_SD_PSEUDONORMAL) {
    W.alloc((size_t)nP, st);
    PseudonormalData pn;
    pseudonormal_precompute(V, nV, F, nF, pn, st);
    pseudonormal_apply(pn, P, nP, V, F, nF, I, C, sqrD.get(), W.get(), N, st);
    mode = 3;
  }
  launch_kernel(combine_kernel, grid, 256, 0, st, (const double*)sqrD.get(),
                (const double*)W.get(), mode, low_sqr_d, up_sqr_d, nP, nF, S, I, C);
  GWN_CUDA(cudaStreamSynchronize(st));
}

}  // namespace gwn
