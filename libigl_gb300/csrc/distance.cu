// Closest triangle and signed distance over a built soup tree.
//
// Reference: igl::signed_distance (include/igl/signed_distance.cpp:20-137,
// 372-440) for 3-D triangle meshes with the sign types UNSIGNED,
// WINDING_NUMBER / DEFAULT and FAST_WINDING_NUMBER, and the closest-point
// query it runs per point, igl::AABB::squared_distance
// (include/igl/AABB.cpp:1135-1205) with point_simplex_squared_distance
// (include/igl/point_simplex_squared_distance.cpp:40-124).
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

struct Best {
  double d2;
  int slot;
  D3 c;
};

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

// FP32 screen of a leaf: true when the triangle cannot be strictly closer
// than the current best (its FP32 distance minus the triangle's stored
// slack and the query-rounding slack 1e-6 (S + d) is still at least it).
__device__ __forceinline__ bool screened_out(const ClosestParams& prm, int slot, float fx,
                                             float fy, float fz, float S, double best) {
  const float4 t0 = __ldg(&prm.tf[(int64_t)slot * 3]);
  const float4 t1 = __ldg(&prm.tf[(int64_t)slot * 3 + 1]);
  const float4 t2 = __ldg(&prm.tf[(int64_t)slot * 3 + 2]);
  const float d = sqrtf(dist2_triangle32(fx, fy, fz, t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z,
                                         t1.w, t2.x));
  const float lower = d - t2.y - 1e-6f * (S + d);
  return lower > 0.f && (double)lower * (double)lower >= best;
}

__device__ __forceinline__ void eval_leaf(const ClosestParams& prm, int slot, D3 q, Best& b) {
  const double* t = prm.td + (int64_t)slot * 9;
  const D3 cp = closest_on_triangle(q, {t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]});
  const D3 d = dsub(q, cp);
  const double d2 = ddot(d, d);
  if (d2 < b.d2) {
    b.d2 = d2;
    b.slot = slot;
    b.c = cp;
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
  Best b{up_sqr_d, -1, {0, 0, 0}};
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
      if (lb > 0.f && (double)lb * (double)lb >= b.d2) {
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
  Best b{up_sqr_d, -1, {0, 0, 0}};
  if (isfinite(q.x) && isfinite(q.y) && isfinite(q.z) && prm.nnodes > 0) {
    const float fx = (float)q.x, fy = (float)q.y, fz = (float)q.z;
    const float S = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) + prm.cmax;
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
      if ((double)lb * (double)lb >= b.d2) continue;
      if (ref < 0) {
        if (!screened_out(prm, ~ref, fx, fy, fz, S, b.d2)) eval_leaf(prm, ~ref, q, b);
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
      if ((double)far_lb * (double)far_lb < b.d2) {
        if (sp == kStack) {
          atomicOr(status, kStatusBadInput);
          break;
        }
        stk_n[sp] = far_n;
        stk_lb[sp] = far_lb;
        ++sp;
      }
      if ((double)near_lb * (double)near_lb < b.d2) {
        if (sp == kStack) {
          atomicOr(status, kStatusBadInput);
          break;
        }
        stk_n[sp] = near_n;
        stk_lb[sp] = near_lb;
        ++sp;
      }
    }
  }
  sqrD[qi] = b.d2;
  I[qi] = b.slot >= 0 ? prm.tri_index[b.slot] : -1;
  C[qi * 3] = b.c.x;
  C[qi * 3 + 1] = b.c.y;
  C[qi * 3 + 2] = b.c.z;
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

void signed_distance_run(const double* P, int64_t nP, const double* V, int64_t nV,
                         const int32_t* F, int64_t nF, int sign_type, double lower_bound,
                         double upper_bound, double* S, int32_t* I, double* C, int precision,
                         cudaStream_t st) {
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
  }
  launch_kernel(combine_kernel, grid, 256, 0, st, (const double*)sqrD.get(),
                (const double*)W.get(), mode, low_sqr_d, up_sqr_d, nP, nF, S, I, C);
  GWN_CUDA(cudaStreamSynchronize(st));
}

}  // namespace gwn
