// Device-side pieces of the triangle-soup Barnes-Hut walk shared by the
// single-mesh evaluation (soup.cu) and the multi-mesh served batches
// (serve.cu): node records -> far field, exact triangle term, and the three
// walks (mixed warp-coherent, plain FP64 warp-coherent, plain FP64 per lane).
//
// Reference: UT_SolidAngle::computeSolidAngle (include/igl/
// FastWindingNumberForSoups.h:7148-7284) and UTsignedSolidAngleTri
// (FastWindingNumberForSoups.h:6070-6110).
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "bh_common.cuh"
#include "gwn_common.cuh"
#include "soup.cuh"

namespace gwn {
namespace soupwalk {

constexpr double kBand = 1e-3;  // |W - 0.5| band re-evaluated in plain FP64
constexpr float kInv4PiF = 0.079577471545947667884f;
constexpr double kInv4Pi = 0.079577471545947667884;

// Far field of one node about its average point, FWNFS.h:7195-7251, with
// (dx,dy,dz) = q - P and r2 = |q - P|^2: the reference's expression, in FP64
// on the FP64 records (the FP32 walk evaluates the packed forms of
// pack_far32 instead, far_field32 below).
template <typename T>
struct Far {
  T N[3], Nii[3], Nxy_yx, Nyz_zy, Nzx_xz, Niii[3], perm, c2[6];
};

template <typename T>
__device__ __forceinline__ T far_field(const Far<T>& m, T dx, T dy, T dz, T r2, int order) {
  // m2 = 1/|q-P|^2, m1 = sqrt(m2), as the reference
  const T m2 = T(1) / r2;
  const T m1 = g_sqrt(m2);
  const T qx = dx * m1, qy = dy * m1, qz = dz * m1;
  T omega = -m2 * (qx * m.N[0] + qy * m.N[1] + qz * m.N[2]);
  if (order >= 1) {
    const T q2x = qx * qx, q2y = qy * qy, q2z = qz * qz;
    const T m3 = m2 * m1;
    omega += m3 * (m.Nii[0] + m.Nii[1] + m.Nii[2] -
                   T(3) * (q2x * m.Nii[0] + q2y * m.Nii[1] + q2z * m.Nii[2] + qx * qy * m.Nxy_yx +
                           qx * qz * m.Nzx_xz + qy * qz * m.Nyz_zy));
    if (order >= 2) {
      const T q3x = q2x * qx, q3y = q2y * qy, q3z = q2z * qz;
      const T m4 = m2 * m2;
      const T t0x = m.c2[3] + m.c2[4], t0y = m.c2[5] + m.c2[0], t0z = m.c2[1] + m.c2[2];
      const T t1x = qy * m.c2[0] + qz * m.c2[1];
      const T t1y = qz * m.c2[2] + qx * m.c2[3];
      const T t1z = qx * m.c2[4] + qy * m.c2[5];
      omega += m4 * (T(1.5) * (qx * (T(3) * m.Niii[0] + t0x) + qy * (T(3) * m.Niii[1] + t0y) +
                               qz * (T(3) * m.Niii[2] + t0z)) -
                     T(7.5) * (q3x * m.Niii[0] + q3y * m.Niii[1] + q3z * m.Niii[2] +
                               qx * qy * qz * m.perm + q2x * t1x + q2y * t1y + q2z * t1z));
    }
  }
  return omega;
}

// Exact triangle solid angle, FWNFS.h:6070-6110 (normalised corner vectors).
template <typename T>
__device__ __forceinline__ T tri_solid_angle(T ax, T ay, T az, T bx, T by, T bz, T cx, T cy,
                                             T cz) {
  const T la2 = ax * ax + ay * ay + az * az;
  const T lb2 = bx * bx + by * by + bz * bz;
  const T lc2 = cx * cx + cy * cy + cz * cz;
  if (la2 == T(0) || lb2 == T(0) || lc2 == T(0)) return T(0);
  if (sizeof(T) == 4) {  // normalise with reciprocal square roots
    const T ia = g_rsqrt(la2), ib = g_rsqrt(lb2), ic = g_rsqrt(lc2);
    ax *= ia; ay *= ia; az *= ia;
    bx *= ib; by *= ib; bz *= ib;
    cx *= ic; cy *= ic; cz *= ic;
  } else {  // FP64: length then divide, as FWNFS.h:6085-6095
    const T la = g_sqrt(la2), lb = g_sqrt(lb2), lc = g_sqrt(lc2);
    ax /= la; ay /= la; az /= la;
    bx /= lb; by /= lb; bz /= lb;
    cx /= lc; cy /= lc; cz /= lc;
  }
  const T ux = bx - ax, uy = by - ay, uz = bz - az;
  const T vx = cx - ax, vy = cy - ay, vz = cz - az;
  const T num = ax * (uy * vz - uz * vy) + ay * (uz * vx - ux * vz) + az * (ux * vy - uy * vx);
  if (num == T(0)) return T(0);
  const T den = T(1) + (ax * bx + ay * by + az * bz) + (ax * cx + ay * cy + az * cz) +
                (bx * cx + by * cy + bz * cz);
  return T(2) * g_atan2(num, den);
}

// FP32 far field of a packed record (pack_far32; b..f its float4s): omega = m2 (m1 (A(q) +
// m1 K(q)) - q.N) with q = (x - P) m1, (dx,dy,dz) = x - P, r2 = |x - P|^2.
__device__ __forceinline__ float far_field32(float4 b, float4 c, float4 d, float4 e, float4 f,
                                             float dx, float dy, float dz, float r2, int order) {
  const float m1 = g_rsqrt(r2), m2 = m1 * m1;
  const float qx = dx * m1, qy = dy * m1, qz = dz * m1;
  const float lin = fmaf(qx, b.x, fmaf(qy, b.y, qz * b.z));
  if (order == 0) return -m2 * lin;
  const float x2 = qx * qx, y2 = qy * qy, z2 = qz * qz, yz = qy * qz;
  const float a = fmaf(qx, fmaf(b.w, qx, fmaf(c.z, qy, c.w * qz)),
                       fmaf(c.x, y2, fmaf(c.y, z2, d.x * yz)));
  float s = a;
  if (order >= 2) {
    const float kx = fmaf(d.y, x2, fmaf(e.z, y2, fmaf(f.x, z2, f.z * yz)));
    const float ky = fmaf(e.x, x2, fmaf(d.z, y2, f.y * z2));
    const float kz = fmaf(e.y, x2, fmaf(e.w, y2, d.w * z2));
    s = fmaf(m1, fmaf(qx, kx, fmaf(qy, ky, qz * kz)), a);
  }
  return m2 * fmaf(m1, s, -lin);
}

__device__ __forceinline__ Far<double> load_far(const SoupNodeD* r) {
  Far<double> m;
  for (int d = 0; d < 3; ++d) {
    m.N[d] = r->N[d];
    m.Nii[d] = r->Nii[d];
    m.Niii[d] = r->Niii[d];
  }
  m.Nxy_yx = r->Nxy_yx;
  m.Nyz_zy = r->Nyz_zy;
  m.Nzx_xz = r->Nzx_xz;
  m.perm = r->perm;
  for (int k = 0; k < 6; ++k) m.c2[k] = r->c2[k];
  return m;
}

// Query i of a launch (through the spatial order perm, or a re-evaluation
// list).  Streaming loads: each query is read once, so its cache lines go
// first and L2 keeps the node records the walks share.
template <typename QT>
__device__ __forceinline__ void read_query(const QT* Q, const int32_t* perm, const int32_t* list,
                                           int64_t i, int64_t& qi, double& x, double& y,
                                           double& z) {
  qi = list ? (int64_t)__ldcs(list + i) : (perm ? (int64_t)__ldcs(perm + i) : i);
  x = (double)__ldcs(Q + qi * 3 + 0);
  y = (double)__ldcs(Q + qi * 3 + 1);
  z = (double)__ldcs(Q + qi * 3 + 2);
}

struct EvalParams {
  const SoupNodeF* nf;
  const SoupNodeD* nd;
  const float4* tf;
  const double* td;
  int nnodes;
  int order;
  float beta2f;
  double beta2d;
  float eps;       // near-field distance (1e-3 * bbox diagonal)
  float cmax;      // max |coordinate| of any node centre
  unsigned* status;
  int ref32;       // open test: the reference's FP32 one (GWN_TREE_REFERENCE)
  int fp64_queue = 0;  // moments bounded: the FP64 walk queues its far fields
};

// The reference's descend test (FWNFS.h:7176-7193) on its FP32 data: q cast
// to float, |q - P|^2 summed as (x^2 + y^2) + z^2 and compared with
// maxP2 * beta^2, each operation rounded on its own as in the SSE code,
// which has no fused multiply-add.  With the reference's P and maxP2 (the
// FP32 records of GWN_TREE_REFERENCE) it decides as the reference does.
__device__ __forceinline__ bool ref_open32(float qx, float qy, float qz, float4 a, float beta2) {
  const float dx = __fsub_rn(qx, a.x), dy = __fsub_rn(qy, a.y), dz = __fsub_rn(qz, a.z);
  const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  return r2 <= __fmul_rn(a.w, beta2);
}

// FP64 solid angle of the triangle t[0..8] (xyz of three corners) seen from
// q, in the unnormalised van Oosterom-Strackee form of igl::solid_angle
// (include/igl/solid_angle.cpp:22-48): with A, B, C the corners relative to
// q, tan(Omega/2) = A.(B x C) / (|A||B||C| + (A.B)|C| + (A.C)|B| + (B.C)|A|).
// Equal to the normalised form of tri_solid_angle up to rounding, without
// its nine divisions.  A corner at q or a zero determinant gives 0, as there.
// The corner vectors, the determinant and the denominator -- where the
// cancellation near the triangle is -- are FP64; the angle is FP32 atan2 of
// the pair scaled by a power of two, so that the pair's rounding to FP32
// moves it by at most 2^-24 rad besides atan2f's own error (a few 1e-7 rad):
// FP64 atan2 would cost as much as the rest of the term at this part's FP64
// rate.
__device__ __forceinline__ double solid_angle_vos64(const double* __restrict__ t, double qx,
                                                    double qy, double qz) {
  const double ax = t[0] - qx, ay = t[1] - qy, az = t[2] - qz;
  const double bx = t[3] - qx, by = t[4] - qy, bz = t[5] - qz;
  const double cx = t[6] - qx, cy = t[7] - qy, cz = t[8] - qz;
  const double la2 = ax * ax + ay * ay + az * az;
  const double lb2 = bx * bx + by * by + bz * bz;
  const double lc2 = cx * cx + cy * cy + cz * cz;
  if (la2 == 0.0 || lb2 == 0.0 || lc2 == 0.0) return 0.0;
  // two coinciding corners: the normalised form's u = b - a (or v, or
  // u x v) is exactly zero there, so its term is 0 (FWNFS.h:6097-6101)
  if ((t[0] == t[3] && t[1] == t[4] && t[2] == t[5]) ||
      (t[0] == t[6] && t[1] == t[7] && t[2] == t[8]) ||
      (t[3] == t[6] && t[4] == t[7] && t[5] == t[8]))
    return 0.0;
  const double det = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
  if (det == 0.0) return 0.0;
  const double la = sqrt(la2), lb = sqrt(lb2), lc = sqrt(lc2);
  const double den = la * lb * lc + (ax * bx + ay * by + az * bz) * lc +
                     (ax * cx + ay * cy + az * cz) * lb + (bx * cx + by * cy + bz * cz) * la;
  // s = 2^-e, e = the binary exponent of max(|det|, |den|), clamped so that
  // s is a normal double
  const int hi = __double2hiint(fmax(fabs(det), fabs(den)));
  const int e = min(max(((hi >> 20) & 0x7ff) - 1023, -1022), 1022);
  const double s = __hiloint2double((1023 - e) << 20, 0);
  return 2.0 * (double)atan2f((float)(det * s), (float)(den * s));
}

// Per-warp queue of FP64 near-field terms (triangle slot, owning lane).
// The walk does not evaluate an FP64 triangle term where it arises: the
// lanes that need one append it here, and when the queue would overflow (and
// at the end of the walk) the warp evaluates up to 32 queued terms at once,
// one per lane, so that each FP64 instruction serves the whole warp instead
// of the few lanes that share a leaf.  Every lane still adds its own terms in
// node order, so the sum does not depend on the other lanes of the warp.
// The lanes' FP64 queries also live here rather than in registers: they are
// read only at the rare FP64 open-test re-checks and at the flushes, and
// the six registers they would hold cost the walk spills (9.60 -> 9.25 ms
// per 10M-query launch with them parked here).
// Each lane keeps the queue positions of its own terms as a bit mask and adds
// their values (v, written by the lanes that evaluated them) in queue order.
struct NearQueue {
  int2 e[32];
  double q[32][3];  // each lane's FP64 query
  double v[32];     // the evaluated terms of one flush
};

__device__ __forceinline__ void flush_near64(const double* __restrict__ td, NearQueue& q, int n,
                                             unsigned mine, double& acc64) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (lane < n) {
    const int2 e = q.e[lane];
    q.v[lane] = solid_angle_vos64(td + (int64_t)e.x * 9, q.q[e.y][0], q.q[e.y][1], q.q[e.y][2]);
  }
  __syncwarp();
  while (mine) {
    acc64 += q.v[__ffs(mine) - 1];
    mine &= mine - 1;
  }
  __syncwarp();
}

// Work counters of the instrumented walk (only touched when kStats).
struct WalkCounters {
  unsigned long long steps = 0, visits = 0, far = 0, exact32 = 0, exact64 = 0, recheck = 0;
};

// Mixed-precision warp-coherent walk of one query per lane.  All 32 lanes of
// the warp must call it together (invalid lanes pass valid = false).  FP32
// records and arithmetic; the open test is redone in FP64 inside the guard
// band; exact triangle terms within eps of the query are taken in FP64
// through the warp's NearQueue `nq` (shared memory).  Returns the
// solid-angle sum as an FP32 part and an FP64 part.  kTree: the tree kind
// (GWN_TREE_REFERENCE / GWN_TREE_BINNED) when known at compile time, -1 to
// read it from prm.ref32.
template <bool kStats, int kTree = -1>
__device__ __forceinline__ void walk_mixed(const EvalParams& prm, bool valid, double qx, double qy,
                                           double qz, float& acc, double& acc64,
                                           WalkCounters& c, NearQueue& nq) {
  const int lane = threadIdx.x & 31;
  nq.q[lane][0] = qx;
  nq.q[lane][1] = qy;
  nq.q[lane][2] = qz;
  const unsigned lt_mask = (1u << lane) - 1u;
  int nqueued = 0;    // warp-uniform
  unsigned mine = 0;  // this lane's queue positions
  const bool ref = kTree < 0 ? prm.ref32 != 0 : kTree == GWN_TREE_REFERENCE;
  const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
  const float S = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) + prm.cmax;
  const float sigma = guard_sigma(S);
  acc = 0.f;
  acc64 = 0.0;
  int resume = valid ? 0 : 0x7fffffff;
  int node = 0;
  const unsigned full = 0xffffffffu;
  while (node < prm.nnodes) {
    // the whole record at once, in three 256-bit loads (records are 96
    // bytes from a 32-byte aligned base): the far field's coefficients
    // arrive with the open test's data instead of one load latency after it
    const SoupNodeF* r = prm.nf + node;
    float4 a, rb, rc, rd, re, rf;
    ldg256(&r->a, a, rb);
    ldg256(&r->c, rc, rd);
    ldg256(&r->e, re, rf);
    const int link = __float_as_int(rf.w);
    bool open = false;
    bool want64 = false;
    int slot64 = 0;
    if (kStats) ++c.steps;
    if (node >= resume) {
      if (kStats) ++c.visits;
      const bool leaf = link < 0;
      if (node == 0 && !leaf) {
        open = true;
      } else {
        const float dx = fx - a.x, dy = fy - a.y, dz = fz - a.z;
        float r2;
        bool near;
        if (ref) {
          // ref_open32's own |q - P|^2, reused by the far field below
          r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
          near = r2 <= __fmul_rn(a.w, prm.beta2f);
        } else {
          r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          const float thr = a.w * prm.beta2f;
          near = r2 <= thr;
          if (in_guard_band(r2, thr, sigma)) {
            const SoupNodeD* r64 = prm.nd + node;
            near = open_test64(nq.q[lane][0], nq.q[lane][1], nq.q[lane][2], r64->P[0],
                               r64->P[1], r64->P[2], r64->maxP2, prm.beta2d);
            if (kStats) ++c.recheck;
          }
        }
        if (!near) {
          if (kStats) ++c.far;
          const float om = far_field32(rb, rc, rd, re, rf, dx, dy, dz, r2, prm.order);
          if (isfinite(om)) {
            acc += om;
            resume = leaf ? node + 1 : link;
          } else {
            near = true;
          }
        }
        if (near) {
          if (leaf) {
            const int slot = ~link;
            const float rad = sqrtf(a.w) + prm.eps;
            if (r2 <= rad * rad * 1.0001f) {
              if (kStats) ++c.exact64;
              want64 = true;
              slot64 = slot;
            } else {
              if (kStats) ++c.exact32;
              const float4 t0 = __ldg(&prm.tf[(int64_t)slot * 3]);
              const float4 t1 = __ldg(&prm.tf[(int64_t)slot * 3 + 1]);
              const float4 t2 = __ldg(&prm.tf[(int64_t)slot * 3 + 2]);
              acc += tri_solid_angle<float>(t0.x - fx, t0.y - fy, t0.z - fz, t0.w - fx, t1.x - fy,
                                            t1.y - fz, t1.z - fx, t1.w - fy, t2.x - fz);
            }
            resume = node + 1;
          } else {
            open = true;
          }
        }
      }
    }
    const unsigned m64 = __ballot_sync(full, want64);
    if (m64) {
      const int k = __popc(m64);
      if (nqueued + k > 32) {
        flush_near64(prm.td, nq, nqueued, mine, acc64);
        nqueued = 0;
        mine = 0;
      }
      if (want64) {
        const int pos = nqueued + __popc(m64 & lt_mask);
        nq.e[pos] = make_int2(slot64, lane);
        mine |= 1u << pos;
      }
      nqueued += k;
    }
    // a lane that opens the node wants node + 1, every other lane is past
    // the node (resume > node): the warp goes to the smallest of them
    node = __reduce_min_sync(full, open ? node + 1 : resume);
  }
  if (nqueued) flush_near64(prm.td, nq, nqueued, mine, acc64);
}

// Winding number from the two parts of walk_mixed.
__device__ __forceinline__ double mixed_result(float acc, double acc64) {
  return acc64 != 0.0 ? ((double)acc + acc64) * kInv4Pi : (double)(acc * kInv4PiF);
}

// Per-warp queue of the plain FP64 walk's terms.  The FP64 pipe charges a
// warp instruction the same for 1 or 32 lanes, and a far field or a
// triangle term arises for the lanes that reach it at one step, so the walk
// appends (term, lane) here and the warp evaluates 32 terms at a time, one
// per lane; each lane adds its own values by its bit mask of queue
// positions, in queue order, which is its walk order: its sum, term by term,
// is the one it would form alone.  A far field is queued only when it cannot
// be non-finite (bounded moments, |q - P|^2 >= 1e-100: every product stays
// within range), because a non-finite one descends instead
// (FWNFS.h:7247-7251); any other far field is evaluated where it arises and
// its value queued.
constexpr int kQueuedValue = INT_MIN;  // entry holding a value, not a term

struct Fp64Queue {
  int2 e[32];       // .x: node (far field), ~slot (triangle) or kQueuedValue; .y: lane
  double q[32][3];  // each lane's query
  double v[32];     // values
};

__device__ __forceinline__ void flush_fp64(const EvalParams& prm, Fp64Queue& fq, int n,
                                           unsigned mine, double& acc) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (lane < n) {
    const int2 e = fq.e[lane];
    if (e.x != kQueuedValue) {
      const double qx = fq.q[e.y][0], qy = fq.q[e.y][1], qz = fq.q[e.y][2];
      double v;
      if (e.x >= 0) {
        const SoupNodeD* r = prm.nd + e.x;
        const double dx = qx - r->P[0], dy = qy - r->P[1], dz = qz - r->P[2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        v = far_field<double>(load_far(r), dx, dy, dz, r2, prm.order);
      } else {
        const double* t = prm.td + (int64_t)(~e.x) * 9;
        v = tri_solid_angle<double>(t[0] - qx, t[1] - qy, t[2] - qz, t[3] - qx, t[4] - qy,
                                    t[5] - qz, t[6] - qx, t[7] - qy, t[8] - qz);
      }
      fq.v[lane] = v;
    }
  }
  __syncwarp();
  while (mine) {
    acc += fq.v[__ffs(mine) - 1];
    mine &= mine - 1;
  }
  __syncwarp();
}

// Plain FP64 warp-coherent walk (same calling rule as walk_mixed, with the
// warp's Fp64Queue); returns the solid-angle sum.
__device__ __forceinline__ double walk_fp64(const EvalParams& prm, bool valid, double qx,
                                            double qy, double qz, Fp64Queue& fq) {
  const int lane = threadIdx.x & 31;
  fq.q[lane][0] = qx;
  fq.q[lane][1] = qy;
  fq.q[lane][2] = qz;
  const unsigned lt_mask = (1u << lane) - 1u;
  double acc = 0.0;
  int nq = 0;         // warp-uniform
  unsigned mine = 0;  // this lane's queue positions
  int resume = valid ? 0 : 0x7fffffff;
  int node = 0;
  const unsigned full = 0xffffffffu;
  while (node < prm.nnodes) {
    const SoupNodeD* r = prm.nd + node;
    bool open = false;
    bool push = false;
    int term = 0;
    double value = 0.0;
    if (node >= resume) {
      const long long link = r->link;
      const bool leaf = link < 0;
      if (node == 0 && !leaf) {
        open = true;
      } else {
        bool near = prm.ref32 ? ref_open32((float)qx, (float)qy, (float)qz,
                                           __ldg(&prm.nf[node].a), prm.beta2f)
                              : open_test64(qx, qy, qz, r->P[0], r->P[1], r->P[2], r->maxP2,
                                            prm.beta2d);
        if (!near) {
          const double dx = qx - r->P[0], dy = qy - r->P[1], dz = qz - r->P[2];
          const double r2 = dx * dx + dy * dy + dz * dz;
          if (prm.fp64_queue && r2 >= 1e-100) {
            push = true;
            term = node;
            resume = leaf ? node + 1 : (int)link;
          } else {
            const double om = far_field<double>(load_far(r), dx, dy, dz, r2, prm.order);
            if (isfinite(om)) {
              push = true;
              term = kQueuedValue;
              value = om;
              resume = leaf ? node + 1 : (int)link;
            } else {
              near = true;
            }
          }
        }
        if (near) {
          if (leaf) {
            push = true;
            term = (int)link;  // ~slot
            resume = node + 1;
          } else {
            open = true;
          }
        }
      }
    }
    const unsigned m = __ballot_sync(full, push);
    if (m) {
      const int k = __popc(m);
      if (nq + k > 32) {
        flush_fp64(prm, fq, nq, mine, acc);
        nq = 0;
        mine = 0;
      }
      if (push) {
        const int pos = nq + __popc(m & lt_mask);
        fq.e[pos] = make_int2(term, lane);
        if (term == kQueuedValue) fq.v[pos] = value;
        mine |= 1u << pos;
      }
      nq += k;
    }
    // a lane that opens the node wants node + 1, every other lane is past
    // the node (resume > node): the warp goes to the smallest of them
    node = __reduce_min_sync(full, open ? node + 1 : resume);
  }
  if (nq) flush_fp64(prm, fq, nq, mine, acc);
  return acc;
}

// Plain FP64 walk of one query by one thread, no warp cooperation (for
// sparse re-evaluation lists whose lanes may belong to different meshes).
// Visits the same nodes and adds the same terms, in the same order, as
// walk_fp64 does for that query.
__device__ inline double walk_fp64_lane(const EvalParams& prm, double qx, double qy, double qz) {
  double acc = 0.0;
  int node = 0;
  while (node < prm.nnodes) {
    const SoupNodeD* r = prm.nd + node;
    const long long link = r->link;
    const bool leaf = link < 0;
    if (node == 0 && !leaf) {
      ++node;
      continue;
    }
    bool near = prm.ref32 ? ref_open32((float)qx, (float)qy, (float)qz, __ldg(&prm.nf[node].a),
                                       prm.beta2f)
                          : open_test64(qx, qy, qz, r->P[0], r->P[1], r->P[2], r->maxP2,
                                        prm.beta2d);
    const double dx = qx - r->P[0], dy = qy - r->P[1], dz = qz - r->P[2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (!near) {
      const double om = far_field<double>(load_far(r), dx, dy, dz, r2, prm.order);
      if (isfinite(om)) {
        acc += om;
        node = leaf ? node + 1 : (int)link;
        continue;
      }
    }
    if (leaf) {
      const double* t = prm.td + (int64_t)(~link) * 9;
      acc += tri_solid_angle<double>(t[0] - qx, t[1] - qy, t[2] - qz, t[3] - qx, t[4] - qy,
                                     t[5] - qz, t[6] - qx, t[7] - qy, t[8] - qz);
    }
    ++node;
  }
  return acc;
}

}  // namespace soupwalk
}  // namespace gwn
