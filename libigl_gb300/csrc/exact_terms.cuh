// Solid-angle terms shared by the exact winding number (exact.cu) and its
// hierarchical form (hier.cu): the packed FP32 triangle record, its FP32
// van Oosterom-Strackee term, and the reference's FP64 term.
#pragma once

#include <cuda_runtime.h>

#include "atan2f.cuh"

namespace gwn {

struct TriF {      // 64 bytes, 16-byte aligned
  float4 r0;       // ax ay az e1x
  float4 r1;       // e1y e1z e2x e2y
  float4 r2;       // e2z nx ny nz
  float4 r3;       // cx cy cz (R+eps)^2
};

// FP64 solid-angle term of the reference, include/igl/solid_angle.cpp:21-54,
// returned as atan2(det, den) (= Omega/2); callers divide the sum by 2 pi.
__device__ __forceinline__ double vos_term64(const double* A, const double* B,
                                             const double* C, double px, double py,
                                             double pz) {
  const double v00 = A[0] - px, v01 = A[1] - py, v02 = A[2] - pz;
  const double v10 = B[0] - px, v11 = B[1] - py, v12 = B[2] - pz;
  const double v20 = C[0] - px, v21 = C[1] - py, v22 = C[2] - pz;
  const double l0 = sqrt(v00 * v00 + (v01 * v01 + v02 * v02));
  const double l1 = sqrt(v10 * v10 + (v11 * v11 + v12 * v12));
  const double l2 = sqrt(v20 * v20 + (v21 * v21 + v22 * v22));
  const double det = v00 * v11 * v22 + v10 * v21 * v02 + v20 * v01 * v12 - v20 * v11 * v02 -
                     v10 * v01 * v22 - v00 * v21 * v12;
  const double dp0 = v10 * v20 + v11 * v21 + v12 * v22;
  const double dp1 = v20 * v00 + v21 * v01 + v22 * v02;
  const double dp2 = v00 * v10 + v01 * v11 + v02 * v12;
  return atan2(det, l0 * l1 * l2 + dp0 * l0 + dp1 * l1 + dp2 * l2);
}

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// FP32 term of one packed triangle seen from (qx,qy,qz): atan2(det, den).

__device__ __forceinline__ float vos_term32(const TriF& t, float qx, float qy, float qz) {
  const float ax = t.r0.x - qx, ay = t.r0.y - qy, az = t.r0.z - qz;
  const float bx = ax + t.r0.w, by = ay + t.r1.x, bz = az + t.r1.y;
  const float cx = ax + t.r1.z, cy = ay + t.r1.w, cz = az + t.r2.x;
  const float det = fmaf(ax, t.r2.y, fmaf(ay, t.r2.z, az * t.r2.w));
  const float la = sqrt_approx(fmaf(ax, ax, fmaf(ay, ay, az * az)));
  const float lb = sqrt_approx(fmaf(bx, bx, fmaf(by, by, bz * bz)));
  const float lc = sqrt_approx(fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
  const float ab = fmaf(ax, bx, fmaf(ay, by, az * bz));
  const float bc = fmaf(bx, cx, fmaf(by, cy, bz * cz));
  const float ca = fmaf(cx, ax, fmaf(cy, ay, cz * az));
  const float den = fmaf(la * lb, lc, fmaf(bc, la, fmaf(ca, lb, ab * lc)));
  return atan2_pairs(det, den);
}

// FP32 record of the triangle p[0], p[1], p[2] (FP64 input): a, e1 = b - a,
// e2 = c - a, n = e1 x e2 (formed in FP64), and the bounding sphere about
// the centroid grown by eps (squared, with a relative margin); a non-finite
// sphere makes every pair with it FP64.
__device__ __forceinline__ TriF make_trif(const double p[3][3], double eps) {
  double e1[3], e2[3], n[3], m[3];
  for (int d = 0; d < 3; ++d) {
    e1[d] = p[1][d] - p[0][d];
    e2[d] = p[2][d] - p[0][d];
    m[d] = (e1[d] + e2[d]) / 3.0;
  }
  n[0] = e1[1] * e2[2] - e1[2] * e2[1];
  n[1] = e1[2] * e2[0] - e1[0] * e2[2];
  n[2] = e1[0] * e2[1] - e1[1] * e2[0];
  // Bounding-sphere radius about the centroid (vertices are the farthest points).
  double r2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
  double t1 = 0, t2 = 0;
  for (int d = 0; d < 3; ++d) {
    t1 += (m[d] - e1[d]) * (m[d] - e1[d]);
    t2 += (m[d] - e2[d]) * (m[d] - e2[d]);
  }
  const double R = sqrt(fmax(r2, fmax(t1, t2)));
  const double rr = (R + eps) * (R + eps) * (1.0 + 1e-5) + 1e-30;
  TriF t;
  t.r0 = make_float4((float)p[0][0], (float)p[0][1], (float)p[0][2], (float)e1[0]);
  t.r1 = make_float4((float)e1[1], (float)e1[2], (float)e2[0], (float)e2[1]);
  t.r2 = make_float4((float)e2[2], (float)n[0], (float)n[1], (float)n[2]);
  t.r3 = make_float4((float)(p[0][0] + m[0]), (float)(p[0][1] + m[1]), (float)(p[0][2] + m[2]),
                     isfinite(rr) ? (float)rr : INFINITY);
  return t;
}

}  // namespace gwn
