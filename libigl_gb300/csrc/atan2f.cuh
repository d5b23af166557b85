// FP32 atan2 shared by the FP32 angle terms of the exact 3-D sum (exact.cu)
// and of the 2-D tree walk (eytzinger.cu).
#pragma once

#include <cuda_runtime.h>

namespace gwn {

// atan2 for the FP32 pair terms.  atan(t) on [0, 1] is t * P(t^2) with P of
// degree 8, its coefficients fitted here to atan(sqrt(s))/sqrt(s) on [0, 1]
// by least squares in the relative error with Lawson reweighting (towards
// the minimax fit); relative fit error 1.5e-8, 2 ulp with FP32 Horner.  The
// octants follow from atan(y/x) = pi/2 - atan(x/y) and the reflection
// x -> -x (angle -> pi - angle); the sign is y's.  (0, 0) gives 0.
// tests/test_oracle.py re-checks these coefficients in FP32 against atan.
__device__ __forceinline__ float atan2_pairs(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float t = __fdividef(mn, mx);
  const float s = t * t;
  float p = 2.849886427e-03f;
  p = fmaf(p, s, -1.606861688e-02f);
  p = fmaf(p, s, 4.269149899e-02f);
  p = fmaf(p, s, -7.504292578e-02f);
  p = fmaf(p, s, 1.064093336e-01f);
  p = fmaf(p, s, -1.420364380e-01f);
  p = fmaf(p, s, 1.999261975e-01f);
  p = fmaf(p, s, -3.333307207e-01f);
  p = fmaf(p, s, 1.0f);
  float r = t * p;
  r = ay > ax ? 1.57079632679489662f - r : r;
  r = x < 0.f ? 3.14159265358979324f - r : r;
  r = copysignf(r, y);
  return mx == 0.f ? 0.f : r;
}

}  // namespace gwn
