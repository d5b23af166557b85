// Pieces shared by the Barnes-Hut paths (triangle soup and point cloud):
// Morton keys, query ordering, and the FP64 decision / guard-band rule that
// keeps the mixed-precision traversal's open/approximate decisions identical
// to the plain FP64 traversal's.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

// Spread the low 10 / 21 bits of x so that two zero bits separate each bit.
__host__ __device__ inline uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
__host__ __device__ inline unsigned long long spread21(unsigned long long x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

// Query ordering for warp coherence: 30-bit Morton key of each query inside
// a box (lo, inv_extent), sorted; the traversal then reads queries through
// the returned permutation.
struct QueryOrder {
  DevBuf<int32_t> perm;
  bool active = false;
};

// Builds `out.perm` (or leaves it inactive for tiny batches).  Q is nQ x 3 of
// QT (float or double), device memory.
void order_queries(const void* Q, int q_dtype, int64_t nQ, const double lo[3],
                   const double hi[3], QueryOrder& out, cudaStream_t st);

#ifdef __CUDACC__
// Precision-exact math for the templated walks: the float versions must not
// promote to double (FP64 is a slow pipe on this GPU).
__device__ __forceinline__ float g_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double g_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float g_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double g_rsqrt(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float g_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double g_atan2(double y, double x) { return atan2(y, x); }
// 256-bit read-only global load (ld.global.nc.v8, sm_100 and later) of the
// 32 bytes at p, which must be 32-byte aligned.
__device__ __forceinline__ void ldg256(const void* p, float4& lo, float4& hi) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z),
        "=f"(hi.w)
      : "l"(p));
}
__device__ __forceinline__ float g_rcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double g_rcp(double x) { return 1.0 / x; }

// The FP64 open test shared by both precisions: open (do not approximate)
// iff |q - c|^2 <= r2max * beta2.  Operations are pinned (no contraction) so
// that every kernel evaluates the identical expression.
__device__ __forceinline__ bool open_test64(double qx, double qy, double qz, double cx,
                                            double cy, double cz, double r2max, double beta2) {
  const double dx = __dsub_rn(qx, cx), dy = __dsub_rn(qy, cy), dz = __dsub_rn(qz, cz);
  const double r2 = __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
  return r2 <= __dmul_rn(r2max, beta2);
}

// Whether an FP32 comparison of r2 against thr may disagree with the FP64
// one.  With u = 2^-24 and S = max|q| + max|c|, the FP32 error of r2 - thr
// is at most (eps + 3u) r2 + 3u thr + 3 delta^2 (1 + 1/eps), delta = 3 u S,
// eps = 1e-5; the band below doubles that bound.
__device__ __forceinline__ bool in_guard_band(float r2, float thr, float sigma) {
  return fabsf(r2 - thr) <= fmaf(2e-5f, r2 + thr, sigma);
}
__host__ __device__ inline float guard_sigma(float S) { return 2e-8f * S * S; }
#endif

}  // namespace gwn
