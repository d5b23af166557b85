// Query ordering for the Barnes-Hut walks: queries grouped by their cell of a
// 256^3 Morton grid over the tree's bounding box (one counting pass), the
// permutation handed to the walk.
#include <cuda_runtime.h>

#include "bh_common.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

constexpr int64_t kMinOrdered = 8192;  // smaller batches are walked in input order

template <typename QT>
__global__ void query_keys_kernel(const QT* __restrict__ Q, int64_t n, float3 lo, float3 inv,
                                  uint32_t* __restrict__ keys) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = (float)Q[i * 3 + 0], y = (float)Q[i * 3 + 1], z = (float)Q[i * 3 + 2];
  auto q = [](float v, float l, float s) -> uint32_t {
    float t = (v - l) * s;
    t = fminf(fmaxf(t, 0.f), 1023.f);  // NaN -> 0 via fmaxf
    return (uint32_t)t;
  };
  // the cell of 256^3 over the box: the top 24 bits of the 30-bit Morton code
  keys[i] = ((spread10(q(x, lo.x, inv.x)) << 2) | (spread10(q(y, lo.y, inv.y)) << 1) |
             spread10(q(z, lo.z, inv.z))) >> 6;
}

}  // namespace

void order_queries(const void* Q, int q_dtype, int64_t nQ, const double lo[3], const double hi[3],
                   QueryOrder& out, cudaStream_t st) {
  out.active = false;
  if (nQ < kMinOrdered) return;
  GWN_REQUIRE(nQ < (int64_t(1) << 31), "at most 2^31-1 queries per call");
  // grow the box a little so queries just outside still spread over keys
  float3 l, inv;
  double c[3], h[3];
  for (int d = 0; d < 3; ++d) {
    c[d] = 0.5 * (lo[d] + hi[d]);
    h[d] = 0.5 * (hi[d] - lo[d]) * 1.25 + 1e-12;
  }
  l = make_float3((float)(c[0] - h[0]), (float)(c[1] - h[1]), (float)(c[2] - h[2]));
  inv = make_float3((float)(1024.0 / (2 * h[0])), (float)(1024.0 / (2 * h[1])),
                    (float)(1024.0 / (2 * h[2])));
  DevBuf<uint32_t> keys((size_t)nQ, st);
  out.perm.alloc((size_t)nQ, st);
  const unsigned grid = (unsigned)((nQ + 255) / 256);
  if (q_dtype == GWN_F64)
    launch_kernel(query_keys_kernel<double>, grid, 256, 0, st, static_cast<const double*>(Q), nQ,
                  l, inv, keys.get());
  else
    launch_kernel(query_keys_kernel<float>, grid, 256, 0, st, static_cast<const float*>(Q), nQ,
                  l, inv, keys.get());
  bucket_order(keys.get(), nQ, 1u << 24, out.perm.get(), st);
  out.active = true;
}

}  // namespace gwn
