// Exact generalized winding number: an n-body sweep of every query against
// every triangle (or edge), summing the per-element solid angle.
//
// Reference semantics: igl::winding_number(V,F,O,W), include/igl/
// winding_number.cpp:17-56, evaluates per query sum_f solid_angle(f, p)
// (winding_number.cpp:58-89 with solid_angle.cpp:16-54).  The reference
// evaluates it through a cap hierarchy (WindingNumberAABB) that returns the
// same sum up to rounding; this kernel sums every element directly.
//
// Layout and schedule (sm_103a):
//  * triangles are pre-packed once per call into 64-byte FP32 records
//    {a, e1=b-a, e2=c-a, n=e1 x e2, centroid, (R+eps)^2} (edges, normal and
//    centroid formed in FP64, then rounded) and grouped into tiles of
//    kTile triangles with a bounding sphere per tile;
//  * each CTA owns 256 queries (one per thread) and streams the triangle
//    tiles through shared memory with 1-D bulk copies (cp.async.bulk) on a
//    3-stage mbarrier ring; every thread reads each triangle as a broadcast;
//  * FP32 per pair: van Oosterom-Strackee tan(Omega/2) = det / den with
//    det = (a-q).n; a tile whose bounding sphere (grown by eps = 1e-3 * bbox
//    diagonal) contains the query of any lane in the warp is swept with a
//    per-pair near test, and near pairs are evaluated in FP64 from the
//    original vertices with the reference's own formula;
//  * queries whose FP32 result lands within 1e-3 of 0.5 are appended to a
//    list and re-evaluated entirely in FP64 by a block-per-query kernel.
// The plain FP64 path uses the reference formula for every pair.
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <mutex>
#include <string>
#include <type_traits>

#include "atan2f.cuh"
#include "exact_terms.cuh"
#include "gwn_common.cuh"
#include "gwn_internal.cuh"

namespace gwn {
namespace {

constexpr int kTile = 128;        // triangles per tile
constexpr int kStages = 3;        // bulk-copy ring depth
constexpr int kThreads = 256;     // queries per CTA
constexpr int kTile64 = 64;       // triangles per FP64 tile
constexpr double kNearFrac = 1e-3;
// Mixed-precision calls with at least this many triangles and queries use
// the cap hierarchy; below, building it costs about what all pairs do.
constexpr int64_t kHierMinTriangles = 4096;
constexpr int64_t kHierMinQueries = 1024;
constexpr double kBand = 1e-3;    // |W - 0.5| band that triggers FP64 re-evaluation
constexpr float kInv2PiF = 0.15915494309189533577f;
constexpr double kInv2Pi = 0.15915494309189533577;




// After a failed wait at tile `stop`, wait (bounded) for every copy that was
// issued into the ring: tiles 0 .. min(stop - 1 + stages, ntiles - 1).
__device__ void drain_ring(uint64_t* bar, int stages, int stop, int ntiles) {
  const int last = min(stop - 1 + stages, ntiles - 1);
  for (int s = 0; s < stages; ++s) {
    int L = -1;
    for (int t = last; t >= 0 && t > last - stages; --t)
      if (t % stages == s) L = t;
    if (L >= 0) (void)mbar_wait_bounded(&bar[s], (uint32_t)((L / stages) & 1));
  }
}


template <typename T>
__device__ __forceinline__ void load_q3(const T* Q, int64_t i, double& x, double& y, double& z) {
  x = (double)Q[i * 3 + 0];
  y = (double)Q[i * 3 + 1];
  z = (double)Q[i * 3 + 2];
}

// ------------------------------------------------------------ preprocessing --
__global__ void bbox_kernel(const double* __restrict__ V, int64_t nV, int dim,
                            unsigned long long* __restrict__ mm /* 2*dim ordered */) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nV;
       i += (int64_t)gridDim.x * blockDim.x) {
    for (int d = 0; d < dim; ++d) {
      const double v = V[i * dim + d];
      if (isfinite(v)) {
        lo[d] = fmin(lo[d], v);
        hi[d] = fmax(hi[d], v);
      }
    }
  }
  for (int d = 0; d < dim; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int d = 0; d < dim; ++d) {
      atomicMin(&mm[d], ordered_bits(lo[d]));
      atomicMax(&mm[dim + d], ordered_bits(hi[d]));
    }
  }
}

__global__ void pack_tris_kernel(const double* __restrict__ V, int64_t nV,
                                 const int32_t* __restrict__ F, int64_t nF, int64_t nPad,
                                 const unsigned long long* __restrict__ mm, TriF* __restrict__ out,
                                 double* __restrict__ out64, unsigned* __restrict__ status) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (f >= nPad) return;
  double diag2 = 0;
  for (int d = 0; d < 3; ++d) {
    const double e = from_ordered_bits(mm[3 + d]) - from_ordered_bits(mm[d]);
    if (isfinite(e) && e > 0) diag2 += e * e;
  }
  const double eps = kNearFrac * sqrt(diag2);
  TriF t;
  if (f >= nF) {  // padding: a zero triangle contributes atan2(0, >=0) = 0
    t.r0 = make_float4(0.f, 0.f, 0.f, 0.f);
    t.r1 = t.r0;
    t.r2 = t.r0;
    t.r3 = make_float4(0.f, 0.f, 0.f, -1.f);
    out[f] = t;
    for (int k = 0; k < 9; ++k) out64[f * 9 + k] = 0.0;
    return;
  }
  int32_t idx[3];
  for (int c = 0; c < 3; ++c) {
    idx[c] = F[f * 3 + c];
    if (idx[c] < 0 || idx[c] >= nV) {
      atomicOr(status, kStatusBadInput);
      idx[c] = 0;
    }
  }
  double p[3][3];
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) p[c][d] = V[(int64_t)idx[c] * 3 + d];
  out[f] = make_trif(p, eps);
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) out64[f * 9 + c * 3 + d] = p[c][d];
}

// Per-tile bounding sphere of the triangles' spheres, grown by eps; stored as
// (centre, radius^2) with a safety margin so FP32 tests stay conservative.
__global__ void tile_meta_kernel(const TriF* __restrict__ tris, int ntiles,
                                 const unsigned long long* __restrict__ mm,
                                 float4* __restrict__ meta) {
  const int tile = blockIdx.x;
  const int i = threadIdx.x;  // kTile threads
  const TriF t = tris[(int64_t)tile * kTile + i];
  const bool pad = t.r3.w < 0.f;
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    const double c = d == 0 ? t.r3.x : (d == 1 ? t.r3.y : t.r3.z);
    lo[d] = pad ? INFINITY : c;
    hi[d] = pad ? -INFINITY : c;
  }
  __shared__ double s_lo[3][kTile / 32], s_hi[3][kTile / 32];
  __shared__ double s_c[3];
  __shared__ double s_r[kTile / 32];
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
    if ((i & 31) == 0) {
      s_lo[d][i >> 5] = lo[d];
      s_hi[d][i >> 5] = hi[d];
    }
  }
  __syncthreads();
  if (i < 3) {
    double l = INFINITY, h = -INFINITY;
    for (int w = 0; w < kTile / 32; ++w) {
      l = fmin(l, s_lo[i][w]);
      h = fmax(h, s_hi[i][w]);
    }
    s_c[i] = (l <= h) ? 0.5 * (l + h) : 0.0;
  }
  __syncthreads();
  double r = 0;
  if (!pad) {
    const double dx = t.r3.x - s_c[0], dy = t.r3.y - s_c[1], dz = t.r3.z - s_c[2];
    r = sqrt(dx * dx + dy * dy + dz * dz) + sqrt((double)t.r3.w);  // r3.w already includes eps
  }
  for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
  if ((i & 31) == 0) s_r[i >> 5] = r;
  __syncthreads();
  if (i == 0) {
    double R = 0;
    for (int w = 0; w < kTile / 32; ++w) R = fmax(R, s_r[w]);
    const double R2 = R * R * (1.0 + 1e-5) + 1e-30;
    meta[tile] = make_float4((float)s_c[0], (float)s_c[1], (float)s_c[2],
                             isfinite(R2) ? (float)R2 : INFINITY);
  }
}

// ------------------------------------------------------------ mixed kernel --
struct Smem3 {
  TriF tiles[kStages][kTile];
  uint64_t bar[kStages];
  int2 near_q[kThreads / 32][32];  // per-warp queue of (triangle, lane) near pairs
};

// Evaluate the n queued near pairs of this warp in FP64, one per lane, so each
// FP64 instruction serves the whole warp instead of the few lanes that share
// a triangle; every lane then adds its own terms in queue (= triangle) order.
__device__ __forceinline__ void flush_near_pairs(const double* __restrict__ tris64,
                                                 const int2* q, int n, double qx, double qy,
                                                 double qz, double& near_acc) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  int2 e = make_int2(0, lane);
  if (lane < n) e = q[lane];
  const double ox = __shfl_sync(full, qx, e.y), oy = __shfl_sync(full, qy, e.y),
               oz = __shfl_sync(full, qz, e.y);
  double v = 0.0;
  if (lane < n) {
    const double* g = tris64 + (int64_t)e.x * 9;
    v = vos_term64(g, g + 3, g + 6, ox, oy, oz);
  }
  for (int k = 0; k < n; ++k) {
    const double vk = __shfl_sync(full, v, k);
    const int ok = __shfl_sync(full, e.y, k);
    if (ok == lane) near_acc += vk;
  }
  __syncwarp();
}

template <typename QT, typename WT>
__global__ void __launch_bounds__(kThreads) exact3_mixed_kernel(
    const TriF* __restrict__ tris, const double* __restrict__ tris64,
    const float4* __restrict__ meta, int ntiles, const QT* __restrict__ Q, int64_t nQ,
    WT* __restrict__ W, int32_t* __restrict__ refine_list, unsigned* __restrict__ refine_count,
    unsigned* __restrict__ status, int withhold) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem3& sm = *reinterpret_cast<Smem3*>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t qi = blockIdx.x * (int64_t)kThreads + tid;
  const bool valid = qi < nQ;
  double qx = 0, qy = 0, qz = 0;
  if (valid) load_q3(Q, qi, qx, qy, qz);
  const float fx = (float)qx, fy = (float)qy, fz = (float)qz;

  constexpr uint32_t kTileBytes = sizeof(TriF) * kTile;
  if (tid == 0) {
    // withhold != 0 (failure-path tests only): stage 0 expects one more
    // arrival than is ever made, so the first wait runs out of its budget.
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.bar[s], (withhold && s == 0) ? 2 : 1);
    fence_mbar_init();
    for (int s = 0; s < kStages && s < ntiles; ++s) {
      mbar_arrive_expect_tx(&sm.bar[s], kTileBytes);
      bulk_g2s(&sm.tiles[s][0], tris + (int64_t)s * kTile, kTileBytes, &sm.bar[s]);
    }
  }
  __syncthreads();

  float acc = 0.f, comp = 0.f;  // Kahan over tile sums
  double near_acc = 0.0;
  bool any_near = false;
  bool ok = true;
  int stop_tile = 0;
  int nqueued = 0;  // warp-uniform length of this warp's near-pair queue
  int2* nq = sm.near_q[tid >> 5];
  const unsigned lane_lt = (1u << (tid & 31)) - 1u;
  for (int t = 0; t < ntiles; ++t) {
    const int s = t % kStages;
    const uint32_t parity = (uint32_t)((t / kStages) & 1);
    const bool got = mbar_wait_bounded(&sm.bar[s], parity);
    if (!__syncthreads_and(got)) {
      ok = false;
      stop_tile = t;
      break;
    }
    const float4 mt = __ldg(&meta[t]);
    const float dx = fx - mt.x, dy = fy - mt.y, dz = fz - mt.z;
    const bool tile_near = valid && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < mt.w;
    float ssum = 0.f;
    const TriF* tile = sm.tiles[s];
    if (__any_sync(0xffffffffu, tile_near)) {
#pragma unroll 2
      for (int k = 0; k < kTile; ++k) {
        const TriF tr = tile[k];
        const float ex = tr.r3.x - fx, ey = tr.r3.y - fy, ez = tr.r3.z - fz;
        const bool near = valid && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < tr.r3.w;
        if (!near) ssum += vos_term32(tr, fx, fy, fz);
        // near pairs go to the warp's queue and are evaluated in FP64 32 at a
        // time, one per lane (flush_near_pairs)
        const unsigned m = __ballot_sync(0xffffffffu, near);
        if (m) {
          const int c = __popc(m);
          if (nqueued + c > 32) {
            flush_near_pairs(tris64, nq, nqueued, qx, qy, qz, near_acc);
            nqueued = 0;
          }
          if (near) nq[nqueued + __popc(m & lane_lt)] = make_int2(t * kTile + k, tid & 31);
          nqueued += c;
          any_near |= near;
        }
      }
    } else {
#pragma unroll 4
      for (int k = 0; k < kTile; ++k) ssum += vos_term32(tile[k], fx, fy, fz);
    }
    const float y = ssum - comp;
    const float tt = acc + y;
    comp = (tt - acc) - y;
    acc = tt;
    __syncthreads();  // every thread is done with stage s
    if (tid == 0 && t + kStages < ntiles) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&sm.bar[s], kTileBytes);
      bulk_g2s(&sm.tiles[s][0], tris + (int64_t)(t + kStages) * kTile, kTileBytes, &sm.bar[s]);
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicOr(status, kStatusWaitTimeout);
      if (withhold) mbar_arrive(&sm.bar[0]);  // the withheld arrival: stage 0 can drain
      drain_ring(sm.bar, kStages, stop_tile, ntiles);
    }
    return;
  }
  if (nqueued) flush_near_pairs(tris64, nq, nqueued, qx, qy, qz, near_acc);
  if (!valid) return;
  double w;
  if (any_near)
    w = ((double)acc + near_acc) * kInv2Pi;
  else
    w = (double)(acc * kInv2PiF);
  W[qi] = (WT)w;
  if (fabs(w - 0.5) <= kBand) {
    const unsigned slot = atomicAdd(refine_count, 1u);
    refine_list[slot] = (int32_t)qi;
  }
}

// ------------------------------------------------------------ FP64 kernels --
struct Smem64 {
  double tiles[kStages][kTile64 * 9];
  uint64_t bar[kStages];
};

template <typename QT, typename WT>
__global__ void __launch_bounds__(kThreads) exact3_fp64_kernel(const double* __restrict__ tris64,
                                                               int ntiles64,
                                                               const QT* __restrict__ Q,
                                                               int64_t nQ, WT* __restrict__ W,
                                                               unsigned* __restrict__ status,
                                                               int withhold) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem64& sm = *reinterpret_cast<Smem64*>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t qi = blockIdx.x * (int64_t)kThreads + tid;
  const bool valid = qi < nQ;
  double qx = 0, qy = 0, qz = 0;
  if (valid) load_q3(Q, qi, qx, qy, qz);
  constexpr uint32_t kBytes = sizeof(double) * 9 * kTile64;
  if (tid == 0) {
    // withhold != 0 (failure-path tests only): stage 0 expects one more
    // arrival than is ever made, so the first wait runs out of its budget.
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.bar[s], (withhold && s == 0) ? 2 : 1);
    fence_mbar_init();
    for (int s = 0; s < kStages && s < ntiles64; ++s) {
      mbar_arrive_expect_tx(&sm.bar[s], kBytes);
      bulk_g2s(&sm.tiles[s][0], tris64 + (int64_t)s * kTile64 * 9, kBytes, &sm.bar[s]);
    }
  }
  __syncthreads();
  double acc = 0.0;
  bool ok = true;
  int stop_tile = 0;
  for (int t = 0; t < ntiles64; ++t) {
    const int s = t % kStages;
    const bool got = mbar_wait_bounded(&sm.bar[s], (uint32_t)((t / kStages) & 1));
    if (!__syncthreads_and(got)) {
      ok = false;
      stop_tile = t;
      break;
    }
    const double* tile = sm.tiles[s];
    for (int k = 0; k < kTile64; ++k) {
      const double* g = tile + k * 9;
      acc += vos_term64(g, g + 3, g + 6, qx, qy, qz);
    }
    __syncthreads();
    if (tid == 0 && t + kStages < ntiles64) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&sm.bar[s], kBytes);
      bulk_g2s(&sm.tiles[s][0], tris64 + (int64_t)(t + kStages) * kTile64 * 9, kBytes,
               &sm.bar[s]);
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicOr(status, kStatusWaitTimeout);
      if (withhold) mbar_arrive(&sm.bar[0]);  // the withheld arrival: stage 0 can drain
      drain_ring(sm.bar, kStages, stop_tile, ntiles64);
    }
    return;
  }
  if (valid) W[qi] = (WT)(acc / (2.0 * kPi));
}

// Block-per-query FP64 re-evaluation of the listed queries (persistent over
// the device-side count, deterministic fixed-order block reduction).
template <typename QT, typename WT>
__global__ void __launch_bounds__(kThreads) exact3_refine_kernel(
    const double* __restrict__ tris64, int64_t nF, const QT* __restrict__ Q,
    WT* __restrict__ W, const int32_t* __restrict__ list, const unsigned* __restrict__ count) {
  __shared__ double red[kThreads / 32];
  const unsigned n = *count;
  for (unsigned j = blockIdx.x; j < n; j += gridDim.x) {
    const int64_t qi = list[j];
    double qx, qy, qz;
    load_q3(Q, qi, qx, qy, qz);
    double acc = 0.0;
    for (int64_t f = threadIdx.x; f < nF; f += kThreads) {
      const double* g = tris64 + f * 9;
      acc += vos_term64(g, g + 3, g + 6, qx, qy, qz);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < kThreads / 32; ++w) s += red[w];
      W[qi] = (WT)(s / (2.0 * kPi));
    }
    __syncthreads();
  }
}

// 2D: sum of signed angles of edges, include/igl/signed_angle.cpp:14-45, FP64.
template <typename QT, typename WT>
__global__ void exact2_kernel(const double* __restrict__ V, int64_t nV,
                              const int32_t* __restrict__ F, int64_t nF,
                              const QT* __restrict__ Q, int64_t nQ, WT* __restrict__ W,
                              unsigned* __restrict__ status) {
  const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (qi >= nQ) return;
  const double px = (double)Q[qi * 2], py = (double)Q[qi * 2 + 1];
  double acc = 0;
  for (int64_t f = 0; f < nF; ++f) {
    int32_t i0 = __ldg(&F[f * 2]), i1 = __ldg(&F[f * 2 + 1]);
    if (i0 < 0 || i0 >= nV || i1 < 0 || i1 >= nV) {
      atomicOr(status, kStatusBadInput);
      continue;
    }
    double ax = px - __ldg(&V[(int64_t)i0 * 2]), ay = py - __ldg(&V[(int64_t)i0 * 2 + 1]);
    double bx = px - __ldg(&V[(int64_t)i1 * 2]), by = py - __ldg(&V[(int64_t)i1 * 2 + 1]);
    const double al = sqrt(ax * ax + ay * ay), bl = sqrt(bx * bx + by * by);
    if (al != 0) {
      ax /= al;
      ay /= al;
    }
    if (bl != 0) {
      bx /= bl;
      by /= bl;
    }
    acc += -atan2(bx * ay - by * ax, bx * ax + by * ay) / (2.0 * kPi);
  }
  W[qi] = (WT)acc;
}

template <typename A, typename B>
__global__ void convert_kernel(const A* __restrict__ in, B* __restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (B)in[i];
}

template <typename QT, typename WT>
void launch_exact3(const ExactArgs& a, cudaStream_t st) {
  // Large meshes: the cap hierarchy (hier.cu), the reference's own algorithm
  // for winding_number (winding_number.cpp:40-53, WindingNumberTree.h:
  // 261-336), gives the all-pairs value up to rounding at a cost that grows
  // far slower than #F; in plain FP64 every term is FP64, in mixed precision
  // the terms are FP32 with FP64 near terms and threshold re-evaluation
  // (within 4.1e-7 of the FP64 sum where the all-pairs mixed sweep reaches
  // 3e-6).  Float32 queries / results are widened / narrowed around it.
  if (a.nF >= kHierMinTriangles && a.nQ >= kHierMinQueries) {
    DeviceStatus status(st, a.host_mode);
    HierTree h;
    hier_build(a.V, a.nV, a.F, a.nF, h, status.ptr(), st, true);
    const double* Qd = static_cast<const double*>(a.Q);
    double* Wd = static_cast<double*>(a.W);
    DevBuf<double> q64, w64;
    if (!std::is_same<QT, double>::value) {
      q64.alloc((size_t)a.nQ * 3, st);
      launch_kernel(convert_kernel<QT, double>, (unsigned)((a.nQ * 3 + 255) / 256), 256, 0, st,
                    static_cast<const QT*>(a.Q), q64.get(), a.nQ * 3);
      Qd = q64.get();
    }
    if (!std::is_same<WT, double>::value) {
      w64.alloc((size_t)a.nQ, st);
      Wd = w64.get();
    }
    hier_eval(h, Qd, a.nQ, Wd, st, a.precision);
    if (!std::is_same<WT, double>::value)
      launch_kernel(convert_kernel<double, WT>, (unsigned)((a.nQ + 255) / 256), 256, 0, st,
                    (const double*)w64.get(), static_cast<WT*>(a.W), a.nQ);
    status.check(st, "winding_number (hierarchy)");
    return;
  }
  const int64_t nPad = ((a.nF + kTile - 1) / kTile) * (int64_t)kTile;
  const int ntiles = (int)(nPad / kTile);
  DeviceStatus status(st, a.host_mode);
  DevBuf<unsigned long long> mm(6, st);
  init_minmax(mm.get(), 3, st);
  launch_kernel(bbox_kernel, std::max(1, std::min(num_sms() * 4, (int)((a.nV + 255) / 256))), 256, 0, st, 
      a.V, a.nV, 3, mm.get());
  DevBuf<TriF> tris((size_t)std::max<int64_t>(nPad, 1), st);
  DevBuf<double> tris64((size_t)std::max<int64_t>(nPad, 1) * 9, st);
  if (nPad > 0) {
    launch_kernel(pack_tris_kernel, (unsigned)((nPad + 255) / 256), 256, 0, st, 
        a.V, a.nV, a.F, a.nF, nPad, mm.get(), tris.get(), tris64.get(), status.ptr());
  }
  const unsigned grid = (unsigned)((a.nQ + kThreads - 1) / kThreads);
  const QT* Q = static_cast<const QT*>(a.Q);
  WT* W = static_cast<WT*>(a.W);
  if (a.precision == GWN_MIXED) {
    DevBuf<float4> meta((size_t)std::max(ntiles, 1), st);
    if (ntiles > 0) launch_kernel(tile_meta_kernel, ntiles, kTile, 0, st, tris.get(), ntiles, mm.get(), meta.get());
    DevBuf<int32_t> list((size_t)std::max<int64_t>(a.nQ, 1), st);
    DevBuf<unsigned> count(1, st);
    count.zero(st);
    if (grid > 0) {
      const size_t smem = sizeof(Smem3);
      GWN_CUDA(cudaFuncSetAttribute(exact3_mixed_kernel<QT, WT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      {
        PhaseTimer ph("nbody", st);
        launch_kernel(exact3_mixed_kernel<QT, WT>, grid, kThreads, smem, st, 
            tris.get(), tris64.get(), meta.get(), ntiles, Q, a.nQ, W, list.get(), count.get(),
            status.ptr(), take_wait_injection());
      }
      GWN_CUDA(cudaGetLastError());
      {
        PhaseTimer ph("refine", st);
        launch_kernel(exact3_refine_kernel<QT, WT>, num_sms() * 4, kThreads, 0, st, 
            tris64.get(), a.nF, Q, W, list.get(), count.get());
      }
      GWN_CUDA(cudaGetLastError());
    }
    status.check(st, "winding_number (mixed)");
  } else {
    const int64_t nPad64 = ((nPad + kTile64 - 1) / kTile64) * (int64_t)kTile64;  // == nPad
    const int ntiles64 = (int)(nPad64 / kTile64);
    if (grid > 0) {
      const size_t smem = sizeof(Smem64);
      GWN_CUDA(cudaFuncSetAttribute(exact3_fp64_kernel<QT, WT>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      PhaseTimer ph("nbody", st);
      launch_kernel(exact3_fp64_kernel<QT, WT>, grid, kThreads, smem, st, tris64.get(), ntiles64, Q,
                                                                a.nQ, W, status.ptr(),
                                                                take_wait_injection());
      GWN_CUDA(cudaGetLastError());
    }
    status.check(st, "winding_number (fp64)");
  }
}

template <typename QT, typename WT>
void launch_exact2(const ExactArgs& a, cudaStream_t st) {
  DeviceStatus status(st, a.host_mode);
  if (a.nQ > 0) {
    launch_kernel(exact2_kernel<QT, WT>, (unsigned)((a.nQ + 127) / 128), 128, 0, st, 
        a.V, a.nV, a.F, a.nF, static_cast<const QT*>(a.Q), a.nQ, static_cast<WT*>(a.W),
        status.ptr());
    GWN_CUDA(cudaGetLastError());
  }
  status.check(st, "winding_number (2d)");
}

}  // namespace

void exact_refine_listed(const double* tris64, int64_t nF, const double* Q, const int32_t* list,
                         const unsigned* count, double* W, cudaStream_t st) {
  launch_kernel(exact3_refine_kernel<double, double>, num_sms() * 4, kThreads, 0, st, tris64, nF, Q,
                W, list, count);
}

void run_exact(const ExactArgs& a, cudaStream_t st) {
  const bool qd = a.q_dtype == GWN_F64, wd = a.w_dtype == GWN_F64;
  if (a.dim == 3) {
    if (qd && wd) launch_exact3<double, double>(a, st);
    else if (qd) launch_exact3<double, float>(a, st);
    else if (wd) launch_exact3<float, double>(a, st);
    else launch_exact3<float, float>(a, st);
  } else {
    if (qd && wd) launch_exact2<double, double>(a, st);
    else if (qd) launch_exact2<double, float>(a, st);
    else if (wd) launch_exact2<float, double>(a, st);
    else launch_exact2<float, float>(a, st);
  }
}


// ---------------------------------------------------------------------------
// No-allocation variant (gwn_winding_number_noalloc).
//
// For callers that must not allocate device memory during a call -- hosts
// that own every device allocation through their own pool and forbid foreign
// cudaMalloc, or latency-critical loops where cudaMalloc / cudaFree would
// synchronize the device.  The caller passes device inputs and outputs; the
// call's scratch (packed FP32 triangle tiles, tile bounding spheres, bbox
// words) lives in the file-scope array below, sized for kNoAllocMaxTris
// triangles (4,203,616 bytes, held by every GPU that loads the library until
// the process exits).  Every call shares the array and leaves its contents
// behind, so calls that overlap on the GPU (different streams) race; calls
// on one stream are ordered.  The first call on a device looks up the
// array's device address (cudaGetSymbolAddress, with that device current);
// make that first call before any stream capture.  The address is kept for
// the life of the process: it does not survive cudaDeviceReset or any other
// teardown of the device's primary context, after which the entry point must
// not be called.
// ---------------------------------------------------------------------------
namespace {

constexpr int64_t kNoAllocMaxTris = 65536;
constexpr int kNoAllocMaxTiles = (int)(kNoAllocMaxTris / kTile);
struct NoAllocScratch {
  TriF tris[kNoAllocMaxTris];          // 4 MiB
  float4 meta[kNoAllocMaxTiles];       // 8 KiB
  unsigned long long mm[6];            // bbox as ordered bits
  // Failures of calls made without a status word of their own.  Never
  // cleared by a call (zero at module load): gwn_device_status reads and
  // clears it together with the library's other sticky word.
  unsigned sticky_status;
};
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__global__ void noalloc_init_kernel(NoAllocScratch* s) {
  const int i = threadIdx.x;
  if (i < 3) s->mm[i] = ~0ull;
  else if (i < 6) s->mm[i] = 0ull;
}

// FP32 packing only (near pairs read the caller's FP64 V/F directly).
__global__ void noalloc_pack_kernel(const double* __restrict__ V, int64_t nV,
                                    const int32_t* __restrict__ F, int64_t nF, int64_t nPad,
                                    const unsigned long long* __restrict__ mm,
                                    TriF* __restrict__ out, unsigned* __restrict__ status) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (f >= nPad) return;
  double diag2 = 0;
  for (int d = 0; d < 3; ++d) {
    const double e = from_ordered_bits(mm[3 + d]) - from_ordered_bits(mm[d]);
    if (isfinite(e) && e > 0) diag2 += e * e;
  }
  const double eps = kNearFrac * sqrt(diag2);
  TriF t;
  if (f >= nF) {
    t.r0 = make_float4(0.f, 0.f, 0.f, 0.f);
    t.r1 = t.r0;
    t.r2 = t.r0;
    t.r3 = make_float4(0.f, 0.f, 0.f, -1.f);
    out[f] = t;
    return;
  }
  int32_t idx[3];
  for (int c = 0; c < 3; ++c) {
    idx[c] = F[f * 3 + c];
    if (idx[c] < 0 || idx[c] >= nV) {
      atomicOr(status, kStatusBadInput);
      idx[c] = 0;
    }
  }
  double p[3][3];
  for (int c = 0; c < 3; ++c)
    for (int d = 0; d < 3; ++d) p[c][d] = V[(int64_t)idx[c] * 3 + d];
  out[f] = make_trif(p, eps);
}

__device__ __forceinline__ double vos_term64_indexed(const double* __restrict__ V,
                                                     const int32_t* __restrict__ F, int64_t nV,
                                                     int64_t f, double qx, double qy, double qz) {
  int32_t i0 = F[f * 3], i1 = F[f * 3 + 1], i2 = F[f * 3 + 2];
  if (i0 < 0 || i0 >= nV) i0 = 0;
  if (i1 < 0 || i1 >= nV) i1 = 0;
  if (i2 < 0 || i2 >= nV) i2 = 0;
  return vos_term64(V + (int64_t)i0 * 3, V + (int64_t)i1 * 3, V + (int64_t)i2 * 3, qx, qy, qz);
}

// The mixed sweep of exact3_mixed_kernel over the static tiles; FP64 near
// pairs read the caller's V/F; no re-evaluation list is kept.
__global__ void __launch_bounds__(kThreads) noalloc_mixed_kernel(
    const TriF* __restrict__ tris, const float4* __restrict__ meta, int ntiles,
    const double* __restrict__ V, int64_t nV, const int32_t* __restrict__ F,
    const double* __restrict__ Q, int64_t nQ, double* __restrict__ W,
    unsigned* __restrict__ status, int withhold) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem3& sm = *reinterpret_cast<Smem3*>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t qi = blockIdx.x * (int64_t)kThreads + tid;
  const bool valid = qi < nQ;
  double qx = 0, qy = 0, qz = 0;
  if (valid) load_q3(Q, qi, qx, qy, qz);
  const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
  constexpr uint32_t kTileBytes = sizeof(TriF) * kTile;
  if (tid == 0) {
    // withhold != 0 (failure-path tests only): stage 0 expects one more
    // arrival than is ever made, so the first wait runs out of its budget.
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.bar[s], (withhold && s == 0) ? 2 : 1);
    fence_mbar_init();
    for (int s = 0; s < kStages && s < ntiles; ++s) {
      mbar_arrive_expect_tx(&sm.bar[s], kTileBytes);
      bulk_g2s(&sm.tiles[s][0], tris + (int64_t)s * kTile, kTileBytes, &sm.bar[s]);
    }
  }
  __syncthreads();
  float acc = 0.f, comp = 0.f;
  double near_acc = 0.0;
  bool any_near = false, ok = true;
  int stop_tile = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int s = t % kStages;
    const bool got = mbar_wait_bounded(&sm.bar[s], (uint32_t)((t / kStages) & 1));
    if (!__syncthreads_and(got)) {
      ok = false;
      stop_tile = t;
      break;
    }
    const float4 mt = __ldg(&meta[t]);
    const float dx = fx - mt.x, dy = fy - mt.y, dz = fz - mt.z;
    const bool tile_near = valid && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < mt.w;
    float ssum = 0.f;
    const TriF* tile = sm.tiles[s];
    if (__any_sync(0xffffffffu, tile_near)) {
      for (int k = 0; k < kTile; ++k) {
        const TriF tr = tile[k];
        const float ex = tr.r3.x - fx, ey = tr.r3.y - fy, ez = tr.r3.z - fz;
        if (valid && fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < tr.r3.w) {
          near_acc += vos_term64_indexed(V, F, nV, (int64_t)t * kTile + k, qx, qy, qz);
          any_near = true;
        } else {
          ssum += vos_term32(tr, fx, fy, fz);
        }
      }
    } else {
#pragma unroll 4
      for (int k = 0; k < kTile; ++k) ssum += vos_term32(tile[k], fx, fy, fz);
    }
    const float y = ssum - comp;
    const float tt = acc + y;
    comp = (tt - acc) - y;
    acc = tt;
    __syncthreads();
    if (tid == 0 && t + kStages < ntiles) {
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&sm.bar[s], kTileBytes);
      bulk_g2s(&sm.tiles[s][0], tris + (int64_t)(t + kStages) * kTile, kTileBytes, &sm.bar[s]);
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicOr(status, kStatusWaitTimeout);
      if (withhold) mbar_arrive(&sm.bar[0]);  // the withheld arrival: stage 0 can drain
      drain_ring(sm.bar, kStages, stop_tile, ntiles);
    }
    return;
  }
  if (!valid) return;
  W[qi] = any_near ? ((double)acc + near_acc) * kInv2Pi : (double)(acc * kInv2PiF);
}

// Warp per query: results within 1e-3 of 0.5 are recomputed in FP64 over
// every triangle (lanes stride the faces; fixed xor-tree reduction).
__global__ void noalloc_refine_kernel(const double* __restrict__ V, int64_t nV,
                                      const int32_t* __restrict__ F, int64_t nF,
                                      const double* __restrict__ Q, int64_t nQ,
                                      double* __restrict__ W) {
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t qi = warp; qi < nQ; qi += nwarps) {
    if (!(fabs(W[qi] - 0.5) <= kBand)) continue;  // uniform across the warp
    double qx, qy, qz;
    load_q3(Q, qi, qx, qy, qz);
    double acc = 0.0;
    for (int64_t f = lane; f < nF; f += 32) acc += vos_term64_indexed(V, F, nV, f, qx, qy, qz);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) W[qi] = acc / (2.0 * kPi);
  }
}

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
NoAllocScratch* g_noalloc_ptr[kNoAllocMaxDevices] = {};  // per device, from cudaGetSymbolAddress

NoAllocScratch* noalloc_scratch_for_current_device() {
  int dev = 0;
  GWN_CUDA(cudaGetDevice(&dev));
  GWN_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    GWN_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    GWN_REQUIRE(p != nullptr, "static scratch has no device address");
    g_noalloc_ptr[dev] = static_cast<NoAllocScratch*>(p);
  }
  return g_noalloc_ptr[dev];
}

}  // namespace

int64_t noalloc_max_triangles() { return kNoAllocMaxTris; }

unsigned noalloc_sticky_status(bool clear) {
  unsigned v = 0;
  const size_t off = offsetof(NoAllocScratch, sticky_status);
  GWN_CUDA(cudaMemcpyFromSymbol(&v, g_noalloc_scratch, sizeof(v), off));
  if (clear && v) {
    const unsigned zero = 0;
    GWN_CUDA(cudaMemcpyToSymbol(g_noalloc_scratch, &zero, sizeof(zero), off));
  }
  return v;
}

void run_exact_noalloc(const double* V, int64_t nV, const int32_t* F, int64_t nF, const double* Q,
                       int64_t nQ, double* W, unsigned* dev_status, cudaStream_t st) {
  GWN_REQUIRE(nF <= kNoAllocMaxTris,
              "gwn_winding_number_noalloc: nF = " + std::to_string(nF) +
                  " exceeds the static scratch limit of " + std::to_string(kNoAllocMaxTris) +
                  " triangles");
  NoAllocScratch* s = noalloc_scratch_for_current_device();
  unsigned* status = dev_status ? dev_status : &s->sticky_status;
  launch_kernel(noalloc_init_kernel, 1, 32, 0, st, s);
  if (nQ == 0) return;
  if (nV > 0)
    launch_kernel(bbox_kernel, std::max(1, std::min(num_sms() * 4, (int)((nV + 255) / 256))), 256,
                  0, st, V, nV, 3, s->mm);
  const int64_t nPad = ((nF + kTile - 1) / kTile) * (int64_t)kTile;
  const int ntiles = (int)(nPad / kTile);
  if (nPad > 0) {
    launch_kernel(noalloc_pack_kernel, (unsigned)((nPad + 255) / 256), 256, 0, st, V, nV, F, nF,
                  nPad, s->mm, s->tris, status);
    launch_kernel(tile_meta_kernel, ntiles, kTile, 0, st, s->tris, ntiles, s->mm, s->meta);
  }
  const size_t smem = sizeof(Smem3);
  GWN_CUDA(cudaFuncSetAttribute(noalloc_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  launch_kernel(noalloc_mixed_kernel, (unsigned)((nQ + kThreads - 1) / kThreads), kThreads, smem,
                st, s->tris, s->meta, ntiles, V, nV, F, Q, nQ, W, status, take_wait_injection());
  launch_kernel(noalloc_refine_kernel, num_sms() * 8, 256, 0, st, V, nV, F, nF, Q, nQ, W);
}

}  // namespace gwn
