// The reference's own triangle-soup tree, built on the GPU node for node,
// with the reference's per-child moments.
//
// igl::fast_winding_number(V,F,order,bvh) (include/igl/fast_winding_number.cpp:
// 380-416) calls UT_SolidAngle<float,float>::init, which builds a 4-wide
// BVH (UT_BVH<4>::init with the BOX_AREA heuristic,
// include/igl/FastWindingNumberForSoups.h:4581-4634) over float copies of the
// vertices and stores, per node, one moment record per child lane
// (FWNFS.h:6543-7133).  This file rebuilds exactly that tree and those FP32
// moments on the device, plus the same moments in FP64, and lays them out as
// the pre-order child-slot records the soup walks read (soup.cuh): slot 0 is
// the root (always opened), then every child lane of every node in
// depth-first order, a lane that is a triangle being a leaf slot.
//
// It is compiled with --fmad=false: every FP32 expression rounds after each
// operation, as the reference's SSE code (no fused multiply-add) does, so
// centres, split heuristics, boxes and moments are bit for bit the
// reference's.
//
// Tree build (UT_BVH<4>::initNode, FWNFS.h:4918-5047), one depth at a time:
//   a node of at most 4 boxes holds them as items; a larger node makes the
//   reference's three binary splits (multiSplit, FWNFS.h:5249-5346: split
//   all, then twice the part with the largest area x count), all nodes of
//   the depth split by split.  A split (FWNFS.h:5350-5800) of
//     <= 32 boxes runs in one thread (2 boxes trivially, <= 6 by trying every
//           partition, else a stable sort of the centres and a sweep),
//     <= 1024 boxes in one CTA (span statistics by shared-memory atomics,
//           the partition done sequentially in shared memory),
//     more boxes across the GPU: span statistics by chunk, and the
//           reference's in-place partition reproduced exactly (below).
//   Span counts and boxes are order-independent (counts, min, max), so
//   every decision equals the serial code's.
//
// The in-place three-way partition (partitionByCentre, FWNFS.h:5903-5944)
// keeps the boxes below the pivot in order at the front; the boxes equal to
// the pivot and those above it form two queues, and each arrival of a box
// below the pivot (or, for the upper queue, below or equal) moves the front
// of a non-empty queue to its back.  The final order of a queue is read off
// a tape of its operations: an append writes the box, the r-th rotation
// writes a copy of tape entry r, and the queue is the tape's last k entries.
// Every box finds its tape positions from prefix counts; the copies are
// resolved by pointer doubling.  nthElement (FWNFS.h:5847-5900), the
// fallback when no span is balanced enough, repeats such partitions.
//
// Moments (UT_SolidAngle::init's per-item data and its post() merge,
// FWNFS.h:6668-7118): bottom-up one depth at a time; a node's lanes are its
// children's data, and its own data is what its parent's lane holds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "gwn_common.cuh"
#include "soup.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

constexpr uint32_t kEmpty = 0xffffffffu;     // empty child lane
constexpr uint32_t kInternal = 0x80000000u;  // child lane that is a node
constexpr int kSpans = 16;
constexpr int kSplits = kSpans - 1;
constexpr uint32_t kMinFraction = 16;
constexpr uint32_t kSmallMax = 2 * kSpans;  // exhaustive / sorted splits
constexpr uint32_t kMedMax = 1024;           // one CTA per split
constexpr uint32_t kChunk = 1024;            // positions per CTA in GPU-wide passes
constexpr uint32_t kTerm = 0x80000000u;      // tape entry holding a box index
constexpr uint32_t kNone = 0xffffffffu;
constexpr double kNearFrac = 1e-3;

struct Box {
  float lo[3], hi[3];
};

__host__ __device__ inline void box_empty(Box& b) {
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = FLT_MAX;
    b.hi[a] = -FLT_MAX;
  }
}
__device__ __forceinline__ void box_add(Box& b, const Box& o) {
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = b.lo[a] < o.lo[a] ? b.lo[a] : o.lo[a];
    b.hi[a] = b.hi[a] > o.hi[a] ? b.hi[a] : o.hi[a];
  }
}
// BOX_AREA heuristic: half the surface area (FWNFS.h:4064-4080).
__device__ __forceinline__ float half_area(const Box& b) {
  const float d0 = b.hi[0] - b.lo[0], d1 = b.hi[1] - b.lo[1], d2 = b.hi[2] - b.lo[2];
  return d0 * d1 + d1 * d2 + d2 * d0;
}
// Twice the box centre along an axis (utBoxCenter).
__device__ __forceinline__ float centre2(const Box& b, int a) { return b.lo[a] + b.hi[a]; }

// The longest axis of a box, the first on ties.
__device__ __forceinline__ int longest_axis(const Box& b, float& len) {
  int axis = 0;
  len = b.hi[0] - b.lo[0];
  for (int a = 1; a < 3; ++a) {
    const float l = b.hi[a] - b.lo[a];
    if (l > len) {
      axis = a;
      len = l;
    }
  }
  return axis;
}

// float -> int as the reference's x86 build converts (cvttss2si): out of
// range or NaN gives INT_MIN.
__device__ __forceinline__ int cvt_x86(float v) {
  return (v >= -2147483648.0f && v < 2147483648.0f) ? (int)v : INT_MIN;
}
__device__ __forceinline__ int span_of(float c2, float min2, float scale) {
  const int s = cvt_x86((c2 - min2) * scale);
  return s < 0 ? 0 : (s > kSpans - 1 ? kSpans - 1 : s);
}

// Order-preserving float keys for atomic min / max (-0 taken as +0, which
// no decision distinguishes).
__device__ __forceinline__ uint32_t fkey(float x) {
  if (x == 0.0f) x = 0.0f;
  const uint32_t u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}
struct BoxKeys {
  uint32_t lo[3], hi[3];
};
__device__ __forceinline__ void keys_init(uint32_t* k) {
  for (int a = 0; a < 3; ++a) {
    k[a] = 0xffffffffu;
    k[3 + a] = 0u;
  }
}
__device__ __forceinline__ void keys_add(uint32_t* k, const Box& b) {
  for (int a = 0; a < 3; ++a) {
    atomicMin(&k[a], fkey(b.lo[a]));
    atomicMax(&k[3 + a], fkey(b.hi[a]));
  }
}
__device__ __forceinline__ Box keys_box(const uint32_t* k) {
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = fkey_inv(k[a]);
    b.hi[a] = fkey_inv(k[3 + a]);
  }
  return b;
}

// One node of the tree under construction (build order: depth by depth).
struct RNode {
  uint32_t start, n;  // its boxes: idx[start .. start + n)
  Box all;            // the box its parent's split handed down
  uint32_t cut[5];    // sub-ranges after the splits made so far
  Box sub[4];
  float area[4];
  int32_t nsub, choice;
  uint32_t child[4];  // item (triangle id), kInternal | node, kEmpty
  // the split of the current round
  uint32_t t_start, t_n, t_mid;
  Box t_box, t_out[2];
};

// --------------------------------------------------------------- boxes --
// A triangle's box as UT_SolidAngle::init makes it: initBounds(v0), then
// enlargeBounds(v1), enlargeBounds(v2) with SYSmin / SYSmax
// (FWNFS.h:255-256, 4023-4028).  (a > b) ? b : a keeps a NaN of the first
// vertex and drops one of a later vertex.
template <typename T>
__device__ __forceinline__ void tri_box(const T* a, const T* b, const T* c, T* lo, T* hi) {
  for (int d = 0; d < 3; ++d) {
    lo[d] = a[d];
    hi[d] = a[d];
    lo[d] = lo[d] > b[d] ? b[d] : lo[d];
    hi[d] = hi[d] < b[d] ? b[d] : hi[d];
    lo[d] = lo[d] > c[d] ? c[d] : lo[d];
    hi[d] = hi[d] < c[d] ? c[d] : hi[d];
  }
}

// Triangle boxes over float copies of the vertices (UT_SolidAngle::init,
// FWNFS.h:6560-6590); a box with a non-finite bound is excluded
// (FWNFS.h:4606-4615).  Triangles with an index outside V are reported and
// excluded.
__global__ void tri_box_kernel(const double* __restrict__ V, int64_t nV,
                               const int32_t* __restrict__ F, int64_t nF, Box* __restrict__ box,
                               uint32_t* __restrict__ keep, unsigned* __restrict__ status) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (f >= nF) return;
  bool ok = true;
  float p[3][3];
  for (int c = 0; c < 3; ++c) {
    const int32_t i = F[f * 3 + c];
    if (i < 0 || i >= nV) {
      atomicOr(status, kStatusBadInput);
      ok = false;
      for (int d = 0; d < 3; ++d) p[c][d] = 0.f;
      continue;
    }
    for (int d = 0; d < 3; ++d) p[c][d] = (float)V[(int64_t)i * 3 + d];
  }
  Box b;
  tri_box(p[0], p[1], p[2], b.lo, b.hi);
  for (int a = 0; a < 3; ++a)
    if (!isfinite(b.lo[a]) || !isfinite(b.hi[a])) ok = false;
  box[f] = b;
  keep[f] = ok ? 1u : 0u;
}

// Kept triangles in input order, and the root box (one atomic per warp).
__global__ void compact_kernel(const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos,
                               int64_t nF, const Box* __restrict__ box, uint32_t* __restrict__ idx,
                               uint32_t* __restrict__ root_keys) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool k = f < nF && keep[f];
  uint32_t kk[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  if (k) {
    idx[pos[f]] = (uint32_t)f;
    const Box b = box[f];
    for (int a = 0; a < 3; ++a) {
      kk[a] = fkey(b.lo[a]);
      kk[3 + a] = fkey(b.hi[a]);
    }
  }
  const unsigned full = 0xffffffffu;
  for (int a = 0; a < 3; ++a) {
    kk[a] = __reduce_min_sync(full, kk[a]);
    kk[3 + a] = __reduce_max_sync(full, kk[3 + a]);
  }
  if ((threadIdx.x & 31) == 0 && kk[0] != 0xffffffffu) {
    for (int a = 0; a < 3; ++a) {
      atomicMin(&root_keys[a], kk[a]);
      atomicMax(&root_keys[3 + a], kk[3 + a]);
    }
  }
}

__global__ void root_init_kernel(RNode* nodes, uint32_t m, const uint32_t* __restrict__ root_keys) {
  RNode& r = nodes[0];
  r.start = 0;
  r.n = m;
  r.all = keys_box(root_keys);
  r.nsub = 1;
  r.choice = 0;
}

// ------------------------------------------------------ split: <= 32 boxes --
// One split of n <= 32 boxes (FWNFS.h:5350-5585) on a local copy of the
// indices; returns the cut (boxes [0, mid) go left).
__device__ void split_small(const Box& all, uint32_t* id, uint32_t n, const Box* __restrict__ tb,
                            uint32_t& mid, Box& o0, Box& o1) {
  if (n == 2) {
    o0 = tb[id[0]];
    o1 = tb[id[1]];
    mid = 1;
    return;
  }
  if (n <= 6) {  // every 2-partition with box 0 on side 0
    Box lb[6];
    for (uint32_t b = 0; b < n; ++b) lb[b] = tb[id[b]];
    const uint32_t lim = 1u << (n - 1);
    uint32_t best = kNone;
    float best_h = 0.f;
    for (uint32_t bits = 1; bits < lim; ++bits) {
      Box s0 = lb[0], s1;
      box_empty(s1);
      uint32_t c0 = 1, c1 = 0;
      for (uint32_t b = 0; b + 1 < n; ++b) {
        if ((bits >> b) & 1u) {
          box_add(s1, lb[b + 1]);
          ++c1;
        } else {
          box_add(s0, lb[b + 1]);
          ++c0;
        }
      }
      const float h = half_area(s0) * (float)c0 + half_area(s1) * (float)c1;
      if (best == kNone || h < best_h) {
        best = bits;
        best_h = h;
        o0 = s0;
        o1 = s1;
      }
    }
    uint32_t rest[5];
    for (uint32_t b = 0; b + 1 < n; ++b) rest[b] = id[b + 1];
    uint32_t w = 1;
    for (uint32_t b = 0; b + 1 < n; ++b)
      if (!((best >> b) & 1u)) id[w++] = rest[b];
    mid = w;
    for (uint32_t b = 0; b + 1 < n; ++b)
      if ((best >> b) & 1u) id[w++] = rest[b];
    return;
  }
  float len;
  const int axis = longest_axis(all, len);
  if (!(len > 0.f)) {  // a single point or NaN: an arbitrary split
    mid = n / 2;
    o0 = all;
    o1 = all;
    return;
  }
  // stable sort by centre (the reference's chunked insertion sort + merges
  // is a stable sort), then sweep
  float c[kSmallMax];
  for (uint32_t i = 0; i < n; ++i) c[i] = centre2(tb[id[i]], axis);
  for (uint32_t i = 1; i < n; ++i) {
    const float v = c[i];
    const uint32_t e = id[i];
    uint32_t j = i;
    while (j > 0 && v < c[j - 1]) {
      c[j] = c[j - 1];
      id[j] = id[j - 1];
      --j;
    }
    c[j] = v;
    id[j] = e;
  }
  const uint32_t ns = n - 1;
  // right boxes as the reference accumulates them: starting from box ns-1,
  // so the last box never enters (FWNFS.h:5560-5565)
  Box R[kSmallMax - 1];
  Box acc = tb[id[ns - 1]];
  R[ns - 1] = acc;
  for (uint32_t i = ns - 1; i > 0; --i) {
    box_add(acc, tb[id[i]]);
    R[i - 1] = acc;
  }
  Box L = tb[id[0]];
  uint32_t best = 0;
  float best_h = half_area(L) + half_area(R[0]) * (float)(n - 1);
  Box bestL = L;
  for (uint32_t s = 1; s < ns; ++s) {
    box_add(L, tb[id[s]]);
    const float h = half_area(L) * (float)(s + 1) + half_area(R[s]) * (float)(n - (s + 1));
    if (h < best_h) {
      best = s;
      best_h = h;
      bestL = L;
    }
  }
  mid = best + 1;
  o0 = bestL;
  o1 = R[best];
}

__global__ void split_small_kernel(RNode* __restrict__ nodes, const uint32_t* __restrict__ list,
                                   uint32_t count, uint32_t* __restrict__ idx,
                                   const Box* __restrict__ tb) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  RNode& N = nodes[list[k]];
  const uint32_t s = N.t_start, n = N.t_n;
  uint32_t id[kSmallMax];
  for (uint32_t i = 0; i < n; ++i) id[i] = idx[s + i];
  uint32_t mid;
  Box o0, o1;
  split_small(N.t_box, id, n, tb, mid, o0, o1);
  for (uint32_t i = 0; i < n; ++i) idx[s + i] = id[i];
  N.t_mid = s + mid;
  N.t_out[0] = o0;
  N.t_out[1] = o1;
}

// ------------------------------------------- the sequential partition --
// partitionByCentre on arrays of (index, centre) pairs, positions [lo, hi):
// returns the first position >= pivot and the first > pivot.
__device__ void partition_seq(uint32_t* id, float* c, uint32_t lo, uint32_t hi, float pivot,
                              uint32_t& ps, uint32_t& pe) {
  uint32_t s = lo, e = lo;
  for (uint32_t p = lo; p < hi; ++p) {
    const float v = c[p];
    if (v < pivot) {
      if (p != s) {
        const uint32_t ti = id[p];
        if (s == e) {
          id[p] = id[s];
          c[p] = c[s];
        } else {
          id[p] = id[e];
          c[p] = c[e];
          id[e] = id[s];
          c[e] = c[s];
        }
        id[s] = ti;
        c[s] = v;
      }
      ++s;
      ++e;
    } else if (v == pivot) {
      if (p != e) {
        const uint32_t ti = id[p];
        id[p] = id[e];
        c[p] = c[e];
        id[e] = ti;
        c[e] = v;
      }
      ++e;
    }
  }
  ps = s;
  pe = e;
}

// Median of three centres as nthElement picks its pivot (FWNFS.h:5852-5870).
__device__ __forceinline__ float median3(float a, float b, float c) {
  float p0 = a, p1 = b, p2 = c, t;
  if (p0 < p1) { t = p0; p0 = p1; p1 = t; }
  if (p0 < p2) { t = p0; p0 = p2; p2 = t; }
  if (p1 < p2) { t = p1; p1 = p2; p2 = t; }
  return p1;
}

// Each step narrows [lo, hi) by at least the pivot's own box, so at most
// hi - lo steps run; the bound only guards against a hang.
__device__ bool nth_seq(uint32_t* id, float* c, uint32_t lo, uint32_t hi, uint32_t nth) {
  for (uint32_t step = 0, limit = hi - lo + 1; step < limit; ++step) {
    const float pv = median3(c[lo], c[lo + (hi - lo) / 2], c[hi - 1]);
    uint32_t ps, pe;
    partition_seq(id, c, lo, hi, pv, ps, pe);
    if (nth < ps) hi = ps;
    else if (nth < pe) return true;
    else lo = pe;
    if (hi <= lo + 1) return true;
  }
  return false;
}

// Span statistics -> chosen span (or -1 when none keeps 1/16 of the boxes on
// each side, FWNFS.h:5684-5706), with the left / right boxes of that span.
__device__ int choose_span(const uint32_t* cnt, const uint32_t (*keys)[6], uint32_t n, Box& Lb,
                           Box& Rb, uint32_t& left_count, uint32_t& lc0, uint32_t& lc14) {
  Box span[kSpans];
  for (int i = 0; i < kSpans; ++i) {
    if (cnt[i]) {
      for (int a = 0; a < 3; ++a) {
        span[i].lo[a] = fkey_inv(keys[i][a]);
        span[i].hi[a] = fkey_inv(keys[i][3 + a]);
      }
    } else {
      box_empty(span[i]);
    }
  }
  Box L[kSplits], R[kSplits];
  uint32_t lc[kSplits];
  Box acc = span[0];
  L[0] = acc;
  for (int i = 1; i < kSplits; ++i) {
    box_add(acc, span[i]);
    L[i] = acc;
  }
  acc = span[kSpans - 1];
  R[kSplits - 1] = acc;
  for (int i = kSplits - 1; i > 0; --i) {
    box_add(acc, span[i]);
    R[i - 1] = acc;
  }
  uint32_t run = cnt[0];
  lc[0] = run;
  for (int i = 1; i < kSplits; ++i) {
    run += cnt[i];
    lc[i] = run;
  }
  const uint32_t min_count = n / kMinFraction;
  const uint32_t max_count = (uint32_t)(((uint64_t)(kMinFraction - 1) * n) / kMinFraction);
  float smallest = INFINITY;
  int si = -1;
  for (int i = 0; i < kSplits; ++i) {
    if (lc[i] < min_count || lc[i] > max_count) continue;
    const float h = (float)lc[i] * half_area(L[i]) + (float)(n - lc[i]) * half_area(R[i]);
    if (h < smallest) {
      smallest = h;
      si = i;
    }
  }
  lc0 = lc[0];
  lc14 = lc[kSplits - 1];
  if (si >= 0) {
    Lb = L[si];
    Rb = R[si];
    left_count = lc[si];
  }
  return si;
}

// The fallback's target order statistic (FWNFS.h:5718-5740).
__device__ __forceinline__ uint32_t nth_target(uint32_t n, uint32_t lc0, uint32_t lc14) {
  const uint32_t min_count = n / kMinFraction;
  const uint32_t max_count = (uint32_t)(((uint64_t)(kMinFraction - 1) * n) / kMinFraction);
  if (lc0 > max_count) return max_count;
  if (lc14 < min_count) return min_count;
  return n / 2;
}

// --------------------------------------------- split: 33..1024 boxes --
__global__ void __launch_bounds__(256) split_medium_kernel(RNode* __restrict__ nodes,
                                                           const uint32_t* __restrict__ list,
                                                           uint32_t* __restrict__ idx,
                                                           const Box* __restrict__ tb,
                                                           unsigned* __restrict__ status) {
  __shared__ uint32_t s_id[kMedMax];
  __shared__ float s_c[kMedMax];
  __shared__ uint32_t s_cnt[kSpans];
  __shared__ uint32_t s_keys[kSpans][6];
  __shared__ uint32_t s_bk[2][6];
  __shared__ uint32_t s_mid;
  __shared__ int s_need;
  const int tid = threadIdx.x;
  RNode& N = nodes[list[blockIdx.x]];
  const uint32_t s = N.t_start, n = N.t_n;
  const Box B = N.t_box;
  float len;
  const int axis = longest_axis(B, len);
  if (!(len > 0.f)) {
    if (tid == 0) {
      N.t_mid = s + n / 2;
      N.t_out[0] = B;
      N.t_out[1] = B;
    }
    return;
  }
  if (tid < kSpans) {
    s_cnt[tid] = 0;
    keys_init(s_keys[tid]);
  }
  if (tid < 2) keys_init(s_bk[tid]);
  __syncthreads();
  const float min2 = 2.0f * B.lo[axis];
  const float scale = (0.5f * (float)kSpans) / len;
  for (uint32_t i = tid; i < n; i += blockDim.x) {
    const uint32_t e = idx[s + i];
    const Box b = tb[e];
    const float c = centre2(b, axis);
    s_id[i] = e;
    s_c[i] = c;
    const int si = span_of(c, min2, scale);
    atomicAdd(&s_cnt[si], 1u);
    keys_add(s_keys[si], b);
  }
  __syncthreads();
  if (tid == 0) {
    Box Lb, Rb;
    uint32_t lcs = 0, lc0, lc14;
    const int si = choose_span(s_cnt, s_keys, n, Lb, Rb, lcs, lc0, lc14);
    uint32_t mid;
    int need = 1;
    if (si < 0) {
      mid = nth_target(n, lc0, lc14);
      if (!nth_seq(s_id, s_c, 0, n, mid)) atomicOr(status, kStatusInternal);
    } else {
      const float pivot = min2 + (float)(si + 1) * len / (float)(kSpans / 2);
      uint32_t ps, pe;
      partition_seq(s_id, s_c, 0, n, pivot, ps, pe);
      mid = lcs;
      if (mid >= ps && mid <= pe) {
        need = 0;
        N.t_out[0] = Lb;
        N.t_out[1] = Rb;
      } else {
        mid = mid < ps ? ps : pe;
        if (mid == 0) ++mid;
        else if (mid == n) --mid;
      }
    }
    s_mid = mid;
    s_need = need;
  }
  __syncthreads();
  const uint32_t mid = s_mid;
  if (s_need) {
    for (uint32_t i = tid; i < n; i += blockDim.x) keys_add(s_bk[i < mid ? 0 : 1], tb[s_id[i]]);
    __syncthreads();
    if (tid == 0) {
      N.t_out[0] = keys_box(s_bk[0]);
      N.t_out[1] = keys_box(s_bk[1]);
    }
  }
  for (uint32_t i = tid; i < n; i += blockDim.x) idx[s + i] = s_id[i];
  if (tid == 0) N.t_mid = s + mid;
}

// ----------------------------------------------- split: > 1024 boxes --
enum LMode : int32_t { kLDone = 0, kLSpan = 1, kLNth = 2 };

struct LTask {
  uint32_t node;
  uint32_t start, n;
  int32_t axis;
  float len, min2, scale;
  uint32_t cnt[kSpans];
  uint32_t keys[kSpans][6];
  Box Lb, Rb;
  uint32_t lcs;
  // the partition job in progress: positions [jlo, jlo + jn) around pivot
  int32_t mode;
  uint32_t jlo, jn, nth;
  float pivot;
  uint32_t firstE, firstG;    // job-relative, kNone if absent
  uint32_t nL, nE;            // job totals
  uint32_t nL_atE, nLE_atG;   // prefix counts at firstE / firstG
  uint32_t mid;
  int32_t need;               // sub boxes must be recomputed
  uint32_t bk[2][6];
};

// 32-bit chunk: CTA b of a GPU-wide pass works on positions
// [chunk[b].y, chunk[b].z) of large task chunk[b].x.

__global__ void large_init_kernel(RNode* __restrict__ nodes, const uint32_t* __restrict__ list,
                                  uint32_t count, LTask* __restrict__ T) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  LTask& t = T[k];
  const uint32_t x = list[k];
  RNode& N = nodes[x];
  t.node = x;
  t.start = N.t_start;
  t.n = N.t_n;
  float len;
  t.axis = longest_axis(N.t_box, len);
  t.len = len;
  t.min2 = 2.0f * N.t_box.lo[t.axis];
  t.scale = (0.5f * (float)kSpans) / len;
  for (int i = 0; i < kSpans; ++i) {
    t.cnt[i] = 0;
    keys_init(t.keys[i]);
  }
  keys_init(t.bk[0]);
  keys_init(t.bk[1]);
  t.need = 0;
  if (!(len > 0.f)) {
    t.mode = kLDone;
    t.mid = t.start + t.n / 2;
    N.t_out[0] = N.t_box;
    N.t_out[1] = N.t_box;
  } else {
    t.mode = kLSpan;
  }
}

__global__ void __launch_bounds__(256) large_span_kernel(const int4* __restrict__ chunks,
                                                         LTask* __restrict__ T,
                                                         const uint32_t* __restrict__ idx,
                                                         const Box* __restrict__ tb) {
  __shared__ uint32_t s_cnt[kSpans];
  __shared__ uint32_t s_keys[kSpans][6];
  const int4 ch = chunks[blockIdx.x];
  LTask& t = T[ch.x];
  const int tid = threadIdx.x;
  if (tid < kSpans) {
    s_cnt[tid] = 0;
    keys_init(s_keys[tid]);
  }
  __syncthreads();
  const int axis = t.axis;
  const float min2 = t.min2, scale = t.scale;
  for (int p = ch.y + tid; p < ch.z; p += blockDim.x) {
    const Box b = tb[idx[p]];
    const int si = span_of(centre2(b, axis), min2, scale);
    atomicAdd(&s_cnt[si], 1u);
    keys_add(s_keys[si], b);
  }
  __syncthreads();
  if (tid < kSpans && s_cnt[tid]) {
    atomicAdd(&t.cnt[tid], s_cnt[tid]);
    for (int a = 0; a < 3; ++a) {
      atomicMin(&t.keys[tid][a], s_keys[tid][a]);
      atomicMax(&t.keys[tid][3 + a], s_keys[tid][3 + a]);
    }
  }
}

__device__ __forceinline__ float centre_at(const uint32_t* idx, const Box* tb, uint32_t p,
                                           int axis) {
  return centre2(tb[idx[p]], axis);
}

__global__ void large_choose_kernel(LTask* __restrict__ T, uint32_t count,
                                    const uint32_t* __restrict__ idx, const Box* __restrict__ tb) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  LTask& t = T[k];
  if (t.mode != kLSpan) return;
  uint32_t lc0, lc14;
  const int si = choose_span(t.cnt, t.keys, t.n, t.Lb, t.Rb, t.lcs, lc0, lc14);
  t.jlo = t.start;
  t.jn = t.n;
  if (si < 0) {
    t.mode = kLNth;
    t.nth = t.start + nth_target(t.n, lc0, lc14);
    t.pivot = median3(centre_at(idx, tb, t.start, t.axis),
                      centre_at(idx, tb, t.start + t.n / 2, t.axis),
                      centre_at(idx, tb, t.start + t.n - 1, t.axis));
  } else {
    t.pivot = t.min2 + (float)(si + 1) * t.len / (float)(kSpans / 2);
  }
}

__global__ void part_init_kernel(LTask* __restrict__ T, uint32_t count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  T[k].firstE = kNone;
  T[k].firstG = kNone;
}

// Pass 1: class of every position (0 below, 1 equal, 2 above the pivot),
// counts per chunk, first equal / first above per job.
__global__ void __launch_bounds__(256) part_classify_kernel(const int4* __restrict__ chunks,
                                                            LTask* __restrict__ T,
                                                            const uint32_t* __restrict__ idx,
                                                            const Box* __restrict__ tb,
                                                            uint8_t* __restrict__ cls,
                                                            uint32_t* __restrict__ chunk_cnt) {
  __shared__ uint32_t s_n[3];
  const int4 ch = chunks[blockIdx.x];
  LTask& t = T[ch.x];
  const int tid = threadIdx.x;
  if (tid < 3) s_n[tid] = 0;
  __syncthreads();
  uint32_t n0 = 0, n1 = 0, n2 = 0, fE = kNone, fG = kNone;
  for (int p = ch.y + tid; p < ch.z; p += blockDim.x) {
    const float c = centre2(tb[idx[p]], t.axis);
    const uint8_t k = c < t.pivot ? 0 : (c == t.pivot ? 1 : 2);
    cls[p] = k;
    const uint32_t rel = (uint32_t)p - t.jlo;
    if (k == 0) ++n0;
    else if (k == 1) {
      ++n1;
      fE = min(fE, rel);
    } else {
      ++n2;
      fG = min(fG, rel);
    }
  }
  atomicAdd(&s_n[0], n0);
  atomicAdd(&s_n[1], n1);
  atomicAdd(&s_n[2], n2);
  if (fE != kNone) atomicMin(&t.firstE, fE);
  if (fG != kNone) atomicMin(&t.firstG, fG);
  __syncthreads();
  if (tid < 3) chunk_cnt[blockIdx.x * 3 + tid] = s_n[tid];
}

// Pass 2: per job, the counts before each of its chunks (its chunks are
// consecutive in the chunk list: jc = (first, count)).
__global__ void part_chunk_scan_kernel(LTask* __restrict__ T, uint32_t count,
                                       const int2* __restrict__ jc,
                                       const uint32_t* __restrict__ chunk_cnt,
                                       uint32_t* __restrict__ chunk_base) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count || jc[k].y == 0) return;
  uint32_t a = 0, b = 0, c = 0;
  for (int i = jc[k].x; i < jc[k].x + jc[k].y; ++i) {
    chunk_base[i * 3 + 0] = a;
    chunk_base[i * 3 + 1] = b;
    chunk_base[i * 3 + 2] = c;
    a += chunk_cnt[i * 3 + 0];
    b += chunk_cnt[i * 3 + 1];
    c += chunk_cnt[i * 3 + 2];
  }
  T[k].nL = a;
  T[k].nE = b;
}

// Pass 3: prefix counts of "below" and "equal" at every position.  Thread t
// of the CTA owns positions 4t .. 4t+3 of the chunk.
__global__ void __launch_bounds__(256) part_prefix_kernel(const int4* __restrict__ chunks,
                                                          LTask* __restrict__ T,
                                                          const uint8_t* __restrict__ cls,
                                                          const uint32_t* __restrict__ chunk_base,
                                                          uint32_t* __restrict__ preL,
                                                          uint32_t* __restrict__ preE) {
  __shared__ uint32_t s_warp[8];
  const int4 ch = chunks[blockIdx.x];
  LTask& t = T[ch.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int p0 = ch.y + 4 * tid;
  uint8_t k[4];
  uint32_t own = 0;  // below in the low 16 bits, equal in the high 16
  for (int j = 0; j < 4; ++j) {
    const int p = p0 + j;
    k[j] = p < ch.z ? cls[p] : 2;
    own += k[j] == 0 ? 1u : (k[j] == 1 ? 0x10000u : 0u);
  }
  uint32_t incl = own;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  uint32_t wbase = 0;
  for (int w = 0; w < warp; ++w) wbase += s_warp[w];
  uint32_t run = wbase + incl - own;
  uint32_t L = chunk_base[blockIdx.x * 3 + 0] + (run & 0xffffu);
  uint32_t E = chunk_base[blockIdx.x * 3 + 1] + (run >> 16);
  for (int j = 0; j < 4; ++j) {
    const int p = p0 + j;
    if (p >= ch.z) break;
    preL[p] = L;
    preE[p] = E;
    const uint32_t rel = (uint32_t)p - t.jlo;
    if (rel == t.firstE) t.nL_atE = L;
    if (rel == t.firstG) t.nLE_atG = L + E;
    if (k[j] == 0) ++L;
    else if (k[j] == 1) ++E;
  }
}

// Pass 4: boxes below the pivot go to their place (in tmp); the equal and
// upper queues' operations are written to their tapes.
__global__ void __launch_bounds__(256) part_tape_kernel(const int4* __restrict__ chunks,
                                                        const LTask* __restrict__ T,
                                                        const uint32_t* __restrict__ idx,
                                                        const uint8_t* __restrict__ cls,
                                                        const uint32_t* __restrict__ preL,
                                                        const uint32_t* __restrict__ preE,
                                                        uint32_t* __restrict__ tmp,
                                                        uint32_t* __restrict__ tapeE,
                                                        uint32_t* __restrict__ tapeG) {
  const int4 ch = chunks[blockIdx.x];
  const LTask& t = T[ch.x];
  const uint32_t jlo = t.jlo, fE = t.firstE, fG = t.firstG;
  for (int p = ch.y + threadIdx.x; p < ch.z; p += blockDim.x) {
    const uint32_t rel = (uint32_t)p - jlo;
    const uint8_t k = cls[p];
    const uint32_t e = idx[p];
    const uint32_t L = preL[p], E = preE[p], G = rel - L - E;
    const bool afterE = fE != kNone && rel > fE, afterG = fG != kNone && rel > fG;
    const uint32_t rotE = afterE ? L - t.nL_atE : 0u;
    const uint32_t rotG = afterG ? (L + E) - t.nLE_atG : 0u;
    // every tape position is below the job's size (a tape holds at most
    // one entry per box of the job); the checks only guard the memory
    const uint32_t te = E + rotE, tg = G + rotG, jn = t.jn;
    if (k == 0) {
      if (L < jn) tmp[jlo + L] = e;
      if (afterE && te < jn) tapeE[jlo + te] = rotE;
      if (afterG && tg < jn) tapeG[jlo + tg] = rotG;
    } else if (k == 1) {
      if (te < jn) tapeE[jlo + te] = kTerm | e;
      if (afterG && tg < jn) tapeG[jlo + tg] = rotG;
    } else {
      if (tg < jn) tapeG[jlo + tg] = kTerm | e;
    }
  }
}

// Pass 5 (repeated): one pointer-doubling step on both tapes.
__global__ void __launch_bounds__(256) part_jump_kernel(const int4* __restrict__ chunks,
                                                        const LTask* __restrict__ T,
                                                        uint32_t* __restrict__ tapeE,
                                                        uint32_t* __restrict__ tapeG) {
  const int4 ch = chunks[blockIdx.x];
  const LTask& t = T[ch.x];
  const uint32_t jlo = t.jlo;
  const uint32_t nG = t.jn - t.nL - t.nE;
  const uint32_t lenE = t.nE + (t.firstE != kNone ? t.nL - t.nL_atE : 0u);
  const uint32_t lenG = nG + (t.firstG != kNone ? (t.nL + t.nE) - t.nLE_atG : 0u);
  for (int p = ch.y + threadIdx.x; p < ch.z; p += blockDim.x) {
    const uint32_t rel = (uint32_t)p - jlo;
    // a copy always refers to an earlier tape entry (v < rel)
    if (rel < lenE) {
      const uint32_t v = tapeE[p];
      if (!(v & kTerm) && v < rel) tapeE[p] = tapeE[jlo + v];
    }
    if (rel < lenG) {
      const uint32_t v = tapeG[p];
      if (!(v & kTerm) && v < rel) tapeG[p] = tapeG[jlo + v];
    }
  }
}

// Pass 6: the partitioned order back into idx: below | equal queue | upper
// queue (each queue = the last k entries of its tape).
__global__ void __launch_bounds__(256) part_scatter_kernel(const int4* __restrict__ chunks,
                                                           const LTask* __restrict__ T,
                                                           const uint32_t* __restrict__ tmp,
                                                           const uint32_t* __restrict__ tapeE,
                                                           const uint32_t* __restrict__ tapeG,
                                                           uint32_t* __restrict__ idx,
                                                           unsigned* __restrict__ status) {
  const int4 ch = chunks[blockIdx.x];
  const LTask& t = T[ch.x];
  const uint32_t jlo = t.jlo;
  const uint32_t RE = t.firstE != kNone ? t.nL - t.nL_atE : 0u;
  const uint32_t RG = t.firstG != kNone ? (t.nL + t.nE) - t.nLE_atG : 0u;
  for (int p = ch.y + threadIdx.x; p < ch.z; p += blockDim.x) {
    const uint32_t rel = (uint32_t)p - jlo;
    uint32_t v = 0;
    if (rel < t.nL) {
      v = tmp[p] | kTerm;
    } else if (rel < t.nL + t.nE) {
      const uint32_t q = RE + (rel - t.nL);
      if (q < t.jn) v = tapeE[jlo + q];
    } else {
      const uint32_t q = RG + (rel - t.nL - t.nE);
      if (q < t.jn) v = tapeG[jlo + q];
    }
    if (!(v & kTerm)) {  // an unresolved queue entry: an internal error, never expected
      atomicOr(status, kStatusInternal);
      v = idx[p] | kTerm;
    }
    idx[p] = v & ~kTerm;
  }
}

// After a partition: the span split takes its cut, or an nthElement step
// narrows its range (and picks the next pivot from the new order).
__global__ void part_update_kernel(LTask* __restrict__ T, uint32_t count,
                                   const uint32_t* __restrict__ idx, const Box* __restrict__ tb) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  LTask& t = T[k];
  if (t.mode == kLDone) return;
  const uint32_t ps = t.jlo + t.nL, pe = ps + t.nE;
  if (t.mode == kLSpan) {
    uint32_t mid = t.start + t.lcs;
    t.mode = kLDone;
    if (mid >= ps && mid <= pe) {
      t.mid = mid;
      t.need = 0;
      return;
    }
    mid = mid < ps ? ps : pe;
    if (mid == t.start) ++mid;
    else if (mid == t.start + t.n) --mid;
    t.mid = mid;
    t.need = 1;
    return;
  }
  // nthElement step
  uint32_t lo = t.jlo, hi = t.jlo + t.jn;
  bool done = false;
  if (t.nth < ps) hi = ps;
  else if (t.nth < pe) done = true;
  else lo = pe;
  if (!done && hi <= lo + 1) done = true;
  if (done) {
    t.mode = kLDone;
    t.mid = t.nth;
    t.need = 1;
    return;
  }
  t.jlo = lo;
  t.jn = hi - lo;
  t.pivot = median3(centre_at(idx, tb, lo, t.axis), centre_at(idx, tb, lo + (hi - lo) / 2, t.axis),
                    centre_at(idx, tb, hi - 1, t.axis));
}

__global__ void __launch_bounds__(256) large_boxes_kernel(const int4* __restrict__ chunks,
                                                          LTask* __restrict__ T,
                                                          const uint32_t* __restrict__ idx,
                                                          const Box* __restrict__ tb) {
  __shared__ uint32_t s_bk[2][6];
  const int4 ch = chunks[blockIdx.x];
  LTask& t = T[ch.x];
  const int tid = threadIdx.x;
  if (tid < 2) keys_init(s_bk[tid]);
  __syncthreads();
  for (int p = ch.y + tid; p < ch.z; p += blockDim.x)
    keys_add(s_bk[(uint32_t)p < t.mid ? 0 : 1], tb[idx[p]]);
  __syncthreads();
  if (tid < 12) {
    const int side = tid / 6, j = tid % 6;
    if (j < 3) atomicMin(&t.bk[side][j], s_bk[side][j]);
    else atomicMax(&t.bk[side][j], s_bk[side][j]);
  }
}

__global__ void large_finish_kernel(RNode* __restrict__ nodes, const LTask* __restrict__ T,
                                    uint32_t count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const LTask& t = T[k];
  RNode& N = nodes[t.node];
  N.t_mid = t.mid;
  if (!(t.len > 0.f)) return;  // t_out already the node box
  if (t.need) {
    N.t_out[0] = keys_box(t.bk[0]);
    N.t_out[1] = keys_box(t.bk[1]);
  } else {
    N.t_out[0] = t.Lb;
    N.t_out[1] = t.Rb;
  }
}

// --------------------------------------------------- rounds and levels --
// The split each node makes this round (multiSplit: round 0 splits the
// whole range; rounds 1 and 2 the part with the largest area x count,
// the first on ties), sorted into the three size classes.
__global__ void prepare_round_kernel(RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                                     int round, uint32_t* __restrict__ lists, uint32_t cap,
                                     uint32_t* __restrict__ counts) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  RNode& N = nodes[x];
  if (N.n <= 4) return;
  uint32_t s, n;
  Box b;
  if (round == 0) {
    s = N.start;
    n = N.n;
    b = N.all;
  } else {
    int choice = -1;
    float best = 0.f;
    for (int i = 0; i < N.nsub; ++i) {
      const uint32_t c = N.cut[i + 1] - N.cut[i];
      if (c > 1) {
        const float h = N.area[i] * (float)c;
        if (choice < 0 || h > best) {
          choice = i;
          best = h;
        }
      }
    }
    N.choice = choice;
    s = N.cut[choice];
    n = N.cut[choice + 1] - s;
    b = N.sub[choice];
  }
  N.t_start = s;
  N.t_n = n;
  N.t_box = b;
  const int cat = n <= kSmallMax ? 0 : (n <= kMedMax ? 1 : 2);
  const uint32_t pos = atomicAdd(&counts[cat], 1u);
  lists[(size_t)cat * cap + pos] = x;
}

__global__ void finish_round_kernel(RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                                    int round) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  RNode& N = nodes[x];
  if (N.n <= 4) return;
  if (round == 0) {
    N.cut[0] = N.start;
    N.cut[1] = N.t_mid;
    N.cut[2] = N.start + N.n;
    N.sub[0] = N.t_out[0];
    N.sub[1] = N.t_out[1];
    N.area[0] = half_area(N.sub[0]);
    N.area[1] = half_area(N.sub[1]);
    N.nsub = 2;
    return;
  }
  const int c = N.choice, ns = N.nsub;
  for (int i = ns; i > c; --i) N.cut[i + 1] = N.cut[i];
  for (int i = ns - 1; i > c; --i) {
    N.sub[i + 1] = N.sub[i];
    N.area[i + 1] = N.area[i];
  }
  N.cut[c + 1] = N.t_mid;
  N.sub[c] = N.t_out[0];
  N.sub[c + 1] = N.t_out[1];
  N.area[c] = half_area(N.sub[c]);
  N.area[c + 1] = half_area(N.sub[c + 1]);
  N.nsub = ns + 1;
}

// Children of a depth: items go into the lanes; every part of two or more
// boxes becomes a node of the next depth (cnt[] = how many).
__global__ void count_children_kernel(RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                                      const uint32_t* __restrict__ idx, uint32_t* __restrict__ cnt) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  RNode& N = nodes[x];
  uint32_t k = 0;
  if (N.n <= 4) {
    for (uint32_t i = 0; i < 4; ++i) N.child[i] = i < N.n ? idx[N.start + i] : kEmpty;
  } else {
    for (int i = 0; i < 4; ++i) {
      const uint32_t c = N.cut[i + 1] - N.cut[i];
      if (c == 1) N.child[i] = idx[N.cut[i]];
      else ++k;
    }
  }
  cnt[x - lb] = k;
}

__global__ void make_children_kernel(RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                                     const uint32_t* __restrict__ offs) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  RNode& N = nodes[x];
  if (N.n <= 4) return;
  uint32_t o = le + offs[x - lb];
  for (int i = 0; i < 4; ++i) {
    const uint32_t c = N.cut[i + 1] - N.cut[i];
    if (c == 1) continue;
    N.child[i] = kInternal | o;
    RNode& C = nodes[o];
    C.start = N.cut[i];
    C.n = c;
    C.all = N.sub[i];
    C.nsub = 1;
    C.choice = 0;
    ++o;
  }
}

// ------------------------------------------------------------- moments --
// Per-node data as the reference's post() returns it to the parent (about
// the node's own average point P), in T = float (the reference's values) or
// double.
template <typename T>
struct Loc {
  T lo[3], hi[3];
  T P[3], areaP[3], N[3], area;
  T Nii[3], Nxy, Nyx, Nyz, Nzy, Nzx, Nxz;
  T Niii[3], perm, c2[6];
};

template <typename T>
__device__ void zero_loc(Loc<T>& L) {
  T* p = reinterpret_cast<T*>(&L);
  for (size_t i = 0; i < sizeof(Loc<T>) / sizeof(T); ++i) p[i] = T(0);
}

// Second-moment integrals of one triangle (FWNFS.h:6727-6884), corners
// A <= B <= C along axis i.
template <typename T>
__device__ void tri_integrals(const T* A, const T* B, const T* C, const T* P, T* ii, T* ij, T* ik,
                              int i) {
  T oab[3], oac[3], ocb[3];
  for (int d = 0; d < 3; ++d) {
    oab[d] = B[d] - A[d];
    oac[d] = C[d] - A[d];
    ocb[d] = B[d] - C[d];
  }
  const T t = oab[i] / oac[i];
  const int j = (i == 2) ? 0 : i + 1, k = (j == 2) ? 0 : j + 1;
  const T jd = t * oac[j] - oab[j], kd = t * oac[k] - oab[k];
  const T xa0 = jd * oab[k] - kd * oab[j], xa1 = kd * oab[i], xa2 = jd * oab[i];
  const T xc0 = jd * ocb[k] - kd * ocb[j], xc1 = kd * ocb[i], xc2 = jd * ocb[i];
  const T sa = sqrt(xa0 * xa0 + xa1 * xa1 + xa2 * xa2);
  const T sc = sqrt(xc0 * xc0 + xc1 * xc1 + xc2 * xc2);
  const T Pai = A[i] - P[i], Pci = C[i] - P[i];
  const T two3 = T(2.0 / 3.0), one3 = T(1.0 / 3.0), half = T(0.5), qtr = T(0.25);
  const T ia = sa * (half * Pai * Pai + two3 * Pai * oab[i] + qtr * oab[i] * oab[i]);
  const T ic = sc * (half * Pci * Pci + two3 * Pci * ocb[i] + qtr * ocb[i] * ocb[i]);
  *ii = ia + ic;
  for (int s = 0; s < 2; ++s) {
    T* out = s == 0 ? ij : ik;
    if (!out) continue;
    const int jk = s == 0 ? j : k;
    const T df = s == 0 ? jd : kd;
    const T mid = B[jk] + half * df;
    const T am = mid - A[jk], cm = mid - C[jk];
    const T Paj = A[jk] - P[jk], Pcj = C[jk] - P[jk];
    const T ija = sa * (half * Pai * Paj + one3 * Pai * am + one3 * Paj * oab[i] + qtr * oab[i] * am);
    const T ijc = sc * (half * Pci * Pcj + one3 * Pci * cm + one3 * Pcj * ocb[i] + qtr * ocb[i] * cm);
    *out = ija + ijc;
  }
}

// Per-triangle data (the reference's item(), FWNFS.h:6668-6890).
template <typename T>
__device__ void item_loc(const T* a, const T* b, const T* c, int order, Loc<T>& L) {
  zero_loc(L);
  tri_box(a, b, c, L.lo, L.hi);
  T ab[3], ac[3];
  for (int d = 0; d < 3; ++d) {
    ab[d] = b[d] - a[d];
    ac[d] = c[d] - a[d];
  }
  L.N[0] = T(0.5) * (ab[1] * ac[2] - ab[2] * ac[1]);
  L.N[1] = T(0.5) * (ab[2] * ac[0] - ab[0] * ac[2]);
  L.N[2] = T(0.5) * (ab[0] * ac[1] - ab[1] * ac[0]);
  const T area = sqrt(L.N[0] * L.N[0] + L.N[1] * L.N[1] + L.N[2] * L.N[2]);
  const T third = T(1) / T(3);
  for (int d = 0; d < 3; ++d) {
    L.P[d] = ((a[d] + b[d]) + c[d]) * third;
    L.areaP[d] = L.P[d] * area;
  }
  L.area = area;
  if (order < 2 || area == T(0)) return;
  const T inv = T(1) / area;
  const T n[3] = {L.N[0] * inv, L.N[1] * inv, L.N[2] * inv};
  const T* v[3] = {a, b, c};
  int o[3][3];
  for (int ax = 0; ax < 3; ++ax) {
    int* q = o[ax];
    q[0] = 0;
    q[1] = 1;
    q[2] = 2;
    int t;
    if (a[ax] > b[ax]) { t = q[0]; q[0] = q[1]; q[1] = t; }
    if (v[q[0]][ax] > c[ax]) { t = q[0]; q[0] = q[2]; q[2] = t; }
    if (v[q[1]][ax] > v[q[2]][ax]) { t = q[1]; q[1] = q[2]; q[2] = t; }
  }
  const T dx = v[o[0][2]][0] - v[o[0][0]][0];
  const T dy = v[o[1][2]][1] - v[o[1][0]][1];
  const T dz = v[o[2][2]][2] - v[o[2][0]][2];
  T xx = 0, xy = 0, yy = 0, yz = 0, zz = 0, zx = 0;
  if (dx > T(0))
    tri_integrals(v[o[0][0]], v[o[0][1]], v[o[0][2]], L.P, &xx,
                  (dx >= dy && dy > T(0)) ? &xy : (T*)nullptr,
                  (dx >= dz && dz > T(0)) ? &zx : (T*)nullptr, 0);
  if (dy > T(0))
    tri_integrals(v[o[1][0]], v[o[1][1]], v[o[1][2]], L.P, &yy,
                  (dy >= dz && dz > T(0)) ? &yz : (T*)nullptr,
                  (dx < dy && dx > T(0)) ? &xy : (T*)nullptr, 1);
  if (dz > T(0))
    tri_integrals(v[o[2][0]], v[o[2][1]], v[o[2][2]], L.P, &zz,
                  (dx < dz && dx > T(0)) ? &zx : (T*)nullptr,
                  (dy < dz && dy > T(0)) ? &yz : (T*)nullptr, 2);
  L.Niii[0] = xx * n[0];
  L.Niii[1] = yy * n[1];
  L.Niii[2] = zz * n[2];
  L.perm = T(2) * (n[0] * yz + n[1] * zx + n[2] * xy);
  const T Nxxy = n[0] * xy, Nxxz = n[0] * zx, Nyyz = n[1] * yz, Nyyx = n[1] * xy, Nzzx = n[2] * zx,
          Nzzy = n[2] * yz;
  L.c2[0] = T(2) * Nxxy + n[1] * xx;
  L.c2[1] = T(2) * Nxxz + n[2] * xx;
  L.c2[2] = T(2) * Nyyz + n[2] * yy;
  L.c2[3] = T(2) * Nyyx + n[0] * yy;
  L.c2[4] = T(2) * Nzzx + n[0] * zz;
  L.c2[5] = T(2) * Nzzy + n[1] * zz;
}

// A lane's maxP^2: the farthest box corner coordinate from P, squared and
// summed (FWNFS.h:6940-6955).
template <typename T>
__device__ __forceinline__ T lane_maxP2(const Loc<T>& C) {
  T m2 = T(0);
  for (int d = 0; d < 3; ++d) {
    const T a = C.P[d] - C.lo[d], b = C.hi[d] - C.P[d];
    const T mx = a > b ? a : b;
    m2 = d == 0 ? mx * mx : m2 + mx * mx;
  }
  return m2;
}

// A node's own data from its children's (the reference's post(),
// FWNFS.h:6892-7118), in the reference's order of operations.
template <typename T>
__device__ void merge_loc(const Loc<T>* ch, int nch, int order, Loc<T>& out) {
  zero_loc(out);
  for (int d = 0; d < 3; ++d) {
    out.N[d] = ch[0].N[d];
    out.areaP[d] = ch[0].areaP[d];
    out.lo[d] = ch[0].lo[d];
    out.hi[d] = ch[0].hi[d];
  }
  out.area = ch[0].area;
  for (int i = 1; i < nch; ++i) {
    for (int d = 0; d < 3; ++d) {
      out.N[d] += ch[i].N[d];
      out.areaP[d] += ch[i].areaP[d];
    }
    out.area += ch[i].area;
  }
  for (int i = 1; i < nch; ++i)
    for (int d = 0; d < 3; ++d) {
      out.lo[d] = out.lo[d] < ch[i].lo[d] ? out.lo[d] : ch[i].lo[d];
      out.hi[d] = out.hi[d] > ch[i].hi[d] ? out.hi[d] : ch[i].hi[d];
    }
  if (out.area > T(0)) {
    const T inv = T(1) / out.area;
    for (int d = 0; d < 3; ++d) out.P[d] = out.areaP[d] * inv;
  } else {
    for (int d = 0; d < 3; ++d) out.P[d] = T(0.5) * (out.lo[d] + out.hi[d]);
  }
  if (order < 1) return;
  for (int d = 0; d < 3; ++d) {
    out.Nii[d] = ch[0].Nii[d];
    out.Niii[d] = ch[0].Niii[d];
  }
  out.perm = ch[0].perm;
  for (int k = 0; k < 6; ++k) out.c2[k] = ch[0].c2[k];
  for (int i = 1; i < nch; ++i) {
    for (int d = 0; d < 3; ++d) {
      out.Nii[d] += ch[i].Nii[d];
      out.Niii[d] += ch[i].Niii[d];
    }
    out.perm += ch[i].perm;
    for (int k = 0; k < 6; ++k) out.c2[k] += ch[i].c2[k];
  }
  for (int i = 0; i < nch; ++i) {
    const Loc<T>& C = ch[i];
    const T dx = C.P[0] - out.P[0], dy = C.P[1] - out.P[1], dz = C.P[2] - out.P[2];
    const T* n = C.N;
    out.Nii[0] += n[0] * dx;
    out.Nii[1] += n[1] * dy;
    out.Nii[2] += n[2] * dz;
    const T Nxy = C.Nxy + n[0] * dy, Nyx = C.Nyx + n[1] * dx, Nyz = C.Nyz + n[1] * dz,
            Nzy = C.Nzy + n[2] * dy, Nzx = C.Nzx + n[2] * dx, Nxz = C.Nxz + n[0] * dz;
    out.Nxy += Nxy;
    out.Nyx += Nyx;
    out.Nyz += Nyz;
    out.Nzy += Nzy;
    out.Nzx += Nzx;
    out.Nxz += Nxz;
    if (order >= 2) {
      const T dd[3] = {dx, dy, dz};
      for (int d = 0; d < 3; ++d) out.Niii[d] += T(2) * dd[d] * C.Nii[d] + dd[d] * dd[d] * n[d];
      out.perm += (dx * (Nyz + Nzy) + dy * (Nzx + Nxz) + dz * (Nxy + Nyx));
      out.c2[0] += T(2) * (dy * C.Nii[0] + dx * C.Nxy + n[0] * dx * dy) + T(2) * C.Nyx * dx + n[1] * dx * dx;
      out.c2[1] += T(2) * (dz * C.Nii[0] + dx * C.Nxz + n[0] * dx * dz) + T(2) * C.Nzx * dx + n[2] * dx * dx;
      out.c2[2] += T(2) * (dz * C.Nii[1] + dy * C.Nyz + n[1] * dy * dz) + T(2) * C.Nzy * dy + n[2] * dy * dy;
      out.c2[3] += T(2) * (dx * C.Nii[1] + dy * C.Nyx + n[1] * dy * dx) + T(2) * C.Nxy * dy + n[0] * dy * dy;
      out.c2[4] += T(2) * (dx * C.Nii[2] + dz * C.Nzx + n[2] * dz * dx) + T(2) * C.Nxz * dz + n[0] * dz * dz;
      out.c2[5] += T(2) * (dy * C.Nii[2] + dz * C.Nzy + n[2] * dz * dy) + T(2) * C.Nyz * dz + n[1] * dz * dz;
    }
  }
}

// Sizes of each node's subtree: nodes, slots (lanes in the walk array) and
// items; bottom-up, one depth per launch.
__global__ void sizes_kernel(const RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                             uint32_t* __restrict__ nsize, uint32_t* __restrict__ nslots,
                             uint32_t* __restrict__ nitems) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  uint32_t sz = 1, sl = 1, it = 0;
  for (int i = 0; i < 4; ++i) {
    const uint32_t c = nodes[x].child[i];
    if (c == kEmpty) continue;
    if (c & kInternal) {
      const uint32_t y = c & ~kInternal;
      sz += nsize[y];
      sl += nslots[y];
      it += nitems[y];
    } else {
      ++sl;
      ++it;
    }
  }
  nsize[x] = sz;
  nslots[x] = sl;
  nitems[x] = it;
}

// Depth-first positions, top-down: the reference's node number (pre-order,
// children in lane order), the node's slot in the walk array, the first
// leaf slot of its subtree.
__global__ void positions_kernel(const RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                                 const uint32_t* __restrict__ nsize,
                                 const uint32_t* __restrict__ nslots,
                                 const uint32_t* __restrict__ nitems, uint32_t* __restrict__ pre,
                                 uint32_t* __restrict__ slot, uint32_t* __restrict__ ibase) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  uint32_t p = pre[x] + 1, sp = slot[x] + 1, ib = ibase[x];
  for (int i = 0; i < 4; ++i) {
    const uint32_t c = nodes[x].child[i];
    if (c == kEmpty) continue;
    if (c & kInternal) {
      const uint32_t y = c & ~kInternal;
      pre[y] = p;
      p += nsize[y];
      slot[y] = sp;
      sp += nslots[y];
      ibase[y] = ib;
      ib += nitems[y];
    } else {
      ++sp;
      ++ib;
    }
  }
}

__device__ void load_tri(const double* __restrict__ V, int64_t nV, const int32_t* __restrict__ F,
                         uint32_t f, double* v) {
  for (int c = 0; c < 3; ++c) {
    int32_t i = F[(int64_t)f * 3 + c];
    if (i < 0 || i >= nV) i = 0;  // reported at the box pass; excluded there
    for (int d = 0; d < 3; ++d) v[c * 3 + d] = V[(int64_t)i * 3 + d];
  }
}

__device__ void write_records(const Loc<float>& C32, const Loc<double>& C64, long long link,
                              SoupNodeF* nf, SoupNodeD* nd) {
  const float m32 = lane_maxP2(C32);
  SoupNodeF R;
  R.a = make_float4(C32.P[0], C32.P[1], C32.P[2], m32);
  {
    // the reference's FP32 moments (with its FP32 sums of the mixed terms),
    // packed into the walk's far-field forms
    double N[3], Nii[3], Niii[3], c2[6];
    for (int d = 0; d < 3; ++d) {
      N[d] = C32.N[d];
      Nii[d] = C32.Nii[d];
      Niii[d] = C32.Niii[d];
    }
    for (int k = 0; k < 6; ++k) c2[k] = C32.c2[k];
    pack_far32(R, N, Nii, (double)(C32.Nxy + C32.Nyx), (double)(C32.Nyz + C32.Nzy),
               (double)(C32.Nzx + C32.Nxz), Niii, (double)C32.perm, c2, (int)link);
  }
  *nf = R;
  SoupNodeD D;
  for (int d = 0; d < 3; ++d) {
    D.P[d] = C64.P[d];
    D.N[d] = C64.N[d];
    D.Nii[d] = C64.Nii[d];
    D.Niii[d] = C64.Niii[d];
  }
  D.maxP2 = lane_maxP2(C64);
  D.Nxy_yx = C64.Nxy + C64.Nyx;
  D.Nyz_zy = C64.Nyz + C64.Nzy;
  D.Nzx_xz = C64.Nzx + C64.Nxz;
  D.perm = C64.perm;
  for (int k = 0; k < 6; ++k) D.c2[k] = C64.c2[k];
  D.link = link;
  *nd = D;
}

// Moments of one depth, bottom-up: each node merges its children's data
// (items computed here) and writes its lanes' slot records; the root also
// writes slot 0.
__global__ void moments_kernel(const RNode* __restrict__ nodes, uint32_t lb, uint32_t le,
                               const double* __restrict__ V, int64_t nV,
                               const int32_t* __restrict__ F, int order,
                               const uint32_t* __restrict__ nslots,
                               const uint32_t* __restrict__ nitems,
                               const uint32_t* __restrict__ slot,
                               const uint32_t* __restrict__ ibase, Loc<float>* __restrict__ L32,
                               Loc<double>* __restrict__ L64, SoupNodeF* __restrict__ nf,
                               SoupNodeD* __restrict__ nd, float4* __restrict__ tf,
                               double* __restrict__ td, int32_t* __restrict__ tri_index) {
  const uint32_t x = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= le) return;
  Loc<float> c32[4];
  Loc<double> c64[4];
  int nch = 0;
  uint32_t sp = slot[x] + 1, ib = ibase[x];
  for (int i = 0; i < 4; ++i) {
    const uint32_t c = nodes[x].child[i];
    if (c == kEmpty) break;
    long long link;
    if (c & kInternal) {
      const uint32_t y = c & ~kInternal;
      c32[nch] = L32[y];
      c64[nch] = L64[y];
      link = (long long)sp + nslots[y];
      write_records(c32[nch], c64[nch], link, nf + sp, nd + sp);
      sp += nslots[y];
      ib += nitems[y];
    } else {
      double v[9];
      load_tri(V, nV, F, c, v);
      float w[9];
      for (int k = 0; k < 9; ++k) w[k] = (float)v[k];
      item_loc<float>(w, w + 3, w + 6, order, c32[nch]);
      item_loc<double>(v, v + 3, v + 6, order, c64[nch]);
      link = ~(long long)ib;
      write_records(c32[nch], c64[nch], link, nf + sp, nd + sp);
      for (int k = 0; k < 9; ++k) td[(int64_t)ib * 9 + k] = v[k];
      tf[(int64_t)ib * 3 + 0] = make_float4(w[0], w[1], w[2], w[3]);
      tf[(int64_t)ib * 3 + 1] = make_float4(w[4], w[5], w[6], w[7]);
      tf[(int64_t)ib * 3 + 2] = make_float4(w[8], tri_screen_slack(v), 0.f, 0.f);
      tri_index[ib] = (int32_t)c;
      ++sp;
      ++ib;
    }
    ++nch;
  }
  Loc<float> o32;
  Loc<double> o64;
  merge_loc(c32, nch, order, o32);
  merge_loc(c64, nch, order, o64);
  L32[x] = o32;
  L64[x] = o64;
  if (x == 0) {  // the root: slot 0, always opened by the walks
    write_records(o32, o64, (long long)nslots[0], nf, nd);
    nf[0].a.w = INFINITY;
    nd[0].maxP2 = INFINITY;
  }
}

// Reference node array: 4 entries per node in the reference's numbering.
__global__ void export_tree_kernel(const RNode* __restrict__ nodes, uint32_t nn,
                                   const uint32_t* __restrict__ pre, uint32_t* __restrict__ out) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nn) return;
  for (int i = 0; i < 4; ++i) {
    const uint32_t c = nodes[x].child[i];
    out[(size_t)pre[x] * 4 + i] = (c != kEmpty && (c & kInternal)) ? (kInternal | pre[c & ~kInternal]) : c;
  }
}

inline unsigned blocks_for(uint64_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

// Host side of one round's large splits.
struct LargeRunner {
  cudaStream_t st;
  RNode* nodes;
  uint32_t* idx;
  uint32_t* tmp;
  uint32_t* tapeE;
  uint32_t* tapeG;
  uint32_t* preL;
  uint32_t* preE;
  uint8_t* cls;
  const Box* tb;
  unsigned* status;

  void run(const uint32_t* list_dev, uint32_t count) {
    DevBuf<LTask> T(count, st);
    launch_kernel(large_init_kernel, blocks_for(count, 64), 64, 0, st, nodes, list_dev, count,
                  T.get());
    std::vector<LTask> h(count);
    GWN_CUDA(cudaMemcpyAsync(h.data(), T.get(), count * sizeof(LTask), cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    // span statistics over every task with a real axis
    {
      std::vector<int4> ch;
      for (uint32_t k = 0; k < count; ++k)
        if (h[k].mode == kLSpan) add_chunks(ch, k, h[k].start, h[k].n);
      if (!ch.empty()) {
        DevBuf<int4> dch(ch.size(), st);
        dch.upload(ch.data(), ch.size(), st);
        launch_kernel(large_span_kernel, (unsigned)ch.size(), 256, 0, st, (const int4*)dch.get(),
                      T.get(), (const uint32_t*)idx, tb);
        launch_kernel(large_choose_kernel, blocks_for(count, 64), 64, 0, st, T.get(), count,
                      (const uint32_t*)idx, tb);
        GWN_CUDA(cudaStreamSynchronize(st));
      }
    }
    // partitions until every span split and nthElement is done (each
    // nthElement step narrows its range, so the count is bounded by its size)
    for (uint64_t iter = 0;; ++iter) {
      GWN_REQUIRE(iter < 100000,
                  "soup_build: the partition loop did not finish");
      GWN_CUDA(cudaMemcpyAsync(h.data(), T.get(), count * sizeof(LTask), cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
      std::vector<int4> ch;
      std::vector<int2> jc(count, make_int2(0, 0));
      uint32_t maxn = 0;
      for (uint32_t k = 0; k < count; ++k) {
        if (h[k].mode == kLDone) continue;
        jc[k].x = (int)ch.size();
        add_chunks(ch, k, h[k].jlo, h[k].jn);
        jc[k].y = (int)ch.size() - jc[k].x;
        maxn = std::max(maxn, h[k].jn);
      }
      if (ch.empty()) break;
      const unsigned nch = (unsigned)ch.size();
      DevBuf<int4> dch(nch, st);
      dch.upload(ch.data(), nch, st);
      DevBuf<int2> djc(count, st);
      djc.upload(jc.data(), count, st);
      DevBuf<uint32_t> ccnt((size_t)nch * 3, st), cbase((size_t)nch * 3, st);
      const int4* c4 = dch.get();
      launch_kernel(part_init_kernel, blocks_for(count, 64), 64, 0, st, T.get(), count);
      launch_kernel(part_classify_kernel, nch, 256, 0, st, c4, T.get(), (const uint32_t*)idx, tb,
                    cls, ccnt.get());
      launch_kernel(part_chunk_scan_kernel, blocks_for(count, 64), 64, 0, st, T.get(), count,
                    (const int2*)djc.get(), (const uint32_t*)ccnt.get(), cbase.get());
      launch_kernel(part_prefix_kernel, nch, 256, 0, st, c4, T.get(), (const uint8_t*)cls,
                    (const uint32_t*)cbase.get(), preL, preE);
      launch_kernel(part_tape_kernel, nch, 256, 0, st, c4, (const LTask*)T.get(),
                    (const uint32_t*)idx, (const uint8_t*)cls, (const uint32_t*)preL,
                    (const uint32_t*)preE, tmp, tapeE, tapeG);
      int rounds = 1;
      while ((1ull << rounds) < (unsigned long long)maxn + 1) ++rounds;
      for (int r = 0; r <= rounds; ++r)
        launch_kernel(part_jump_kernel, nch, 256, 0, st, c4, (const LTask*)T.get(), tapeE, tapeG);
      launch_kernel(part_scatter_kernel, nch, 256, 0, st, c4, (const LTask*)T.get(),
                    (const uint32_t*)tmp, (const uint32_t*)tapeE, (const uint32_t*)tapeG, idx,
                    status);
      launch_kernel(part_update_kernel, blocks_for(count, 64), 64, 0, st, T.get(), count,
                    (const uint32_t*)idx, tb);
    }
    // sub boxes where the cut moved off the span's (or came from nthElement)
    {
      std::vector<int4> ch;
      for (uint32_t k = 0; k < count; ++k)
        if (h[k].need) add_chunks(ch, k, h[k].start, h[k].n);
      if (!ch.empty()) {
        DevBuf<int4> dch(ch.size(), st);
        dch.upload(ch.data(), ch.size(), st);
        launch_kernel(large_boxes_kernel, (unsigned)ch.size(), 256, 0, st,
                      (const int4*)dch.get(), T.get(), (const uint32_t*)idx, tb);
      }
    }
    launch_kernel(large_finish_kernel, blocks_for(count, 64), 64, 0, st, nodes,
                  (const LTask*)T.get(), count);
    GWN_CUDA(cudaStreamSynchronize(st));  // chunk lists live on this stack frame
  }

  static void add_chunks(std::vector<int4>& ch, uint32_t k, uint32_t lo, uint32_t n) {
    for (uint32_t b = 0; b < n; b += kChunk)
      ch.push_back(make_int4((int)k, (int)(lo + b), (int)(lo + std::min(n, b + kChunk)), 0));
  }
};

__global__ void iota3_kernel(int32_t* F, int64_t m) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < m * 3) F[i] = (int32_t)i;
}

__global__ void remap_kernel(const int32_t* __restrict__ map, int32_t* __restrict__ I, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && I[i] >= 0) I[i] = map[I[i]];
}

}  // namespace

void soup_build_search(const gwn_soup_impl& ref, gwn_soup_impl& search, cudaStream_t st) {
  const int64_t m = ref.n;
  DevBuf<int32_t> F((size_t)std::max<int64_t>(m * 3, 1), st);
  if (m) launch_kernel(iota3_kernel, blocks_for((uint64_t)m * 3), 256, 0, st, F.get(), m);
  soup_build(search, ref.td.get(), m * 3, F.get(), m, ref.order, false, st);
  GWN_CUDA(cudaStreamSynchronize(st));
}

void soup_remap_index(const int32_t* map, int32_t* I, int64_t n, cudaStream_t st) {
  if (n) launch_kernel(remap_kernel, blocks_for((uint64_t)n), 256, 0, st, map, I, n);
}

void soup_build_ref(gwn_soup_impl& s, const double* V, int64_t nV, const int32_t* F, int64_t nF,
                    int order, bool host_mode, cudaStream_t st) {
  GWN_REQUIRE(order >= 0 && order <= 2, "order must be 0, 1 or 2");
  GWN_REQUIRE(nF < (int64_t(1) << 30), "at most 2^30 triangles");
  s.order = order;
  s.n_input = nF;
  s.tree = GWN_TREE_REFERENCE;
  DeviceStatus status(st, host_mode);
  const size_t nF1 = (size_t)std::max<int64_t>(nF, 1);
  DevBuf<Box> tb(nF1, st);
  DevBuf<uint32_t> keep(nF1, st), pos(nF1, st), idx(nF1, st), root_keys(6, st);
  uint32_t m = 0;
  if (nF > 0) {
    launch_kernel(tri_box_kernel, blocks_for((uint64_t)nF), 256, 0, st, V, nV, F, nF, tb.get(),
                  keep.get(), status.ptr());
    exclusive_scan_u32(keep.get(), pos.get(), nF, st);
    std::vector<uint32_t> init = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    root_keys.upload(init.data(), 6, st);
    launch_kernel(compact_kernel, blocks_for((uint64_t)nF), 256, 0, st, (const uint32_t*)keep.get(),
                  (const uint32_t*)pos.get(), nF, (const Box*)tb.get(), idx.get(), root_keys.get());
    uint32_t last[2];
    GWN_CUDA(cudaMemcpyAsync(&last[0], pos.get() + (nF - 1), 4, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaMemcpyAsync(&last[1], keep.get() + (nF - 1), 4, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    m = last[0] + last[1];
  }
  if (host_mode) status.check(st, "soup_build");
  s.n = m;
  if (m == 0) {
    s.nnodes = 0;
    s.ref_nodes = 0;
    for (int d = 0; d < 3; ++d) s.lo[d] = s.hi[d] = 0;
    return;
  }
  // ---- tree, depth by depth
  const size_t cap = (size_t)std::max<uint32_t>(m, 1);
  DevBuf<RNode> nodes(cap, st);
  DevBuf<uint32_t> tmp(cap, st), tapeE(cap, st), tapeG(cap, st), preL(cap, st), preE(cap, st);
  DevBuf<uint8_t> cls(cap, st);
  DevBuf<uint32_t> lists(cap * 3, st), counts(3, st), ccount(cap, st), coffs(cap, st);
  launch_kernel(root_init_kernel, 1, 1, 0, st, nodes.get(), m, (const uint32_t*)root_keys.get());
  LargeRunner large{st,        nodes.get(), idx.get(),  tmp.get(),
                    tapeE.get(), tapeG.get(), preL.get(), preE.get(),
                    cls.get(),  tb.get(),    status.ptr()};
  std::vector<uint32_t> level = {0, 1};  // depth d holds nodes [level[d], level[d + 1])
  uint32_t lb = 0, le = 1;
  while (true) {
    const uint32_t nl = le - lb;
    for (int round = 0; round < 3; ++round) {
      counts.zero(st);
      launch_kernel(prepare_round_kernel, blocks_for(nl), 256, 0, st, nodes.get(), lb, le, round,
                    lists.get(), (uint32_t)cap, counts.get());
      uint32_t hc[3];
      GWN_CUDA(cudaMemcpyAsync(hc, counts.get(), sizeof(hc), cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
      if (hc[0] + hc[1] + hc[2] == 0) break;  // every node of this depth holds <= 4 items
      if (hc[0])
        launch_kernel(split_small_kernel, blocks_for(hc[0], 128), 128, 0, st, nodes.get(),
                      (const uint32_t*)lists.get(), hc[0], idx.get(), (const Box*)tb.get());
      if (hc[1])
        launch_kernel(split_medium_kernel, hc[1], 256, 0, st, nodes.get(),
                      (const uint32_t*)(lists.get() + cap), idx.get(), (const Box*)tb.get(),
                      status.ptr());
      if (hc[2]) large.run(lists.get() + 2 * cap, hc[2]);
      launch_kernel(finish_round_kernel, blocks_for(nl), 256, 0, st, nodes.get(), lb, le, round);
    }
    launch_kernel(count_children_kernel, blocks_for(nl), 256, 0, st, nodes.get(), lb, le,
                  (const uint32_t*)idx.get(), ccount.get());
    exclusive_scan_u32(ccount.get(), coffs.get(), nl, st);
    uint32_t lastc[2];
    GWN_CUDA(cudaMemcpyAsync(&lastc[0], coffs.get() + (nl - 1), 4, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaMemcpyAsync(&lastc[1], ccount.get() + (nl - 1), 4, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    const uint32_t added = lastc[0] + lastc[1];
    GWN_REQUIRE((size_t)le + added <= cap, "soup_build: tree larger than its bound");
    if (added == 0) break;
    launch_kernel(make_children_kernel, blocks_for(nl), 256, 0, st, nodes.get(), lb, le,
                  (const uint32_t*)coffs.get());
    lb = le;
    le += added;
    level.push_back(le);
  }
  const uint32_t nn = le;
  const int depth = (int)level.size() - 1;  // number of depths
  if (host_mode) status.check(st, "soup_build");
  // ---- sizes (bottom-up) and depth-first positions (top-down)
  DevBuf<uint32_t> nsize(nn, st), nslots(nn, st), nitems(nn, st), pre(nn, st), slot(nn, st),
      ibase(nn, st);
  for (int d = depth - 1; d >= 0; --d)
    launch_kernel(sizes_kernel, blocks_for(level[d + 1] - level[d]), 256, 0, st,
                  (const RNode*)nodes.get(), level[d], level[d + 1], nsize.get(), nslots.get(),
                  nitems.get());
  GWN_CUDA(cudaMemsetAsync(pre.get(), 0, 4, st));
  GWN_CUDA(cudaMemsetAsync(slot.get(), 0, 4, st));
  GWN_CUDA(cudaMemsetAsync(ibase.get(), 0, 4, st));
  for (int d = 0; d < depth; ++d)
    launch_kernel(positions_kernel, blocks_for(level[d + 1] - level[d]), 256, 0, st,
                  (const RNode*)nodes.get(), level[d], level[d + 1], (const uint32_t*)nsize.get(),
                  (const uint32_t*)nslots.get(), (const uint32_t*)nitems.get(), pre.get(),
                  slot.get(), ibase.get());
  uint32_t total_slots = 0;
  GWN_CUDA(cudaMemcpyAsync(&total_slots, nslots.get(), 4, cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  // ---- moments and the walk's slot records
  s.nnodes = total_slots;
  s.ref_nodes = nn;
  s.max_depth = depth;
  s.tri_index.alloc(m);
  s.nf.alloc(total_slots);
  // the walk reads records with 256-bit loads
  if (reinterpret_cast<uintptr_t>(s.nf.get()) % 32)
    throw Error(GWN_ERR_INTERNAL, "node records are not 32-byte aligned");
  s.nd.alloc(total_slots);
  s.tf.alloc((size_t)m * 3);
  s.td.alloc((size_t)m * 9);
  s.ref_child.alloc((size_t)nn * 4);
  {
    DevBuf<Loc<float>> L32(nn, st);
    DevBuf<Loc<double>> L64(nn, st);
    for (int d = depth - 1; d >= 0; --d)
      launch_kernel(moments_kernel, blocks_for(level[d + 1] - level[d], 128), 128, 0, st,
                    (const RNode*)nodes.get(), level[d], level[d + 1], V, nV, F, order,
                    (const uint32_t*)nslots.get(), (const uint32_t*)nitems.get(),
                    (const uint32_t*)slot.get(), (const uint32_t*)ibase.get(), L32.get(),
                    L64.get(), s.nf.get(), s.nd.get(),
                    s.tf.get(), s.td.get(), s.tri_index.get());
    launch_kernel(export_tree_kernel, blocks_for(nn), 256, 0, st, (const RNode*)nodes.get(), nn,
                  (const uint32_t*)pre.get(), s.ref_child.get());
    Loc<double> root;
    GWN_CUDA(cudaMemcpyAsync(&root, L64.get(), sizeof(root), cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    double diag2 = 0, cmax = 0;
    for (int d = 0; d < 3; ++d) {
      s.lo[d] = root.lo[d];
      s.hi[d] = root.hi[d];
      const double e = root.hi[d] - root.lo[d];
      diag2 += e * e;
      cmax = fmax(cmax, fmax(fabs(root.lo[d]), fabs(root.hi[d])));
    }
    s.eps = kNearFrac * sqrt(diag2);
    s.cmax = cmax;
  }
  soup_check_moments(s, st);
  if (host_mode) status.check(st, "soup_build");
  s.bytes = s.nf.bytes() + s.nd.bytes() + s.tf.bytes() + s.td.bytes() + s.tri_index.bytes() +
            s.ref_child.bytes();
}

}  // namespace gwn
