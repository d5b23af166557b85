// Point-cloud fast winding number: order-0/1/2 dipole expansion precompute
// (segmented warp-shuffle reduction, FP64) and a warp-coherent stackless
// Barnes-Hut walk.
//
// Reference: include/igl/fast_winding_number.cpp:17-124 (precompute) and
// :126-311 (evaluate).  Per cell with points:
//   CM = sum A p / sum A, EC[0:3] = sum A n, R = max |p - CM|,
//   EC[3+u+3v] = sum A (p-CM)_u n_v,
//   EC[12+9k+u+3v] = sum 0.5 (p-CM)_k A (p-CM)_u n_v,
// an empty cell gets CM = NaN (:70-75).  Evaluation descends from the root:
// a child with points is approximated when |CM - q| > beta R (:266) -- a leaf
// child by its points' dipoles, an internal child by expansion_eval
// (:174-228) -- and otherwise opened; an opened leaf adds its points'
// dipoles (:253-262); a dipole at distance 0 contributes 0.5 (:164-166).
//
// Precompute on the device: every non-empty cell's point list (a contiguous
// range of the octree's point order, or a caller CSR list) is cut into
// chunks of at most 1024 points; one warp sums a chunk (lanes stride the
// points, a fixed xor-shuffle tree combines lanes) and a second kernel adds
// each cell's chunk partials in chunk order.  Two passes: mass centre first,
// then R and the moments about it.  All accumulation is FP64.
//
// Walk: pre-order of the non-empty cells (order of (first point, depth));
// the same warp-coherent scheme as the soup path.  Mixed precision: FP32
// records and arithmetic; the approximate/open test is redone in FP64 with
// the reference's own expression inside a proven FP32 error band; dipoles
// within 1e-3 * bbox diagonal of the query are evaluated in FP64; results
// within 1e-3 of 0.5 are recomputed by the plain FP64 walk.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "bh_common.cuh"
#include "cloud.cuh"
#include "gwn_common.cuh"
#include "octree.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

constexpr int kChunk = 1024;
// Cells with at most kSmallCell points are summed by one thread each (both
// passes, points in list order); larger cells by warps over 1024-point
// chunks.  Most cells of an octree are small: giving each a warp spent the
// time in 37-value FP64 warp reductions for a handful of points.
constexpr int kSmallCell = 64;
constexpr double kNearFrac = 1e-3;
constexpr double kBand = 1e-3;
constexpr double kPi4 = 4.0 * kPi;
constexpr float kInvPi4F = (float)(1.0 / (4.0 * kPi));

inline unsigned blocks(int64_t n, int t = 256) {
  return (unsigned)std::max<int64_t>(1, (n + t - 1) / t);
}

__global__ void an_kernel(const double* __restrict__ N, const double* __restrict__ A, int64_t n,
                          double* __restrict__ AN) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = A[i];
  for (int d = 0; d < 3; ++d) AN[i * 3 + d] = N[i * 3 + d] * a;  // N.row(i)*A(i), :257
}

__global__ void chunk_count_kernel(const int32_t* __restrict__ count, int64_t ncells,
                                   unsigned* __restrict__ nch) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c < ncells) nch[c] = count[c] > kSmallCell ? (unsigned)((count[c] + kChunk - 1) / kChunk) : 0u;
}

__global__ void chunk_fill_kernel(const unsigned* __restrict__ nch,
                                  const unsigned* __restrict__ base, int64_t ncells,
                                  int32_t* __restrict__ chunk_cell) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  for (unsigned j = 0; j < nch[c]; ++j) chunk_cell[base[c] + j] = (int32_t)c;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

struct CsrView {
  const int64_t* start;
  const int32_t* count;
  const int32_t* idx;
};

// Pass 1: sum A, A p, A n over each chunk (7 doubles per chunk).
__global__ void pass1_kernel(CsrView v, const int32_t* __restrict__ chunk_cell,
                             const unsigned* __restrict__ chunk_base, int64_t nchunks,
                             const double* __restrict__ P, const double* __restrict__ N,
                             const double* __restrict__ A, double* __restrict__ part) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const int32_t c = chunk_cell[w];
  const int64_t off = (w - chunk_base[c]) * (int64_t)kChunk;
  const int64_t s = v.start[c] + off;
  const int32_t cnt = (int32_t)min((int64_t)kChunk, (int64_t)v.count[c] - off);
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int j = lane; j < cnt; j += 32) {
    const int64_t p = v.idx[s + j];
    const double a = A[p];
    acc[0] += a;
    for (int d = 0; d < 3; ++d) {
      acc[1 + d] += a * P[p * 3 + d];
      acc[4 + d] += a * N[p * 3 + d];
    }
  }
  for (int k = 0; k < 7; ++k) acc[k] = warp_sum(acc[k]);
  if (lane < 7) {
    double v0 = acc[0];
#pragma unroll
    for (int k = 1; k < 7; ++k)
      if (lane == k) v0 = acc[k];
    part[w * 8 + lane] = v0;
  }
}

// Cells with more than kSmallCell points: one warp per cell (the warp that
// owns the cell's first chunk) sums the chunk partials, lanes striding the
// chunks, then a fixed xor tree: a deterministic order that does not leave
// one thread summing thousands of partials of the largest cells.
__global__ void combine1_kernel(const int32_t* __restrict__ chunk_cell,
                                const unsigned* __restrict__ chunk_base,
                                const unsigned* __restrict__ nch, int64_t nchunks,
                                const double* __restrict__ part, int num_terms,
                                double* __restrict__ CM, double* __restrict__ EC,
                                double* __restrict__ area) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const int32_t c = chunk_cell[w];
  if ((unsigned)w != chunk_base[c]) return;  // not the cell's first chunk
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (unsigned j = lane; j < nch[c]; j += 32)
    for (int k = 0; k < 7; ++k) s[k] += part[(chunk_base[c] + j) * 8 + k];
  for (int k = 0; k < 7; ++k) s[k] = warp_sum(s[k]);
  if (lane != 0) return;
  area[c] = s[0];
  for (int d = 0; d < 3; ++d) {
    CM[c * 3 + d] = s[1 + d] / s[0];
    EC[c * num_terms + d] = s[4 + d];
  }
}

// Empty cells: CM = 0/0 (NaN) and zero area, as the reference's sums give.
__global__ void empty_cells_kernel(const int32_t* __restrict__ count, int64_t ncells,
                                   double* __restrict__ CM, double* __restrict__ area) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells || count[c] != 0) return;
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  CM[c * 3] = CM[c * 3 + 1] = CM[c * 3 + 2] = nan;
  area[c] = 0.0;
}

// Pass 2: max |p - CM| and the order-1/2 moments about CM (1 + 36 doubles).
template <int NT>
__global__ void pass2_kernel(CsrView v, const int32_t* __restrict__ chunk_cell,
                             const unsigned* __restrict__ chunk_base, int64_t nchunks,
                             const double* __restrict__ P, const double* __restrict__ N,
                             const double* __restrict__ A, const double* __restrict__ CM,
                             double* __restrict__ part) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const int32_t c = chunk_cell[w];
  const int64_t off = (w - chunk_base[c]) * (int64_t)kChunk;
  const int64_t s = v.start[c] + off;
  const int32_t cnt = (int32_t)min((int64_t)kChunk, (int64_t)v.count[c] - off);
  const double cm[3] = {CM[c * 3], CM[c * 3 + 1], CM[c * 3 + 2]};
  double mx = 0;
  double acc[NT > 3 ? NT - 3 : 1];
#pragma unroll
  for (int k = 0; k < NT - 3; ++k) acc[k] = 0;
  for (int j = lane; j < cnt; j += 32) {
    const int64_t p = v.idx[s + j];
    const double a = A[p];
    double pt[3], n[3];
    for (int d = 0; d < 3; ++d) {
      pt[d] = P[p * 3 + d] - cm[d];
      n[d] = N[p * 3 + d];
    }
    const double nrm = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(pt[0], pt[0]), __dmul_rn(pt[1], pt[1])),
                                      __dmul_rn(pt[2], pt[2])));
    mx = fmax(mx, nrm);
    if (NT >= 12) {
#pragma unroll
      for (int vv = 0; vv < 3; ++vv)
#pragma unroll
        for (int u = 0; u < 3; ++u) acc[u + 3 * vv] += (a * pt[u]) * n[vv];
    }
    if (NT == 39) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double h = 0.5 * pt[k];
#pragma unroll
        for (int vv = 0; vv < 3; ++vv)
#pragma unroll
          for (int u = 0; u < 3; ++u) acc[9 + 9 * k + u + 3 * vv] += h * ((a * pt[u]) * n[vv]);
      }
    }
  }
  mx = warp_max(mx);
#pragma unroll
  for (int k = 0; k < NT - 3; ++k) acc[k] = warp_sum(acc[k]);
  if (lane == 0) {
    double* o = part + w * 37;
    o[0] = mx;
#pragma unroll
    for (int k = 0; k < NT - 3; ++k) o[1 + k] = acc[k];
  }
}

__global__ void combine2_kernel(const int32_t* __restrict__ chunk_cell,
                                const unsigned* __restrict__ chunk_base,
                                const unsigned* __restrict__ nch, int64_t nchunks,
                                const double* __restrict__ part, int num_terms,
                                double* __restrict__ R, double* __restrict__ EC) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nchunks) return;
  const int32_t c = chunk_cell[w];
  if ((unsigned)w != chunk_base[c]) return;  // not the cell's first chunk
  double mx = 0;
  for (unsigned j = lane; j < nch[c]; j += 32) mx = fmax(mx, part[(chunk_base[c] + j) * 37]);
  mx = warp_max(mx);
  if (lane == 0) R[c] = mx;
  for (int k = 3; k < num_terms; ++k) {
    double s = 0;
    for (unsigned j = lane; j < nch[c]; j += 32) s += part[(chunk_base[c] + j) * 37 + (k - 2)];
    s = warp_sum(s);
    if (lane == 0) EC[c * num_terms + k] = s;
  }
}

// Both passes for one small cell per thread: the same terms as pass1 /
// combine1 / pass2 / combine2, summed over the cell's points in list order
// (the reference's loop order, fast_winding_number.cpp:57-120).
template <int NT>
__device__ __forceinline__ void small_cell_moments(CsrView v, int64_t c, int32_t cnt,
                                                        const double* __restrict__ P,
                                                        const double* __restrict__ N,
                                                        const double* __restrict__ A,
                                                        double* __restrict__ CM,
                                                        double* __restrict__ R,
                                                        double* __restrict__ area,
                                                        double* __restrict__ row) {
  const int64_t s0 = v.start[c];
  double s[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j < cnt; ++j) {
    const int64_t p = v.idx[s0 + j];
    const double a = A[p];
    s[0] += a;
    for (int d = 0; d < 3; ++d) {
      s[1 + d] += a * P[p * 3 + d];
      s[4 + d] += a * N[p * 3 + d];
    }
  }
  area[c] = s[0];
  double cm[3];
  for (int d = 0; d < 3; ++d) {
    cm[d] = s[1 + d] / s[0];
    CM[c * 3 + d] = cm[d];
    row[d] = s[4 + d];
  }
  double mx = 0;
  double acc[NT > 3 ? NT - 3 : 1];
#pragma unroll
  for (int k = 0; k < NT - 3; ++k) acc[k] = 0;
  for (int j = 0; j < cnt; ++j) {
    const int64_t p = v.idx[s0 + j];
    const double a = A[p];
    double pt[3], n[3];
    for (int d = 0; d < 3; ++d) {
      pt[d] = P[p * 3 + d] - cm[d];
      n[d] = N[p * 3 + d];
    }
    const double nrm = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(pt[0], pt[0]), __dmul_rn(pt[1], pt[1])),
                                      __dmul_rn(pt[2], pt[2])));
    mx = fmax(mx, nrm);
    if (NT >= 12) {
#pragma unroll
      for (int vv = 0; vv < 3; ++vv)
#pragma unroll
        for (int u = 0; u < 3; ++u) acc[u + 3 * vv] += (a * pt[u]) * n[vv];
    }
    if (NT == 39) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double h = 0.5 * pt[k];
#pragma unroll
        for (int vv = 0; vv < 3; ++vv)
#pragma unroll
          for (int u = 0; u < 3; ++u) acc[9 + 9 * k + u + 3 * vv] += h * ((a * pt[u]) * n[vv]);
      }
    }
  }
  R[c] = mx;
#pragma unroll
  for (int k = 0; k < NT - 3; ++k) row[3 + k] = acc[k];
}

// Small non-empty cells grouped by point count (a counting sort on
// 1..kSmallCell): the lanes of a warp then loop over the same number of
// points, where consecutive cell ids (mostly empty cells, and counts from 1
// to 64 side by side) left two lanes in three idle on the FP64 pipe.
// 4,096 cells per block (256 threads x 16): the global counters then take
// one atomic per block and count instead of one per cell, since thousands of
// same-address atomics serialize.
constexpr int kListThreads = 256, kListPer = 16;
constexpr int64_t kListCells = (int64_t)kListThreads * kListPer;

__global__ void __launch_bounds__(kListThreads) small_hist_kernel(const int32_t* __restrict__ count,
                                                                  int64_t ncells,
                                                                  unsigned* __restrict__ hist) {
  __shared__ unsigned h[kSmallCell + 1];
  for (int k = threadIdx.x; k <= kSmallCell; k += blockDim.x) h[k] = 0;
  __syncthreads();
  for (int j = 0; j < kListPer; ++j) {
    const int64_t c = blockIdx.x * kListCells + (int64_t)j * kListThreads + threadIdx.x;
    if (c < ncells) {
      const int32_t n = count[c];
      if (n > 0 && n <= kSmallCell) atomicAdd(&h[n], 1u);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k <= kSmallCell; k += blockDim.x)
    if (h[k]) atomicAdd(&hist[k], h[k]);
}

// hist[0..kSmallCell] -> exclusive offsets, total in hist[kSmallCell + 1]
// (one thread; 65 entries)
__global__ void small_offsets_kernel(unsigned* __restrict__ hist) {
  unsigned run = 0;
  for (int k = 0; k <= kSmallCell; ++k) {
    const unsigned v = hist[k];
    hist[k] = run;
    run += v;
  }
  hist[kSmallCell + 1] = run;
}

__global__ void __launch_bounds__(kListThreads) small_scatter_kernel(const int32_t* __restrict__ count,
                                                                     int64_t ncells,
                                                                     unsigned* __restrict__ next,
                                                                     int32_t* __restrict__ list) {
  __shared__ unsigned h[kSmallCell + 1], base[kSmallCell + 1];
  for (int k = threadIdx.x; k <= kSmallCell; k += blockDim.x) h[k] = 0;
  __syncthreads();
  int32_t n[kListPer];
  unsigned rank[kListPer];
#pragma unroll
  for (int j = 0; j < kListPer; ++j) {
    const int64_t c = blockIdx.x * kListCells + (int64_t)j * kListThreads + threadIdx.x;
    n[j] = c < ncells ? count[c] : 0;
    rank[j] = (n[j] > 0 && n[j] <= kSmallCell) ? atomicAdd(&h[n[j]], 1u) : 0u;
  }
  __syncthreads();
  for (int k = threadIdx.x; k <= kSmallCell; k += blockDim.x)
    base[k] = h[k] ? atomicAdd(&next[k], h[k]) : 0u;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kListPer; ++j) {
    const int64_t c = blockIdx.x * kListCells + (int64_t)j * kListThreads + threadIdx.x;
    if (n[j] > 0 && n[j] <= kSmallCell) list[base[n[j]] + rank[j]] = (int32_t)c;
  }
}

// One thread per listed small cell (both passes over the cell's points in
// list order); each warp stages its 32 EC rows in shared memory and writes
// them row by row, each row one coalesced store of NT doubles.
template <int NT>
__global__ void __launch_bounds__(128) small_cells_kernel(CsrView v, const int32_t* __restrict__ list,
                                                          int64_t n,
                                                          const double* __restrict__ P,
                                                          const double* __restrict__ N,
                                                          const double* __restrict__ A,
                                                          double* __restrict__ CM,
                                                          double* __restrict__ R,
                                                          double* __restrict__ EC,
                                                          double* __restrict__ area) {
  __shared__ double rows[4][32 * NT];
  __shared__ int32_t cells[4][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t i0 = (blockIdx.x * (int64_t)blockDim.x) + warp * 32;  // first entry of the warp
  if (i0 >= n) return;  // the whole warp
  const int64_t i = i0 + lane;
  const int32_t c = i < n ? list[i] : -1;
  cells[warp][lane] = c;
  if (c >= 0)
    small_cell_moments<NT>(v, c, v.count[c], P, N, A, CM, R, area, rows[warp] + lane * NT);
  __syncwarp();
  const int nrows = n - i0 < 32 ? (int)(n - i0) : 32;
  for (int r = 0; r < nrows; ++r) {
    double* out = EC + (int64_t)cells[warp][r] * NT;
    for (int e = lane; e < NT; e += 32) out[e] = rows[warp][r * NT + e];
  }
}


// ----------------------------------------------------------------- layout --
__global__ void nonempty_keys_kernel(const int64_t* __restrict__ start,
                                     const int32_t* __restrict__ count,
                                     const int32_t* __restrict__ depth, int64_t ncells,
                                     unsigned long long* __restrict__ key,
                                     int32_t* __restrict__ val) {
  const int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (x >= ncells) return;
  key[x] = count[x] > 0 ? (((unsigned long long)start[x] << 15) | (unsigned long long)depth[x])
                        : ((1ull << 48) - 1);
  val[x] = (int32_t)x;
}

__device__ __forceinline__ int64_t lower_bound_key(const unsigned long long* keys, int64_t n,
                                                   unsigned long long k) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

struct LayoutIn {
  const int32_t* order;   // traversal position -> cell id
  const int32_t* first_by_pos;  // traversal position -> first point slot (or null: cell start)
  const int64_t* skip;    // traversal position -> one past subtree (or null: compute from keys)
  const unsigned long long* keys;  // sorted (start, depth) keys (when skip is null)
  int64_t nnodes;
  const int64_t* start;
  const int32_t* count;
  const int32_t* ch;
  const int32_t* depth;
  const double* CM;
  const double* R;
  const double* EC;
  int num_terms;
  const double* area;  // per cell, for the FP64 near-field radius
  double eps, cmax;
};

// FP64 near-field radius of a dipole (or expansion) of strength `area`: a
// point dipole's field grows as area / r^2, so the FP32 rounding of q - p
// (delta = 4 u cmax) costs area * delta / (4 pi r^3); below
// r = (area * delta / (4 pi tau))^(1/3), tau = 2e-7 per term, or below the
// 1e-3 * bbox-diagonal rule, the term is evaluated in FP64.
__device__ __forceinline__ float near_radius2(double area, double eps, double cmax) {
  const double delta = 4.0 * 5.9604644775390625e-08 * cmax;
  const double r = fmax(eps, cbrt(fabs(area) * delta / (4.0 * kPi * 2e-7)));
  return (float)(r * r * 1.0001);
}

__global__ void emit_nodes_kernel(LayoutIn in, CloudNodeF* __restrict__ nf,
                                  CloudNodeD* __restrict__ nd) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= in.nnodes) return;
  const int32_t c = in.order[p];
  int64_t skip;
  if (in.skip) {
    skip = in.skip[p];
  } else {
    const unsigned long long end = (unsigned long long)(in.start[c] + in.count[c]);
    skip = lower_bound_key(in.keys, in.nnodes, end << 15);
  }
  const bool leaf = in.ch[(int64_t)c * 8] == -1;
  CloudNodeD D;
  for (int d = 0; d < 3; ++d) D.cm[d] = in.CM[(int64_t)c * 3 + d];
  D.r = in.R[c];
  {
    double ec[39];
    for (int k = 0; k < 39; ++k) ec[k] = k < in.num_terms ? in.EC[(int64_t)c * in.num_terms + k] : 0.0;
    pack_cloud(ec, in.num_terms, D.pk);
  }
  D.pad = 0;
  const int first = in.first_by_pos ? in.first_by_pos[p] : (int)in.start[c];
  D.l = make_int4((int)skip, first, in.count[c], leaf ? 1 : 0);
  nd[p] = D;
  CloudNodeF Fr;
  Fr.a = make_float4((float)D.cm[0], (float)D.cm[1], (float)D.cm[2], (float)D.r);
  const double* pk = D.pk;
  Fr.b = make_float4((float)pk[0], (float)pk[1], (float)pk[2], (float)pk[3]);
  Fr.c = make_float4((float)pk[4], (float)pk[5], (float)pk[6], (float)pk[7]);
  Fr.d = make_float4((float)pk[8], (float)pk[9], (float)pk[10], (float)pk[11]);
  Fr.e = make_float4((float)pk[12], (float)pk[13], (float)pk[14],
                     near_radius2(in.area[c], in.eps, in.cmax));
  Fr.l = D.l;
  nf[p] = Fr;
}

__global__ void emit_points_kernel(const int32_t* __restrict__ slot_point, int64_t nslots,
                                   const double* __restrict__ P, const double* __restrict__ AN,
                                   double eps, double cmax, float4* __restrict__ pf,
                                   double* __restrict__ pd) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= nslots) return;
  const int64_t p = slot_point[j];
  double v[6];
  for (int d = 0; d < 3; ++d) {
    v[d] = P[p * 3 + d];
    v[3 + d] = AN[p * 3 + d];
  }
  for (int k = 0; k < 6; ++k) pd[j * 6 + k] = v[k];
  const double strength = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
  pf[j * 2] = make_float4((float)v[0], (float)v[1], (float)v[2], near_radius2(strength, eps, cmax));
  pf[j * 2 + 1] = make_float4((float)v[3], (float)v[4], (float)v[5], 0.f);
}

// --------------------------------------------------------------- evaluate --
// direct_eval, fast_winding_number.cpp:159-172 (FP64, reference expression order).
__device__ __forceinline__ double dipole64(double lx, double ly, double lz, double ax, double ay,
                                           double az) {
  const double ln = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(lx, lx), __dmul_rn(ly, ly)), __dmul_rn(lz, lz)));
  if (ln == 0) return 0.5;
  return (lx * ax + ly * ay + lz * az) / (kPi4 * (ln * ln * ln));
}

// FP64 expansion from a packed record (pack_cloud), loc = CM - q: the same
// forms as the FP32 walk's, in FP64.
__device__ __forceinline__ double expansion_packed64(const double* pk, double lx, double ly,
                                                     double lz, int num_terms) {
  const double ir = 1.0 / sqrt(lx * lx + ly * ly + lz * lz), ir2 = ir * ir;
  const double ux = lx * ir, uy = ly * ir, uz = lz * ir;
  const double lin = ux * pk[0] + uy * pk[1] + uz * pk[2];
  if (num_terms <= 3) return ir2 * lin;
  const double x2 = ux * ux, y2 = uy * uy, z2 = uz * uz, yz = uy * uz;
  const double qzz = -(pk[3] + pk[4]);
  double s = ux * (pk[3] * ux + pk[5] * uy + pk[6] * uz) + pk[4] * y2 + qzz * z2 + pk[7] * yz;
  if (num_terms > 12) {
    const double kxzz = -(3 * pk[8] + pk[12]), kyzz = -(3 * pk[9] + pk[10]);
    const double kzzz = -(pk[11] + pk[13]) / 3;
    const double kx = pk[8] * x2 + pk[12] * y2 + kxzz * z2 + pk[14] * yz;
    const double ky = pk[10] * x2 + pk[9] * y2 + kyzz * z2;
    const double kz = pk[11] * x2 + pk[13] * y2 + kzzz * z2;
    s += ir * (ux * kx + uy * ky + uz * kz);
  }
  return ir2 * (lin + ir * s);
}

// FP32 expansion from a packed record (pack_cloud): loc = CM - q,
// r2 = |loc|^2; W = (u.N + (Q(u) + K(u)/r)/r) / r^2 with u = loc/r.
__device__ __forceinline__ float expansion_packed32(float4 b, float4 c, float4 d, float4 e,
                                                    float lx, float ly, float lz, float r2,
                                                    int num_terms) {
  const float ir = rsqrtf(r2), ir2 = ir * ir;
  const float ux = lx * ir, uy = ly * ir, uz = lz * ir;
  const float lin = fmaf(ux, b.x, fmaf(uy, b.y, uz * b.z));
  if (num_terms <= 3) return ir2 * lin;
  const float x2 = ux * ux, y2 = uy * uy, z2 = uz * uz, yz = uy * uz;
  const float qzz = -(b.w + c.x);
  float s = fmaf(ux, fmaf(b.w, ux, fmaf(c.y, uy, c.z * uz)), fmaf(c.x, y2, fmaf(qzz, z2, c.w * yz)));
  if (num_terms > 12) {
    const float kxzz = -fmaf(3.f, d.x, e.x), kyzz = -fmaf(3.f, d.y, d.z);
    const float kzzz = -(d.w + e.y) * (1.f / 3.f);
    const float kx = fmaf(d.x, x2, fmaf(e.x, y2, fmaf(kxzz, z2, e.z * yz)));
    const float ky = fmaf(d.z, x2, fmaf(d.y, y2, kyzz * z2));
    const float kz = fmaf(d.w, x2, fmaf(e.y, y2, kzzz * z2));
    s = fmaf(ir, fmaf(ux, kx, fmaf(uy, ky, uz * kz)), s);
  }
  return ir2 * fmaf(ir, s, lin);
}

// The reference's test `|CM - q| > beta R` (:265-266), FP64, pinned order.
__device__ __forceinline__ bool far64(double qx, double qy, double qz, const double* cm, double r,
                                      double beta) {
  const double dx = __dsub_rn(cm[0], qx), dy = __dsub_rn(cm[1], qy), dz = __dsub_rn(cm[2], qz);
  const double nrm = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
  return nrm > __dmul_rn(beta, r);
}

struct CloudEvalParams {
  const CloudNodeF* nf;
  const CloudNodeD* nd;
  const float4* pf;
  const double* pd;
  int nnodes;
  int num_terms;
  double beta;
  float beta_f;
  float eps;
  float cmax;
};

template <typename QT>
__device__ __forceinline__ void read_q(const QT* Q, const int32_t* perm, const int32_t* list,
                                       int64_t i, int64_t& qi, double& x, double& y, double& z) {
  qi = list ? (int64_t)list[i] : (perm ? (int64_t)perm[i] : i);
  x = (double)Q[qi * 3];
  y = (double)Q[qi * 3 + 1];
  z = (double)Q[qi * 3 + 2];
}

// Per-warp queue of FP64 terms: code >= 0 is a point slot (exact dipole
// term), code < 0 is ~node (the node's expansion in FP64).  Lanes append the
// terms they need and the warp evaluates up to 32 queued terms at once, one
// per lane, so each FP64 instruction serves the whole warp; each lane adds
// its own values by its bit mask of queue positions, in queue order, which
// is its walk order.  The mixed walk queues its FP64 near-field terms here,
// the plain FP64 walk every term.  The lanes' FP64 queries live here too
// (read only at FP64 re-checks and flushes), and the mixed walk runs 8
// blocks of 128 threads per SM (64 registers; with the division-free FP32
// terms, 18.2 -> 17.4 ms for C3's 8M queries against 6).
struct CloudNearQueue {
  int2 e[32];
  double q[32][3];  // each lane's FP64 query
  double v[32];     // the values of one flush
};

__device__ __forceinline__ void flush_cloud64(const CloudEvalParams& prm, CloudNearQueue& q,
                                              int n, unsigned mine, double& acc64) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (lane < n) {
    const int2 e = q.e[lane];
    const double ox = q.q[e.y][0], oy = q.q[e.y][1], oz = q.q[e.y][2];
    double v;
    if (e.x >= 0) {
      const double* pd = prm.pd + (int64_t)e.x * 6;
      v = dipole64(pd[0] - ox, pd[1] - oy, pd[2] - oz, pd[3], pd[4], pd[5]);
    } else {
      const CloudNodeD* rd = prm.nd + ~e.x;
      const double lx = __dsub_rn(rd->cm[0], ox), ly = __dsub_rn(rd->cm[1], oy),
                   lz = __dsub_rn(rd->cm[2], oz);
      v = expansion_packed64(rd->pk, lx, ly, lz, prm.num_terms);
    }
    q.v[lane] = v;
  }
  __syncwarp();
  while (mine) {
    acc64 += q.v[__ffs(mine) - 1];
    mine &= mine - 1;
  }
  __syncwarp();
}

// Appends this lane's term `code` if `want` (all 32 lanes call together).
__device__ __forceinline__ void queue_cloud64(const CloudEvalParams& prm, CloudNearQueue& q,
                                              int& nqueued, unsigned& mine, bool want, int code,
                                              double& acc64) {
  const unsigned full = 0xffffffffu;
  const unsigned m = __ballot_sync(full, want);
  if (!m) return;
  const int k = __popc(m);
  if (nqueued + k > 32) {
    flush_cloud64(prm, q, nqueued, mine, acc64);
    nqueued = 0;
    mine = 0;
  }
  const int lane = threadIdx.x & 31;
  if (want) {
    const int pos = nqueued + __popc(m & ((1u << lane) - 1u));
    q.e[pos] = make_int2(code, lane);
    mine |= 1u << pos;
  }
  nqueued += k;
}

// Appends cnt dipole terms of this lane (point slots first, first + 1, ...)
// after the lower lanes' terms, flushing whenever the queue fills (all 32
// lanes call together).
__device__ __forceinline__ void queue_points64(const CloudEvalParams& prm, CloudNearQueue& q,
                                               int& nqueued, unsigned& mine, int cnt, int first,
                                               double& acc64) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int incl = cnt;
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(full, incl, d);
    if (lane >= d) incl += y;
  }
  const int total = __shfl_sync(full, incl, 31);
  const int excl = incl - cnt;
  for (int done = 0; done < total;) {
    const int take = min(32 - nqueued, total - done);
    const int k0 = max(0, done - excl), k1 = min(cnt, done + take - excl);
    for (int k = k0; k < k1; ++k) {
      const int pos = nqueued + excl + k - done;
      q.e[pos] = make_int2(first + k, lane);
      mine |= 1u << pos;
    }
    nqueued += take;
    done += take;
    if (nqueued == 32) {
      flush_cloud64(prm, q, 32, mine, acc64);
      nqueued = 0;
      mine = 0;
    }
  }
}

template <typename QT, typename WT>
__global__ void __launch_bounds__(128, 8) cloud_eval_mixed_kernel(CloudEvalParams prm, const QT* __restrict__ Q,
                                                               const int32_t* __restrict__ perm,
                                                               int64_t nQ, WT* __restrict__ W,
                                                               int32_t* __restrict__ refine_list,
                                                               unsigned* __restrict__ refine_count) {
  __shared__ CloudNearQueue near_q[4];
  CloudNearQueue& nq = near_q[threadIdx.x >> 5];
  int nqueued = 0;    // warp-uniform
  unsigned mine = 0;  // this lane's queue positions
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < nQ;
  int64_t qi = 0;
  double qx = 0, qy = 0, qz = 0;
  if (valid) read_q(Q, perm, (const int32_t*)nullptr, i, qi, qx, qy, qz);
  const int lane = threadIdx.x & 31;
  nq.q[lane][0] = qx;
  nq.q[lane][1] = qy;
  nq.q[lane][2] = qz;
  const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
  const float S = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) + prm.cmax;
  const float sigma = guard_sigma(S);
  float acc = 0.f;
  double acc64 = 0.0;
  int resume = valid ? 0 : 0x7fffffff;
  int node = 0;
  const unsigned full = 0xffffffffu;
  while (node < prm.nnodes) {
    // the whole record in three 256-bit loads (96-byte records, 32-byte
    // aligned base)
    const CloudNodeF* r = prm.nf + node;
    float4 a, rb, rc, rd, re, lf;
    ldg256(&r->a, a, rb);
    ldg256(&r->c, rc, rd);
    ldg256(&r->e, re, lf);
    const int4 l = make_int4(__float_as_int(lf.x), __float_as_int(lf.y), __float_as_int(lf.z),
                             __float_as_int(lf.w));
    const bool visit = node >= resume;
    bool open = false;
    if (l.w != 0) {  // leaf (the node, hence the branch, is warp-uniform)
      for (int j = 0; j < l.z; ++j) {
        const int64_t slot = (int64_t)l.y + j;
        bool want = false;
        if (visit) {
          const float4 p = __ldg(&prm.pf[slot * 2]);
          const float lx = p.x - fx, ly = p.y - fy, lz = p.z - fz;
          const float r2 = fmaf(lz, lz, fmaf(ly, ly, lx * lx));
          if (r2 <= p.w) {
            want = true;
          } else {
            const float4 an = __ldg(&prm.pf[slot * 2 + 1]);
            const float ir = rsqrtf(r2);
            acc += fmaf(lx, an.x, fmaf(ly, an.y, lz * an.z)) * (ir * ir * ir * kInvPi4F);
          }
        }
        queue_cloud64(prm, nq, nqueued, mine, want, (int)slot, acc64);
      }
      if (visit) resume = l.x;
    } else if (node == 0) {
      open = visit;
    } else {
      bool want = false;
      if (visit) {
        const float dx = a.x - fx, dy = a.y - fy, dz = a.z - fz;
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float br = prm.beta_f * a.w;
        const float thr = br * br;
        bool far = r2 > thr;
        if (in_guard_band(r2, thr, sigma)) {
          const CloudNodeD* rd = prm.nd + node;
          far = far64(nq.q[lane][0], nq.q[lane][1], nq.q[lane][2], rd->cm, rd->r, prm.beta);
        }
        if (far) {
          if (r2 <= re.w) {  // strong expansion close to the query: FP64
            want = true;
          } else {
            acc += expansion_packed32(rb, rc, rd, re, dx, dy, dz, r2, prm.num_terms);
          }
          resume = l.x;
        } else {
          open = true;
        }
      }
      queue_cloud64(prm, nq, nqueued, mine, want, ~node, acc64);
    }
    // a lane that opens the node wants node + 1, every other lane is past
    // the node (resume > node): the warp goes to the smallest of them
    node = __reduce_min_sync(full, open ? node + 1 : resume);
  }
  if (nqueued) flush_cloud64(prm, nq, nqueued, mine, acc64);
  if (!valid) return;
  const double w = acc64 != 0.0 ? (double)acc + acc64 : (double)acc;
  W[qi] = (WT)w;
  if (fabs(w - 0.5) <= kBand) {
    const unsigned s = atomicAdd(refine_count, 1u);
    refine_list[s] = (int32_t)qi;
  }
}

template <typename QT, typename WT>
__global__ void __launch_bounds__(128) cloud_eval_fp64_kernel(CloudEvalParams prm, const QT* __restrict__ Q,
                                                              const int32_t* __restrict__ perm,
                                                              const int32_t* __restrict__ list,
                                                              const unsigned* __restrict__ list_count,
                                                              int64_t nQ, WT* __restrict__ W) {
  const int64_t n = list ? (int64_t)*list_count : nQ;
  if (list && blockIdx.x * (int64_t)blockDim.x >= n) return;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < n;
  int64_t qi = 0;
  double qx = 0, qy = 0, qz = 0;
  if (valid) read_q(Q, perm, list, i, qi, qx, qy, qz);
  // every term through the warp's FP64 queue (see CloudNearQueue)
  __shared__ CloudNearQueue fp64_q[4];
  CloudNearQueue& fq = fp64_q[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  fq.q[lane][0] = qx;
  fq.q[lane][1] = qy;
  fq.q[lane][2] = qz;
  int nqueued = 0;    // warp-uniform
  unsigned mine = 0;  // this lane's queue positions
  double acc = 0.0;
  int resume = valid ? 0 : 0x7fffffff;
  int node = 0;
  const unsigned full = 0xffffffffu;
  while (node < prm.nnodes) {
    const CloudNodeD* r = prm.nd + node;
    const int4 l = r->l;
    const bool visit = node >= resume;
    bool open = false;
    if (l.w) {  // leaf (the node, hence the branch, is warp-uniform)
      queue_points64(prm, fq, nqueued, mine, visit ? l.z : 0, l.y, acc);
      if (visit) resume = l.x;
    } else if (node == 0) {
      open = visit;
    } else {
      bool want = false;
      if (visit) {
        if (far64(qx, qy, qz, r->cm, r->r, prm.beta)) {
          want = true;
          resume = l.x;
        } else {
          open = true;
        }
      }
      queue_cloud64(prm, fq, nqueued, mine, want, ~node, acc);
    }
    // a lane that opens the node wants node + 1, every other lane is past
    // the node (resume > node): the warp goes to the smallest of them
    node = __reduce_min_sync(full, open ? node + 1 : resume);
  }
  if (nqueued) flush_cloud64(prm, fq, nqueued, mine, acc);
  if (valid) W[qi] = (WT)acc;
}

// FP64 re-evaluation of the listed queries (results within the band of
// 0.5), one warp per query: the lanes share the query's walk (the listed
// queries lie anywhere on the surface, so a warp of 32 of them would walk
// the union of 32 walks); a leaf's dipoles are split over the lanes, a far
// cell's expansion is evaluated by one lane, and the lanes' sums are added
// at the end.
template <typename QT, typename WT>
__global__ void __launch_bounds__(128) cloud_refine_warp_kernel(CloudEvalParams prm,
                                                                const QT* __restrict__ Q,
                                                                const int32_t* __restrict__ list,
                                                                const unsigned* __restrict__ count,
                                                                WT* __restrict__ W) {
  const unsigned n = *count;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w < (int64_t)n;
       w += nwarps) {
    const int64_t qi = list[w];
    const double qx = (double)Q[qi * 3], qy = (double)Q[qi * 3 + 1], qz = (double)Q[qi * 3 + 2];
    double acc = 0.0;
    int node = 0;
    while (node < prm.nnodes) {
      const CloudNodeD* r = prm.nd + node;
      const int4 l = r->l;
      if (l.w) {
        for (int j = lane; j < l.z; j += 32) {
          const double* pd = prm.pd + ((int64_t)l.y + j) * 6;
          acc += dipole64(pd[0] - qx, pd[1] - qy, pd[2] - qz, pd[3], pd[4], pd[5]);
        }
        node = l.x;
      } else if (node == 0) {
        node = 1;
      } else if (far64(qx, qy, qz, r->cm, r->r, prm.beta)) {
        if (lane == 0) {
          const double lx = __dsub_rn(r->cm[0], qx), ly = __dsub_rn(r->cm[1], qy),
                       lz = __dsub_rn(r->cm[2], qz);
          acc += expansion_packed64(r->pk, lx, ly, lz, prm.num_terms);
        }
        node = l.x;
      } else {
        node = node + 1;
      }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) W[qi] = (WT)acc;
  }
}

// beta <= 0: direct sum over every point (:300-310).  FP64 plain, or FP32
// with FP64 near-field dipoles.
template <typename QT, typename WT, bool kMixed>
__global__ void __launch_bounds__(256) cloud_direct_kernel(const float4* __restrict__ pf,
                                                           const double* __restrict__ pd,
                                                           int64_t n, float eps, const QT* __restrict__ Q,
                                                           int64_t nQ, WT* __restrict__ W) {
  const int64_t qi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (qi >= nQ) return;
  const double qx = (double)Q[qi * 3], qy = (double)Q[qi * 3 + 1], qz = (double)Q[qi * 3 + 2];
  const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
  double acc64 = 0;
  float acc = 0;
  for (int64_t j = 0; j < n; ++j) {
    if (kMixed) {
      const float4 p = __ldg(&pf[j * 2]);
      const float lx = p.x - fx, ly = p.y - fy, lz = p.z - fz;
      const float r2 = fmaf(lz, lz, fmaf(ly, ly, lx * lx));
      if (r2 <= p.w) {
        const double* d = pd + j * 6;
        acc64 += dipole64(d[0] - qx, d[1] - qy, d[2] - qz, d[3], d[4], d[5]);
      } else {
        const float4 an = __ldg(&pf[j * 2 + 1]);
        const float ir = rsqrtf(r2);
        acc += fmaf(lx, an.x, fmaf(ly, an.y, lz * an.z)) * (ir * ir * ir * kInvPi4F);
      }
    } else {
      const double* d = pd + j * 6;
      acc64 += dipole64(d[0] - qx, d[1] - qy, d[2] - qz, d[3], d[4], d[5]);
    }
  }
  W[qi] = (WT)((double)acc + acc64);
}

template <typename WT>
__global__ void fill_zero(WT* w, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) w[i] = WT(0);
}

// Precompute CM/R/EC for every cell of a CSR view.
void precompute(gwn_cloud_impl& c, const CsrView& v, int64_t ncells, const double* P,
                const double* N, const double* A, cudaStream_t st) {
  c.CM.alloc((size_t)std::max<int64_t>(ncells, 1) * 3);
  c.R.alloc((size_t)std::max<int64_t>(ncells, 1));
  c.EC.alloc((size_t)std::max<int64_t>(ncells, 1) * c.num_terms);
  c.area.alloc((size_t)std::max<int64_t>(ncells, 1));
  if (ncells == 0) return;
  // empty cells keep R = 0 and EC = 0; the kernels below write the others
  GWN_CUDA(cudaMemsetAsync(c.EC.get(), 0, c.EC.bytes(), st));
  GWN_CUDA(cudaMemsetAsync(c.R.get(), 0, c.R.bytes(), st));
  DevBuf<unsigned> nch((size_t)ncells, st), cbase((size_t)ncells, st);
  launch_kernel(chunk_count_kernel, blocks(ncells), 256, 0, st, v.count, ncells, nch.get());
  exclusive_scan_u32(nch.get(), cbase.get(), ncells, st);
  // the small cells' list, grouped by point count
  DevBuf<unsigned> hist(kSmallCell + 2, st);
  hist.zero(st);
  const unsigned list_blocks = (unsigned)((ncells + kListCells - 1) / kListCells);
  launch_kernel(small_hist_kernel, list_blocks, kListThreads, 0, st, v.count, ncells, hist.get());
  launch_kernel(small_offsets_kernel, 1, 1, 0, st, hist.get());
  unsigned* sizes_h = pinned_words();
  GWN_CUDA(cudaMemcpyAsync(sizes_h, nch.get() + ncells - 1, 4, cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaMemcpyAsync(sizes_h + 1, cbase.get() + ncells - 1, 4, cudaMemcpyDeviceToHost,
                           st));
  GWN_CUDA(cudaMemcpyAsync(sizes_h + 2, hist.get() + kSmallCell + 1, 4,
                           cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  const unsigned last_n = sizes_h[0], last_b = sizes_h[1], nsmall = sizes_h[2];
  DevBuf<int32_t> small((size_t)std::max<unsigned>(nsmall, 1u), st);
  if (nsmall)
    launch_kernel(small_scatter_kernel, list_blocks, kListThreads, 0, st, v.count, ncells,
                  hist.get(), small.get());
  const int64_t nchunks = (int64_t)last_n + last_b;
  DevBuf<int32_t> chunk_cell((size_t)std::max<int64_t>(nchunks, 1), st);
  launch_kernel(chunk_fill_kernel, blocks(ncells), 256, 0, st, nch.get(), cbase.get(), ncells, chunk_cell.get());
  DevBuf<double> part((size_t)std::max<int64_t>(nchunks, 1) * 37, st);
  if (nchunks)
    launch_kernel(pass1_kernel, blocks(nchunks * 32), 256, 0, st, v, chunk_cell.get(), cbase.get(), nchunks, P,
                                                      N, A, part.get());
  if (nchunks)
    launch_kernel(combine1_kernel, blocks(nchunks * 32), 256, 0, st, (const int32_t*)chunk_cell.get(),
                  (const unsigned*)cbase.get(), (const unsigned*)nch.get(), nchunks,
                  (const double*)part.get(), c.num_terms, c.CM.get(), c.EC.get(), c.area.get());
  launch_kernel(empty_cells_kernel, blocks(ncells), 256, 0, st, v.count, ncells, c.CM.get(),
                c.area.get());
  GWN_CUDA(cudaGetLastError());
  if (nchunks) {
    if (c.num_terms == 39)
      launch_kernel(pass2_kernel<39>, blocks(nchunks * 32), 256, 0, st, v, chunk_cell.get(), cbase.get(),
                                                            nchunks, P, N, A, c.CM.get(), part.get());
    else if (c.num_terms == 12)
      launch_kernel(pass2_kernel<12>, blocks(nchunks * 32), 256, 0, st, v, chunk_cell.get(), cbase.get(),
                                                            nchunks, P, N, A, c.CM.get(), part.get());
    else
      launch_kernel(pass2_kernel<3>, blocks(nchunks * 32), 256, 0, st, v, chunk_cell.get(), cbase.get(),
                                                           nchunks, P, N, A, c.CM.get(), part.get());
  }
  if (nchunks)
    launch_kernel(combine2_kernel, blocks(nchunks * 32), 256, 0, st, (const int32_t*)chunk_cell.get(),
                  (const unsigned*)cbase.get(), (const unsigned*)nch.get(), nchunks,
                  (const double*)part.get(), c.num_terms, c.R.get(), c.EC.get());
  if (nsmall) {
    const int32_t* sl = small.get();
    if (c.num_terms == 39)
      launch_kernel(small_cells_kernel<39>, blocks(nsmall, 128), 128, 0, st, v, sl, (int64_t)nsmall,
                    P, N, A, c.CM.get(), c.R.get(), c.EC.get(), c.area.get());
    else if (c.num_terms == 12)
      launch_kernel(small_cells_kernel<12>, blocks(nsmall, 128), 128, 0, st, v, sl, (int64_t)nsmall,
                    P, N, A, c.CM.get(), c.R.get(), c.EC.get(), c.area.get());
    else
      launch_kernel(small_cells_kernel<3>, blocks(nsmall, 128), 128, 0, st, v, sl, (int64_t)nsmall,
                    P, N, A, c.CM.get(), c.R.get(), c.EC.get(), c.area.get());
  }
}

__global__ void count_nonempty_kernel(const int32_t* __restrict__ count, int64_t n,
                                      unsigned long long* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool ne = i < n && count[i] > 0;
  const unsigned b = __ballot_sync(0xffffffffu, ne);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, (unsigned long long)__popc(b));
}

__global__ void bbox3_kernel(const double* __restrict__ P, int64_t n,
                             unsigned long long* __restrict__ mm) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) {
      const double v = P[i * 3 + d];
      if (isfinite(v)) {
        lo[d] = fmin(lo[d], v);
        hi[d] = fmax(hi[d], v);
      }
    }
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
    if ((threadIdx.x & 31) == 0 && lo[d] <= hi[d]) {
      atomicMin(&mm[d], ordered_bits(lo[d]));
      atomicMax(&mm[3 + d], ordered_bits(hi[d]));
    }
  }
}

void points_bbox(const double* P, int64_t n, double lo[3], double hi[3], cudaStream_t st) {
  DevBuf<unsigned long long> mm(6, st);
  init_minmax(mm.get(), 3, st);
  if (n) launch_kernel(bbox3_kernel, std::min<unsigned>(blocks(n), 1024u), 256, 0, st, P, n, mm.get());
  unsigned long long h[6];
  GWN_CUDA(cudaMemcpyAsync(h, mm.get(), sizeof(h), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  for (int d = 0; d < 3; ++d) {
    lo[d] = n ? from_ordered_bits(h[d]) : 0.0;
    hi[d] = n ? from_ordered_bits(h[3 + d]) : 0.0;
    if (!(lo[d] <= hi[d])) lo[d] = hi[d] = 0.0;
  }
}

void finish_extent(gwn_cloud_impl& c, cudaStream_t st) {
  points_bbox(c.P.get(), c.n, c.lo, c.hi, st);
  double diag2 = 0, cmax = 0;
  for (int d = 0; d < 3; ++d) {
    diag2 += (c.hi[d] - c.lo[d]) * (c.hi[d] - c.lo[d]);
    cmax = std::max(cmax, std::max(std::fabs(c.lo[d]), std::fabs(c.hi[d])));
  }
  c.eps = kNearFrac * std::sqrt(diag2);
  c.cmax = cmax;
  c.bytes = c.CM.bytes() + c.R.bytes() + c.EC.bytes() + c.area.bytes() + c.P.bytes() + c.AN.bytes();
}

}  // namespace

void cloud_build(gwn_cloud_impl& c, const gwn_octree_impl& t, const double* N, const double* A,
                 int order, cudaStream_t st) {
  GWN_REQUIRE(order >= 0 && order <= 2, "expansion order must be 0, 1 or 2");
  c.order = order;
  c.num_terms = order == 0 ? 3 : (order == 1 ? 12 : 39);
  c.n = t.n;
  c.ncells = t.ncells;
  const int64_t n = t.n, ncells = t.ncells;
  c.P.alloc((size_t)std::max<int64_t>(n, 1) * 3);
  c.AN.alloc((size_t)std::max<int64_t>(n, 1) * 3);
  if (n) {
    GWN_CUDA(cudaMemcpyAsync(c.P.get(), t.P.get(), (size_t)n * 3 * 8, cudaMemcpyDeviceToDevice, st));
    launch_kernel(an_kernel, blocks(n), 256, 0, st, N, A, n, c.AN.get());
  }
  CsrView v{t.start.get(), t.count.get(), t.perm.get()};
  precompute(c, v, ncells, c.P.get(), N, A, st);
  // traversal order of non-empty cells
  DevBuf<unsigned long long> key((size_t)ncells, st), key_tmp((size_t)ncells, st);
  DevBuf<int32_t> val((size_t)ncells, st), val_tmp((size_t)ncells, st);
  launch_kernel(nonempty_keys_kernel, blocks(ncells), 256, 0, st, t.start.get(), t.count.get(), t.depth.get(),
                                                       ncells, key.get(), val.get());
  radix_sort_pairs<unsigned long long>(key.get(), val.get(), key_tmp.get(), val_tmp.get(), ncells, 0,
                                       48, st);
  int64_t nnodes = 0;
  {
    DevBuf<unsigned long long> cnt(1, st);
    cnt.zero(st);
    launch_kernel(count_nonempty_kernel, blocks(ncells), 256, 0, st, t.count.get(), ncells, cnt.get());
    unsigned long long h = 0;
    GWN_CUDA(cudaMemcpyAsync(&h, cnt.get(), 8, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    nnodes = (int64_t)h;
  }
  c.nnodes = nnodes;
  c.nf.alloc((size_t)std::max<int64_t>(nnodes, 1));
  // the walk reads records with 256-bit loads
  if (reinterpret_cast<uintptr_t>(c.nf.get()) % 32)
    throw Error(GWN_ERR_INTERNAL, "cloud records are not 32-byte aligned");
  c.nd.alloc((size_t)std::max<int64_t>(nnodes, 1));
  finish_extent(c, st);
  LayoutIn in{val.get(), nullptr, nullptr, key.get(), nnodes, t.start.get(), t.count.get(), t.ch.get(),
              t.depth.get(), c.CM.get(), c.R.get(), c.EC.get(), c.num_terms, c.area.get(), c.eps,
              c.cmax};
  if (nnodes) launch_kernel(emit_nodes_kernel, blocks(nnodes), 256, 0, st, in, c.nf.get(), c.nd.get());
  c.pf.alloc((size_t)std::max<int64_t>(n, 1) * 2);
  c.pd.alloc((size_t)std::max<int64_t>(n, 1) * 6);
  if (n)
    launch_kernel(emit_points_kernel, blocks(n), 256, 0, st, t.perm.get(), n, c.P.get(), c.AN.get(),
                  c.eps, c.cmax, c.pf.get(), c.pd.get());
  c.bytes += c.nf.bytes() + c.nd.bytes() + c.pf.bytes() + c.pd.bytes();
}


// Drop-in form: caller CSR lists and CH (host copies for the pre-order walk
// of the tree, device copies for the kernels).
__global__ void csr_count_kernel(const int64_t* __restrict__ off, int64_t n,
                                 int32_t* __restrict__ cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = (int32_t)(off[i + 1] - off[i]);
}

void cloud_build_arrays(gwn_cloud_impl& c, const double* P, const double* N, const double* A,
                        int64_t nP, const int64_t* pi_off_d, const int32_t* pi_idx_d,
                        const int32_t* CH_d, int64_t ncells, int order, bool compute_moments,
                        const int64_t* pi_off_h, const int32_t* pi_idx_h, const int32_t* CH_h,
                        cudaStream_t st) {
  GWN_REQUIRE(order >= 0 && order <= 2, "expansion order must be 0, 1 or 2");
  GWN_REQUIRE(ncells >= 1, "the octree needs at least the root cell");
  c.order = order;
  c.num_terms = order == 0 ? 3 : (order == 1 ? 12 : 39);
  c.n = nP;
  c.ncells = ncells;
  c.P.alloc((size_t)std::max<int64_t>(nP, 1) * 3);
  c.AN.alloc((size_t)std::max<int64_t>(nP, 1) * 3);
  if (nP) {
    GWN_CUDA(cudaMemcpyAsync(c.P.get(), P, (size_t)nP * 24, cudaMemcpyDeviceToDevice, st));
    launch_kernel(an_kernel, blocks(nP), 256, 0, st, N, A, nP, c.AN.get());
  }
  DevBuf<int32_t> cnt((size_t)ncells, st);
  launch_kernel(csr_count_kernel, blocks(ncells), 256, 0, st, pi_off_d, ncells, cnt.get());
  // the moments are computed even when the caller supplies CM/R/EC: the
  // per-cell areas set the FP64 near-field radii of the walk
  (void)compute_moments;
  {
    CsrView v{pi_off_d, cnt.get(), pi_idx_d};
    precompute(c, v, ncells, c.P.get(), N, A, st);
  }
  if (!pi_off_h) return;
  finish_extent(c, st);
  // depth-first pre-order of the non-empty cells (children in octant order,
  // as the reference's recursion visits them) with subtree ends and leaf slots
  std::vector<int32_t> order_h, first_h;
  std::vector<int64_t> skip_h;
  std::vector<int32_t> slot_point;
  order_h.reserve((size_t)ncells);
  struct Fr { int32_t cell; int64_t pos; int child; };
  std::vector<Fr> stack;
  auto nonempty = [&](int32_t x) { return pi_off_h[x + 1] > pi_off_h[x]; };
  auto push_node = [&](int32_t x) {
    const int64_t pos = (int64_t)order_h.size();
    order_h.push_back(x);
    skip_h.push_back(0);
    const bool leaf = CH_h[(int64_t)x * 8] == -1;
    first_h.push_back(leaf ? (int32_t)slot_point.size() : 0);
    if (leaf)
      for (int64_t j = pi_off_h[x]; j < pi_off_h[x + 1]; ++j) slot_point.push_back(pi_idx_h[j]);
    stack.push_back({x, pos, leaf ? 8 : 0});
  };
  push_node(0);
  while (!stack.empty()) {
    Fr& f = stack.back();
    if (f.child >= 8) {
      skip_h[(size_t)f.pos] = (int64_t)order_h.size();
      stack.pop_back();
      continue;
    }
    const int32_t ch = CH_h[(int64_t)f.cell * 8 + f.child];
    ++f.child;
    GWN_REQUIRE(ch > 0 && ch < ncells, "CH holds a child id out of range");
    if (nonempty(ch)) {
      GWN_REQUIRE((int64_t)order_h.size() < ncells, "CH does not describe a tree");
      push_node(ch);
    }
  }
  const int64_t nnodes = (int64_t)order_h.size();
  c.nnodes = nnodes;
  DevBuf<int32_t> order_d((size_t)nnodes, st), first_d((size_t)nnodes, st);
  DevBuf<int64_t> skip_d((size_t)nnodes, st);
  order_d.upload(order_h.data(), (size_t)nnodes, st);
  first_d.upload(first_h.data(), (size_t)nnodes, st);
  skip_d.upload(skip_h.data(), (size_t)nnodes, st);
  const int64_t nslots = (int64_t)slot_point.size();
  DevBuf<int32_t> slot_d((size_t)std::max<int64_t>(nslots, 1), st);
  slot_d.upload(slot_point.data(), (size_t)nslots, st);
  for (int32_t sp : slot_point) GWN_REQUIRE(sp >= 0 && sp < nP, "point index out of range");
  c.nf.alloc((size_t)std::max<int64_t>(nnodes, 1));
  // the walk reads records with 256-bit loads
  if (reinterpret_cast<uintptr_t>(c.nf.get()) % 32)
    throw Error(GWN_ERR_INTERNAL, "cloud records are not 32-byte aligned");
  c.nd.alloc((size_t)std::max<int64_t>(nnodes, 1));
  DevBuf<int64_t> start_d((size_t)ncells, st);
  GWN_CUDA(cudaMemcpyAsync(start_d.get(), pi_off_d, (size_t)ncells * 8, cudaMemcpyDeviceToDevice, st));
  c.pf.alloc((size_t)std::max<int64_t>(nslots, 1) * 2);
  c.pd.alloc((size_t)std::max<int64_t>(nslots, 1) * 6);
  if (nslots)
    launch_kernel(emit_points_kernel, blocks(nslots), 256, 0, st, slot_d.get(), nslots, c.P.get(),
                  c.AN.get(), c.eps, c.cmax, c.pf.get(), c.pd.get());
  // node records need CM/R/EC: emitted by cloud_emit_arrays once moments exist
  c.layout_order = std::move(order_d);
  c.layout_first = std::move(first_d);
  c.layout_skip = std::move(skip_d);
  c.layout_start = std::move(start_d);
  c.layout_count = std::move(cnt);
  c.layout_ch = CH_d;
  GWN_CUDA(cudaStreamSynchronize(st));  // host vectors outlive their uploads
}

void cloud_emit_arrays(gwn_cloud_impl& c, cudaStream_t st) {
  LayoutIn in{c.layout_order.get(), c.layout_first.get(), c.layout_skip.get(), nullptr, c.nnodes,
              c.layout_start.get(), c.layout_count.get(), c.layout_ch, nullptr, c.CM.get(),
              c.R.get(), c.EC.get(), c.num_terms, c.area.get(), c.eps, c.cmax};
  if (c.nnodes) launch_kernel(emit_nodes_kernel, blocks(c.nnodes), 256, 0, st, in, c.nf.get(), c.nd.get());
  GWN_CUDA(cudaGetLastError());
}

void cloud_set_moments(gwn_cloud_impl& c, const double* CM, const double* R, const double* EC,
                       cudaStream_t st) {
  c.CM.alloc((size_t)std::max<int64_t>(c.ncells, 1) * 3);
  c.R.alloc((size_t)std::max<int64_t>(c.ncells, 1));
  c.EC.alloc((size_t)std::max<int64_t>(c.ncells, 1) * c.num_terms);
  GWN_CUDA(cudaMemcpyAsync(c.CM.get(), CM, (size_t)c.ncells * 24, cudaMemcpyDeviceToDevice, st));
  GWN_CUDA(cudaMemcpyAsync(c.R.get(), R, (size_t)c.ncells * 8, cudaMemcpyDeviceToDevice, st));
  GWN_CUDA(cudaMemcpyAsync(c.EC.get(), EC, (size_t)c.ncells * c.num_terms * 8,
                           cudaMemcpyDeviceToDevice, st));
}

template <typename QT, typename WT>
static void cloud_eval_t(const gwn_cloud_impl& c, double beta, const void* Qv, int64_t nQ, void* Wv,
                         int precision, cudaStream_t st) {
  const QT* Q = static_cast<const QT*>(Qv);
  WT* W = static_cast<WT*>(Wv);
  if (nQ == 0) return;
  if (c.n == 0 || c.nnodes == 0) {
    launch_kernel(fill_zero<WT>, blocks(nQ), 256, 0, st, W, nQ);
    GWN_CUDA(cudaGetLastError());
    return;
  }
  if (!(beta > 0)) {
    if (precision == GWN_MIXED)
      launch_kernel(cloud_direct_kernel<QT, WT, true>, blocks(nQ), 256, 0, st, c.pf.get(), c.pd.get(), c.n,
                                                                   (float)c.eps, Q, nQ, W);
    else
      launch_kernel(cloud_direct_kernel<QT, WT, false>, blocks(nQ), 256, 0, st, c.pf.get(), c.pd.get(), c.n,
                                                                    (float)c.eps, Q, nQ, W);
    GWN_CUDA(cudaGetLastError());
    return;
  }
  CloudEvalParams prm;
  prm.nf = c.nf.get();
  prm.nd = c.nd.get();
  prm.pf = c.pf.get();
  prm.pd = c.pd.get();
  prm.nnodes = (int)c.nnodes;
  prm.num_terms = c.num_terms;
  prm.beta = beta;
  prm.beta_f = (float)beta;
  prm.eps = (float)c.eps;
  prm.cmax = (float)c.cmax;
  QueryOrder qo;
  {
    PhaseTimer ph("order_queries", st);
    order_queries(Qv, sizeof(QT) == 8 ? GWN_F64 : GWN_F32, nQ, c.lo, c.hi, qo, st);
  }
  const int32_t* perm = qo.active ? qo.perm.get() : nullptr;
  const unsigned grid = blocks(nQ, 128);
  if (precision == GWN_MIXED) {
    DevBuf<int32_t> list((size_t)nQ, st);
    DevBuf<unsigned> count(1, st);
    count.zero(st);
    {
      PhaseTimer ph("walk", st);
      launch_kernel(cloud_eval_mixed_kernel<QT, WT>, grid, 128, 0, st, prm, Q, perm, nQ, W, list.get(),
                                                            count.get());
    }
    GWN_CUDA(cudaGetLastError());
    {
      PhaseTimer ph("refine", st);
      launch_kernel(cloud_refine_warp_kernel<QT, WT>, (unsigned)(num_sms() * 8), 128, 0, st, prm,
                    Q, (const int32_t*)list.get(), (const unsigned*)count.get(), W);
    }
    GWN_CUDA(cudaGetLastError());
  } else {
    PhaseTimer ph("walk", st);
    launch_kernel(cloud_eval_fp64_kernel<QT, WT>, grid, 128, 0, st, prm, Q, perm, nullptr, nullptr, nQ, W);
    GWN_CUDA(cudaGetLastError());
  }
}

void cloud_eval(const gwn_cloud_impl& c, double beta, const void* Q, int q_dtype, int64_t nQ,
                void* W, int w_dtype, int precision, cudaStream_t st) {
  const bool qd = q_dtype == GWN_F64, wd = w_dtype == GWN_F64;
  if (qd && wd) cloud_eval_t<double, double>(c, beta, Q, nQ, W, precision, st);
  else if (qd) cloud_eval_t<double, float>(c, beta, Q, nQ, W, precision, st);
  else if (wd) cloud_eval_t<float, double>(c, beta, Q, nQ, W, precision, st);
  else cloud_eval_t<float, float>(c, beta, Q, nQ, W, precision, st);
}

}  // namespace gwn
