// k nearest points through the octree (igl::knn).
//
// Reference: include/igl/knn.cpp:24-136.  For every query row of P the k
// points of V nearest to it, nearest first; when #V <= k every point, sorted
// (:41-51).  The reference runs a best-first search over the octree of V with
// one priority queue of cells and points; the result does not depend on the
// search, only on the distances (the norm of V.row(j) - p, :86-90) -- and, for
// equal distances, on the queue's order, which the reference leaves to
// std::priority_queue.  Here equal distances are ordered by point index (the
// reference's own test, tests/include/igl/knn.cpp:35-41, has such a tie and
// expects that order).  As in the reference (:121-125, "leaves either have
// one point, or none"), a leaf contributes only the first point of its list:
// duplicates beyond the first (which no octree can separate) are never
// returned, and a row may then hold fewer than k points (the rest is -1,
// where the reference's loop would run past its empty queue).  When #V <= k
// every point is returned, duplicates included (:41-51).
//
// One thread per query searches the octree of V depth-first, nearer child
// first (children ordered by the FP32 distance to their box, rounded outward,
// minus a slack covering the query's FP32 rounding), skipping empty cells and
// cells whose lower bound exceeds the k-th distance so far, with the k best
// (distance, index) pairs in a max-heap; point distances are FP64 with the
// operations pinned.  For k above kKnnMaxK, or a query whose search stack
// would overflow (an octree much deeper than any dense cloud gives), a plain
// scan of all points per query is used instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "bh_common.cuh"
#include "gwn_common.cuh"
#include "gwn_internal.cuh"
#include "octree.cuh"

namespace gwn {
namespace {

constexpr int kKnnMaxK = 64;
constexpr int kKnnStack = 192;

struct KnnTree {
  const float4* box;  // per cell: {lo.xyz, count}, {hi.xyz, 0}, FP32 rounded outward
  const int32_t* ch;
  const int64_t* start;
  const int32_t* count;
  const int32_t* perm;
  const double* P;
  int64_t n;
  float cmax;
};

__device__ __forceinline__ double point_dist(const double* __restrict__ P, int32_t j, double qx,
                                             double qy, double qz) {
  const double dx = __dsub_rn(P[(int64_t)j * 3], qx), dy = __dsub_rn(P[(int64_t)j * 3 + 1], qy),
               dz = __dsub_rn(P[(int64_t)j * 3 + 2], qz);
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// (d, i) before (e, j) in the result order
__device__ __forceinline__ bool before(double d, int32_t i, double e, int32_t j) {
  return d < e || (d == e && i < j);
}

// Max-heap of the best k (root = the worst kept pair).
struct Heap {
  double* d;
  int32_t* i;
  int n, k;
  __device__ void offer(double dd, int32_t ii) {
    if (n < k) {
      int c = n++;
      while (c > 0) {  // sift up
        const int p = (c - 1) >> 1;
        if (!before(d[p], i[p], dd, ii)) break;
        d[c] = d[p];
        i[c] = i[p];
        c = p;
      }
      d[c] = dd;
      i[c] = ii;
      return;
    }
    if (!before(dd, ii, d[0], i[0])) return;
    int c = 0;
    for (;;) {  // sift down
      const int l = 2 * c + 1, r = l + 1;
      int m = c;
      double md = dd;
      int32_t mi = ii;
      if (l < n && before(md, mi, d[l], i[l])) {
        m = l;
        md = d[l];
        mi = i[l];
      }
      if (r < n && before(md, mi, d[r], i[r])) m = r;
      if (m == c) break;
      d[c] = d[m];
      i[c] = i[m];
      c = m;
    }
    d[c] = dd;
    i[c] = ii;
  }
  // ascending (d, i) into out
  __device__ void write_sorted(int32_t* out) {
    // heap sort in place: repeatedly move the root (max) to the end
    for (int end = n - 1; end > 0; --end) {
      const double td = d[0];
      const int32_t ti = i[0];
      d[0] = d[end];
      i[0] = i[end];
      d[end] = td;
      i[end] = ti;
      int c = 0;
      for (;;) {
        const int l = 2 * c + 1, r = l + 1;
        int m = c;
        if (l < end && before(d[m], i[m], d[l], i[l])) m = l;
        if (r < end && before(d[m], i[m], d[r], i[r])) m = r;
        if (m == c) break;
        const double sd = d[c];
        const int32_t si = i[c];
        d[c] = d[m];
        i[c] = i[m];
        d[m] = sd;
        i[m] = si;
        c = m;
      }
    }
    for (int j = 0; j < n; ++j) out[j] = i[j];
    for (int j = n; j < k; ++j) out[j] = -1;
  }
};

// Cell boxes for the search: the cube (centre cn, width w) rounded outward
// to FP32, and the cell's point count.
__global__ void cell_boxes_kernel(const double* __restrict__ cn, const double* __restrict__ w,
                                  const int32_t* __restrict__ count, int64_t ncells,
                                  float4* __restrict__ box) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const double h = 0.5 * w[c];
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    const double cc = cn[c * 3 + a];
    lo[a] = __double2float_rd(cc - h);
    hi[a] = __double2float_ru(cc + h);
  }
  box[2 * c] = make_float4(lo[0], lo[1], lo[2], __int_as_float(count[c]));
  box[2 * c + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
}

// FP32 lower bound of the distance from q to a cell's box; minus 1e-6 (S + d)
// for the query's rounding.
__device__ __forceinline__ float cell_lower_bound(float4 lo, float4 hi, float fx, float fy,
                                                  float fz, float S) {
  const float ex = fmaxf(fmaxf(lo.x - fx, fx - hi.x), 0.f);
  const float ey = fmaxf(fmaxf(lo.y - fy, fy - hi.y), 0.f);
  const float ez = fmaxf(fmaxf(lo.z - fz, fz - hi.z), 0.f);
  const float d = sqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex)));
  return fmaxf(d - 1e-6f * (S + d), 0.f);
}

// KMAX: the heap's capacity (k <= KMAX), so that small k keep a small
// per-thread frame in local memory.
template <typename QT, int KMAX>
__global__ void __launch_bounds__(128) knn_octree_kernel(KnnTree t, const QT* __restrict__ Q,
                                                         int64_t nQ,
                                                         const int32_t* __restrict__ perm, int k,
                                                         int32_t* __restrict__ I,
                                                         int32_t* __restrict__ overflow,
                                                         unsigned* __restrict__ n_overflow) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nQ) return;
  const int64_t q = perm ? (int64_t)perm[i] : i;
  const double qx = (double)Q[q * 3], qy = (double)Q[q * 3 + 1], qz = (double)Q[q * 3 + 2];
  const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
  const float S = fmaxf(fabsf(fx), fmaxf(fabsf(fy), fabsf(fz))) + t.cmax;
  double hd[KMAX];
  int32_t hi[KMAX];
  Heap heap{hd, hi, 0, k};
  // FP32 upper bound of the k-th distance once the heap is full (pruning
  // only what is strictly farther)
  float kbound = INFINITY;
  // the stack holds cells only: a popped cell's bound is computed again from
  // its box (the same value as when it was pushed), which keeps the
  // thread's frame in local memory small
  int stk[kKnnStack];
  int sp = 0;
  stk[sp++] = 0;  // the root, bound 0
  while (sp > 0) {
    const int c = stk[--sp];
    if (c != 0) {
      const float lb = cell_lower_bound(__ldg(&t.box[2 * (int64_t)c]),
                                        __ldg(&t.box[2 * (int64_t)c + 1]), fx, fy, fz, S);
      if (lb > kbound) continue;
    }
    if (t.ch[(int64_t)c * 8] < 0) {  // leaf: its first point (knn.cpp:121-125)
      const int32_t p = t.perm[t.start[c]];
      heap.offer(point_dist(t.P, p, qx, qy, qz), p);
      if (heap.n == k) kbound = __double2float_ru(heap.d[0]);
      continue;
    }
    int cc[8];
    float cl[8];
    int m = 0;
    for (int o = 0; o < 8; ++o) {
      const int x = t.ch[(int64_t)c * 8 + o];
      const float4 blo = __ldg(&t.box[2 * (int64_t)x]);
      if (__float_as_int(blo.w) == 0) continue;  // empty cell
      const float l = cell_lower_bound(blo, __ldg(&t.box[2 * (int64_t)x + 1]), fx, fy, fz, S);
      if (l > kbound) continue;
      int j = m++;  // insertion by descending bound: the nearest ends up last (popped first)
      while (j > 0 && cl[j - 1] < l) {
        cc[j] = cc[j - 1];
        cl[j] = cl[j - 1];
        --j;
      }
      cc[j] = x;
      cl[j] = l;
    }
    if (sp + m > kKnnStack) {  // too deep for the stack: scanned separately
      overflow[atomicAdd(n_overflow, 1u)] = (int32_t)q;
      return;
    }
    for (int j = 0; j < m; ++j) stk[sp++] = cc[j];
  }
  heap.write_sorted(I + q * k);
}

// Every point against query `q` (listed queries, or all when list is null),
// heap in scratch (k pairs per thread).
// `rep` (optional): only points flagged 1 take part (the first point of each
// leaf, as the octree search sees them).
template <typename QT>
__global__ void knn_scan_kernel(const double* __restrict__ P, int64_t n, const QT* __restrict__ Q,
                                int64_t nQ, const int32_t* __restrict__ list,
                                const unsigned* __restrict__ n_list, int k,
                                const unsigned char* __restrict__ rep,
                                double* __restrict__ sd, int32_t* __restrict__ si,
                                int32_t* __restrict__ I) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t cnt = list ? (int64_t)*n_list : nQ;
  if (t >= cnt) return;
  const int64_t q = list ? (int64_t)list[t] : t;
  const double qx = (double)Q[q * 3], qy = (double)Q[q * 3 + 1], qz = (double)Q[q * 3 + 2];
  Heap heap{sd + t * (int64_t)k, si + t * (int64_t)k, 0, k};
  for (int64_t j = 0; j < n; ++j)
    if (!rep || rep[j]) heap.offer(point_dist(P, (int32_t)j, qx, qy, qz), (int32_t)j);
  heap.write_sorted(I + q * k);
}

// rep[p] = 1 for the first point of every non-empty leaf (rep zeroed first).
__global__ void leaf_first_kernel(const int32_t* __restrict__ ch, const int64_t* __restrict__ start,
                                  const int32_t* __restrict__ count,
                                  const int32_t* __restrict__ perm, int64_t ncells,
                                  unsigned char* __restrict__ rep) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells || ch[c * 8] >= 0 || count[c] == 0) return;
  rep[perm[start[c]]] = 1;
}

__global__ void max_abs_kernel(const double* __restrict__ P, int64_t n,
                               unsigned long long* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double m = 0;
  if (i < n) m = fmax(fabs(P[i * 3]), fmax(fabs(P[i * 3 + 1]), fabs(P[i * 3 + 2])));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

}  // namespace

int64_t knn_columns(int64_t n, int64_t k) { return std::min<int64_t>(n, k); }

template <typename QT>
static void knn_t(const gwn_octree_impl& tree, const QT* Q, int64_t nQ, int64_t k, int32_t* I,
                  cudaStream_t st) {
  const int64_t kk = knn_columns(tree.n, k);
  if (nQ == 0 || kk == 0) return;
  // scratch heaps for the scan path, in batches of at most 256 MB
  const int64_t batch = std::max<int64_t>(1, std::min<int64_t>(nQ, (int64_t(256) << 20) / (12 * kk)));
  // the octree search's point set: first points of the leaves (#V > k)
  DevBuf<unsigned char> rep;
  if (tree.n > k) {
    rep.alloc((size_t)tree.n, st);
    rep.zero(st);
    launch_kernel(leaf_first_kernel, (unsigned)((tree.ncells + 255) / 256), 256, 0, st,
                  (const int32_t*)tree.ch.get(), (const int64_t*)tree.start.get(),
                  (const int32_t*)tree.count.get(), (const int32_t*)tree.perm.get(), tree.ncells,
                  rep.get());
  }
  if (kk > kKnnMaxK || tree.n <= k) {  // scan (every point when #V <= k)
    DevBuf<double> sd((size_t)(batch * kk), st);
    DevBuf<int32_t> si((size_t)(batch * kk), st);
    for (int64_t b = 0; b < nQ; b += batch) {
      const int64_t m = std::min(batch, nQ - b);
      launch_kernel(knn_scan_kernel<QT>, (unsigned)((m + 127) / 128), 128, 0, st,
                    (const double*)tree.P.get(), tree.n, Q + b * 3, m, (const int32_t*)nullptr,
                    (const unsigned*)nullptr, (int)kk, (const unsigned char*)rep.get(), sd.get(),
                    si.get(), I + b * kk);
    }
    return;
  }
  DevBuf<unsigned long long> mx(1, st);
  mx.zero(st);
  launch_kernel(max_abs_kernel, (unsigned)((tree.n + 255) / 256), 256, 0, st,
                (const double*)tree.P.get(), tree.n, mx.get());
  unsigned long long mxh = 0;
  GWN_CUDA(cudaMemcpyAsync(&mxh, mx.get(), 8, cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  double cmax;
  std::memcpy(&cmax, &mxh, 8);
  DevBuf<float4> box((size_t)tree.ncells * 2, st);
  launch_kernel(cell_boxes_kernel, (unsigned)((tree.ncells + 255) / 256), 256, 0, st,
                (const double*)tree.cn.get(), (const double*)tree.w.get(),
                (const int32_t*)tree.count.get(), tree.ncells, box.get());
  KnnTree t{box.get(), tree.ch.get(), tree.start.get(), tree.count.get(), tree.perm.get(),
            tree.P.get(), tree.n, (float)cmax};
  // queries grouped by Morton cell of the root cube, so neighbouring threads
  // walk the same cells
  double root[4];
  GWN_CUDA(cudaMemcpyAsync(root, tree.cn.get(), 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaMemcpyAsync(root + 3, tree.w.get(), sizeof(double), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  const double lo[3] = {root[0] - 0.5 * root[3], root[1] - 0.5 * root[3], root[2] - 0.5 * root[3]};
  const double hi[3] = {root[0] + 0.5 * root[3], root[1] + 0.5 * root[3], root[2] + 0.5 * root[3]};
  QueryOrder qo;
  order_queries(Q, std::is_same<QT, double>::value ? GWN_F64 : GWN_F32, nQ, lo, hi, qo, st);
  DevBuf<int32_t> over((size_t)nQ, st);
  DevBuf<unsigned> nover(1, st);
  nover.zero(st);
  const int32_t* qperm = qo.active ? qo.perm.get() : nullptr;
  const unsigned grid = (unsigned)((nQ + 127) / 128);
  if (kk <= 16)
    launch_kernel(knn_octree_kernel<QT, 16>, grid, 128, 0, st, t, Q, nQ, qperm, (int)kk, I,
                  over.get(), nover.get());
  else if (kk <= 32)
    launch_kernel(knn_octree_kernel<QT, 32>, grid, 128, 0, st, t, Q, nQ, qperm, (int)kk, I,
                  over.get(), nover.get());
  else
    launch_kernel(knn_octree_kernel<QT, kKnnMaxK>, grid, 128, 0, st, t, Q, nQ, qperm, (int)kk, I,
                  over.get(), nover.get());
  unsigned no = 0;
  GWN_CUDA(cudaMemcpyAsync(&no, nover.get(), 4, cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  if (no == 0) return;
  // overflowed queries: scan, in batches of the scratch size
  const int64_t b2 = std::min<int64_t>(batch, no);
  DevBuf<double> sd((size_t)(b2 * kk), st);
  DevBuf<int32_t> si((size_t)(b2 * kk), st);
  for (int64_t b = 0; b < (int64_t)no; b += b2) {
    const unsigned m = (unsigned)std::min<int64_t>(b2, (int64_t)no - b);
    DevBuf<unsigned> nm(1, st);
    GWN_CUDA(cudaMemcpyAsync(nm.get(), &m, 4, cudaMemcpyHostToDevice, st));
    launch_kernel(knn_scan_kernel<QT>, (unsigned)((m + 127) / 128), 128, 0, st,
                  (const double*)tree.P.get(), tree.n, Q, nQ, (const int32_t*)over.get() + b,
                  (const unsigned*)nm.get(), (int)kk, (const unsigned char*)rep.get(), sd.get(),
                  si.get(), I);
    GWN_CUDA(cudaStreamSynchronize(st));  // m lives on this frame
  }
}

void octree_knn(const gwn_octree_impl& tree, const void* Q, int q_dtype, int64_t nQ, int64_t k,
                int32_t* I, cudaStream_t st) {
  if (q_dtype == GWN_F64) knn_t(tree, static_cast<const double*>(Q), nQ, k, I, st);
  else knn_t(tree, static_cast<const float*>(Q), nQ, k, I, st);
}

}  // namespace gwn
