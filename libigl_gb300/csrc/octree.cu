// GPU octree build, bit-exact with igl::octree (include/igl/octree.cpp:5-170).
//
// Reference semantics restated: the root cube is the points' AABB (centre =
// (min+max)/2, width = largest extent, :142-153); a cell with more than one
// point and depth < 30000 (:16, :98) gets 8 children whose centres are
// parent + (+-h/2 per axis), h = width/2 (:59-81, :104-113, octant bits x=1,
// y=2, z=4 from `>=` against the parent centre, :32-53); every cell's point
// list is the parent's list filtered in order (:117-122), so lists are
// ascending; child ids are m..m+7 handed out when a cell is visited in
// depth-first pre-order (:100-131).
//
// Device algorithm:
//  * level by level, the points of the cells being split form one array of
//    (segment, point) entries in segment order; the octant of each point is
//    found with the same FP64 `>=` tests, and a stable radix sort on
//    segment*8+octant performs every cell's stable partition at once; child
//    cells are emitted with the same FP64 centre recurrence;
//  * a cell whose points can never separate again (all identical, or a
//    centre that no longer moves in FP64 with all points in one octant)
//    would recurse to depth 30000 one octant at a time: such chains are
//    emitted by one thread each instead of one level per launch;
//  * ids: the i-th internal cell in depth-first pre-order owns ids
//    1+8i..8+8i.  Internal cells of different depths nest and cells of one
//    depth have disjoint point ranges, so pre-order is the order of
//    (first point position, depth); one sort of that key gives every rank.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "gwn_common.cuh"
#include "octree.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

constexpr int kMaxDepth = 30000;

// Creation-order cell records (SoA).
struct Cells {
  DevBuf<double> c;       // 3 per cell
  DevBuf<double> w;
  DevBuf<int64_t> start;
  DevBuf<int32_t> count;
  DevBuf<int32_t> depth;
  DevBuf<int32_t> parent;
  DevBuf<int32_t> oct;
  int64_t size = 0, cap = 0;

  template <typename T>
  static void grow(DevBuf<T>& b, size_t old_n, size_t new_n, cudaStream_t st) {
    DevBuf<T> nb(new_n, st);
    if (old_n)
      GWN_CUDA(cudaMemcpyAsync(nb.get(), b.get(), old_n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    b = std::move(nb);
  }
  void reserve(int64_t need, cudaStream_t st) {
    if (need <= cap) return;
    int64_t nc = std::max<int64_t>(need, cap * 2 + 64);
    grow(c, (size_t)size * 3, (size_t)nc * 3, st);
    grow(w, (size_t)size, (size_t)nc, st);
    grow(start, (size_t)size, (size_t)nc, st);
    grow(count, (size_t)size, (size_t)nc, st);
    grow(depth, (size_t)size, (size_t)nc, st);
    grow(parent, (size_t)size, (size_t)nc, st);
    grow(oct, (size_t)size, (size_t)nc, st);
    cap = nc;
  }
};

__global__ void root_kernel(const unsigned long long* __restrict__ mm, int64_t n, double* c,
                            double* w, int64_t* start, int32_t* count, int32_t* depth,
                            int32_t* parent, int32_t* oct) {
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = n > 0 ? from_ordered_bits(mm[d]) : 0.0;
    hi[d] = n > 0 ? from_ordered_bits(mm[3 + d]) : 0.0;
  }
  for (int d = 0; d < 3; ++d) c[d] = (lo[d] + hi[d]) / 2.0;
  double width = hi[0] - lo[0];
  for (int d = 1; d < 3; ++d) {
    const double e = hi[d] - lo[d];
    if (e > width) width = e;
  }
  *w = width;
  *start = 0;
  *count = (int32_t)n;
  *depth = 0;
  *parent = -1;
  *oct = 0;
}

// min/max over all points (NaN coordinates take part as in a plain compare
// loop: they never win a min/max).
__global__ void point_bbox_kernel(const double* __restrict__ P, int64_t n,
                                  unsigned long long* __restrict__ mm) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) {
      const double v = P[i * 3 + d];
      lo[d] = fmin(lo[d], v);
      hi[d] = fmax(hi[d], v);
    }
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&mm[d], ordered_bits(lo[d]));
      atomicMax(&mm[3 + d], ordered_bits(hi[d]));
    }
  }
}

__global__ void iota_kernel(int32_t* a, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = (int32_t)i;
}

__global__ void fill_i32_kernel(int32_t* a, int64_t n, int32_t v) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// Octant of every active entry against its segment's centre; flags whether a
// segment's points occupy one octant only and whether they are all equal.
__global__ void octant_kernel(const double* __restrict__ P, const int32_t* __restrict__ act_pt,
                              const int32_t* __restrict__ act_seg, int64_t M,
                              const int32_t* __restrict__ seg_cell,
                              const int32_t* __restrict__ seg_first,
                              const double* __restrict__ cc, unsigned* __restrict__ key,
                              unsigned* __restrict__ seg_mask, unsigned* __restrict__ seg_diff) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= M) return;
  const int k = act_seg[m];
  const int cell = seg_cell[k];
  const int32_t p = act_pt[m];
  const double px = P[(int64_t)p * 3], py = P[(int64_t)p * 3 + 1], pz = P[(int64_t)p * 3 + 2];
  int o = 0;
  if (px >= cc[(int64_t)cell * 3 + 0]) o += 1;
  if (py >= cc[(int64_t)cell * 3 + 1]) o += 2;
  if (pz >= cc[(int64_t)cell * 3 + 2]) o += 4;
  key[m] = (unsigned)k * 8u + (unsigned)o;
  // All points of a segment hit the same two words: read first and skip the
  // atomic once the bit is set (at the top levels millions of points share
  // one segment, and same-address atomics serialize).
  const unsigned bit = 1u << o;
  if ((*(volatile unsigned*)&seg_mask[k] & bit) == 0u) atomicOr(&seg_mask[k], bit);
  const int32_t f = act_pt[seg_first[k]];
  if ((px != P[(int64_t)f * 3] || py != P[(int64_t)f * 3 + 1] || pz != P[(int64_t)f * 3 + 2]) &&
      *(volatile unsigned*)&seg_diff[k] == 0u)
    atomicOr(&seg_diff[k], 1u);
}

// Points per child from the sorted keys: each run of equal keys adds its end
// and subtracts its start (two uncontended atomics per run; child_count is
// zero on entry).
__global__ void child_count_kernel(const unsigned* __restrict__ key, int64_t M,
                                   unsigned* __restrict__ child_count) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= M) return;
  const unsigned k = key[m];
  if (m == 0 || key[m - 1] != k) atomicSub(&child_count[k], (unsigned)m);
  if (m == M - 1 || key[m + 1] != k) atomicAdd(&child_count[k], (unsigned)(m + 1));
}

// Whether the FP64 centre recurrence can no longer move `c` on any axis:
// c + w/4 and c - w/4 both round back to c.
__device__ __forceinline__ bool centre_stuck(const double* c, double w) {
  const double q = __dmul_rn(__dmul_rn(w, 0.5), 0.5);
  for (int d = 0; d < 3; ++d)
    if (__dadd_rn(c[d], q) != c[d] || __dadd_rn(c[d], -q) != c[d]) return false;
  return true;
}

// Emit the 8 children of every segment (thread per (segment, octant)).
// child_state: 0 = leaf, 1 = active next level, 2 = chain.
__global__ void emit_children_kernel(int K, const int32_t* __restrict__ seg_cell,
                                     const int64_t* __restrict__ seg_pstart,
                                     const unsigned* __restrict__ seg_mask,
                                     const unsigned* __restrict__ seg_diff,
                                     const unsigned* __restrict__ child_count, int64_t base,
                                     double* cc, double* cw, int64_t* cstart, int32_t* ccount,
                                     int32_t* cdepth, int32_t* cparent, int32_t* coct,
                                     unsigned* __restrict__ child_state) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)K * 8) return;
  const int k = (int)(t >> 3), o = (int)(t & 7);
  const int cell = seg_cell[k];
  const double pc[3] = {cc[(int64_t)cell * 3], cc[(int64_t)cell * 3 + 1], cc[(int64_t)cell * 3 + 2]};
  const double h = __dmul_rn(cw[cell], 0.5);
  const double hh = __dmul_rn(h, 0.5);
  int64_t s = seg_pstart[k];
  for (int j = 0; j < o; ++j) s += child_count[(int64_t)k * 8 + j];
  const unsigned cnt = child_count[t];
  const int64_t x = base + t;
  cc[x * 3 + 0] = __dadd_rn(pc[0], (o & 1) ? hh : -hh);
  cc[x * 3 + 1] = __dadd_rn(pc[1], (o == 2 || o == 3 || o == 6 || o == 7) ? hh : -hh);
  cc[x * 3 + 2] = __dadd_rn(pc[2], (o > 3) ? hh : -hh);
  cw[x] = h;
  cstart[x] = s;
  ccount[x] = (int32_t)cnt;
  const int d = cdepth[cell] + 1;
  cdepth[x] = d;
  cparent[x] = cell;
  coct[x] = o;
  unsigned state = 0;
  if (cnt > 1 && d < kMaxDepth) {
    const bool one_octant = __popc(seg_mask[k]) == 1;
    const bool chain = one_octant && (seg_diff[k] == 0 || centre_stuck(pc, cw[cell]));
    state = chain ? 2u : 1u;
  }
  child_state[t] = state;
}

// Scatter the sorted entries of this level into perm and compact the entries
// of children that stay active into the next level's arrays.
__global__ void advance_kernel(const int32_t* __restrict__ pt_sorted,
                               const unsigned* __restrict__ key_sorted, int64_t M,
                               const int32_t* __restrict__ seg_first,
                               const int64_t* __restrict__ seg_pstart,
                               const unsigned* __restrict__ child_state,
                               const unsigned* __restrict__ child_newseg,
                               const unsigned* __restrict__ entry_pos, int32_t* __restrict__ perm,
                               int32_t* __restrict__ next_pt, int32_t* __restrict__ next_seg) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= M) return;
  const unsigned key = key_sorted[m];
  const int k = (int)(key >> 3);
  const int32_t p = pt_sorted[m];
  perm[seg_pstart[k] + (m - seg_first[k])] = p;
  if (child_state[key] == 1u) {
    const unsigned pos = entry_pos[m];
    next_pt[pos] = p;
    next_seg[pos] = (int32_t)child_newseg[key];
  }
}

__global__ void entry_flag_kernel(const unsigned* __restrict__ key_sorted, int64_t M,
                                  const unsigned* __restrict__ child_state,
                                  unsigned* __restrict__ flag) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m < M) flag[m] = child_state[key_sorted[m]] == 1u ? 1u : 0u;
}

__global__ void state_flag_kernel(const unsigned* __restrict__ child_state, int64_t n, unsigned v,
                                  unsigned* __restrict__ flag) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) flag[i] = child_state[i] == v ? 1u : 0u;
}

// The level's totals in one word array, read by the host with one copy:
// {last child state, new segments before the last child, chains before it,
//  last entry's flag, entries before it}.
__global__ void level_totals_kernel(const unsigned* __restrict__ child_state,
                                    const unsigned* __restrict__ child_newseg,
                                    const unsigned* __restrict__ child_chainslot, int64_t K8,
                                    const unsigned* __restrict__ eflag,
                                    const unsigned* __restrict__ epos, int64_t M,
                                    unsigned* __restrict__ out) {
  out[0] = child_state[K8 - 1];
  out[1] = child_newseg[K8 - 1];
  out[2] = child_chainslot[K8 - 1];
  out[3] = eflag[M - 1];
  out[4] = epos[M - 1];
}

// Next level's segment table and the chain list.
__global__ void next_segments_kernel(int64_t K8, const unsigned* __restrict__ child_state,
                                     const unsigned* __restrict__ child_newseg,
                                     const unsigned* __restrict__ child_chainslot,
                                     const unsigned* __restrict__ entry_pos_of_child,
                                     int64_t base, const int64_t* __restrict__ cstart,
                                     const int32_t* __restrict__ ccount,
                                     int32_t* __restrict__ nseg_cell,
                                     int32_t* __restrict__ nseg_first,
                                     int64_t* __restrict__ nseg_pstart,
                                     int32_t* __restrict__ chain_cell) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= K8) return;
  const unsigned s = child_state[t];
  if (s == 1u) {
    const unsigned j = child_newseg[t];
    nseg_cell[j] = (int32_t)(base + t);
    nseg_first[j] = (int32_t)entry_pos_of_child[t];
    nseg_pstart[j] = cstart[base + t];
  } else if (s == 2u) {
    chain_cell[child_chainslot[t]] = (int32_t)(base + t);
  }
}

// First entry position (in the next level's compacted array) of each active
// child: the number of active entries before it = exclusive scan of the
// active children's counts.
__global__ void active_count_kernel(const unsigned* __restrict__ child_state,
                                    const unsigned* __restrict__ child_count, int64_t K8,
                                    unsigned* __restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < K8) out[t] = child_state[t] == 1u ? child_count[t] : 0u;
}

// One thread per chain: the cell's points share one octant at every deeper
// level; emit 8 children per level down to depth 30000.
__global__ void chain_kernel(const double* __restrict__ P, const int32_t* __restrict__ perm,
                             const int32_t* __restrict__ chain_cell, int nchains,
                             const int64_t* __restrict__ chain_base, double* cc, double* cw,
                             int64_t* cstart, int32_t* ccount, int32_t* cdepth, int32_t* cparent,
                             int32_t* coct) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nchains) return;
  int64_t cur = chain_cell[i];
  const int64_t s = cstart[cur];
  const int32_t cnt = ccount[cur];
  const int32_t rep = perm[s];
  const double px = P[(int64_t)rep * 3], py = P[(int64_t)rep * 3 + 1], pz = P[(int64_t)rep * 3 + 2];
  double c[3] = {cc[cur * 3], cc[cur * 3 + 1], cc[cur * 3 + 2]};
  double w = cw[cur];
  int d = cdepth[cur];
  int64_t x = chain_base[i];
  while (d < kMaxDepth) {
    int o = 0;
    if (px >= c[0]) o += 1;
    if (py >= c[1]) o += 2;
    if (pz >= c[2]) o += 4;
    const double h = __dmul_rn(w, 0.5);
    const double hh = __dmul_rn(h, 0.5);
    int64_t next = -1;
    for (int j = 0; j < 8; ++j, ++x) {
      cc[x * 3 + 0] = __dadd_rn(c[0], (j & 1) ? hh : -hh);
      cc[x * 3 + 1] = __dadd_rn(c[1], (j == 2 || j == 3 || j == 6 || j == 7) ? hh : -hh);
      cc[x * 3 + 2] = __dadd_rn(c[2], (j > 3) ? hh : -hh);
      cw[x] = h;
      cstart[x] = s;
      ccount[x] = j == o ? cnt : 0;
      cdepth[x] = d + 1;
      cparent[x] = (int32_t)cur;
      coct[x] = j;
      if (j == o) next = x;
    }
    cur = next;
    c[0] = cc[cur * 3];
    c[1] = cc[cur * 3 + 1];
    c[2] = cc[cur * 3 + 2];
    w = h;
    ++d;
  }
}

__global__ void internal_keys_kernel(const int64_t* __restrict__ cstart,
                                     const int32_t* __restrict__ ccount,
                                     const int32_t* __restrict__ cdepth, int64_t ncells,
                                     unsigned long long* __restrict__ key, int32_t* __restrict__ val,
                                     unsigned* __restrict__ is_internal) {
  const int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (x >= ncells) return;
  const bool internal = ccount[x] > 1 && cdepth[x] < kMaxDepth;
  is_internal[x] = internal ? 1u : 0u;
  // non-internal cells sort after every internal one
  key[x] = internal ? (((unsigned long long)cstart[x] << 15) | (unsigned long long)cdepth[x])
                    : ((1ull << 48) - 1);
  val[x] = (int32_t)x;
}

__global__ void rank_kernel(const int32_t* __restrict__ sorted_cell, int64_t ninternal,
                            int32_t* __restrict__ rank) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < ninternal) rank[sorted_cell[r]] = (int32_t)r;
}

__global__ void final_layout_kernel(int64_t ncells, const double* __restrict__ cc,
                                    const double* __restrict__ cw,
                                    const int64_t* __restrict__ cstart,
                                    const int32_t* __restrict__ ccount,
                                    const int32_t* __restrict__ cdepth,
                                    const int32_t* __restrict__ cparent,
                                    const int32_t* __restrict__ coct,
                                    const int32_t* __restrict__ rank, double* __restrict__ cn,
                                    double* __restrict__ w, int32_t* __restrict__ ch,
                                    int64_t* __restrict__ start, int32_t* __restrict__ count,
                                    int32_t* __restrict__ depth) {
  const int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (x >= ncells) return;
  const int32_t par = cparent[x];
  const int64_t id = par < 0 ? 0 : 1 + 8 * (int64_t)rank[par] + coct[x];
  for (int d = 0; d < 3; ++d) cn[id * 3 + d] = cc[x * 3 + d];
  w[id] = cw[x];
  start[id] = cstart[x];
  count[id] = ccount[x];
  depth[id] = cdepth[x];
  const bool internal = ccount[x] > 1 && cdepth[x] < kMaxDepth;
  for (int j = 0; j < 8; ++j) ch[id * 8 + j] = internal ? (int32_t)(1 + 8 * (int64_t)rank[x] + j) : -1;
}

// Gather each cell's point range into the CSR index array (warp per cell),
// with a (cell id, point id) sort key: a cell's range in perm is ordered by
// octant path, the reference's lists are ascending (octree.cpp:117-122).
__global__ void csr_gather_kernel(const int64_t* __restrict__ off, const int64_t* __restrict__ start,
                                  const int32_t* __restrict__ count, const int32_t* __restrict__ perm,
                                  int64_t ncells, int32_t* __restrict__ idx,
                                  unsigned long long* __restrict__ key) {
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncells) return;
  const int64_t o = off[warp], s = start[warp];
  const int32_t c = count[warp];
  for (int32_t j = lane; j < c; j += 32) {
    const int32_t p = perm[s + j];
    idx[o + j] = p;
    key[o + j] = ((unsigned long long)warp << 30) | (unsigned long long)p;
  }
}

// 64-bit exclusive scan of per-cell counts (block-partials, recursive).
__global__ void scan64_partials(const int32_t* __restrict__ cnt, int64_t n,
                                int64_t* __restrict__ part) {
  __shared__ int64_t s[1024];
  const int64_t base = blockIdx.x * 4096LL;
  int64_t v = 0;
  for (int k = 0; k < 4; ++k) {
    const int64_t i = base + threadIdx.x * 4 + k;
    if (i < n) v += cnt[i];
  }
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = 512; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void scan64_tiles(const int32_t* __restrict__ cnt, int64_t n,
                             const int64_t* __restrict__ part_off, int64_t* __restrict__ off) {
  __shared__ int64_t s[1024];
  const int64_t base = blockIdx.x * 4096LL;
  int64_t v[4], t = 0;
  for (int k = 0; k < 4; ++k) {
    const int64_t i = base + threadIdx.x * 4 + k;
    v[k] = i < n ? cnt[i] : 0;
    t += v[k];
  }
  s[threadIdx.x] = t;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int64_t a = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
    __syncthreads();
    s[threadIdx.x] += a;
    __syncthreads();
  }
  int64_t run = s[threadIdx.x] - t + (part_off ? part_off[blockIdx.x] : 0);
  for (int k = 0; k < 4; ++k) {
    const int64_t i = base + threadIdx.x * 4 + k;
    if (i < n) off[i] = run;
    run += v[k];
  }
  if (base + 4096 >= n && threadIdx.x == 1023) off[n] = run;
}

void exclusive_scan_counts64(const int32_t* cnt, int64_t n, int64_t* off, cudaStream_t st) {
  const int64_t nb = (n + 4095) / 4096;
  if (nb <= 1) {
    launch_kernel(scan64_tiles, 1, 1024, 0, st, cnt, n, nullptr, off);
    GWN_CUDA(cudaGetLastError());
    return;
  }
  DevBuf<int64_t> part((size_t)nb, st), part_off((size_t)nb + 1, st);
  launch_kernel(scan64_partials, (unsigned)nb, 1024, 0, st, cnt, n, part.get());
  // partials are few (<= 2^20 for 2^32 cells); scan them on the host
  std::vector<int64_t> h((size_t)nb), ho((size_t)nb + 1);
  GWN_CUDA(cudaMemcpyAsync(h.data(), part.get(), (size_t)nb * sizeof(int64_t),
                           cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  ho[0] = 0;
  for (int64_t i = 0; i < nb; ++i) ho[(size_t)i + 1] = ho[(size_t)i] + h[(size_t)i];
  GWN_CUDA(cudaMemcpyAsync(part_off.get(), ho.data(), ((size_t)nb + 1) * sizeof(int64_t),
                           cudaMemcpyHostToDevice, st));
  launch_kernel(scan64_tiles, (unsigned)nb, 1024, 0, st, cnt, n, part_off.get(), off);
  GWN_CUDA(cudaGetLastError());
  GWN_CUDA(cudaStreamSynchronize(st));  // ho must outlive the copy
}

inline unsigned blocks(int64_t n, int t = 256) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

int bits_for(uint64_t maxval) {
  int b = 1;
  while (b < 64 && (maxval >> b)) ++b;
  return b;
}

}  // namespace

void octree_build(gwn_octree_impl& t, const double* P, int64_t n, bool host_mode, cudaStream_t st) {
  (void)host_mode;
  GWN_REQUIRE(n <= (int64_t(1) << 29), "at most 2^29 points");
  t.n = n;
  t.P.alloc((size_t)std::max<int64_t>(n, 1) * 3);
  if (n)
    GWN_CUDA(cudaMemcpyAsync(t.P.get(), P, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  const double* dP = t.P.get();
  Cells cells;
  cells.reserve(std::max<int64_t>(64, 9 + n / 2), st);
  DevBuf<unsigned long long> mm(6, st);
  init_minmax(mm.get(), 3, st);
  if (n > 0) {
    launch_kernel(point_bbox_kernel, std::min<unsigned>(blocks(n), 1024u), 256, 0, st, dP, n, mm.get());
    GWN_CUDA(cudaGetLastError());
  }
  launch_kernel(root_kernel, 1, 1, 0, st, mm.get(), n, cells.c.get(), cells.w.get(), cells.start.get(),
                               cells.count.get(), cells.depth.get(), cells.parent.get(),
                               cells.oct.get());
  GWN_CUDA(cudaGetLastError());
  cells.size = 1;
  DevBuf<int32_t> perm((size_t)std::max<int64_t>(n, 1), st);
  launch_kernel(iota_kernel, blocks(n), 256, 0, st, perm.get(), n);

  // level state
  int64_t M = n >= 2 ? n : 0;  // active entries
  int K = n >= 2 ? 1 : 0;      // active segments
  DevBuf<int32_t> act_pt((size_t)std::max<int64_t>(M, 1), st), act_seg((size_t)std::max<int64_t>(M, 1), st);
  DevBuf<int32_t> seg_cell(1, st), seg_first(1, st);
  DevBuf<int64_t> seg_pstart(1, st);
  if (K) {
    launch_kernel(iota_kernel, blocks(M), 256, 0, st, act_pt.get(), M);
    launch_kernel(fill_i32_kernel, blocks(M), 256, 0, st, act_seg.get(), M, 0);
    launch_kernel(fill_i32_kernel, 1, 32, 0, st, seg_cell.get(), 1, 0);
    launch_kernel(fill_i32_kernel, 1, 32, 0, st, seg_first.get(), 1, 0);
    GWN_CUDA(cudaMemsetAsync(seg_pstart.get(), 0, sizeof(int64_t), st));
  }
  bool had_chain = false;
  int levels = 0;
  DevBuf<unsigned> totals_d(8, st);
  unsigned* totals_h = pinned_words();
  while (K > 0) {
    ++levels;
    const int64_t K8 = (int64_t)K * 8;
    DevBuf<unsigned> key((size_t)M, st), key_tmp((size_t)M, st);
    DevBuf<int32_t> pt_tmp((size_t)M, st);
    DevBuf<unsigned> seg_mask((size_t)K, st), seg_diff((size_t)K, st), child_count((size_t)K8, st);
    seg_mask.zero(st);
    seg_diff.zero(st);
    child_count.zero(st);
    launch_kernel(octant_kernel, blocks(M), 256, 0, st, dP, act_pt.get(), act_seg.get(), M, seg_cell.get(),
                                             seg_first.get(), cells.c.get(), key.get(),
                                             seg_mask.get(), seg_diff.get());
    GWN_CUDA(cudaGetLastError());
    radix_sort_pairs<uint32_t>(key.get(), act_pt.get(), key_tmp.get(), pt_tmp.get(), M, 0,
                               bits_for((uint64_t)K8 - 1), st);
    launch_kernel(child_count_kernel, blocks(M), 256, 0, st, key.get(), M, child_count.get());
    cells.reserve(cells.size + K8, st);
    const int64_t base = cells.size;
    DevBuf<unsigned> child_state((size_t)K8, st);
    launch_kernel(emit_children_kernel, blocks(K8), 256, 0, st, 
        K, seg_cell.get(), seg_pstart.get(), seg_mask.get(), seg_diff.get(), child_count.get(), base,
        cells.c.get(), cells.w.get(), cells.start.get(), cells.count.get(), cells.depth.get(),
        cells.parent.get(), cells.oct.get(), child_state.get());
    GWN_CUDA(cudaGetLastError());
    cells.size += K8;
    // scans: new segment ids, chain slots, first entry of each active child,
    // compacted entry positions
    DevBuf<unsigned> child_newseg((size_t)K8, st), child_chainslot((size_t)K8, st),
        child_firstpos((size_t)K8, st), tmp((size_t)K8, st);
    launch_kernel(state_flag_kernel, blocks(K8), 256, 0, st, child_state.get(), K8, 1u, tmp.get());
    exclusive_scan_u32(tmp.get(), child_newseg.get(), K8, st);
    launch_kernel(state_flag_kernel, blocks(K8), 256, 0, st, child_state.get(), K8, 2u, tmp.get());
    exclusive_scan_u32(tmp.get(), child_chainslot.get(), K8, st);
    launch_kernel(active_count_kernel, blocks(K8), 256, 0, st, child_state.get(), child_count.get(), K8,
                                                    tmp.get());
    exclusive_scan_u32(tmp.get(), child_firstpos.get(), K8, st);
    DevBuf<unsigned> eflag((size_t)M, st), epos((size_t)M, st);
    launch_kernel(entry_flag_kernel, blocks(M), 256, 0, st, key.get(), M, child_state.get(), eflag.get());
    exclusive_scan_u32(eflag.get(), epos.get(), M, st);
    // totals: one small kernel and one copy into pinned memory per level
    launch_kernel(level_totals_kernel, 1, 1, 0, st, (const unsigned*)child_state.get(),
                  (const unsigned*)child_newseg.get(), (const unsigned*)child_chainslot.get(), K8,
                  (const unsigned*)eflag.get(), (const unsigned*)epos.get(), M, totals_d.get());
    GWN_CUDA(cudaMemcpyAsync(totals_h, totals_d.get(), 5 * sizeof(unsigned),
                             cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    const unsigned last_state = totals_h[0], last_newseg = totals_h[1],
                   last_chain = totals_h[2], last_eflag = totals_h[3],
                   last_epos = totals_h[4];
    const int nK = (int)(last_newseg + (last_state == 1u ? 1u : 0u));
    const int nChains = (int)(last_chain + (last_state == 2u ? 1u : 0u));
    const int64_t nM = (int64_t)last_epos + last_eflag;
    DevBuf<int32_t> next_pt((size_t)std::max<int64_t>(nM, 1), st),
        next_seg((size_t)std::max<int64_t>(nM, 1), st);
    launch_kernel(advance_kernel, blocks(M), 256, 0, st, act_pt.get(), key.get(), M, seg_first.get(),
                                              seg_pstart.get(), child_state.get(),
                                              child_newseg.get(), epos.get(), perm.get(),
                                              next_pt.get(), next_seg.get());
    GWN_CUDA(cudaGetLastError());
    DevBuf<int32_t> nseg_cell((size_t)std::max(nK, 1), st), nseg_first((size_t)std::max(nK, 1), st);
    DevBuf<int64_t> nseg_pstart((size_t)std::max(nK, 1), st);
    DevBuf<int32_t> chain_cell((size_t)std::max(nChains, 1), st);
    launch_kernel(next_segments_kernel, blocks(K8), 256, 0, st, 
        K8, child_state.get(), child_newseg.get(), child_chainslot.get(), child_firstpos.get(), base,
        cells.start.get(), cells.count.get(), nseg_cell.get(), nseg_first.get(), nseg_pstart.get(),
        chain_cell.get());
    GWN_CUDA(cudaGetLastError());
    if (nChains > 0) {
      had_chain = true;
      std::vector<int32_t> cc_h((size_t)nChains), cd_h((size_t)nChains);
      GWN_CUDA(cudaMemcpyAsync(cc_h.data(), chain_cell.get(), (size_t)nChains * 4,
                               cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
      // depth of each chain head: all chains created at this level have the same depth
      int32_t dh = 0;
      GWN_CUDA(cudaMemcpy(&dh, cells.depth.get() + cc_h[0], 4, cudaMemcpyDeviceToHost));
      const int64_t per = 8LL * (kMaxDepth - dh);
      std::vector<int64_t> cb((size_t)nChains);
      for (int i = 0; i < nChains; ++i) cb[(size_t)i] = cells.size + per * i;
      cells.reserve(cells.size + per * nChains, st);
      DevBuf<int64_t> chain_base((size_t)nChains, st);
      chain_base.upload(cb.data(), (size_t)nChains, st);
      launch_kernel(chain_kernel, blocks(nChains, 64), 64, 0, st, 
          dP, perm.get(), chain_cell.get(), nChains, chain_base.get(), cells.c.get(), cells.w.get(),
          cells.start.get(), cells.count.get(), cells.depth.get(), cells.parent.get(),
          cells.oct.get());
      GWN_CUDA(cudaGetLastError());
      GWN_CUDA(cudaStreamSynchronize(st));  // cb outlives its copy
      cells.size += per * nChains;
    }
    act_pt = std::move(next_pt);
    act_seg = std::move(next_seg);
    seg_cell = std::move(nseg_cell);
    seg_first = std::move(nseg_first);
    seg_pstart = std::move(nseg_pstart);
    M = nM;
    K = nK;
  }
  // ids
  const int64_t ncells = cells.size;
  GWN_REQUIRE(ncells < (int64_t(1) << 31), "octree has more than 2^31 cells");
  DevBuf<unsigned long long> ikey((size_t)ncells, st), ikey_tmp((size_t)ncells, st);
  DevBuf<int32_t> ival((size_t)ncells, st), ival_tmp((size_t)ncells, st);
  DevBuf<unsigned> is_internal((size_t)ncells, st);
  launch_kernel(internal_keys_kernel, blocks(ncells), 256, 0, st, cells.start.get(), cells.count.get(),
                                                       cells.depth.get(), ncells, ikey.get(),
                                                       ival.get(), is_internal.get());
  GWN_CUDA(cudaGetLastError());
  radix_sort_pairs<unsigned long long>(ikey.get(), ival.get(), ikey_tmp.get(), ival_tmp.get(),
                                       ncells, 0, 48, st);
  const int64_t ninternal = (ncells - 1) / 8;
  DevBuf<int32_t> rank((size_t)ncells, st);
  if (ninternal > 0)
    launch_kernel(rank_kernel, blocks(ninternal), 256, 0, st, ival.get(), ninternal, rank.get());
  t.ncells = ncells;
  t.cn.alloc((size_t)ncells * 3);
  t.w.alloc((size_t)ncells);
  t.ch.alloc((size_t)ncells * 8);
  t.start.alloc((size_t)ncells);
  t.count.alloc((size_t)ncells);
  t.depth.alloc((size_t)ncells);
  launch_kernel(final_layout_kernel, blocks(ncells), 256, 0, st, 
      ncells, cells.c.get(), cells.w.get(), cells.start.get(), cells.count.get(), cells.depth.get(),
      cells.parent.get(), cells.oct.get(), rank.get(), t.cn.get(), t.w.get(), t.ch.get(),
      t.start.get(), t.count.get(), t.depth.get());
  GWN_CUDA(cudaGetLastError());
  t.perm.alloc((size_t)std::max<int64_t>(n, 1));
  if (n)
    GWN_CUDA(cudaMemcpyAsync(t.perm.get(), perm.get(), (size_t)n * 4, cudaMemcpyDeviceToDevice, st));
  // total index count
  DevBuf<int64_t> off((size_t)ncells + 1, st);
  exclusive_scan_counts64(t.count.get(), ncells, off.get(), st);
  GWN_CUDA(cudaMemcpyAsync(&t.nindices, off.get() + ncells, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  // deepest cell: a chain reaches 30000, otherwise one level per iteration
  t.max_depth = had_chain ? kMaxDepth : levels;
}

void octree_export_csr(const gwn_octree_impl& t, int64_t* pi_offsets, int32_t* pi_indices,
                       cudaStream_t st) {
  exclusive_scan_counts64(t.count.get(), t.ncells, pi_offsets, st);
  if (pi_indices && t.nindices > 0) {
    GWN_REQUIRE(t.nindices < (int64_t(1) << 32), "point lists exceed 2^32 entries");
    const int64_t threads = t.ncells * 32;
    DevBuf<unsigned long long> key((size_t)t.nindices, st), key_tmp((size_t)t.nindices, st);
    DevBuf<int32_t> tmp((size_t)t.nindices, st);
    launch_kernel(csr_gather_kernel, blocks(threads), 256, 0, st, pi_offsets, t.start.get(), t.count.get(),
                                                       t.perm.get(), t.ncells, pi_indices,
                                                       key.get());
    GWN_CUDA(cudaGetLastError());
    // entries are already grouped by cell; sort by the full key to order
    // every cell's points ascending
    radix_sort_pairs<unsigned long long>(key.get(), pi_indices, key_tmp.get(), tmp.get(),
                                         t.nindices, 0, 30 + bits_for((uint64_t)t.ncells), st);
  }
}

}  // namespace gwn
