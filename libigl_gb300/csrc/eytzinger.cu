// 2-D winding numbers over an Eytzinger AABB tree of segments:
//   igl::eytzinger_aabb                      include/igl/eytzinger_aabb.cpp:16-100
//   igl::eytzinger_aabb_winding_number_tree  include/igl/eytzinger_aabb_winding_number_tree.cpp:17-118
//   igl::eytzinger_aabb_winding_number       include/igl/eytzinger_aabb_winding_number.cpp:9-125
//
// Build.  The reference splits recursively at the median box centre along
// the longest axis.  Here the tree is built one level at a time over all
// nodes of the level: every node's primitives sit in a contiguous range of a
// list kept in the reference's list order (`cur`), and, per axis, in a second
// list sorted by that axis's centre (`A[a]`), so a node's median is read at
// the middle of its range instead of selected.  A split is a stable
// partition of both lists (scans), which keeps every child range sorted.
// Child sizes depend only on the parent's size (left n/2, right n - n/2: the
// reference's tie rule always balances), so ranges follow from m alone.
//
// Pair lists.  A vertex's net count over the segments under node r is the
// sum of +1 (segment start) / -1 (segment end) over its incident segments
// whose leaf lies under r.  Leaves are numbered by their position on the
// bottom level (each subtree covers a contiguous range), incidences are
// sorted by (vertex, position), and each (vertex, node) with a non-zero count
// is emitted once, by the first incidence of the vertex under the node.
// Records sorted by (node, sign, vertex) give each node's pairs: positive
// vertices ascending, paired in order with negative vertices ascending (the
// reference pairs in unordered_map order; any pairing gives the same sum).
//
// Evaluation.  One thread per query (grouped by Morton cell), a stackless
// walk of the implicit tree in the reference's visiting order (right child
// first); the mixed walk moves warp by warp.  FP64 form: the reference's
// arithmetic on the caller's arrays.  Mixed form: FP32
// boxes rounded outward (a box test may only say "outside" when the query is
// outside), segment / pair endpoints and the query as hi + lo FP32 pairs in a
// frame centred on the root box, FP32 angle summed with compensation; FP64
// only for a term whose FP32 angle may be off by 2 pi (query almost on the
// segment) or whose query sits on an endpoint, and again for a result within
// 1e-3 of 0.5.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "atan2f.cuh"
#include "gwn_internal.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

constexpr int kT = 256;
inline unsigned nblk(int64_t n, int t = kT) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

constexpr double kTwoPi = 6.283185307179586476925286766559;

int depth_of(int64_t m) {
  int d = 0;
  while ((int64_t(1) << d) < m) ++d;
  return d;
}

// ------------------------------------------------------------------ build --
// Range [s, s+n) at level d of the element at list position j; false when the
// element already sits in a leaf above level d.
__device__ __forceinline__ bool locate(int64_t j, int64_t m, int d, int64_t& node, int64_t& s,
                                       int64_t& n) {
  node = 0;
  s = 0;
  n = m;
  for (int t = 0; t < d; ++t) {
    if (n < 2) return false;
    const int64_t h = n >> 1;
    if (j < s + h) {
      node = 2 * node + 1;
      n = h;
    } else {
      node = 2 * node + 2;
      s += h;
      n -= h;
    }
  }
  return true;
}

// Range of slot i at level d; false for a slot with no node.
__device__ __forceinline__ bool node_range(int64_t i, int d, int64_t m, int64_t& s, int64_t& n) {
  const int64_t k = i + 1;
  s = 0;
  n = m;
  for (int t = d - 1; t >= 0; --t) {
    if (n < 2) return false;
    const int64_t h = n >> 1;
    if ((k >> t) & 1) {
      s += h;
      n -= h;
    } else {
      n = h;
    }
  }
  return n >= 1;
}

__global__ void init_tree_kernel(double* B1, double* B2, int32_t* leaf, int64_t nb, int dim) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nb) return;
  leaf[i] = -2;
  for (int a = 0; a < dim; ++a) B1[i * dim + a] = B2[i * dim + a] = __longlong_as_double(0x7ff8000000000000ll);
}

__global__ void centres_kernel(const double* __restrict__ PB1, const double* __restrict__ PB2,
                               int64_t m, int dim, double* __restrict__ PBC) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= m * dim) return;
  PBC[i] = (PB1[i] + PB2[i]) / 2;
}

__global__ void axis_keys_kernel(const double* __restrict__ PBC, int64_t m, int dim, int a,
                                 unsigned long long* __restrict__ key, int32_t* __restrict__ val) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  key[i] = ordered_bits(PBC[i * dim + a] + 0.0);  // -0 and +0 compare equal
  val[i] = (int32_t)i;
}

__global__ void iota_kernel(int32_t* p, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = (int32_t)i;
}

__global__ void level_init_kernel(unsigned long long* B1b, unsigned long long* B2b, int64_t m,
                                  int d, int dim) {
  const int64_t base = (int64_t(1) << d) - 1;
  const int64_t i = base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 2 * base + 1) return;
  int64_t s, n;
  if (!node_range(i, d, m, s, n)) return;
  for (int a = 0; a < dim; ++a) {
    B1b[i * dim + a] = ordered_bits(INFINITY);
    B2b[i * dim + a] = ordered_bits(-INFINITY);
  }
}

// Node boxes of level d: warp-segmented min / max over consecutive list
// positions of the same node, one atomic per node and warp.
__global__ void level_box_kernel(const int32_t* __restrict__ cur, const double* __restrict__ PB1,
                                 const double* __restrict__ PB2, int64_t m, int dim, int d,
                                 unsigned long long* B1b, unsigned long long* B2b) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int64_t node = -1, s, n;
  if (j < m && !locate(j, m, d, node, s, n)) node = -1;
  const int64_t e = node >= 0 ? cur[j] : 0;
  const int64_t next = __shfl_down_sync(0xffffffffu, node, 1);
  const bool tail = lane == 31 || next != node;
  for (int a = 0; a < dim; ++a) {
    unsigned long long lo = node >= 0 ? ordered_bits(PB1[e * dim + a]) : ~0ull;
    unsigned long long hi = node >= 0 ? ordered_bits(PB2[e * dim + a]) : 0ull;
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long lo_o = __shfl_up_sync(0xffffffffu, lo, off);
      const unsigned long long hi_o = __shfl_up_sync(0xffffffffu, hi, off);
      const int64_t node_o = __shfl_up_sync(0xffffffffu, node, off);
      if (lane >= off && node_o == node) {
        lo = lo_o < lo ? lo_o : lo;
        hi = hi_o > hi ? hi_o : hi;
      }
    }
    if (tail && node >= 0) {
      atomicMin(&B1b[node * dim + a], lo);
      atomicMax(&B2b[node * dim + a], hi);
    }
  }
}

// Level d nodes: boxes back to doubles, leaf / internal, split axis and
// median (the reference's 0.5*(v[n/2] + v[n/2-1]) for an even count).
__global__ void level_finish_kernel(unsigned long long* B1b, unsigned long long* B2b,
                                    const int32_t* __restrict__ cur,
                                    const int32_t* __restrict__ A, const double* __restrict__ PBC,
                                    int64_t m, int dim, int d, int32_t* leaf,
                                    int8_t* __restrict__ ldir, double* __restrict__ lmed) {
  const int64_t base = (int64_t(1) << d) - 1;
  const int64_t i = base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 2 * base + 1) return;
  int64_t s, n;
  if (!node_range(i, d, m, s, n)) return;
  double lo[3], hi[3];
  for (int a = 0; a < dim; ++a) {
    lo[a] = from_ordered_bits(B1b[i * dim + a]);
    hi[a] = from_ordered_bits(B2b[i * dim + a]);
    reinterpret_cast<double*>(B1b)[i * dim + a] = lo[a];
    reinterpret_cast<double*>(B2b)[i * dim + a] = hi[a];
  }
  if (n == 1) {
    leaf[i] = cur[s];
    return;
  }
  leaf[i] = -1;
  int dir = 0;
  double best = hi[0] - lo[0];
  for (int a = 1; a < dim; ++a)
    if (hi[a] - lo[a] > best) {
      best = hi[a] - lo[a];
      dir = a;
    }
  const int32_t* Ad = A + (int64_t)dir * m;
  const double zh = PBC[(int64_t)Ad[s + n / 2] * dim + dir];
  double med = zh;
  if ((n & 1) == 0) med = 0.5 * (zh + PBC[(int64_t)Ad[s + n / 2 - 1] * dim + dir]);
  ldir[i - base] = (int8_t)dir;
  lmed[i - base] = med;
}

__global__ void level_classify_kernel(const int32_t* __restrict__ cur,
                                      const double* __restrict__ PBC, int64_t m, int dim, int d,
                                      const int8_t* __restrict__ ldir,
                                      const double* __restrict__ lmed, uint32_t* __restrict__ lt,
                                      uint32_t* __restrict__ eq) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j > m) return;
  uint32_t fl = 0, fe = 0;
  int64_t node, s, n;
  if (j < m && locate(j, m, d, node, s, n) && n >= 2) {
    const int64_t k = node - ((int64_t(1) << d) - 1);
    const double z = PBC[(int64_t)cur[j] * dim + ldir[k]];
    fl = z < lmed[k];
    fe = z == lmed[k];
  }
  lt[j] = fl;
  eq[j] = fe;
}

// Split of the reference list: below-median in order, then the equal ones
// (each to the smaller side, right on a tie) on the left; above-median in
// order, then the equal ones on the right.
__global__ void level_partition_kernel(const int32_t* __restrict__ cur, int64_t m, int d,
                                       const uint32_t* __restrict__ lt,
                                       const uint32_t* __restrict__ eq,
                                       int32_t* __restrict__ ncur, uint8_t* __restrict__ side) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int32_t e = cur[j];
  int64_t node, s, n;
  if (!locate(j, m, d, node, s, n) || n < 2) {
    ncur[j] = e;
    side[e] = 2;
    return;
  }
  const int64_t h = n >> 1;
  const int64_t L = lt[s + n] - lt[s], Eq = eq[s + n] - eq[s], G = n - L - Eq;
  const int64_t rl = lt[j] - lt[s], re = eq[j] - eq[s], rg = (j - s) - rl - re;
  int64_t pos;
  uint8_t sd;
  if (lt[j + 1] != lt[j]) {
    pos = s + rl;
    sd = 0;
  } else if (eq[j + 1] != eq[j]) {
    const int64_t k0 = std::min<int64_t>(Eq, L < G ? G - L : L - G);
    const bool small_left = L < G;
    int64_t before;
    if (re < k0) {
      sd = small_left ? 0 : 1;
      before = re;
    } else {
      const int64_t ep = re - k0;
      if (ep & 1) {
        sd = 0;
        before = (small_left ? k0 : 0) + ep / 2;
      } else {
        sd = 1;
        before = (small_left ? 0 : k0) + (ep - ep / 2);
      }
    }
    pos = sd == 0 ? s + L + before : s + h + G + before;
  } else {
    pos = s + h + rg;
    sd = 1;
  }
  ncur[pos] = e;
  side[e] = sd;
}

__global__ void axis_flags_kernel(const int32_t* __restrict__ A, int64_t m, int d,
                                  const uint8_t* __restrict__ side, uint32_t* __restrict__ f) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p > m) return;
  uint32_t v = 0;
  int64_t node, s, n;
  if (p < m && locate(p, m, d, node, s, n) && n >= 2) v = side[A[p]] == 1;
  f[p] = v;
}

__global__ void axis_scatter_kernel(const int32_t* __restrict__ A, int64_t m, int d,
                                    const uint8_t* __restrict__ side,
                                    const uint32_t* __restrict__ r, int32_t* __restrict__ nA) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= m) return;
  const int32_t e = A[p];
  int64_t node, s, n;
  if (!locate(p, m, d, node, s, n) || n < 2) {
    nA[p] = e;
    return;
  }
  const int64_t rr = r[p] - r[s];
  nA[side[e] == 1 ? s + (n >> 1) + rr : p - rr] = e;
}

// -------------------------------------------------------------- pair lists --
__device__ __forceinline__ int depth_of_slot(int64_t s) { return 63 - __clzll(s + 1); }
// Position on the bottom level (depth D) of the leftmost leaf under slot s.
__device__ __forceinline__ int64_t bottom_of(int64_t s, int D) {
  const int ds = depth_of_slot(s);
  return ((s + 1) << (D - ds)) - (int64_t(1) << D);
}

__global__ void slot_of_kernel(const int32_t* __restrict__ leaf, int64_t nb, int64_t nE,
                               int32_t* __restrict__ slot_of, unsigned* status) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nb) return;
  const int32_t e = leaf[s];
  if (e >= 0) {
    if (e < nE) slot_of[e] = (int32_t)s;
    else atomicOr(status, kStatusBadInput);
  } else if (e < -2) {
    atomicOr(status, kStatusBadInput);
  }
}

__global__ void max_vertex_kernel(const int32_t* __restrict__ E, int64_t n, int* mx,
                                  unsigned* status) {
  int v = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int x = E[i];
    if (x < 0) atomicOr(status, kStatusBadInput);
    v = max(v, x);
  }
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, v);
}

// Incidences: key (vertex << D) + bottom position of the segment's leaf;
// segments in no leaf get a key above every valid one.
__global__ void incidence_kernel(const int32_t* __restrict__ E, int64_t nE,
                                 const int32_t* __restrict__ slot_of, int D, int vbits,
                                 unsigned long long* __restrict__ key, int32_t* __restrict__ val) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 2 * nE) return;
  const int64_t e = i >> 1;
  const int32_t s = slot_of[e];
  const int v = max(E[i], 0);
  key[i] = s < 0 ? (1ull << (vbits + D))
                 : (((unsigned long long)v << D) | (unsigned long long)bottom_of(s, D));
  val[i] = (int32_t)i;
}

__global__ void sign_flags_kernel(const int32_t* __restrict__ val, int64_t n,
                                  uint32_t* __restrict__ f) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  f[i] = i < n ? ((val[i] & 1) ? 0u : 2u) : 0u;  // 1 + sign: start +1, end -1
}

__device__ __forceinline__ int64_t lower_bound_u64(const unsigned long long* k, int64_t lo,
                                                   int64_t hi, unsigned long long x) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (k[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// emit == false: count this incidence's (vertex, node) records into cnt;
// emit == true: write them at off.
template <bool kEmit>
__global__ void pair_records_kernel(const unsigned long long* __restrict__ key,
                                    const int32_t* __restrict__ val, int64_t n,
                                    const int32_t* __restrict__ slot_of,
                                    const int32_t* __restrict__ leaf,
                                    const uint32_t* __restrict__ ps, int D, int vbits,
                                    uint32_t* __restrict__ cnt, const uint32_t* __restrict__ off,
                                    unsigned long long* __restrict__ rkey,
                                    int32_t* __restrict__ rval) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned long long k = key[t];
  const unsigned long long invalid = 1ull << (vbits + D);
  uint32_t c = 0;
  if (k < invalid) {
    const unsigned long long v = k >> D;
    const int64_t mask = (int64_t(1) << D) - 1;
    const bool prev_same = t > 0 && (key[t - 1] >> D) == v;
    const int64_t prev_pos = prev_same ? (int64_t)(key[t - 1] & mask) : -1;
    int64_t r = slot_of[val[t] >> 1];
    uint64_t w = kEmit ? off[t] : 0;
    while (r > 0) {
      r = (r - 1) >> 1;
      const int dr = depth_of_slot(r);
      const int64_t lo = bottom_of(r, D), hi = lo + (int64_t(1) << (D - dr));
      if (prev_same && prev_pos >= lo) break;  // the previous incidence of v emits for r and above
      const int64_t b = lower_bound_u64(key, t, n, (v << D) + (unsigned long long)hi);
      const int64_t net = ((int64_t)ps[b] - (int64_t)ps[t]) - (b - t);
      if (net != 0 && leaf[r] == -1) {
        if (kEmit) {
          rkey[w] = ((unsigned long long)r << (vbits + 1)) |
                    ((unsigned long long)(net < 0) << vbits) | v;
          rval[w] = (int32_t)(net < 0 ? -net : net);
          ++w;
        }
        ++c;
      }
    }
  }
  if (!kEmit) cnt[t] = c;
}

__global__ void record_groups_kernel(const unsigned long long* __restrict__ rkey,
                                     const int32_t* __restrict__ rval, int64_t n, int vbits,
                                     uint32_t* __restrict__ npos, int32_t* __restrict__ first_pos,
                                     int32_t* __restrict__ first_neg, uint32_t* __restrict__ rc) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t > n) return;
  if (t == n) {
    rc[t] = 0;
    return;
  }
  const unsigned long long k = rkey[t];
  const int64_t r = (int64_t)(k >> (vbits + 1));
  const int cls = (int)((k >> vbits) & 1);
  rc[t] = (uint32_t)rval[t];
  if (cls == 0) atomicAdd(&npos[r], (uint32_t)rval[t]);
  const bool new_node = t == 0 || (int64_t)(rkey[t - 1] >> (vbits + 1)) != r;
  if (new_node && cls == 0) first_pos[r] = (int32_t)t;
  if (cls == 1 && (new_node || ((rkey[t - 1] >> vbits) & 1) == 0)) first_neg[r] = (int32_t)t;
}

__global__ void pair_counts_kernel(const uint32_t* __restrict__ npos, int64_t nb,
                                   uint32_t* __restrict__ c2) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r > nb) return;
  c2[r] = r < nb ? 2 * npos[r] : 0;
}

__global__ void to_i32_kernel(const uint32_t* __restrict__ a, int64_t n, int32_t* __restrict__ o) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) o[i] = (int32_t)a[i];
}

__global__ void write_pairs_kernel(const unsigned long long* __restrict__ rkey,
                                   const int32_t* __restrict__ rval, int64_t n, int vbits,
                                   const uint32_t* __restrict__ rc,
                                   const int32_t* __restrict__ first_pos,
                                   const int32_t* __restrict__ first_neg,
                                   const uint32_t* __restrict__ C, const uint32_t* __restrict__ npos,
                                   int32_t* __restrict__ I, unsigned* status) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const unsigned long long k = rkey[t];
  const int64_t r = (int64_t)(k >> (vbits + 1));
  const int cls = (int)((k >> vbits) & 1);
  const int32_t v = (int32_t)(k & ((1ull << vbits) - 1));
  const int32_t f = cls ? first_neg[r] : first_pos[r];
  const int64_t o = (int64_t)rc[t] - (int64_t)rc[f];
  for (int32_t u = 0; u < rval[t]; ++u) {
    if (o + u >= (int64_t)npos[r]) {
      atomicOr(status, kStatusBadInput);
      break;
    }
    I[(int64_t)C[r] + 2 * (o + u) + cls] = v;
  }
}

// -------------------------------------------------------------- evaluation --

// The reference's term: atan2(cross, dot) of (V[a]-p, V[b]-p), products and
// differences rounded separately (no contraction).
__device__ __forceinline__ double seg_angle64(const double* __restrict__ V, int64_t a, int64_t b,
                                              double px, double py) {
  const double x0 = __dsub_rn(V[2 * a], px), y0 = __dsub_rn(V[2 * a + 1], py);
  const double x1 = __dsub_rn(V[2 * b], px), y1 = __dsub_rn(V[2 * b + 1], py);
  const double cr = __dsub_rn(__dmul_rn(x0, y1), __dmul_rn(y0, x1));
  const double dt = __dadd_rn(__dmul_rn(x0, x1), __dmul_rn(y0, y1));
  return atan2(cr, dt);
}

// Next slot after slot r is finished, in the reference's order (a right
// child's left sibling, else up); -1 when the walk is done.
__device__ __forceinline__ int64_t walk_next(int64_t r) {
  for (;;) {
    if (r == 0) return -1;
    if (r & 1) r = (r - 1) >> 1;
    else return r - 1;
  }
}

struct EvalTree {
  const double* V;
  int64_t nV;
  const int32_t* E;
  int64_t nE;
  const double* B1;
  const double* B2;
  const int32_t* leaf;
  int64_t nb;
  const int32_t* I;
  const int32_t* C;
  int64_t nI;
};

// FP64: the reference's walk and arithmetic on the caller's arrays.
__device__ double eval64(const EvalTree& T, double px, double py, unsigned* status) {
  double wn = 0;
  if (T.nb == 0) return 0;
  int64_t r = 0;
  while (r >= 0) {
    if (r >= T.nb) {
      atomicOr(status, kStatusBadInput);
      break;
    }
    const int32_t lf = T.leaf[r];
    if (lf >= 0) {
      if (lf < T.nE) {
        const int64_t a = T.E[2 * (int64_t)lf], b = T.E[2 * (int64_t)lf + 1];
        if (a >= 0 && a < T.nV && b >= 0 && b < T.nV) wn += seg_angle64(T.V, a, b, px, py) / kTwoPi;
        else atomicOr(status, kStatusBadInput);
      } else {
        atomicOr(status, kStatusBadInput);
      }
      r = walk_next(r);
      continue;
    }
    if (px < T.B1[2 * r] || px > T.B2[2 * r] || py < T.B1[2 * r + 1] || py > T.B2[2 * r + 1]) {
      const int64_t c0 = T.C[r], c1 = T.C[r + 1];
      if (c0 < 0 || c1 > T.nI || c1 < c0) {
        atomicOr(status, kStatusBadInput);
      } else {
        for (int64_t i = c0; i + 1 < c1; i += 2) {
          const int64_t a = T.I[i], b = T.I[i + 1];
          if (a >= 0 && a < T.nV && b >= 0 && b < T.nV) wn += seg_angle64(T.V, a, b, px, py) / kTwoPi;
          else atomicOr(status, kStatusBadInput);
        }
      }
      r = walk_next(r);
      continue;
    }
    r = 2 * r + 2;
  }
  return wn;
}

__global__ void eval64_kernel(EvalTree T, const double* __restrict__ P, int64_t nP,
                              const int32_t* __restrict__ perm, double* __restrict__ W,
                              unsigned* status) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nP) return;
  const int64_t q = perm ? perm[i] : i;
  W[q] = eval64(T, P[2 * q], P[2 * q + 1], status);
}

// Mixed-precision frame: coordinates relative to the root box centre c,
// scaled by a power of two so the root box diagonal is in [0.5, 1] (exact,
// and FP32 stays far from overflow and underflow for any input scale).
// Vertices and queries are held as hi + lo FP32 pairs (x = hi + lo to ~2^-48
// relative), so a difference V - p is accurate to FP32 rounding of the
// difference itself however close V and p are.
struct Frame {
  double cx, cy, scale;
};
// The frame and the query cells' origin and scale, computed on the device
// from the root box (so a call never waits for the device).
struct EvalFrame {
  Frame f;
  float klx, kly, ksx, ksy;
};

__global__ void frame_kernel(const double* __restrict__ B1, const double* __restrict__ B2,
                             EvalFrame* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double cx = 0.5 * (B1[0] + B2[0]), cy = 0.5 * (B1[1] + B2[1]);
  double ex = B2[0] - B1[0], ey = B2[1] - B1[1];
  if (!isfinite(cx) || !isfinite(cy) || !isfinite(ex) || !isfinite(ey)) {
    cx = cy = 0;
    ex = ey = 1;
  }
  const double diag = sqrt(ex * ex + ey * ey);
  int e2 = 0;
  if (diag > 0) frexp(diag, &e2);  // diag = f 2^e2, f in [0.5, 1)
  EvalFrame r;
  r.f = Frame{cx, cy, ldexp(1.0, -e2)};
  // 1024 x 1024 Morton cells over the root box grown 25%
  const double hx = 0.625 * ex + 1e-300, hy = 0.625 * ey + 1e-300;
  r.klx = (float)(cx - hx);
  r.kly = (float)(cy - hy);
  r.ksx = (float)(1024.0 / (2 * hx));
  r.ksy = (float)(1024.0 / (2 * hy));
  *out = r;
}
__device__ __forceinline__ void split_coord(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

// Node (32 bytes, one sector): box in the frame (rounded outward) and meta =
// (leaf, a | c0, b | c1, 0).  A leaf's segment endpoints (hi, lo) sit in a
// per-segment array, a pair's in a per-pair array (32 bytes each).
struct NodeF {
  float4 box;
  int4 meta;
};
struct PairF {
  float4 hi;
  float4 lo;
};

__device__ __forceinline__ void seg_hilo(const double* V, int64_t a, int64_t b, const Frame& f,
                                         float4& hi, float4& lo) {
  split_coord((V[2 * a] - f.cx) * f.scale, hi.x, lo.x);
  split_coord((V[2 * a + 1] - f.cy) * f.scale, hi.y, lo.y);
  split_coord((V[2 * b] - f.cx) * f.scale, hi.z, lo.z);
  split_coord((V[2 * b + 1] - f.cy) * f.scale, hi.w, lo.w);
}

__global__ void prep_nodes_kernel(EvalTree T, const EvalFrame* __restrict__ fr,
                                  NodeF* __restrict__ nodes, PairF* __restrict__ segs,
                                  unsigned* status) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= T.nb) return;
  const Frame f = fr->f;
  NodeF nd;
  const int32_t lf = T.leaf[r];
  nd.box = make_float4(__double2float_rd((T.B1[2 * r] - f.cx) * f.scale),
                       __double2float_rd((T.B1[2 * r + 1] - f.cy) * f.scale),
                       __double2float_ru((T.B2[2 * r] - f.cx) * f.scale),
                       __double2float_ru((T.B2[2 * r + 1] - f.cy) * f.scale));
  nd.meta = make_int4(lf, 0, 0, 0);
  if (lf >= 0) {
    int64_t a = -1, b = -1;
    if (lf < T.nE) {
      a = T.E[2 * (int64_t)lf];
      b = T.E[2 * (int64_t)lf + 1];
    }
    if (a < 0 || a >= T.nV || b < 0 || b >= T.nV) {
      atomicOr(status, kStatusBadInput);
      nd.meta = make_int4(-3, 0, 0, 0);  // skipped by the walk
    } else {
      PairF sg;
      seg_hilo(T.V, a, b, f, sg.hi, sg.lo);
      segs[lf] = sg;
      nd.meta = make_int4(lf, (int)a, (int)b, 0);
    }
  } else if (lf == -1) {
    const int64_t c0 = T.C[r], c1 = T.C[r + 1];
    if (2 * r + 2 >= T.nb || c0 < 0 || c1 > T.nI || c1 < c0 || (c0 & 1)) {
      atomicOr(status, kStatusBadInput);
      nd.meta = make_int4(-3, 0, 0, 0);
    } else {
      nd.meta = make_int4(-1, (int)c0, (int)(c0 + ((c1 - c0) & ~int64_t(1))), 0);
    }
  }
  nodes[r] = nd;
}

// Pair i: both endpoints in the frame (hi, lo); (ida, idb) for FP64 terms.
__global__ void prep_pairs_kernel(EvalTree T, const EvalFrame* __restrict__ fr,
                                  PairF* __restrict__ pf, int2* __restrict__ pid, int64_t npairs,
                                  unsigned* status) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= npairs) return;
  const Frame f = fr->f;
  int64_t a = T.I[2 * i], b = T.I[2 * i + 1];
  if (a < 0 || a >= T.nV || b < 0 || b >= T.nV) {
    atomicOr(status, kStatusBadInput);
    a = b = 0;  // a zero-length pair adds nothing
  }
  PairF pr;
  seg_hilo(T.V, a, b, f, pr.hi, pr.lo);
  pf[i] = pr;
  pid[i] = make_int2((int)a, (int)b);
}

struct MixedTree {
  const NodeF* nodes;
  const PairF* segs;
  const PairF* pf;
  const int2* pid;
  const double* V;
  int64_t nb;
  const EvalFrame* fr;
};

// An FP32 angle term is trusted unless (a) the query is within 1e-9 of the
// frame's scale of an endpoint, or (b) the angle is near +-pi (dot < 0) with
// |cross| <= 8 u |v0||v1| (u = 2^-24): there rounding may flip the sign of
// the cross product and the angle by 2 pi.  Elsewhere the error of the
// computed angle is a few u (the differences are accurate to u, the cross
// and dot products to 2u |v0||v1|), independent of the distance to the
// segment.
constexpr float kTiny2 = 1e-18f;
constexpr float kTau2 = 64.f * 5.9604645e-8f * 5.9604645e-8f;

// Compensated FP32 sum (Neumaier): a walk can add thousands of angles of up
// to pi each (dense self-intersecting curves), which a plain FP32 sum rounds
// to ~1e-5 of a turn.
struct Sum32 {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x);
    c = __fadd_rn(c, fabsf(s) >= fabsf(x) ? __fadd_rn(__fsub_rn(s, t), x)
                                          : __fadd_rn(__fsub_rn(x, t), s));
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ void term_mixed(const MixedTree& T, float4 h, float4 l, int a, int b,
                                           float2 qh, float2 ql, double px, double py,
                                           Sum32& acc, double& acc64) {
  const float x0 = (h.x - qh.x) + (l.x - ql.x), y0 = (h.y - qh.y) + (l.y - ql.y);
  const float x1 = (h.z - qh.x) + (l.z - ql.x), y1 = (h.w - qh.y) + (l.w - ql.y);
  const float cr = x0 * y1 - y0 * x1;
  const float dt = fmaf(x0, x1, y0 * y1);
  const float l0 = fmaf(x0, x0, y0 * y0), l1 = fmaf(x1, x1, y1 * y1);
  if (fminf(l0, l1) < kTiny2 || (dt < 0.f && cr * cr <= kTau2 * (l0 * l1)))
    acc64 += seg_angle64(T.V, a, b, px, py);
  else
    acc.add(atan2_pairs(cr, dt));
}

// Warp-coherent walk: the lanes of a warp (Morton-ordered queries) share the
// walk position r.  At an internal node each active lane outside the box adds
// the node's pairs (all such lanes read the same pairs) and waits for the
// walk to come back out of the subtree (at walk_next(r)); the warp descends
// if any active lane is inside.  Every lane adds exactly the terms, in the
// same order, of its own walk.
// 6 blocks of 256 per SM (48 warps, 40 registers): 3.07 -> 3.01 ms per 10M
// queries against the 4 blocks that 52 registers allow.
__global__ void __launch_bounds__(kT, 12 * 128 / kT) eval_mixed_kernel(MixedTree T, const double* __restrict__ P,
                                                        int64_t nP,
                                                        const int32_t* __restrict__ perm,
                                                        double* __restrict__ W,
                                                        int32_t* __restrict__ redo,
                                                        uint32_t* __restrict__ nredo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < nP;
  const int64_t q = valid ? (perm ? perm[i] : i) : 0;
  const double px = valid ? P[2 * q] : 0.0, py = valid ? P[2 * q + 1] : 0.0;
  const Frame f = T.fr->f;
  float2 qh, ql;
  split_coord((px - f.cx) * f.scale, qh.x, ql.x);
  split_coord((py - f.cy) * f.scale, qh.y, ql.y);
  Sum32 acc;
  double acc64 = 0.0;
  bool active = valid;
  int64_t resume = -1;
  int64_t r = T.nb > 0 ? 0 : -1;
  while (r >= 0) {
    if (resume == r) active = true;
    const NodeF* nd = T.nodes + r;
    const int4 meta = __ldg(&nd->meta);
    if (meta.x >= 0) {
      if (active) {
        const PairF* sg = T.segs + meta.x;
        term_mixed(T, __ldg(&sg->hi), __ldg(&sg->lo), meta.y, meta.z, qh, ql, px, py, acc, acc64);
      }
      r = walk_next(r);
      continue;
    }
    if (meta.x != -1) {
      r = walk_next(r);
      continue;
    }
    const float4 box = __ldg(&nd->box);
    const bool outside =
        active && (qh.x < box.x || qh.x > box.z || qh.y < box.y || qh.y > box.w);
    const int64_t after = walk_next(r);
    if (outside) {
      for (int k = meta.y; k < meta.z; k += 2) {
        const PairF* pr = T.pf + (k >> 1);
        const int2 id = __ldg(&T.pid[k >> 1]);
        term_mixed(T, __ldg(&pr->hi), __ldg(&pr->lo), id.x, id.y, qh, ql, px, py, acc, acc64);
      }
      active = false;
      resume = after;
    }
    r = __any_sync(0xffffffffu, active) ? 2 * r + 2 : after;
  }
  if (!valid) return;
  const double w = (acc.value() + acc64) / kTwoPi;
  W[q] = w;
  if (fabs(w - 0.5) < 1e-3) redo[atomicAdd(nredo, 1u)] = (int32_t)q;
}

__global__ void redo64_kernel(EvalTree T, const double* __restrict__ P,
                              const int32_t* __restrict__ redo, const uint32_t* __restrict__ nredo,
                              double* __restrict__ W, unsigned* status) {
  const uint32_t n = *nredo;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int64_t q = redo[i];
    W[q] = eval64(T, P[2 * q], P[2 * q + 1], status);
  }
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

__global__ void keys2_kernel(const double* __restrict__ P, int64_t n,
                             const EvalFrame* __restrict__ fr, uint32_t* __restrict__ key) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float lx = fr->klx, ly = fr->kly, sx = fr->ksx, sy = fr->ksy;
  auto qz = [](float v, float l, float s) -> uint32_t {
    const float t = fminf(fmaxf((v - l) * s, 0.f), 1023.f);  // NaN -> 0
    return (uint32_t)t;
  };
  key[i] = (spread10(qz((float)P[2 * i + 1], ly, sy)) << 1) | spread10(qz((float)P[2 * i], lx, sx));
}

void scan_into(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t st) {
  exclusive_scan_u32(in, out, n, st);
}

}  // namespace

// ============================================================ host entries ==
int64_t eytzinger_slots(int64_t m) { return m <= 0 ? 0 : (int64_t(2) << depth_of(m)); }

void eytzinger_build(const double* PB1, const double* PB2, int64_t m, int dim, double* B1,
                     double* B2, int32_t* leaf, cudaStream_t st) {
  const int64_t nb = eytzinger_slots(m);
  if (nb == 0) return;
  launch_kernel(init_tree_kernel, nblk(nb), kT, 0, st, B1, B2, leaf, nb, dim);
  const int D = depth_of(m);
  DevBuf<double> pbc((size_t)(m * dim), st), lmed((size_t)1 << D, st);
  DevBuf<int8_t> ldir((size_t)1 << D, st);
  DevBuf<int32_t> cur((size_t)m, st), ncur((size_t)m, st), A((size_t)(m * dim), st),
      nA((size_t)(m * dim), st);
  DevBuf<uint8_t> side((size_t)m, st);
  DevBuf<uint32_t> f1((size_t)m + 1, st), f2((size_t)m + 1, st);
  launch_kernel(centres_kernel, nblk(m * dim), kT, 0, st, PB1, PB2, m, dim, pbc.get());
  {
    DevBuf<unsigned long long> k((size_t)m, st), kt((size_t)m, st);
    DevBuf<int32_t> vt((size_t)m, st);
    for (int a = 0; a < dim; ++a) {
      launch_kernel(axis_keys_kernel, nblk(m), kT, 0, st, pbc.get(), m, dim, a, k.get(),
                    A.get() + (int64_t)a * m);
      radix_sort_pairs<unsigned long long>(k.get(), A.get() + (int64_t)a * m, kt.get(), vt.get(),
                                           m, 0, 64, st);
    }
  }
  launch_kernel(iota_kernel, nblk(m), kT, 0, st, cur.get(), m);
  auto* B1b = reinterpret_cast<unsigned long long*>(B1);
  auto* B2b = reinterpret_cast<unsigned long long*>(B2);
  for (int d = 0; d <= D; ++d) {
    const int64_t width = int64_t(1) << d;
    launch_kernel(level_init_kernel, nblk(width), kT, 0, st, B1b, B2b, m, d, dim);
    launch_kernel(level_box_kernel, nblk(m), kT, 0, st, cur.get(), PB1, PB2, m, dim, d, B1b, B2b);
    launch_kernel(level_finish_kernel, nblk(width), kT, 0, st, B1b, B2b, cur.get(), A.get(),
                  pbc.get(), m, dim, d, leaf, ldir.get(), lmed.get());
    if (d == D) break;
    launch_kernel(level_classify_kernel, nblk(m + 1), kT, 0, st, cur.get(), pbc.get(), m, dim, d,
                  ldir.get(), lmed.get(), f1.get(), f2.get());
    scan_into(f1.get(), f1.get(), m + 1, st);
    scan_into(f2.get(), f2.get(), m + 1, st);
    launch_kernel(level_partition_kernel, nblk(m), kT, 0, st, cur.get(), m, d, f1.get(), f2.get(),
                  ncur.get(), side.get());
    for (int a = 0; a < dim; ++a) {
      const int32_t* Aa = A.get() + (int64_t)a * m;
      launch_kernel(axis_flags_kernel, nblk(m + 1), kT, 0, st, Aa, m, d, side.get(), f1.get());
      scan_into(f1.get(), f1.get(), m + 1, st);
      launch_kernel(axis_scatter_kernel, nblk(m), kT, 0, st, Aa, m, d, side.get(), f1.get(),
                    nA.get() + (int64_t)a * m);
    }
    std::swap(cur, ncur);
    std::swap(A, nA);
  }
}

int64_t eytzinger_pairs(const int32_t* E, int64_t nE, const int32_t* leaf, int64_t nb, int32_t* C,
                        int32_t* I, unsigned* status, cudaStream_t st) {
  if (nb == 0) {
    GWN_CUDA(cudaMemsetAsync(C, 0, sizeof(int32_t), st));
    return 0;
  }
  int D = 0;
  while ((int64_t(2) << D) < nb) ++D;
  GWN_REQUIRE((int64_t(2) << D) == nb, "the number of tree slots must be a power of two");
  DevBuf<int32_t> slot_of((size_t)std::max<int64_t>(nE, 1), st);
  GWN_CUDA(cudaMemsetAsync(slot_of.get(), 0xff, slot_of.bytes(), st));
  launch_kernel(slot_of_kernel, nblk(nb), kT, 0, st, leaf, nb, nE, slot_of.get(), status);
  DevBuf<int> mx(1, st);
  mx.zero(st);
  if (nE)
    launch_kernel(max_vertex_kernel, std::min<unsigned>(nblk(2 * nE), 4096u), kT, 0, st, E, 2 * nE,
                  mx.get(), status);
  int maxv = 0;
  GWN_CUDA(cudaMemcpyAsync(&maxv, mx.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  int vbits = 1;
  while ((int64_t(1) << vbits) <= (int64_t)maxv) ++vbits;
  GWN_REQUIRE(vbits + D + 2 <= 64, "tree too deep for this many vertices");
  const int64_t n = 2 * nE;
  DevBuf<unsigned long long> key((size_t)std::max<int64_t>(n, 1), st),
      key_tmp((size_t)std::max<int64_t>(n, 1), st);
  DevBuf<int32_t> val((size_t)std::max<int64_t>(n, 1), st), val_t((size_t)std::max<int64_t>(n, 1), st);
  DevBuf<uint32_t> ps((size_t)n + 1, st), cnt((size_t)n + 1, st);
  DevBuf<uint32_t> npos((size_t)nb + 1, st);
  npos.zero(st);
  int64_t nrec = 0;
  DevBuf<unsigned long long> rkey, rkey_t;
  DevBuf<int32_t> rval, rval_t;
  if (n) {
    launch_kernel(incidence_kernel, nblk(n), kT, 0, st, E, nE, slot_of.get(), D, vbits, key.get(),
                  val.get());
    radix_sort_pairs<unsigned long long>(key.get(), val.get(), key_tmp.get(), val_t.get(), n, 0,
                                         vbits + D + 1, st);
    launch_kernel(sign_flags_kernel, nblk(n + 1), kT, 0, st, val.get(), n, ps.get());
    scan_into(ps.get(), ps.get(), n + 1, st);
    launch_kernel(pair_records_kernel<false>, nblk(n), kT, 0, st, key.get(), val.get(), n,
                  slot_of.get(), leaf, ps.get(), D, vbits, cnt.get(), nullptr, nullptr, nullptr);
    GWN_CUDA(cudaMemsetAsync(cnt.get() + n, 0, sizeof(uint32_t), st));
    scan_into(cnt.get(), cnt.get(), n + 1, st);
    uint32_t tot = 0;
    GWN_CUDA(cudaMemcpyAsync(&tot, cnt.get() + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    nrec = tot;
  }
  DevBuf<uint32_t> rc((size_t)nrec + 1, st);
  DevBuf<int32_t> first_pos((size_t)nb, st), first_neg((size_t)nb, st);
  if (nrec) {
    rkey.alloc((size_t)nrec, st);
    rkey_t.alloc((size_t)nrec, st);
    rval.alloc((size_t)nrec, st);
    rval_t.alloc((size_t)nrec, st);
    launch_kernel(pair_records_kernel<true>, nblk(n), kT, 0, st, key.get(), val.get(), n,
                  slot_of.get(), leaf, ps.get(), D, vbits, nullptr, cnt.get(), rkey.get(),
                  rval.get());
    radix_sort_pairs<unsigned long long>(rkey.get(), rval.get(), rkey_t.get(), rval_t.get(), nrec,
                                         0, D + 2 + vbits, st);
    launch_kernel(record_groups_kernel, nblk(nrec + 1), kT, 0, st, rkey.get(), rval.get(), nrec,
                  vbits, npos.get(), first_pos.get(), first_neg.get(), rc.get());
    scan_into(rc.get(), rc.get(), nrec + 1, st);
  }
  DevBuf<uint32_t> c2((size_t)nb + 1, st);
  launch_kernel(pair_counts_kernel, nblk(nb + 1), kT, 0, st, npos.get(), nb, c2.get());
  scan_into(c2.get(), c2.get(), nb + 1, st);
  uint32_t total = 0;
  GWN_CUDA(cudaMemcpyAsync(&total, c2.get() + nb, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  launch_kernel(to_i32_kernel, nblk(nb + 1), kT, 0, st, c2.get(), nb + 1, C);
  GWN_CUDA(cudaStreamSynchronize(st));
  GWN_REQUIRE(total < (uint32_t)INT32_MAX, "pair list longer than 2^31-1 entries");
  if (I && nrec)
    launch_kernel(write_pairs_kernel, nblk(nrec), kT, 0, st, rkey.get(), rval.get(), nrec, vbits,
                  rc.get(), first_pos.get(), first_neg.get(), c2.get(), npos.get(), I, status);
  return total;
}

void eytzinger_eval(const double* P, int64_t nP, const double* V, int64_t nV, const int32_t* E,
                    int64_t nE, const double* B1, const double* B2, const int32_t* leaf,
                    int64_t nb, const int32_t* I, const int32_t* C, int64_t nI, double* W,
                    int precision, unsigned* status, cudaStream_t st) {
  if (nP == 0) return;
  EvalTree T{V, nV, E, nE, B1, B2, leaf, nb, I, C, nI};
  if (nb == 0) {
    GWN_CUDA(cudaMemsetAsync(W, 0, (size_t)nP * sizeof(double), st));
    return;
  }
  DevBuf<EvalFrame> frame(1, st);
  launch_kernel(frame_kernel, 1, 32, 0, st, B1, B2, frame.get());
  DevBuf<int32_t> perm;
  if (nP >= 8192) {
    PhaseTimer ph("order_queries", st);
    GWN_REQUIRE(nP < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    DevBuf<uint32_t> key((size_t)nP, st);
    perm.alloc((size_t)nP, st);
    launch_kernel(keys2_kernel, nblk(nP), kT, 0, st, P, nP, (const EvalFrame*)frame.get(),
                  key.get());
    bucket_order(key.get(), nP, 1u << 20, perm.get(), st);
  }
  if (precision == GWN_PLAIN_FP64) {
    PhaseTimer ph("walk", st);
    launch_kernel(eval64_kernel, nblk(nP), kT, 0, st, T, P, nP, perm.get(), W, status);
    return;
  }
  const int64_t npairs = nI / 2;
  DevBuf<NodeF> nodes((size_t)nb, st);
  DevBuf<PairF> segs((size_t)std::max<int64_t>(nE, 1), st);
  DevBuf<PairF> pf((size_t)std::max<int64_t>(npairs, 1), st);
  DevBuf<int2> pid((size_t)std::max<int64_t>(npairs, 1), st);
  {
    PhaseTimer ph("prep", st);
    launch_kernel(prep_nodes_kernel, nblk(nb), kT, 0, st, T, (const EvalFrame*)frame.get(),
                  nodes.get(), segs.get(), status);
    if (npairs)
      launch_kernel(prep_pairs_kernel, nblk(npairs), kT, 0, st, T, (const EvalFrame*)frame.get(),
                    pf.get(), pid.get(), npairs, status);
  }
  MixedTree M{nodes.get(), segs.get(), pf.get(), pid.get(), V, nb, frame.get()};
  DevBuf<int32_t> redo((size_t)nP, st);
  DevBuf<uint32_t> nredo(1, st);
  nredo.zero(st);
  {
    PhaseTimer ph("walk", st);
    launch_kernel(eval_mixed_kernel, nblk(nP), kT, 0, st, M, P, nP, perm.get(), W, redo.get(),
                  nredo.get());
  }
  PhaseTimer ph("refine", st);
  launch_kernel(redo64_kernel, 4 * num_sms(), kT, 0, st, T, P, redo.get(), nredo.get(), W, status);
}

}  // namespace gwn
