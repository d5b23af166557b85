// Hierarchical exact winding number of a triangle mesh, the GPU form of
// igl::WindingNumberAABB / igl::WindingNumberTree (include/igl/WindingNumberTree.h:
// 180-350, WindingNumberAABB.h): seen from a point outside a node's box, the
// node's triangles subtend the same solid angle as a cap closing their
// boundary, so the sum over the node's triangles can be replaced by a sum
// over the cap's triangles.  The value is the all-pairs sum's up to
// rounding.
//
// Build.  Triangles are ordered along a Morton curve of their centroids (a
// 1024^3 grid over the mesh box; ties by input order) and
// a binary radix tree is built over that order (every internal node covers
// a contiguous range of leaves); nodes are laid out in pre-order with a link
// one past each subtree.  A node's boundary: over its triangles' directed
// edges (a, b), the net count of each undirected edge {u < v} (+1 for u -> v,
// -1 for v -> u); edges with a non-zero count are the boundary, with that
// multiplicity and orientation.  Incidences (edge, leaf position) are sorted
// by edge (stable, so leaf order within an edge), and each (edge, node) with
// a non-zero count is emitted once, by the edge's first incidence under the
// node.  The cap is the fan from one boundary vertex (the apex) over the
// boundary edges: W(node) = sum over boundary edges (u -> v) of
// W(apex, u, v) (fan triangles through the apex vanish and are dropped).  A
// closed patch has no boundary and adds nothing from outside its box.  As in
// the reference, a node's cap is used only when it has fewer triangles than
// the node.
//
// Walk (mixed precision).  One thread per query (cell-ordered queries), the
// warp moves through the pre-order nodes with per-lane resume positions (a
// lane takes exactly its own walk).  At a node whose box, grown by the
// larger of the near distance eps = 1e-3 x the mesh diagonal and 5% of the
// box's diagonal, excludes the query (FP32, boxes rounded outward) and whose
// cap is usable, the lane adds the cap's FP32 terms and skips the subtree
// (every cap triangle is then seen from at least 1/20 of the node's size
// away); otherwise the lane descends.  Measured against the FP64 all-pairs
// sum on 5k-330k triangles: max |dW| <= 4.1e-7 (margin 0: 7.7e-5, 1.5x
// faster; half the diagonal: 7e-8, 2.5x slower).  A leaf's triangle is FP32 unless the query
// is inside its bounding sphere grown by eps, then FP64 (the reference's
// formula).  Coordinates are relative to the mesh box centre; vertex a of
// every record and the query are hi + lo FP32 pairs, so every difference
// a - q is accurate to FP32 rounding of the difference itself; terms are
// summed with compensation.  Results within 1e-3 of 0.5 are redone by the
// FP64 all-pairs kernel, one block per query.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>

#include "bh_common.cuh"
#include "exact_terms.cuh"
#include "gwn_internal.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

constexpr int kT = 256;
constexpr int kMaxSplit = 8;  // subtrees walked in parallel when queries are few
constexpr double kNearFrac = 1e-3;
constexpr double kBand = 1e-3;
constexpr double kInv2Pi = 0.15915494309189533577;
inline unsigned nblk(int64_t n, int t = kT) { return (unsigned)std::max<int64_t>(1, (n + t - 1) / t); }

__device__ __forceinline__ uint64_t spread21(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

__global__ void mesh_bbox_kernel(const double* __restrict__ V, int64_t nV,
                                 unsigned long long* __restrict__ mm) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nV;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) {
      const double v = V[i * 3 + d];
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
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&mm[d], ordered_bits(lo[d]));
      atomicMax(&mm[3 + d], ordered_bits(hi[d]));
    }
  }
}

__global__ void tri_keys_kernel(const double* __restrict__ V, int64_t nV,
                                const int32_t* __restrict__ F, int64_t nF,
                                const unsigned long long* __restrict__ mm,
                                unsigned long long* __restrict__ key, int32_t* __restrict__ val,
                                unsigned* status) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (f >= nF) return;
  double c[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k) {
    int64_t v = F[f * 3 + k];
    if (v < 0 || v >= nV) {
      atomicOr(status, kStatusBadInput);
      v = 0;
    }
    for (int d = 0; d < 3; ++d) c[d] += V[v * 3 + d];
  }
  uint64_t code = 0;
  for (int d = 0; d < 3; ++d) {
    const double lo = from_ordered_bits(mm[d]), hi = from_ordered_bits(mm[3 + d]);
    const double ext = hi - lo;
    double t = ext > 0 ? (c[d] / 3.0 - lo) / ext : 0.0;
    t = fmin(fmax(t, 0.0), 1.0);  // NaN -> 0
    code |= spread21((uint64_t)(t * 1023.0)) << (2 - d);
  }
  key[f] = code;
  val[f] = (int32_t)f;
}

// Common prefix length of sorted keys i and j, ties broken by index.
__device__ __forceinline__ int delta_key(const unsigned long long* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const unsigned long long a = keys[i], b = keys[j];
  if (a == b) return 64 + __clz((unsigned)(i ^ j));
  return __clzll((long long)(a ^ b));
}

// Binary radix tree over n sorted keys: internal nodes 0..n-2 (range of
// leaves [first, last]), leaf j is node n-1+j.
__global__ void radix_tree_kernel(const unsigned long long* __restrict__ keys, int n,
                                  int32_t* __restrict__ left, int32_t* __restrict__ right,
                                  int32_t* __restrict__ parent, int32_t* __restrict__ first,
                                  int32_t* __restrict__ last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta_key(keys, n, i, i + 1) - delta_key(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta_key(keys, n, i, i - d);
  int lmax = 2;
  while (delta_key(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta_key(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta_key(keys, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) >> 1;
    if (delta_key(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  const int lc = (lo == gamma) ? (n - 1 + gamma) : gamma;
  const int rc = (hi == gamma + 1) ? (n - 1 + gamma + 1) : (gamma + 1);
  left[i] = lc;
  right[i] = rc;
  parent[lc] = i;
  parent[rc] = i;
  first[i] = lo;
  last[i] = hi;
}

// Subtree sizes (nodes) and boxes (FP64) bottom-up: the second
// child to arrive at a parent merges.
__global__ void bottom_up_kernel(const double* __restrict__ V, const int32_t* __restrict__ F,
                                 int64_t nV, const int32_t* __restrict__ sorted_tri, int n,
                                 const int32_t* __restrict__ left,
                                 const int32_t* __restrict__ right,
                                 const int32_t* __restrict__ parent, double* __restrict__ box,
                                 int32_t* __restrict__ size, unsigned* __restrict__ flags) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int node = n - 1 + j;
  {
    const int64_t f = sorted_tri[j];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 3; ++k) {
      int64_t v = F[f * 3 + k];
      if (v < 0 || v >= nV) v = 0;
      for (int d = 0; d < 3; ++d) {
        lo[d] = fmin(lo[d], V[v * 3 + d]);
        hi[d] = fmax(hi[d], V[v * 3 + d]);
      }
    }
    for (int d = 0; d < 3; ++d) {
      box[(int64_t)node * 6 + d] = lo[d];
      box[(int64_t)node * 6 + 3 + d] = hi[d];
    }
    size[node] = 1;
  }
  if (n == 1) return;
  int cur = node;
  while (true) {
    const int p = parent[cur];
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0) return;  // the first child to arrive stops
    __threadfence();
    const int lc = left[p], rc = right[p];
    for (int d = 0; d < 3; ++d) {
      box[(int64_t)p * 6 + d] = fmin(box[(int64_t)lc * 6 + d], box[(int64_t)rc * 6 + d]);
      box[(int64_t)p * 6 + 3 + d] =
          fmax(box[(int64_t)lc * 6 + 3 + d], box[(int64_t)rc * 6 + 3 + d]);
    }
    size[p] = 1 + size[lc] + size[rc];
    if (p == 0) return;
    cur = p;
  }
}

__global__ void preorder_kernel(const int32_t* __restrict__ left,
                                const int32_t* __restrict__ parent,
                                const int32_t* __restrict__ size, int nnodes,
                                int32_t* __restrict__ pre) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nnodes) return;
  int p = 0, cur = x;
  while (cur != 0) {
    const int par = parent[cur];
    const int lc = left[par];
    p += 1 + (lc == cur ? 0 : size[lc]);
    cur = par;
  }
  pre[x] = p;
}

// Directed-edge incidences of the sorted triangles: key {u < v} packed, value
// 3 j + c (leaf position j, corner c: edge from corner c to corner c+1).
// (Indices out of range, already reported by tri_keys_kernel, read as 0.)
__global__ void edge_incidence_kernel(const int32_t* __restrict__ F,
                                      const int32_t* __restrict__ sorted_tri, int n, int64_t nV,
                                      unsigned long long* __restrict__ key,
                                      int32_t* __restrict__ val) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 3 * (int64_t)n) return;
  const int64_t j = i / 3, c = i % 3;
  const int64_t f = sorted_tri[j];
  const int32_t fa = F[f * 3 + c], fb = F[f * 3 + (c + 1) % 3];
  const uint32_t a = (fa < 0 || fa >= nV) ? 0u : (uint32_t)fa;
  const uint32_t b = (fb < 0 || fb >= nV) ? 0u : (uint32_t)fb;
  const uint32_t u = min(a, b), v = max(a, b);
  key[i] = ((unsigned long long)u << 32) | v;
  val[i] = (int32_t)i;
}

__device__ __forceinline__ int edge_sign(const int32_t* F, const int32_t* sorted_tri, int32_t e) {
  const int64_t j = e / 3, c = e % 3;
  const int64_t f = sorted_tri[j];
  return F[f * 3 + c] < F[f * 3 + (c + 1) % 3] ? 1 : -1;  // orientation of {u < v}
}

__global__ void sign_flags_kernel(const int32_t* __restrict__ F,
                                  const int32_t* __restrict__ sorted_tri,
                                  const int32_t* __restrict__ val, int64_t n,
                                  uint32_t* __restrict__ fl) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  fl[i] = i < n ? (uint32_t)(1 + edge_sign(F, sorted_tri, val[i])) : 0u;
}

// First index in [lo, hi) whose (key, leaf position) is past (k, jmax).
__device__ __forceinline__ int64_t past(const unsigned long long* key, const int32_t* val,
                                        int64_t lo, int64_t hi, unsigned long long k, int jmax) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    const unsigned long long km = key[mid];
    const bool before = km < k || (km == k && val[mid] / 3 <= jmax);
    if (before) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// kEmit == false: count the (edge, node) records each incidence emits;
// true: write them (node pre-order index, record value = incidence index,
// net count).
template <bool kEmit>
__global__ void boundary_records_kernel(const unsigned long long* __restrict__ key,
                                        const int32_t* __restrict__ val, int64_t m, int n,
                                        const int32_t* __restrict__ parent,
                                        const int32_t* __restrict__ first,
                                        const int32_t* __restrict__ last,
                                        const int32_t* __restrict__ pre,
                                        const uint32_t* __restrict__ ps,
                                        uint32_t* __restrict__ cnt,
                                        const uint32_t* __restrict__ off,
                                        int32_t* __restrict__ rnode, int32_t* __restrict__ rinc,
                                        int32_t* __restrict__ rnet) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= m) return;
  const unsigned long long k = key[t];
  const int j = val[t] / 3;
  const bool prev_same = t > 0 && key[t - 1] == k;
  const int pj = prev_same ? val[t - 1] / 3 : -1;
  uint32_t c = 0;
  uint64_t w = kEmit ? off[t] : 0;
  int cur = n - 1 + j;
  while (cur != 0) {
    const int r = parent[cur];
    if (prev_same && pj >= first[r]) break;  // an earlier incidence of the edge emits here
    const int64_t b = past(key, val, t, m, k, last[r]);
    const int64_t net = ((int64_t)ps[b] - (int64_t)ps[t]) - (b - t);
    if (net != 0) {
      if (kEmit) {
        rnode[w] = pre[r];
        rinc[w] = (int32_t)t;
        rnet[w] = (int32_t)net;
        ++w;
      }
      ++c;
    }
    cur = r;
  }
  if (!kEmit) cnt[t] = c;
}

__global__ void iota_records_kernel(int32_t* __restrict__ p, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = (int32_t)i;
}

__global__ void record_mult_kernel(const int32_t* __restrict__ rnet, const int32_t* __restrict__ order,
                                   int64_t nrec, uint32_t* __restrict__ mult) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i > nrec) return;
  mult[i] = i < nrec ? (uint32_t)abs(rnet[order[i]]) : 0u;
}

// Triangle record of the walk (64 bytes), coordinates relative to the mesh
// box centre: vertex a as an FP32 hi + lo pair (a = hi + lo to ~2^-48),
// e1 = b - a, e2 = c - a and n = e1 x e2 formed in FP64 and rounded; near2 =
// the squared radius about the centroid within which a leaf's term is taken
// in FP64 (bounding sphere grown by eps), -1 for a cap triangle.
//   r0 = ahi.xyz, e1.x   r1 = e1.yz, e2.xy   r2 = e2.z, n.xyz   r3 = alo.xyz, near2
struct TriH {
  float4 r0, r1, r2, r3;
};

__device__ __forceinline__ TriH make_trih(const double p[3][3], double eps, bool cap) {
  double e1[3], e2[3], n[3], m[3];
  for (int d = 0; d < 3; ++d) {
    e1[d] = p[1][d] - p[0][d];
    e2[d] = p[2][d] - p[0][d];
    m[d] = (e1[d] + e2[d]) / 3.0;
  }
  n[0] = e1[1] * e2[2] - e1[2] * e2[1];
  n[1] = e1[2] * e2[0] - e1[0] * e2[2];
  n[2] = e1[0] * e2[1] - e1[1] * e2[0];
  double r2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2], t1 = 0, t2 = 0;
  for (int d = 0; d < 3; ++d) {
    t1 += (m[d] - e1[d]) * (m[d] - e1[d]);
    t2 += (m[d] - e2[d]) * (m[d] - e2[d]);
  }
  const double R = sqrt(fmax(r2, fmax(t1, t2)));
  const double near2 = (R + eps) * (R + eps) * (1.0 + 1e-5) + 1e-30;
  float hi[3], lo[3];
  for (int d = 0; d < 3; ++d) {
    hi[d] = (float)p[0][d];
    lo[d] = (float)(p[0][d] - (double)hi[d]);
  }
  TriH t;
  t.r0 = make_float4(hi[0], hi[1], hi[2], (float)e1[0]);
  t.r1 = make_float4((float)e1[1], (float)e1[2], (float)e2[0], (float)e2[1]);
  t.r2 = make_float4((float)e2[2], (float)n[0], (float)n[1], (float)n[2]);
  t.r3 = make_float4(lo[0], lo[1], lo[2], cap ? -1.f : (isfinite(near2) ? (float)near2 : INFINITY));
  return t;
}

__device__ __forceinline__ TriH zero_trih() {
  TriH t;
  t.r0 = t.r1 = t.r2 = make_float4(0.f, 0.f, 0.f, 0.f);
  t.r3 = make_float4(0.f, 0.f, 0.f, -1.f);
  return t;
}

// a - q from the hi + lo pairs of both: accurate to FP32 rounding of the
// difference itself.
__device__ __forceinline__ float3 rel_a(const TriH& t, float3 qh, float3 ql) {
  return make_float3((t.r0.x - qh.x) + (t.r3.x - ql.x), (t.r0.y - qh.y) + (t.r3.y - ql.y),
                     (t.r0.z - qh.z) + (t.r3.z - ql.z));
}

// atan2(det, den) of the van Oosterom-Strackee formula, a = vertex a - q.
__device__ __forceinline__ float trih_term32(const TriH& t, float3 a) {
  const float bx = a.x + t.r0.w, by = a.y + t.r1.x, bz = a.z + t.r1.y;
  const float cx = a.x + t.r1.z, cy = a.y + t.r1.w, cz = a.z + t.r2.x;
  const float det = fmaf(a.x, t.r2.y, fmaf(a.y, t.r2.z, a.z * t.r2.w));
  const float la = sqrt_approx(fmaf(a.x, a.x, fmaf(a.y, a.y, a.z * a.z)));
  const float lb = sqrt_approx(fmaf(bx, bx, fmaf(by, by, bz * bz)));
  const float lc = sqrt_approx(fmaf(cx, cx, fmaf(cy, cy, cz * cz)));
  const float ab = fmaf(a.x, bx, fmaf(a.y, by, a.z * bz));
  const float bc = fmaf(bx, cx, fmaf(by, cy, bz * cz));
  const float ca = fmaf(cx, a.x, fmaf(cy, a.y, cz * a.z));
  const float den = fmaf(la * lb, lc, fmaf(bc, la, fmaf(ca, lb, ab * lc)));
  return atan2_pairs(det, den);
}

// Compensated FP32 sum (Neumaier): caps add many large angles that cancel.
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

// Node record of the walk (32 bytes): box (FP32 in the centred frame, grown
// by max(eps, 5% of the box diagonal), rounded outward) with the link in
// lo.w; hi.w = cap start (>= 0: usable cap of capn triangles), -1 (descend),
// or -2 - slot (leaf).
struct NodeH {
  float4 lo;
  float4 hi;
};

struct HierDev {
  const NodeH* nodes;
  const int32_t* capn;
  const TriH* caps;      // cap triangles
  const TriH* tris;      // leaf triangles by slot
  const double* tris64;  // leaf triangles by slot, 9 doubles
  int nnodes;
  const double* box64;   // FP64 node boxes (pre-order), 6 doubles
  const double* caps64;  // FP64 cap triangles, 9 doubles
};

__global__ void node_records_kernel(const double* __restrict__ box,
                                    const int32_t* __restrict__ pre,
                                    const int32_t* __restrict__ size, int n,
                                    const uint32_t* __restrict__ cap_off,
                                    const uint32_t* __restrict__ cap_cnt, double cx, double cy,
                                    double cz, double eps, NodeH* __restrict__ nodes,
                                    int32_t* __restrict__ capn, double* __restrict__ box64) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int nnodes = 2 * n - 1;
  if (x >= nnodes) return;
  const int p = pre[x];
  const bool leaf = x >= n - 1;
  NodeH h;
  const double c[3] = {cx, cy, cz};
  float lo[3], hi[3];
  double diag2 = 0;
  for (int d = 0; d < 3; ++d) {
    const double e = box[(int64_t)x * 6 + 3 + d] - box[(int64_t)x * 6 + d];
    diag2 += e * e;
  }
  // a cap is seen from at least eps and at least 5% of the node's diagonal away
  const double margin = fmax(eps, 0.05 * sqrt(diag2));
  for (int d = 0; d < 3; ++d) {
    lo[d] = __double2float_rd(box[(int64_t)x * 6 + d] - c[d] - margin);
    hi[d] = __double2float_ru(box[(int64_t)x * 6 + 3 + d] - c[d] + margin);
  }
  int meta;
  int cn = 0;
  if (leaf) {
    meta = -2 - (x - (n - 1));
  } else {
    cn = (int)cap_cnt[p];
    const int tris_under = (size[x] + 1) / 2;
    meta = cn < tris_under ? (int)cap_off[p] : -1;
  }
  h.lo = make_float4(lo[0], lo[1], lo[2], __int_as_float(p + size[x]));
  h.hi = make_float4(hi[0], hi[1], hi[2], __int_as_float(meta));
  nodes[p] = h;
  capn[p] = cn;
  for (int k = 0; k < 6; ++k) box64[(int64_t)p * 6 + k] = box[(int64_t)x * 6 + k];
}

// Cap triangles of every node: for the records of node r (in node order,
// each repeated |net| times) the fan triangle (apex, u, v) oriented by the
// record's sign, the apex being the first record's u; triangles through the
// apex get a zero record.
__global__ void cap_tris_kernel(const double* __restrict__ V, const int32_t* __restrict__ F,
                                const int32_t* __restrict__ sorted_tri,
                                const unsigned long long* __restrict__ key,
                                const int32_t* __restrict__ order,
                                const int32_t* __restrict__ rnode,
                                const int32_t* __restrict__ rinc, const int32_t* __restrict__ rnet,
                                int64_t nrec, const uint32_t* __restrict__ mult_off,
                                const uint32_t* __restrict__ cap_off,
                                const int32_t* __restrict__ first_rec, double cx, double cy,
                                double cz, double eps, TriH* __restrict__ caps,
                                double* __restrict__ caps64) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const int32_t rec = order[i];
  const int node = rnode[rec];
  const unsigned long long k = key[rinc[rec]];
  const uint32_t u0 = (uint32_t)(k >> 32), v0 = (uint32_t)(k & 0xffffffffu);
  const int net = rnet[rec];
  const uint32_t a = net > 0 ? u0 : v0, b = net > 0 ? v0 : u0;
  const unsigned long long k0 = key[rinc[order[first_rec[node]]]];
  const uint32_t apex = (uint32_t)(k0 >> 32);
  const double c[3] = {cx, cy, cz};
  double p[3][3];
  const uint32_t vid[3] = {apex, a, b};
  for (int s = 0; s < 3; ++s)
    for (int d = 0; d < 3; ++d) p[s][d] = V[(int64_t)vid[s] * 3 + d] - c[d];
  const bool degenerate = a == apex || b == apex;
  // a zero record adds atan2(0, >= 0) = 0
  const TriH t = degenerate ? zero_trih() : make_trih(p, eps, true);
  double t64[9];
  for (int s = 0; s < 3; ++s)
    for (int d = 0; d < 3; ++d) t64[s * 3 + d] = degenerate ? 0.0 : V[(int64_t)vid[s] * 3 + d];
  const int reps = abs(net);
  for (int r = 0; r < reps; ++r) {
    caps[(int64_t)mult_off[i] + r] = t;
    for (int k = 0; k < 9; ++k) caps64[((int64_t)mult_off[i] + r) * 9 + k] = t64[k];
  }
  (void)cap_off;
}

// Per node with records: its first record (position in the node-sorted
// order) and the offset of its cap triangles.
__global__ void first_record_kernel(const int32_t* __restrict__ order,
                                    const int32_t* __restrict__ rnode, int64_t nrec,
                                    int32_t* __restrict__ first_rec,
                                    const uint32_t* __restrict__ mult_off,
                                    uint32_t* __restrict__ cap_off) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const int node = rnode[order[i]];
  if (i == 0 || rnode[order[i - 1]] != node) {
    first_rec[node] = (int32_t)i;
    cap_off[node] = mult_off[i];
  }
}

// Per node with records: the number of its cap triangles (launched after
// first_record_kernel, whose offsets it reads).
__global__ void cap_count_kernel(const int32_t* __restrict__ order,
                                 const int32_t* __restrict__ rnode, int64_t nrec,
                                 const uint32_t* __restrict__ mult_off,
                                 const uint32_t* __restrict__ cap_off,
                                 uint32_t* __restrict__ cap_cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const int node = rnode[order[i]];
  if (i == nrec - 1 || rnode[order[i + 1]] != node)
    cap_cnt[node] = mult_off[i + 1] - cap_off[node];
}

__global__ void leaf_tris_kernel(const double* __restrict__ V, const int32_t* __restrict__ F,
                                 int64_t nV, const int32_t* __restrict__ sorted_tri, int n,
                                 double cx, double cy, double cz, double eps,
                                 TriH* __restrict__ tris, double* __restrict__ tris64) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t f = sorted_tri[j];
  const double c[3] = {cx, cy, cz};
  double p[3][3];
  for (int s = 0; s < 3; ++s) {
    int64_t v = F[f * 3 + s];
    if (v < 0 || v >= nV) v = 0;
    for (int d = 0; d < 3; ++d) {
      const double x = V[v * 3 + d];
      tris64[(int64_t)j * 9 + s * 3 + d] = x;
      p[s][d] = x - c[d];
    }
  }
  tris[j] = make_trih(p, eps, false);
}

// ----------------------------------------------------------------- walk ---
__device__ __forceinline__ double tri64_term(const double* t, double px, double py, double pz) {
  return vos_term64(t, t + 3, t + 6, px, py, pz);
}

// Per-warp queue of the FP64 leaf terms: the lanes that need one append
// (slot, lane); when the queue would overflow, and at the end, the warp
// evaluates up to 32 queued terms at once, one per lane, and every lane adds
// its own terms in queue order (its walk order), so that the FP64
// instructions run with the whole warp instead of the few lanes near a leaf.
struct HierQueue {
  int2 e[32];
  double q[32][3];  // each lane's FP64 query
};

__device__ __forceinline__ void flush_hier64(const double* __restrict__ tris64,
                                             const HierQueue& hq, int n, double& acc64) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  int2 e = make_int2(0, lane);
  if (lane < n) e = hq.e[lane];
  double v = 0.0;
  if (lane < n)
    v = tri64_term(tris64 + (int64_t)e.x * 9, hq.q[e.y][0], hq.q[e.y][1], hq.q[e.y][2]);
  for (int k = 0; k < n; ++k) {
    const double vk = __shfl_sync(full, v, k);
    const int ok = __shfl_sync(full, e.y, k);
    if (ok == lane) acc64 += vk;
  }
  __syncwarp();
}

template <typename QT>
__global__ void __launch_bounds__(kT, 4) hier_walk_kernel(HierDev H, const QT* __restrict__ Q,
                                                       int64_t nQ,
                                                       const int32_t* __restrict__ perm,
                                                       double cx, double cy, double cz,
                                                       double* __restrict__ W,
                                                       int32_t* __restrict__ redo,
                                                       uint32_t* __restrict__ nredo,
                                                       const int2* __restrict__ ranges,
                                                       const int* __restrict__ nranges,
                                                       double* __restrict__ part) {
  // ranges: walk only the subtree [ranges[y].x, ranges[y].y) of y = blockIdx.y
  // and write the partial sum (solid angle) to part[y * nQ + q]
  int x0 = 0, x1 = H.nnodes;
  if (ranges) {
    if ((int)blockIdx.y >= *nranges) return;
    const int2 rg = ranges[blockIdx.y];
    x0 = rg.x;
    x1 = rg.y;
  }
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < nQ;
  const int64_t q = valid ? (perm ? perm[i] : i) : 0;
  const double px = valid ? (double)Q[q * 3] : 0.0, py = valid ? (double)Q[q * 3 + 1] : 0.0,
               pz = valid ? (double)Q[q * 3 + 2] : 0.0;
  float3 qh, ql;
  {
    const double rx = px - cx, ry = py - cy, rz = pz - cz;
    qh = make_float3((float)rx, (float)ry, (float)rz);
    ql = make_float3((float)(rx - (double)qh.x), (float)(ry - (double)qh.y),
                     (float)(rz - (double)qh.z));
  }
  Sum32 acc;
  double acc64 = 0.0;
  __shared__ HierQueue hqs[kT / 32];
  HierQueue& hq = hqs[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  hq.q[lane][0] = px;
  hq.q[lane][1] = py;
  hq.q[lane][2] = pz;
  int nqueued = 0;  // warp-uniform
  int resume = valid ? x0 : 0x7fffffff;
  if (ranges && valid) {
    // a query outside the root's box takes the root's cap alone (in
    // subtree 0), as the whole-tree walk does, instead of one cap per subtree
    const NodeH r0 = H.nodes[0];
    const int meta0 = __float_as_int(r0.hi.w);
    if (meta0 >= 0 && (qh.x < r0.lo.x || qh.x > r0.hi.x || qh.y < r0.lo.y || qh.y > r0.hi.y ||
                       qh.z < r0.lo.z || qh.z > r0.hi.z)) {
      if (blockIdx.y == 0) {
        const int cn = H.capn[0];
        for (int k = 0; k < cn; ++k) {
          const TriH t = H.caps[meta0 + k];
          acc.add(trih_term32(t, rel_a(t, qh, ql)));
        }
      }
      resume = 0x7fffffff;
    }
  }
  int x = x0;
  while (x < x1) {
    bool want64 = false;
    int slot64 = 0;
    if (x >= resume) {
      const NodeH nd = H.nodes[x];
      const int meta = __float_as_int(nd.hi.w);
      if (meta <= -2) {
        const int slot = -2 - meta;
        const TriH t = H.tris[slot];
        const float3 a = rel_a(t, qh, ql);
        // centroid - q
        const float mx = a.x + (t.r0.w + t.r1.z) * (1.f / 3.f);
        const float my = a.y + (t.r1.x + t.r1.w) * (1.f / 3.f);
        const float mz = a.z + (t.r1.y + t.r2.x) * (1.f / 3.f);
        if (fmaf(mx, mx, fmaf(my, my, mz * mz)) < t.r3.w) {
          want64 = true;
          slot64 = slot;
        } else {
          acc.add(trih_term32(t, a));
        }
        resume = x + 1;
      } else if (meta >= 0 && (qh.x < nd.lo.x || qh.x > nd.hi.x || qh.y < nd.lo.y ||
                               qh.y > nd.hi.y || qh.z < nd.lo.z || qh.z > nd.hi.z)) {
        const int cn = H.capn[x];
        for (int k = 0; k < cn; ++k) {
          const TriH t = H.caps[meta + k];
          acc.add(trih_term32(t, rel_a(t, qh, ql)));
        }
        resume = __float_as_int(nd.lo.w);
      } else {
        resume = x + 1;
      }
    }
    const unsigned m64 = __ballot_sync(0xffffffffu, want64);
    if (m64) {
      const int k = __popc(m64);
      if (nqueued + k > 32) {
        flush_hier64(H.tris64, hq, nqueued, acc64);
        nqueued = 0;
      }
      if (want64) hq.e[nqueued + __popc(m64 & ((1u << lane) - 1u))] = make_int2(slot64, lane);
      nqueued += k;
    }
    x = __reduce_min_sync(0xffffffffu, resume);
  }
  if (nqueued) flush_hier64(H.tris64, hq, nqueued, acc64);
  if (!valid) return;
  if (part) {
    part[(int64_t)blockIdx.y * nQ + q] = acc.value() + acc64;
    return;
  }
  const double w = (acc.value() + acc64) * kInv2Pi;
  W[q] = w;
  if (fabs(w - 0.5) <= kBand) redo[atomicAdd(nredo, 1u)] = (int32_t)q;
}

// Per-warp queue of the plain FP64 walk's triangle terms.  Every leaf and
// cap triangle a lane needs is appended as (triangle, lane): triangle >= 0 a
// cap triangle (caps64), < 0 the leaf ~triangle (tris64).  Whenever 32 are
// queued (and at the end) the warp evaluates them, one per lane, so each
// FP64 instruction serves the whole warp instead of the lanes that happen to
// leave a node at the same step (a warp instruction costs the narrow FP64
// pipe the same with 1 or 32 lanes).  A lane adds its own values by its bit
// mask of queue positions, in queue order, which is its walk order: its sum
// is the one it would form alone.
struct Hier64Queue {
  int2 e[32];
  double q[32][3];  // each lane's query
  double v[32];     // the values of one flush
};

__device__ __forceinline__ void flush_queue64(const HierDev& H, Hier64Queue& hq, int n,
                                              unsigned mine, double& acc) {
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if (lane < n) {
    const int2 e = hq.e[lane];
    const double* t = e.x >= 0 ? H.caps64 + (int64_t)e.x * 9 : H.tris64 + (int64_t)(~e.x) * 9;
    hq.v[lane] = tri64_term(t, hq.q[e.y][0], hq.q[e.y][1], hq.q[e.y][2]);
  }
  __syncwarp();
  while (mine) {
    acc += hq.v[__ffs(mine) - 1];
    mine &= mine - 1;
  }
  __syncwarp();
}

// Appends cnt terms of this lane (tri, tri + 1, ... for a cap; the single
// leaf ~slot when tri < 0) after the lower lanes' terms of this step,
// flushing every time the queue fills.  All 32 lanes call it together.
__device__ __forceinline__ void enqueue64(const HierDev& H, Hier64Queue& hq, int cnt, int tri,
                                          int& nq, unsigned& mine, double& acc) {
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
    const int take = min(32 - nq, total - done);
    const int k0 = max(0, done - excl), k1 = min(cnt, done + take - excl);
    for (int k = k0; k < k1; ++k) {
      const int pos = nq + excl + k - done;
      hq.e[pos] = make_int2(tri >= 0 ? tri + k : tri, lane);
      mine |= 1u << pos;
    }
    nq += take;
    done += take;
    if (nq == 32) {
      flush_queue64(H, hq, 32, mine, acc);
      nq = 0;
      mine = 0;
    }
  }
}

// Plain FP64 walk, the reference's (WindingNumberTree.h:261-336): a node's
// cap for a point strictly outside its FP64 box (the conservative test of
// WindingNumberAABB.h:253-268) when the cap has fewer triangles than the
// node, else its children; leaf and cap triangles in FP64 with the
// reference's formula (solid_angle.cpp:16-54), through the warp's queue.
// Same warp walk, subtree split and partial sums as hier_walk_kernel.
__global__ void __launch_bounds__(kT, 4) hier_walk64_kernel(HierDev H, const double* __restrict__ Q,
                                                         int64_t nQ,
                                                         const int32_t* __restrict__ perm,
                                                         double* __restrict__ W,
                                                         const int2* __restrict__ ranges,
                                                         const int* __restrict__ nranges,
                                                         double* __restrict__ part) {
  int x0 = 0, x1 = H.nnodes;
  if (ranges) {
    if ((int)blockIdx.y >= *nranges) return;
    const int2 rg = ranges[blockIdx.y];
    x0 = rg.x;
    x1 = rg.y;
  }
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < nQ;
  const int64_t q = valid ? (perm ? perm[i] : i) : 0;
  const double px = valid ? Q[q * 3] : 0.0, py = valid ? Q[q * 3 + 1] : 0.0,
               pz = valid ? Q[q * 3 + 2] : 0.0;
  __shared__ Hier64Queue hqs[kT / 32];
  Hier64Queue& hq = hqs[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  hq.q[lane][0] = px;
  hq.q[lane][1] = py;
  hq.q[lane][2] = pz;
  auto outside = [&](int x) {
    const double* b = H.box64 + (int64_t)x * 6;
    return px < b[0] || px > b[3] || py < b[1] || py > b[4] || pz < b[2] || pz > b[5];
  };
  double acc = 0.0;
  int nq = 0;         // warp-uniform
  unsigned mine = 0;  // this lane's queue positions
  int resume = valid ? x0 : 0x7fffffff;
  if (ranges) {
    // outside the root's box: the root's cap alone, in subtree 0
    const int meta0 = __float_as_int(H.nodes[0].hi.w);
    int cnt = 0;
    if (valid && meta0 >= 0 && outside(0)) {
      if (blockIdx.y == 0) cnt = H.capn[0];
      resume = 0x7fffffff;
    }
    enqueue64(H, hq, cnt, meta0, nq, mine, acc);
  }
  int x = x0;
  while (x < x1) {
    int cnt = 0, tri = 0;
    if (x >= resume) {
      const NodeH nd = H.nodes[x];
      const int meta = __float_as_int(nd.hi.w);
      if (meta <= -2) {
        cnt = 1;
        tri = ~(-2 - meta);
        resume = x + 1;
      } else if (meta >= 0 && outside(x)) {
        cnt = H.capn[x];
        tri = meta;
        resume = __float_as_int(nd.lo.w);
      } else {
        resume = x + 1;
      }
    }
    if (__any_sync(0xffffffffu, cnt > 0)) enqueue64(H, hq, cnt, tri, nq, mine, acc);
    x = __reduce_min_sync(0xffffffffu, resume);
  }
  if (nq) flush_queue64(H, hq, nq, mine, acc);
  if (!valid) return;
  if (part) {
    part[(int64_t)blockIdx.y * nQ + q] = acc;
    return;
  }
  W[q] = acc * kInv2Pi;
}

// W from the subtrees' partial sums in a fixed order (plain FP64: no
// re-evaluation list).
__global__ void hier_sum64_kernel(const double* __restrict__ part, int S, int64_t nQ,
                                  double* __restrict__ W) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nQ) return;
  double a = 0.0;
  for (int y = 0; y < S; ++y) a += part[(int64_t)y * nQ + q];
  W[q] = a * kInv2Pi;
}

// The top of the tree cut into at most S subtrees (breadth first; a leaf
// above the cut stays whole): ranges of pre-order positions.  One thread.
__global__ void frontier_kernel(const NodeH* __restrict__ nodes, int S, int2* __restrict__ ranges,
                                int* __restrict__ nranges) {
  auto end_of = [&](int y) {
    const int meta = __float_as_int(nodes[y].hi.w);
    return meta <= -2 ? y + 1 : __float_as_int(nodes[y].lo.w);
  };
  int cur[8], nxt[8];
  int nc = 1;
  cur[0] = 0;
  bool grew = true;
  while (grew && nc * 2 <= S) {
    grew = false;
    int m = 0;
    for (int i = 0; i < nc; ++i) {
      const int y = cur[i];
      if (__float_as_int(nodes[y].hi.w) <= -2) {
        nxt[m++] = y;
      } else {
        nxt[m++] = y + 1;
        nxt[m++] = end_of(y + 1);
        grew = true;
      }
    }
    for (int i = 0; i < m; ++i) cur[i] = nxt[i];
    nc = m;
  }
  for (int i = 0; i < nc; ++i) ranges[i] = make_int2(cur[i], end_of(cur[i]));
  *nranges = nc;
}

// W from the subtrees' partial sums (fixed order), and the FP64 re-check list.
__global__ void hier_sum_kernel(const double* __restrict__ part, int S, int64_t nQ,
                                double* __restrict__ W, int32_t* __restrict__ redo,
                                uint32_t* __restrict__ nredo) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nQ) return;
  double a = 0.0;
  for (int y = 0; y < S; ++y) a += part[(int64_t)y * nQ + q];
  const double w = a * kInv2Pi;
  W[q] = w;
  if (fabs(w - 0.5) <= kBand) redo[atomicAdd(nredo, 1u)] = (int32_t)q;
}



}  // namespace

void hier_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, HierTree& h,
                unsigned* status, cudaStream_t st, bool per_call) {
  if (per_call) {
    h.nodes.ordered(st);
    h.capn.ordered(st);
    h.caps.ordered(st);
    h.tris.ordered(st);
    h.tris64.ordered(st);
    h.box64.ordered(st);
    h.caps64.ordered(st);
  }
  h.V = V;
  h.nV = nV;
  h.F = F;
  h.nF = nF;
  h.n = (int)nF;
  if (nF == 0) return;
  GWN_REQUIRE(nF < (int64_t(1) << 29), "at most 2^29-1 triangles");
  GWN_REQUIRE(nV < (int64_t(1) << 31), "at most 2^31-1 vertices");
  const int n = (int)nF;
  const int nn = 2 * n - 1;
  PhaseTimer ph_all("hier_build", st);
  auto ph_part = std::make_unique<PhaseTimer>("hier_build_tree", st);
  DevBuf<unsigned long long> mm(6, st);
  init_minmax(mm.get(), 3, st);
  launch_kernel(mesh_bbox_kernel, std::min<unsigned>(nblk(nV), 1024u), kT, 0, st, V, nV, mm.get());
  // small host reads go through pinned words (a copy into pageable memory
  // is staged by the driver on every call)
  unsigned* pin = pinned_words();
  unsigned long long* mmh = reinterpret_cast<unsigned long long*>(pin);
  GWN_CUDA(cudaMemcpyAsync(mmh, mm.get(), 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           st));
  GWN_CUDA(cudaStreamSynchronize(st));
  double diag2 = 0;
  for (int d = 0; d < 3; ++d) {
    const double lo = from_ordered_bits(mmh[d]), hi = from_ordered_bits(mmh[3 + d]);
    h.lo[d] = lo;
    h.hi[d] = hi;
    h.c[d] = std::isfinite(lo) && std::isfinite(hi) ? 0.5 * (lo + hi) : 0.0;
    if (std::isfinite(hi - lo) && hi > lo) diag2 += (hi - lo) * (hi - lo);
  }
  h.eps = kNearFrac * std::sqrt(diag2);
  // Morton order of the triangles
  DevBuf<unsigned long long> key((size_t)n, st), key_t((size_t)n, st);
  DevBuf<int32_t> sorted((size_t)n, st), val_t((size_t)n, st);
  launch_kernel(tri_keys_kernel, nblk(n), kT, 0, st, V, nV, F, nF, (const unsigned long long*)mm.get(),
                key.get(), sorted.get(), status);
  radix_sort_pairs<unsigned long long>(key.get(), sorted.get(), key_t.get(), val_t.get(), n, 0, 30,
                                       st);
  // radix tree, sizes, boxes, pre-order
  DevBuf<int32_t> left((size_t)std::max(n - 1, 1), st), right((size_t)std::max(n - 1, 1), st),
      first((size_t)std::max(n - 1, 1), st), last((size_t)std::max(n - 1, 1), st),
      parent((size_t)nn, st), size((size_t)nn, st), pre((size_t)nn, st);
  DevBuf<double> box((size_t)nn * 6, st);
  DevBuf<unsigned> flags((size_t)std::max(n - 1, 1), st);
  flags.zero(st);
  if (n > 1)
    launch_kernel(radix_tree_kernel, nblk(n - 1), kT, 0, st, (const unsigned long long*)key.get(),
                  n, left.get(), right.get(), parent.get(), first.get(), last.get());
  launch_kernel(bottom_up_kernel, nblk(n), kT, 0, st, V, F, nV, (const int32_t*)sorted.get(), n,
                (const int32_t*)left.get(), (const int32_t*)right.get(),
                (const int32_t*)parent.get(), box.get(), size.get(), flags.get());
  launch_kernel(preorder_kernel, nblk(nn), kT, 0, st, (const int32_t*)left.get(),
                (const int32_t*)parent.get(), (const int32_t*)size.get(), nn, pre.get());
  // boundary records
  ph_part = std::make_unique<PhaseTimer>("hier_build_records", st);
  const int64_t m = 3 * (int64_t)n;
  DevBuf<unsigned long long> ekey((size_t)m, st), ekey_t((size_t)m, st);
  DevBuf<int32_t> eval((size_t)m, st), eval_t((size_t)m, st);
  DevBuf<uint32_t> ps((size_t)m + 1, st), cnt((size_t)m + 1, st);
  launch_kernel(edge_incidence_kernel, nblk(m), kT, 0, st, F, (const int32_t*)sorted.get(), n,
                nV, ekey.get(), eval.get());
  int vbits = 1;
  while (vbits < 31 && (int64_t(1) << vbits) < nV) ++vbits;
  // key = u << 32 | v: sort the low vbits of v, then of u
  radix_sort_pairs<unsigned long long>(ekey.get(), eval.get(), ekey_t.get(), eval_t.get(), m, 0,
                                       (vbits + 7) / 8 * 8, st);
  radix_sort_pairs<unsigned long long>(ekey.get(), eval.get(), ekey_t.get(), eval_t.get(), m, 32,
                                       32 + (vbits + 7) / 8 * 8, st);
  launch_kernel(sign_flags_kernel, nblk(m + 1), kT, 0, st, F, (const int32_t*)sorted.get(),
                (const int32_t*)eval.get(), m, ps.get());
  exclusive_scan_u32(ps.get(), ps.get(), m + 1, st);
  int64_t nrec = 0;
  if (n > 1) {
    launch_kernel(boundary_records_kernel<false>, nblk(m), kT, 0, st,
                  (const unsigned long long*)ekey.get(), (const int32_t*)eval.get(), m, n,
                  (const int32_t*)parent.get(), (const int32_t*)first.get(),
                  (const int32_t*)last.get(), (const int32_t*)pre.get(), (const uint32_t*)ps.get(),
                  cnt.get(), (const uint32_t*)nullptr, (int32_t*)nullptr, (int32_t*)nullptr,
                  (int32_t*)nullptr);
    GWN_CUDA(cudaMemsetAsync(cnt.get() + m, 0, sizeof(uint32_t), st));
    exclusive_scan_u32(cnt.get(), cnt.get(), m + 1, st);
    GWN_CUDA(cudaMemcpyAsync(pin + 12, cnt.get() + m, sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
    nrec = pin[12];
  }
  DevBuf<uint32_t> cap_off((size_t)nn, st), cap_cnt((size_t)nn, st);
  cap_off.zero(st);
  cap_cnt.zero(st);
  int64_t ncap = 0;
  DevBuf<int32_t> rnode, rinc, rnet, order, order_t, first_rec;
  DevBuf<uint32_t> mult;
  if (nrec > 0) {
    rnode.alloc((size_t)nrec, st);
    rinc.alloc((size_t)nrec, st);
    rnet.alloc((size_t)nrec, st);
    launch_kernel(boundary_records_kernel<true>, nblk(m), kT, 0, st,
                  (const unsigned long long*)ekey.get(), (const int32_t*)eval.get(), m, n,
                  (const int32_t*)parent.get(), (const int32_t*)first.get(),
                  (const int32_t*)last.get(), (const int32_t*)pre.get(), (const uint32_t*)ps.get(),
                  (uint32_t*)nullptr, (const uint32_t*)cnt.get(), rnode.get(), rinc.get(),
                  rnet.get());
    // records grouped by node (stable: edge order within a node)
    DevBuf<uint32_t> nk((size_t)nrec, st), nk_t((size_t)nrec, st);
    order.alloc((size_t)nrec, st);
    order_t.alloc((size_t)nrec, st);
    GWN_CUDA(cudaMemcpyAsync(nk.get(), rnode.get(), (size_t)nrec * 4, cudaMemcpyDeviceToDevice, st));
    int nbits = 1;
    while ((1 << nbits) < nn) ++nbits;
    launch_kernel(iota_records_kernel, nblk(nrec), kT, 0, st, order.get(), nrec);
    radix_sort_pairs<uint32_t>(nk.get(), order.get(), nk_t.get(), order_t.get(), nrec, 0, nbits, st);
    mult.alloc((size_t)nrec + 1, st);
    launch_kernel(record_mult_kernel, nblk(nrec + 1), kT, 0, st, (const int32_t*)rnet.get(),
                  (const int32_t*)order.get(), nrec, mult.get());
    exclusive_scan_u32(mult.get(), mult.get(), nrec + 1, st);
    GWN_CUDA(cudaMemcpyAsync(pin + 13, mult.get() + nrec, sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, st));
    first_rec.alloc((size_t)nn, st);
    launch_kernel(first_record_kernel, nblk(nrec), kT, 0, st, (const int32_t*)order.get(),
                  (const int32_t*)rnode.get(), nrec, first_rec.get(), (const uint32_t*)mult.get(),
                  cap_off.get());
    launch_kernel(cap_count_kernel, nblk(nrec), kT, 0, st, (const int32_t*)order.get(),
                  (const int32_t*)rnode.get(), nrec, (const uint32_t*)mult.get(),
                  (const uint32_t*)cap_off.get(), cap_cnt.get());
    GWN_CUDA(cudaStreamSynchronize(st));
    ncap = pin[13];
  }
  ph_part = std::make_unique<PhaseTimer>("hier_build_emit", st);
  h.nnodes = nn;
  h.ncap = ncap;
  h.nodes.alloc((size_t)nn * 2);
  h.capn.alloc((size_t)nn);
  h.caps.alloc((size_t)std::max<int64_t>(ncap, 1) * 4);
  h.tris.alloc((size_t)n * 4);
  h.tris64.alloc((size_t)n * 9);
  h.box64.alloc((size_t)nn * 6);
  h.caps64.alloc((size_t)std::max<int64_t>(ncap, 1) * 9);
  NodeH* nodes = reinterpret_cast<NodeH*>(h.nodes.get());
  TriH* caps = reinterpret_cast<TriH*>(h.caps.get());
  TriH* tris = reinterpret_cast<TriH*>(h.tris.get());
  if (ncap > 0)
    launch_kernel(cap_tris_kernel, nblk(nrec), kT, 0, st, V, F, (const int32_t*)sorted.get(),
                  (const unsigned long long*)ekey.get(), (const int32_t*)order.get(),
                  (const int32_t*)rnode.get(), (const int32_t*)rinc.get(),
                  (const int32_t*)rnet.get(), nrec, (const uint32_t*)mult.get(),
                  (const uint32_t*)cap_off.get(), (const int32_t*)first_rec.get(), h.c[0], h.c[1],
                  h.c[2], h.eps, caps, h.caps64.get());
  launch_kernel(node_records_kernel, nblk(nn), kT, 0, st, (const double*)box.get(),
                (const int32_t*)pre.get(), (const int32_t*)size.get(), n,
                (const uint32_t*)cap_off.get(), (const uint32_t*)cap_cnt.get(), h.c[0], h.c[1],
                h.c[2], h.eps, nodes, h.capn.get(), h.box64.get());
  launch_kernel(leaf_tris_kernel, nblk(n), kT, 0, st, V, F, nV, (const int32_t*)sorted.get(), n,
                h.c[0], h.c[1], h.c[2], h.eps, tris, h.tris64.get());
}

void hier_eval(const HierTree& h, const double* Q, int64_t nQ, double* W, cudaStream_t st,
               int precision) {
  if (nQ == 0) return;
  if (h.nF == 0) {
    GWN_CUDA(cudaMemsetAsync(W, 0, (size_t)nQ * 8, st));
    return;
  }
  GWN_REQUIRE(nQ < (int64_t(1) << 31), "at most 2^31-1 queries per call");
  QueryOrder qo;
  order_queries(Q, GWN_F64, nQ, h.lo, h.hi, qo, st);
  DevBuf<int32_t> redo((size_t)nQ, st);
  DevBuf<uint32_t> nredo(1, st);
  nredo.zero(st);
  const HierDev H{reinterpret_cast<const NodeH*>(h.nodes.get()), h.capn.get(),
                  reinterpret_cast<const TriH*>(h.caps.get()),
                  reinterpret_cast<const TriH*>(h.tris.get()), h.tris64.get(), (int)h.nnodes,
                  h.box64.get(), h.caps64.get()};
  // Too few queries to fill the GPU: each warp of queries walks one of up to
  // 8 subtrees (blockIdx.y), and the partial sums are added in a fixed order.
  const int64_t warps = (nQ + 31) / 32;
  const int64_t want = 3 * (int64_t)num_sms() * 32;
  int S = 1;
  while (S < kMaxSplit && warps * S < want) S *= 2;
  const int32_t* perm = qo.active ? qo.perm.get() : nullptr;
  if (precision == GWN_PLAIN_FP64) {
    PhaseTimer ph("hier_walk", st);
    if (S == 1) {
      launch_kernel(hier_walk64_kernel, nblk(nQ), kT, 0, st, H, Q, nQ, perm, W,
                    (const int2*)nullptr, (const int*)nullptr, (double*)nullptr);
    } else {
      DevBuf<int2> ranges(kMaxSplit, st);
      DevBuf<int> nranges(1, st);
      DevBuf<double> part((size_t)S * nQ, st);
      part.zero(st);
      launch_kernel(frontier_kernel, 1, 1, 0, st, H.nodes, S, ranges.get(), nranges.get());
      launch_kernel(hier_walk64_kernel, dim3(nblk(nQ), S), kT, 0, st, H, Q, nQ, perm, W,
                    (const int2*)ranges.get(), (const int*)nranges.get(), part.get());
      launch_kernel(hier_sum64_kernel, nblk(nQ), kT, 0, st, (const double*)part.get(), S, nQ, W);
    }
    return;
  }
  {
    PhaseTimer ph("hier_walk", st);
    if (S == 1) {
      launch_kernel(hier_walk_kernel<double>, nblk(nQ), kT, 0, st, H, Q, nQ,
                    (const int32_t*)(qo.active ? qo.perm.get() : nullptr), h.c[0], h.c[1],
                    h.c[2], W, redo.get(), nredo.get(), (const int2*)nullptr,
                    (const int*)nullptr, (double*)nullptr);
    } else {
      DevBuf<int2> ranges(kMaxSplit, st);
      DevBuf<int> nranges(1, st);
      DevBuf<double> part((size_t)S * nQ, st);
      part.zero(st);
      launch_kernel(frontier_kernel, 1, 1, 0, st, H.nodes, S, ranges.get(), nranges.get());
      launch_kernel(hier_walk_kernel<double>, dim3(nblk(nQ), S), kT, 0, st, H, Q, nQ,
                    (const int32_t*)(qo.active ? qo.perm.get() : nullptr), h.c[0], h.c[1],
                    h.c[2], W, redo.get(), nredo.get(), (const int2*)ranges.get(),
                    (const int*)nranges.get(), part.get());
      launch_kernel(hier_sum_kernel, nblk(nQ), kT, 0, st, (const double*)part.get(), S, nQ, W,
                    redo.get(), nredo.get());
    }
  }
  // FP64 all-pairs re-evaluation of the results within the band, one block
  // per listed query
  PhaseTimer ph("hier_refine", st);
  exact_refine_listed(h.tris64.get(), h.nF, Q, redo.get(), nredo.get(), W, st);
}

}  // namespace gwn
