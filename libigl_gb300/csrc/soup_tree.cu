// Binned top-down build of the triangle soup's binary tree.
//
// The reference builds its own 4-wide BVH on the CPU (UT_BVH<4>::init,
// include/igl/FastWindingNumberForSoups.h:4581-5800, a surface-area split
// search); the tree is an internal detail of the opaque FastWindingNumberBVH,
// and the walk's cost follows its shape: a node is opened when the query lies
// within beta * sqrt(maxPDist2) of the node's average point, so nodes with
// small, tight boxes are opened by fewer queries.  This builder splits every
// node where the children's boxes are smallest: the cost of a split is
// sum over the two sides of (triangles x squared box diagonal).  On the C2
// soup (1.3M triangles, beta 2) it takes 19% fewer node visits per query than
// the radix tree over Morton keys that this library built before.
//
//  * Segments of more than kSmall triangles, level by level: every triangle's
//    centroid is binned (kBins bins per axis over the segment's range) into
//    per-segment counts and vertex boxes; one warp per segment scans the
//    bins of each axis and picks the cheapest boundary; the triangles are
//    stably partitioned (device-wide scan).  A segment whose centroids all
//    fall into one bin on every axis, and every segment from level
//    kMedianLevel on, is split at its middle position instead.
//  * Segments of 2..kSmall triangles: one warp each sweeps every object
//    split on every axis exactly (triangles sorted by centroid) and recurses
//    with a stack in shared memory.
//
// Output, in the id scheme of the rest of soup.cu: leaf j is node n-1+j (slot
// j of vals), internal node ids are the split positions m-1 (between slots
// m-1 and m), with the root's id swapped with id 0 so that the root is 0.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <utility>

#include "gwn_common.cuh"
#include "soup.cuh"
#include "sort.cuh"

namespace gwn {

namespace {

constexpr int kBins = 32;         // one bin per lane of the split warp
constexpr int kSmall = 32;        // one triangle per lane of the small-segment warp
constexpr int kMedianLevel = 40;  // bounds the depth of the binned levels
constexpr int kMaxBinnedSegs = 1 << 18;  // a wider level splits at the median (bins <= 705 MB)

struct Seg {
  int l, r;            // slot range [l, r)
  int parent;          // internal node id of the parent, -1 for the root
  int side;            // 0: left child of the parent, 1: right child
  float lo[3], hi[3];  // binning range: contains every centroid of the segment
};

struct SplitRec {
  int axis;                  // -1: split at the middle position, order kept
  int bin;                   // left side = bins [0, bin) on axis
  int nl;                    // triangles on the left side
  int child[2];              // next level's segment index of each side, or -1
  float lo[2][3], hi[2][3];  // binning ranges of the two sides
};

__device__ __forceinline__ unsigned fkey(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fval(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Bin of centroid coordinate c in [lo, hi]; the same expression decides the
// bins and the partition.
__device__ __forceinline__ int bin_of(float c, float lo, float hi) {
  const float ext = hi - lo;
  if (!(ext > 0.f)) return 0;
  const int b = (int)((c - lo) * ((float)kBins / ext));
  return min(max(b, 0), kBins - 1);
}

__device__ __forceinline__ float diag2(const float* lo, const float* hi) {
  const float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
  return x * x + y * y + z * z;
}

__device__ __forceinline__ int node_id(int gap, int root_m) {
  const int kr = root_m - 1;
  return gap == kr ? 0 : (gap == 0 ? kr : gap);
}

__host__ __device__ inline double clamp_f32_range(double x) { return fmin(fmax(x, -3.0e38), 3.0e38); }

// FP32 centroid and vertex box of each kept triangle in slot order.
__global__ void bt_init_kernel(const double* __restrict__ V, int64_t nV,
                               const int32_t* __restrict__ F, const int32_t* __restrict__ vals,
                               int n, float4* __restrict__ rc,
                               float4* __restrict__ rlo, float4* __restrict__ rhi,
                               int* __restrict__ segid, int first_seg) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int32_t f = vals[p];
  double c[3] = {0, 0, 0}, lo[3], hi[3];
  for (int k = 0; k < 3; ++k) {
    int64_t v = F[(int64_t)f * 3 + k];
    if (v < 0 || v >= nV) v = 0;  // reported by the caller's own checks
    for (int d = 0; d < 3; ++d) {
      const double x = clamp_f32_range(V[v * 3 + d]);
      c[d] += x;
      lo[d] = k ? fmin(lo[d], x) : x;
      hi[d] = k ? fmax(hi[d], x) : x;
    }
  }
  rc[p] = make_float4((float)(c[0] / 3.0), (float)(c[1] / 3.0), (float)(c[2] / 3.0),
                      __int_as_float(f));
  rlo[p] = make_float4(__double2float_rd(lo[0]), __double2float_rd(lo[1]),
                       __double2float_rd(lo[2]), 0.f);
  rhi[p] = make_float4(__double2float_ru(hi[0]), __double2float_ru(hi[1]),
                       __double2float_ru(hi[2]), 0.f);
  segid[p] = first_seg;
}

__global__ void bt_root_kernel(Seg root, Seg* __restrict__ dst, unsigned* __restrict__ count) {
  dst[0] = root;
  if (count) *count = 1;
}

// Bin counts and vertex boxes per (segment, axis, bin).  Neighbouring slots
// mostly share a segment and a bin: each warp reduces the lanes of one key
// at a time and one lane issues the atomics.
__global__ void bt_bin_kernel(const float4* __restrict__ rc, const float4* __restrict__ rlo,
                              const float4* __restrict__ rhi, const int* __restrict__ segid, int n,
                              const Seg* __restrict__ segs, unsigned* __restrict__ cnt,
                              unsigned* __restrict__ blo, unsigned* __restrict__ bhi) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int p = base + threadIdx.x;
    const int s = p < n ? segid[p] : -1;
    float c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (s >= 0) {
      const float4 a = rc[p], b = rlo[p], h = rhi[p];
      c[0] = a.x; c[1] = a.y; c[2] = a.z;
      lo[0] = b.x; lo[1] = b.y; lo[2] = b.z;
      hi[0] = h.x; hi[1] = h.y; hi[2] = h.z;
    }
    for (int ax = 0; ax < 3; ++ax) {
      int key = -1;
      if (s >= 0) key = (s * 3 + ax) * kBins + bin_of(c[ax], segs[s].lo[ax], segs[s].hi[ax]);
      unsigned todo = __ballot_sync(full, key >= 0);
      while (todo) {
        const int leader = __ffs(todo) - 1;
        const int k = __shfl_sync(full, key, leader);
        const bool mine = key == k;
        const unsigned grp = __ballot_sync(full, mine);
        unsigned mn[3], mx[3];
        for (int d = 0; d < 3; ++d) {
          mn[d] = __reduce_min_sync(full, mine ? fkey(lo[d]) : 0xffffffffu);
          mx[d] = __reduce_max_sync(full, mine ? fkey(hi[d]) : 0u);
        }
        if (lane == leader) {
          atomicAdd(&cnt[k], (unsigned)__popc(grp));
          for (int d = 0; d < 3; ++d) {
            atomicMin(&blo[(int64_t)k * 3 + d], mn[d]);
            atomicMax(&bhi[(int64_t)k * 3 + d], mx[d]);
          }
        }
        todo &= ~grp;
      }
    }
  }
}

// One warp per segment: the cheapest bin boundary over the three axes (ties:
// lower axis, then lower boundary), else the middle position.
__global__ void bt_split_kernel(const Seg* __restrict__ segs, int S,
                                const unsigned* __restrict__ cnt, const unsigned* __restrict__ blo,
                                const unsigned* __restrict__ bhi, SplitRec* __restrict__ out,
                                int median_only) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (w >= S) return;
  const Seg sg = segs[w];
  const int n = sg.r - sg.l;
  float best = INFINITY;
  int bax = -1, bbin = 0, bnl = n / 2;
  float bl[2][3], bh[2][3];
  for (int d = 0; d < 3; ++d) {
    bl[0][d] = bl[1][d] = sg.lo[d];
    bh[0][d] = bh[1][d] = sg.hi[d];
  }
  for (int ax = 0; ax < 3 && !median_only; ++ax) {
    const int64_t k = ((int64_t)w * 3 + ax) * kBins + lane;
    const unsigned c = cnt[k];
    float lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = c ? fval(blo[k * 3 + d]) : INFINITY;
      hi[d] = c ? fval(bhi[k * 3 + d]) : -INFINITY;
    }
    // inclusive prefix (bins 0..lane) and suffix (bins lane..31)
    unsigned pc = c, sc = c;
    float pl[3], ph[3], sl[3], sh[3];
    for (int d = 0; d < 3; ++d) {
      pl[d] = sl[d] = lo[d];
      ph[d] = sh[d] = hi[d];
    }
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned uc = __shfl_up_sync(full, pc, off), dc = __shfl_down_sync(full, sc, off);
      if (lane >= off) pc += uc;
      if (lane + off < 32) sc += dc;
      for (int d = 0; d < 3; ++d) {
        const float ul = __shfl_up_sync(full, pl[d], off), uh = __shfl_up_sync(full, ph[d], off);
        const float dl = __shfl_down_sync(full, sl[d], off), dh = __shfl_down_sync(full, sh[d], off);
        if (lane >= off) {
          pl[d] = fminf(pl[d], ul);
          ph[d] = fmaxf(ph[d], uh);
        }
        if (lane + off < 32) {
          sl[d] = fminf(sl[d], dl);
          sh[d] = fmaxf(sh[d], dh);
        }
      }
    }
    // boundary after bin `lane`: left = prefix(lane), right = suffix(lane + 1)
    const unsigned rc_ = __shfl_down_sync(full, sc, 1);
    float rl[3], rh[3];
    for (int d = 0; d < 3; ++d) {
      rl[d] = __shfl_down_sync(full, sl[d], 1);
      rh[d] = __shfl_down_sync(full, sh[d], 1);
    }
    const bool valid = lane < 31 && pc > 0 && rc_ > 0;
    const float cost =
        valid ? (float)pc * diag2(pl, ph) + (float)rc_ * diag2(rl, rh) : INFINITY;
    float mc = cost;
    for (int off = 16; off > 0; off >>= 1) mc = fminf(mc, __shfl_xor_sync(full, mc, off));
    const unsigned win = __ballot_sync(full, valid && cost == mc);
    if (win && mc < best) {
      const int wl = __ffs(win) - 1;
      best = mc;
      bax = ax;
      bbin = wl + 1;
      bnl = (int)__shfl_sync(full, pc, wl);
      for (int d = 0; d < 3; ++d) {
        bl[0][d] = __shfl_sync(full, pl[d], wl);
        bh[0][d] = __shfl_sync(full, ph[d], wl);
        bl[1][d] = __shfl_sync(full, rl[d], wl);
        bh[1][d] = __shfl_sync(full, rh[d], wl);
      }
    }
  }
  if (lane == 0) {
    SplitRec x;
    x.axis = bax;
    x.bin = bbin;
    x.nl = bnl;
    x.child[0] = x.child[1] = -1;
    for (int s = 0; s < 2; ++s)
      for (int d = 0; d < 3; ++d) {
        x.lo[s][d] = bl[s][d];
        x.hi[s][d] = bh[s][d];
      }
    out[w] = x;
  }
}

// One thread per segment: the node's id and links, and the two children
// (leaf, small segment or next-level segment).
__global__ void bt_children_kernel(const Seg* __restrict__ segs, int S, SplitRec* __restrict__ sp,
                                   int n, Seg* __restrict__ next, unsigned* __restrict__ next_count,
                                   Seg* __restrict__ small, unsigned* __restrict__ small_count,
                                   int32_t* __restrict__ left, int32_t* __restrict__ right,
                                   int32_t* __restrict__ parent, int* __restrict__ root_m) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const Seg sg = segs[s];
  SplitRec& x = sp[s];
  const int m = sg.l + x.nl;
  int id;
  if (sg.parent < 0) {
    *root_m = m;
    id = 0;
  } else {
    id = node_id(m - 1, *root_m);
    (sg.side ? right : left)[sg.parent] = id;
    parent[id] = sg.parent;
  }
  for (int c = 0; c < 2; ++c) {
    const int a = c ? m : sg.l, b = c ? sg.r : m;
    x.child[c] = -1;
    if (b - a == 1) {
      const int leaf = n - 1 + a;
      (c ? right : left)[id] = leaf;
      parent[leaf] = id;
      continue;
    }
    Seg ch;
    ch.l = a;
    ch.r = b;
    ch.parent = id;
    ch.side = c;
    for (int d = 0; d < 3; ++d) {
      ch.lo[d] = x.lo[c][d];
      ch.hi[d] = x.hi[c][d];
    }
    if (b - a <= kSmall) {
      small[atomicAdd(small_count, 1u)] = ch;
    } else {
      const unsigned j = atomicAdd(next_count, 1u);
      next[j] = ch;
      x.child[c] = (int)j;
    }
  }
}

__global__ void bt_flag_kernel(const float4* __restrict__ rc, const int* __restrict__ segid, int n,
                               const Seg* __restrict__ segs, const SplitRec* __restrict__ sp,
                               uint32_t* __restrict__ flag) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int s = segid[p];
  uint32_t f = 0;
  if (s >= 0) {
    const SplitRec& x = sp[s];
    if (x.axis >= 0) {
      const float4 a = rc[p];
      const float c = x.axis == 0 ? a.x : (x.axis == 1 ? a.y : a.z);
      f = bin_of(c, segs[s].lo[x.axis], segs[s].hi[x.axis]) < x.bin;
    } else {
      f = (p - segs[s].l) < x.nl;
    }
  }
  flag[p] = f;
}

// Stable partition of every split segment (left side first); other slots
// are copied through.
__global__ void bt_scatter_kernel(const float4* __restrict__ rc, const float4* __restrict__ rlo,
                                  const float4* __restrict__ rhi, const int* __restrict__ segid,
                                  int n, const Seg* __restrict__ segs,
                                  const SplitRec* __restrict__ sp, const uint32_t* __restrict__ flag,
                                  const uint32_t* __restrict__ scan, float4* __restrict__ rc2,
                                  float4* __restrict__ rlo2, float4* __restrict__ rhi2,
                                  int* __restrict__ segid2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int s = segid[p];
  if (s < 0) {
    rc2[p] = rc[p];
    rlo2[p] = rlo[p];
    rhi2[p] = rhi[p];
    segid2[p] = -1;
    return;
  }
  const int l = segs[s].l;
  const SplitRec& x = sp[s];
  const int rl = (int)(scan[p] - scan[l]);
  const bool goes_left = flag[p] != 0;
  const int np = goes_left ? l + rl : l + x.nl + (p - l - rl);
  rc2[np] = rc[p];
  rlo2[np] = rlo[p];
  rhi2[np] = rhi[p];
  segid2[np] = x.child[goes_left ? 0 : 1];
}

__global__ void bt_vals_kernel(const float4* __restrict__ rc, int n, int32_t* __restrict__ vals) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) vals[p] = __float_as_int(rc[p].w);
}

// One warp per segment of 2..kSmall triangles, one triangle per lane: every
// object split on every axis is costed exactly; the chosen axis's centroid
// order becomes the slot order.
__global__ void __launch_bounds__(128) bt_small_kernel(const float4* __restrict__ rc,
                                                       const float4* __restrict__ rlo,
                                                       const float4* __restrict__ rhi,
                                                       const Seg* __restrict__ small, int nsmall,
                                                       int n, int32_t* __restrict__ vals,
                                                       int32_t* __restrict__ left,
                                                       int32_t* __restrict__ right,
                                                       int32_t* __restrict__ parent,
                                                       const int* __restrict__ root_m_dev) {
  __shared__ int4 stk[4][kSmall];
  __shared__ float xb[4][kSmall][10];
  const unsigned full = 0xffffffffu;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * 4 + wib;
  if (gw >= nsmall) return;
  const Seg sg = small[gw];
  const int len = sg.r - sg.l;
  float c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int tri = 0;
  if (lane < len) {
    const float4 a = rc[sg.l + lane], b = rlo[sg.l + lane], h = rhi[sg.l + lane];
    c[0] = a.x; c[1] = a.y; c[2] = a.z;
    tri = __float_as_int(a.w);
    lo[0] = b.x; lo[1] = b.y; lo[2] = b.z;
    hi[0] = h.x; hi[1] = h.y; hi[2] = h.z;
  }
  int root_m = sg.parent < 0 ? 0 : *root_m_dev;
  if (lane == 0) stk[wib][0] = make_int4(0, len, sg.parent, sg.side);
  int top = 1;
  __syncwarp();
  while (top > 0) {
    --top;
    const int4 e = stk[wib][top];
    const int a = e.x, b = e.y, k = b - a;
    const bool in = lane >= a && lane < b;
    float best = INFINITY;
    int bax = -1, bj = k / 2;
    int rk[3];
    for (int ax = 0; ax < 3; ++ax) {
      int r = 0;
      for (int j = a; j < b; ++j) {
        const float cj = __shfl_sync(full, c[ax], j);
        if (cj < c[ax] || (cj == c[ax] && j < lane)) ++r;
      }
      rk[ax] = r;
      __syncwarp();
      if (in)
        for (int d = 0; d < 3; ++d) {
          xb[wib][r][d] = lo[d];
          xb[wib][r][3 + d] = hi[d];
        }
      __syncwarp();
      float pl[3], ph[3];
      for (int d = 0; d < 3; ++d) {
        pl[d] = lane < k ? xb[wib][lane][d] : INFINITY;
        ph[d] = lane < k ? xb[wib][lane][3 + d] : -INFINITY;
      }
      float sl[3] = {pl[0], pl[1], pl[2]}, sh[3] = {ph[0], ph[1], ph[2]};
      for (int off = 1; off < 32; off <<= 1) {
        for (int d = 0; d < 3; ++d) {
          const float ul = __shfl_up_sync(full, pl[d], off), uh = __shfl_up_sync(full, ph[d], off);
          const float dl = __shfl_down_sync(full, sl[d], off),
                      dh = __shfl_down_sync(full, sh[d], off);
          if (lane >= off) {
            pl[d] = fminf(pl[d], ul);
            ph[d] = fmaxf(ph[d], uh);
          }
          if (lane + off < 32) {
            sl[d] = fminf(sl[d], dl);
            sh[d] = fmaxf(sh[d], dh);
          }
        }
      }
      float rl[3], rh[3];
      for (int d = 0; d < 3; ++d) {
        rl[d] = __shfl_down_sync(full, sl[d], 1);
        rh[d] = __shfl_down_sync(full, sh[d], 1);
      }
      // left = sorted 0..lane, right = sorted lane+1..k-1
      const bool valid = lane < k - 1;
      const float cost = valid ? (float)(lane + 1) * diag2(pl, ph) +
                                     (float)(k - 1 - lane) * diag2(rl, rh)
                               : INFINITY;
      float mc = cost;
      for (int off = 16; off > 0; off >>= 1) mc = fminf(mc, __shfl_xor_sync(full, mc, off));
      const unsigned win = __ballot_sync(full, valid && cost == mc);
      if (win && mc < best) {
        best = mc;
        bax = ax;
        bj = __ffs(win);
      }
    }
    // new order inside [a, b): the chosen axis's centroid order, else kept
    const int dst = a + (bax >= 0 ? rk[bax] : lane - a);
    __syncwarp();
    if (in) {
      float* o = xb[wib][dst];
      o[0] = c[0]; o[1] = c[1]; o[2] = c[2];
      o[3] = lo[0]; o[4] = lo[1]; o[5] = lo[2];
      o[6] = hi[0]; o[7] = hi[1]; o[8] = hi[2];
      o[9] = __int_as_float(tri);
    }
    __syncwarp();
    if (in) {
      const float* o = xb[wib][lane];
      c[0] = o[0]; c[1] = o[1]; c[2] = o[2];
      lo[0] = o[3]; lo[1] = o[4]; lo[2] = o[5];
      hi[0] = o[6]; hi[1] = o[7]; hi[2] = o[8];
      tri = __float_as_int(o[9]);
    }
    const int m = sg.l + a + bj;  // absolute split position
    int id;
    if (e.z < 0) {
      root_m = m;
      id = 0;
    } else {
      id = node_id(m - 1, root_m);
    }
    if (lane == 0) {
      if (e.z >= 0) {
        (e.w ? right : left)[e.z] = id;
        parent[id] = e.z;
      }
      int t = top;
      for (int side = 0; side < 2; ++side) {
        const int ra = side ? a + bj : a, rb = side ? b : a + bj;
        if (rb - ra == 1) {
          const int leaf = n - 1 + sg.l + ra;
          (side ? right : left)[id] = leaf;
          parent[leaf] = id;
        } else {
          stk[wib][t++] = make_int4(ra, rb, id, side);
        }
      }
    }
    top += (bj > 1) + (k - bj > 1);
    __syncwarp();
  }
  if (lane < len) vals[sg.l + lane] = tri;
}

}  // namespace

void soup_tree_build(const double* V, int64_t nV, const int32_t* F, int32_t* vals, int n,
                     const double* clo,
                     const double* chi, int32_t* left, int32_t* right, int32_t* parent,
                     cudaStream_t st) {
  if (n < 2) return;
  DevBuf<float4> rc((size_t)n, st), rlo((size_t)n, st), rhi((size_t)n, st);
  DevBuf<float4> rc2((size_t)n, st), rlo2((size_t)n, st), rhi2((size_t)n, st);
  DevBuf<int> segid((size_t)n, st), segid2((size_t)n, st);
  DevBuf<uint32_t> flag((size_t)n, st), scan((size_t)n, st);
  DevBuf<int> root_m(1, st);
  DevBuf<unsigned> counts(2, st);  // small segments, next level's segments
  counts.zero(st);
  const int max_small = n / 2 + 1;
  const int max_large = n / (kSmall + 1) + 1;
  DevBuf<Seg> small((size_t)max_small, st);
  DevBuf<Seg> segA((size_t)max_large, st), segB((size_t)max_large, st);
  DevBuf<SplitRec> sp((size_t)max_large, st);
  Seg root;
  root.l = 0;
  root.r = n;
  root.parent = -1;
  root.side = 0;
  for (int d = 0; d < 3; ++d) {
    root.lo[d] = (float)clamp_f32_range(clo[d]);
    root.hi[d] = (float)clamp_f32_range(chi[d]);
    if (!(root.lo[d] <= root.hi[d])) root.lo[d] = root.hi[d] = 0.f;
  }
  const bool large = n > kSmall;
  const unsigned gridN = (unsigned)((n + 255) / 256);
  launch_kernel(bt_init_kernel, gridN, 256, 0, st, V, nV, F, (const int32_t*)vals, n, rc.get(),
                rlo.get(), rhi.get(), segid.get(), large ? 0 : -1);
  if (large) {
    launch_kernel(bt_root_kernel, 1, 1, 0, st, root, segA.get(), (unsigned*)nullptr);
  } else {
    launch_kernel(bt_root_kernel, 1, 1, 0, st, root, small.get(), counts.get());
  }
  int S = large ? 1 : 0;
  const unsigned gridBin = (unsigned)std::min<int64_t>(gridN, (int64_t)num_sms() * 8);
  for (int level = 0; S > 0; ++level) {
    const bool median_only = level >= kMedianLevel || S > kMaxBinnedSegs;
    const size_t nb = median_only ? 0 : (size_t)S * 3 * kBins;
    DevBuf<unsigned> cnt(nb, st), blo(nb * 3, st), bhi(nb * 3, st);
    if (!median_only) {
      cnt.zero(st);
      GWN_CUDA(cudaMemsetAsync(blo.get(), 0xff, blo.bytes(), st));
      bhi.zero(st);
      launch_kernel(bt_bin_kernel, gridBin, 256, 0, st, (const float4*)rc.get(),
                    (const float4*)rlo.get(), (const float4*)rhi.get(), (const int*)segid.get(),
                    n, (const Seg*)segA.get(), cnt.get(), blo.get(), bhi.get());
    }
    launch_kernel(bt_split_kernel, (unsigned)((S + 3) / 4), 128, 0, st, (const Seg*)segA.get(), S,
                  (const unsigned*)cnt.get(), (const unsigned*)blo.get(),
                  (const unsigned*)bhi.get(), sp.get(), median_only ? 1 : 0);
    GWN_CUDA(cudaMemsetAsync(counts.get() + 1, 0, sizeof(unsigned), st));
    launch_kernel(bt_children_kernel, (unsigned)((S + 127) / 128), 128, 0, st,
                  (const Seg*)segA.get(), S, sp.get(), n, segB.get(), counts.get() + 1,
                  small.get(), counts.get(), left, right, parent, root_m.get());
    launch_kernel(bt_flag_kernel, gridN, 256, 0, st, (const float4*)rc.get(),
                  (const int*)segid.get(), n, (const Seg*)segA.get(), (const SplitRec*)sp.get(),
                  flag.get());
    exclusive_scan_u32(flag.get(), scan.get(), n, st);
    launch_kernel(bt_scatter_kernel, gridN, 256, 0, st, (const float4*)rc.get(),
                  (const float4*)rlo.get(), (const float4*)rhi.get(), (const int*)segid.get(), n,
                  (const Seg*)segA.get(), (const SplitRec*)sp.get(), (const uint32_t*)flag.get(),
                  (const uint32_t*)scan.get(), rc2.get(), rlo2.get(), rhi2.get(), segid2.get());
    std::swap(rc, rc2);
    std::swap(rlo, rlo2);
    std::swap(rhi, rhi2);
    std::swap(segid, segid2);
    std::swap(segA, segB);
    unsigned next = 0;
    GWN_CUDA(cudaMemcpyAsync(&next, counts.get() + 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                             st));
    GWN_CUDA(cudaStreamSynchronize(st));
    S = (int)next;
  }
  unsigned nsmall = 0;
  GWN_CUDA(cudaMemcpyAsync(&nsmall, counts.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  launch_kernel(bt_vals_kernel, gridN, 256, 0, st, (const float4*)rc.get(), n, vals);
  GWN_CUDA(cudaStreamSynchronize(st));
  if (nsmall)
    launch_kernel(bt_small_kernel, (nsmall + 3) / 4, 128, 0, st, (const float4*)rc.get(),
                  (const float4*)rlo.get(), (const float4*)rhi.get(), (const Seg*)small.get(),
                  (int)nsmall, n, vals, left, right, parent, (const int*)root_m.get());
}

}  // namespace gwn
