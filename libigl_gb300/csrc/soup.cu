// Triangle-soup fast winding number: GPU tree build, HDK moments, and a
// warp-coherent stackless Barnes-Hut traversal.
//
// Reference: UT_SolidAngle (include/igl/FastWindingNumberForSoups.h) behind
// igl::fast_winding_number(V,F,order,bvh) / (bvh,accuracy_scale,Q,W)
// (include/igl/fast_winding_number.cpp:380-455).  The reference builds a
// 4-wide SAH BVH on the CPU; the tree is an internal detail of the opaque
// FastWindingNumberBVH, so this path builds its own:
//
//  build (all on the device)
//   1. per triangle: FP64 bounding box and centroid; boxes with a non-finite
//      coordinate are excluded, as UT_BVH::init does (FWNFS.h:4606-4615);
//   2. 63-bit Morton key of the centroid, stable radix sort (the starting
//      order of the build);
//   3. binary tree, top-down: binned splits that minimise the children's
//      (triangles x squared box diagonal), exact object splits below 33
//      triangles (soup_tree.cu);
//   4. one bottom-up pass: each leaf computes the HDK per-triangle data
//      (area-weighted normal N, centroid P, the second-moment integrals
//      Nijk; FWNFS.h:6668-6890), and the second thread to reach an internal
//      node merges its two children with the parallel-axis shifts of
//      FWNFS.h:6892-7118, all accumulated in FP64;
//   5. pre-order positions (pre(child) = pre(parent) + 1 [+ size(left)]),
//      then the nodes are written in pre-order as 96-byte FP32 records and
//      192-byte FP64 records with a skip link (= end of subtree) or, for
//      leaves, the triangle slot.
//
//  evaluate
//   * queries are sorted by a 30-bit Morton key so that a warp's 32 queries
//     are close together; the warp walks the pre-order node array as one:
//     every lane evaluates the current node (a broadcast load) if it is
//     still interested in it (node >= its resume index); the warp moves to
//     node+1 when any lane opens the node, otherwise to the smallest resume
//     index of the warp.  No stack, no per-lane divergence in the walk;
//   * per node: open iff |q - P|^2 <= maxPDist2 * beta^2 (FWNFS.h:7176-7193);
//     the root is always opened; otherwise the order-0/1/2 far field of
//     FWNFS.h:7195-7251 is added (a non-finite value forces opening);
//     opened leaves add the exact triangle solid angle (FWNFS.h:6070-6110);
//   * mixed precision: FP32 records and arithmetic; the open test is redone
//     in FP64 whenever the FP32 margin is inside a proven error band, so the
//     mixed walk makes exactly the plain FP64 walk's decisions; exact
//     triangle terms within 1e-3 * bbox diagonal of the query are computed
//     from the original vertices with FP64 corner vectors, determinant and
//     denominator (the angle from FP32 atan2 of the scaled pair); results
//     within 1e-3 of 0.5 are recomputed by the plain FP64 walk.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "bh_common.cuh"
#include "gwn_common.cuh"
#include "soup.cuh"
#include "soup_walk.cuh"
#include "sort.cuh"

namespace gwn {

namespace {

constexpr double kNearFrac = 1e-3;
using soupwalk::EvalParams;
using soupwalk::kBand;
using soupwalk::kInv4Pi;

// Per-node FP64 build data (moments about the node's own average point P).
struct BuildM {
  double P[3], area, areaP[3], N[3], lo[3], hi[3];
  double Nii[3], Nxy, Nyx, Nyz, Nzy, Nzx, Nxz;
  double Niii[3], perm, c2[6];  // c2: 2Nxxy+Nyxx, 2Nxxz+Nzxx, 2Nyyz+Nzyy, 2Nyyx+Nxyy, 2Nzzx+Nxzz, 2Nzzy+Nyzz
};

// ------------------------------------------------------------- leaf data --
// HDK per-triangle data, FWNFS.h:6668-6890, in FP64.
__device__ void compute_integrals(const double* a, const double* b, const double* c,
                                  const double* P, double* ii, double* ij, double* ik, int i) {
  double oab[3], oac[3], ocb[3];
  for (int d = 0; d < 3; ++d) {
    oab[d] = b[d] - a[d];
    oac[d] = c[d] - a[d];
    ocb[d] = b[d] - c[d];
  }
  const double t = oab[i] / oac[i];
  const int j = (i == 2) ? 0 : (i + 1);
  const int k = (j == 2) ? 0 : (j + 1);
  const double jdiff = t * oac[j] - oab[j];
  const double kdiff = t * oac[k] - oab[k];
  double ca0 = jdiff * oab[k] - kdiff * oab[j], ca1 = kdiff * oab[i], ca2 = jdiff * oab[i];
  double cc0 = jdiff * ocb[k] - kdiff * ocb[j], cc1 = kdiff * ocb[i], cc2 = jdiff * ocb[i];
  const double asa = sqrt(ca0 * ca0 + ca1 * ca1 + ca2 * ca2);
  const double asc = sqrt(cc0 * cc0 + cc1 * cc1 + cc2 * cc2);
  const double Pai = a[i] - P[i], Pci = c[i] - P[i];
  const double ia = asa * (0.5 * Pai * Pai + (2.0 / 3.0) * Pai * oab[i] + 0.25 * oab[i] * oab[i]);
  const double ic = asc * (0.5 * Pci * Pci + (2.0 / 3.0) * Pci * ocb[i] + 0.25 * ocb[i] * ocb[i]);
  *ii = ia + ic;
  for (int pass = 0; pass < 2; ++pass) {
    double* out = pass == 0 ? ij : ik;
    const int jk = pass == 0 ? j : k;
    const double diff = pass == 0 ? jdiff : kdiff;
    if (!out) continue;
    const double obmid = b[jk] + 0.5 * diff;
    const double oabmid = obmid - a[jk];
    const double ocbmid = obmid - c[jk];
    const double Paj = a[jk] - P[jk], Pcj = c[jk] - P[jk];
    const double ija = asa * (0.5 * Pai * Paj + (1.0 / 3.0) * Pai * oabmid +
                              (1.0 / 3.0) * Paj * oab[i] + 0.25 * oab[i] * oabmid);
    const double ijc = asc * (0.5 * Pci * Pcj + (1.0 / 3.0) * Pci * ocbmid +
                              (1.0 / 3.0) * Pcj * ocb[i] + 0.25 * ocb[i] * ocbmid);
    *out = ija + ijc;
  }
}

__device__ void sort3_axis(const double* v[3], int axis, int o[3]) {
  o[0] = 0;
  o[1] = 1;
  o[2] = 2;
  int t;
  if (v[0][axis] > v[1][axis]) { t = o[0]; o[0] = o[1]; o[1] = t; }
  if (v[o[0]][axis] > v[2][axis]) { t = o[0]; o[0] = o[2]; o[2] = t; }
  if (v[o[1]][axis] > v[o[2]][axis]) { t = o[1]; o[1] = o[2]; o[2] = t; }
}

__device__ void leaf_moments(const double* a, const double* b, const double* c, int order,
                             BuildM& m) {
  double ab[3], ac[3];
  for (int d = 0; d < 3; ++d) {
    ab[d] = b[d] - a[d];
    ac[d] = c[d] - a[d];
    m.lo[d] = fmin(a[d], fmin(b[d], c[d]));
    m.hi[d] = fmax(a[d], fmax(b[d], c[d]));
  }
  m.N[0] = 0.5 * (ab[1] * ac[2] - ab[2] * ac[1]);
  m.N[1] = 0.5 * (ab[2] * ac[0] - ab[0] * ac[2]);
  m.N[2] = 0.5 * (ab[0] * ac[1] - ab[1] * ac[0]);
  const double area = sqrt(m.N[0] * m.N[0] + m.N[1] * m.N[1] + m.N[2] * m.N[2]);
  for (int d = 0; d < 3; ++d) {
    m.P[d] = (a[d] + b[d] + c[d]) / 3;
    m.areaP[d] = m.P[d] * area;
    m.Nii[d] = 0;
    m.Niii[d] = 0;
  }
  m.area = area;
  m.Nxy = m.Nyx = m.Nyz = m.Nzy = m.Nzx = m.Nxz = 0;
  m.perm = 0;
  for (int k = 0; k < 6; ++k) m.c2[k] = 0;
  if (order < 2 || area == 0) return;
  double n[3] = {m.N[0] / area, m.N[1] / area, m.N[2] / area};
  const double* v[3] = {a, b, c};
  int ox[3], oy[3], oz[3];
  sort3_axis(v, 0, ox);
  sort3_axis(v, 1, oy);
  sort3_axis(v, 2, oz);
  const double dx = v[ox[2]][0] - v[ox[0]][0];
  const double dy = v[oy[2]][1] - v[oy[0]][1];
  const double dz = v[oz[2]][2] - v[oz[0]][2];
  double xx = 0, xy = 0, yy = 0, yz = 0, zz = 0, zx = 0;
  if (dx > 0)
    compute_integrals(v[ox[0]], v[ox[1]], v[ox[2]], m.P, &xx, (dx >= dy && dy > 0) ? &xy : nullptr,
                      (dx >= dz && dz > 0) ? &zx : nullptr, 0);
  if (dy > 0)
    compute_integrals(v[oy[0]], v[oy[1]], v[oy[2]], m.P, &yy, (dy >= dz && dz > 0) ? &yz : nullptr,
                      (dx < dy && dx > 0) ? &xy : nullptr, 1);
  if (dz > 0)
    compute_integrals(v[oz[0]], v[oz[1]], v[oz[2]], m.P, &zz, (dx < dz && dx > 0) ? &zx : nullptr,
                      (dy < dz && dy > 0) ? &yz : nullptr, 2);
  m.Niii[0] = xx * n[0];
  m.Niii[1] = yy * n[1];
  m.Niii[2] = zz * n[2];
  m.perm = 2 * (n[0] * yz + n[1] * zx + n[2] * xy);
  m.c2[0] = 2 * (n[0] * xy) + n[1] * xx;
  m.c2[1] = 2 * (n[0] * zx) + n[2] * xx;
  m.c2[2] = 2 * (n[1] * yz) + n[2] * yy;
  m.c2[3] = 2 * (n[1] * xy) + n[0] * yy;
  m.c2[4] = 2 * (n[2] * zx) + n[0] * zz;
  m.c2[5] = 2 * (n[2] * yz) + n[1] * zz;
}

// Merge children (FWNFS.h:6892-7118 for two children).
__device__ void merge_moments(const BuildM& L, const BuildM& R, BuildM& m) {
  const BuildM* ch[2] = {&L, &R};
  m.area = L.area + R.area;
  for (int d = 0; d < 3; ++d) {
    m.N[d] = L.N[d] + R.N[d];
    m.areaP[d] = L.areaP[d] + R.areaP[d];
    m.lo[d] = fmin(L.lo[d], R.lo[d]);
    m.hi[d] = fmax(L.hi[d], R.hi[d]);
  }
  for (int d = 0; d < 3; ++d)
    m.P[d] = m.area > 0 ? m.areaP[d] / m.area : 0.5 * (m.lo[d] + m.hi[d]);
  for (int d = 0; d < 3; ++d) {
    m.Nii[d] = 0;
    m.Niii[d] = 0;
  }
  m.Nxy = m.Nyx = m.Nyz = m.Nzy = m.Nzx = m.Nxz = 0;
  m.perm = 0;
  for (int k = 0; k < 6; ++k) m.c2[k] = 0;
  for (int c = 0; c < 2; ++c) {
    const BuildM& C = *ch[c];
    const double dx = C.P[0] - m.P[0], dy = C.P[1] - m.P[1], dz = C.P[2] - m.P[2];
    const double* N = C.N;
    m.Nii[0] += C.Nii[0] + N[0] * dx;
    m.Nii[1] += C.Nii[1] + N[1] * dy;
    m.Nii[2] += C.Nii[2] + N[2] * dz;
    const double Nxy = C.Nxy + N[0] * dy, Nyx = C.Nyx + N[1] * dx;
    const double Nyz = C.Nyz + N[1] * dz, Nzy = C.Nzy + N[2] * dy;
    const double Nzx = C.Nzx + N[2] * dx, Nxz = C.Nxz + N[0] * dz;
    m.Nxy += Nxy;
    m.Nyx += Nyx;
    m.Nyz += Nyz;
    m.Nzy += Nzy;
    m.Nzx += Nzx;
    m.Nxz += Nxz;
    m.Niii[0] += C.Niii[0] + 2 * dx * C.Nii[0] + dx * dx * N[0];
    m.Niii[1] += C.Niii[1] + 2 * dy * C.Nii[1] + dy * dy * N[1];
    m.Niii[2] += C.Niii[2] + 2 * dz * C.Nii[2] + dz * dz * N[2];
    m.perm += C.perm + (dx * (Nyz + Nzy) + dy * (Nzx + Nxz) + dz * (Nxy + Nyx));
    m.c2[0] += C.c2[0] + 2 * (dy * C.Nii[0] + dx * C.Nxy + N[0] * dx * dy) + 2 * C.Nyx * dx +
               N[1] * dx * dx;
    m.c2[1] += C.c2[1] + 2 * (dz * C.Nii[0] + dx * C.Nxz + N[0] * dx * dz) + 2 * C.Nzx * dx +
               N[2] * dx * dx;
    m.c2[2] += C.c2[2] + 2 * (dz * C.Nii[1] + dy * C.Nyz + N[1] * dy * dz) + 2 * C.Nzy * dy +
               N[2] * dy * dy;
    m.c2[3] += C.c2[3] + 2 * (dx * C.Nii[1] + dy * C.Nyx + N[1] * dy * dx) + 2 * C.Nxy * dy +
               N[0] * dy * dy;
    m.c2[4] += C.c2[4] + 2 * (dx * C.Nii[2] + dz * C.Nzx + N[2] * dz * dx) + 2 * C.Nxz * dz +
               N[0] * dz * dz;
    m.c2[5] += C.c2[5] + 2 * (dy * C.Nii[2] + dz * C.Nzy + N[2] * dz * dy) + 2 * C.Nyz * dz +
               N[1] * dz * dz;
  }
}

// ------------------------------------------------------------ build kernels --
__global__ void tri_keys_kernel(const double* __restrict__ V, int64_t nV,
                                const int32_t* __restrict__ F, int64_t nF,
                                unsigned long long* __restrict__ cmm, int phase,
                                unsigned long long* __restrict__ keys, int32_t* __restrict__ vals,
                                unsigned* __restrict__ valid_count, unsigned* __restrict__ status) {
  const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool ok = f < nF;
  double cen[3] = {0, 0, 0};
  if (ok) {
    for (int c = 0; c < 3; ++c) {
      const int32_t idx = F[f * 3 + c];
      if (idx < 0 || idx >= nV) {
        atomicOr(status, kStatusBadInput);
        ok = false;
        break;
      }
      for (int d = 0; d < 3; ++d) {
        const double v = V[(int64_t)idx * 3 + d];
        if (!isfinite(v)) ok = false;
        cen[d] += v;
      }
    }
    for (int d = 0; d < 3; ++d) cen[d] /= 3.0;
  }
  if (phase == 0) {
    // centroid bounding box of the kept triangles
    for (int d = 0; d < 3; ++d) {
      double lo = ok ? cen[d] : INFINITY, hi = ok ? cen[d] : -INFINITY;
      for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      }
      if ((threadIdx.x & 31) == 0 && lo <= hi) {
        atomicMin(&cmm[d], ordered_bits(lo));
        atomicMax(&cmm[3 + d], ordered_bits(hi));
      }
    }
    return;
  }
  if (f >= nF) return;
  unsigned long long key = ~0ull;  // excluded triangles sort last
  if (ok) {
    key = 0;
    for (int d = 0; d < 3; ++d) {
      const double lo = from_ordered_bits(cmm[d]), hi = from_ordered_bits(cmm[3 + d]);
      const double ext = hi - lo;
      double t = ext > 0 ? (cen[d] - lo) / ext : 0.0;
      t = fmin(fmax(t, 0.0), 1.0);
      const unsigned long long q = (unsigned long long)fmin(t * 2097152.0, 2097151.0);
      key |= spread21(q) << (2 - d);
    }
    atomicAdd(valid_count, 1u);
  }
  keys[f] = key;
  vals[f] = (int32_t)f;
}

__global__ void bottom_up_kernel(const double* __restrict__ V, const int32_t* __restrict__ F,
                                 const int32_t* __restrict__ sorted_tri, int n, int order,
                                 const int32_t* __restrict__ left,
                                 const int32_t* __restrict__ right,
                                 const int32_t* __restrict__ parent, BuildM* __restrict__ M,
                                 int32_t* __restrict__ size, unsigned* __restrict__ flags,
                                 int32_t* __restrict__ depth_max) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int node = n - 1 + j;
  {
    const int32_t f = sorted_tri[j];
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
      a[d] = V[(int64_t)F[(int64_t)f * 3 + 0] * 3 + d];
      b[d] = V[(int64_t)F[(int64_t)f * 3 + 1] * 3 + d];
      c[d] = V[(int64_t)F[(int64_t)f * 3 + 2] * 3 + d];
    }
    BuildM m;
    leaf_moments(a, b, c, order, m);
    M[node] = m;
    size[node] = 1;
  }
  if (n == 1) return;
  int cur = node;
  int levels = 0;
  while (levels < n) {  // a tree over n leaves is less than n deep
    const int p = parent[cur];
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0) return;  // first child to arrive stops here
    __threadfence();
    const int lc = left[p], rc = right[p];
    BuildM m;
    merge_moments(M[lc], M[rc], m);
    M[p] = m;
    size[p] = 1 + size[lc] + size[rc];
    ++levels;
    if (p == 0) {
      atomicMax(depth_max, levels);
      return;
    }
    cur = p;
  }
}

// pre-order position of every node: walk up, adding 1 per level plus the
// left sibling's subtree size whenever the path enters a right child.
__global__ void preorder_kernel(const int32_t* __restrict__ left,
                                const int32_t* __restrict__ parent,
                                const int32_t* __restrict__ size, int nnodes, int root,
                                int32_t* __restrict__ pre, int32_t* __restrict__ depth,
                                int32_t* __restrict__ depth_max) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nnodes) return;
  int p = 0, dep = 0, cur = x;
  while (cur != root && dep < nnodes) {
    const int par = parent[cur];
    const int lc = left[par];
    p += 1 + (lc == cur ? 0 : size[lc]);
    ++dep;
    cur = par;
  }
  pre[x] = p;
  depth[x] = dep;
  atomicMax(depth_max, dep);
}

// Closest-point search nodes (see gwn_soup_impl::snode), one thread per
// internal node.
__global__ void search_nodes_kernel(const BuildM* __restrict__ M, const int32_t* __restrict__ left,
                                    const int32_t* __restrict__ right, int n,
                                    float4* __restrict__ snode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int l = left[i], r = right[i];
  const int ref_l = l >= n - 1 ? ~(l - (n - 1)) : l;
  const int ref_r = r >= n - 1 ? ~(r - (n - 1)) : r;
  const BuildM& ml = M[l];
  const BuildM& mr = M[r];
  float4* o = snode + 4 * (int64_t)i;
  o[0] = make_float4(__double2float_rd(ml.lo[0]), __double2float_rd(ml.lo[1]),
                     __double2float_rd(ml.lo[2]), __int_as_float(ref_l));
  o[1] = make_float4(__double2float_ru(ml.hi[0]), __double2float_ru(ml.hi[1]),
                     __double2float_ru(ml.hi[2]), __int_as_float(ref_r));
  o[2] = make_float4(__double2float_rd(mr.lo[0]), __double2float_rd(mr.lo[1]),
                     __double2float_rd(mr.lo[2]), 0.f);
  o[3] = make_float4(__double2float_ru(mr.hi[0]), __double2float_ru(mr.hi[1]),
                     __double2float_ru(mr.hi[2]), 0.f);
}

__global__ void emit_kernel(const BuildM* __restrict__ M, const int32_t* __restrict__ pre,
                            const int32_t* __restrict__ size, int n,
                            const double* __restrict__ V, const int32_t* __restrict__ F,
                            const int32_t* __restrict__ sorted_tri, SoupNodeF* __restrict__ nf,
                            SoupNodeD* __restrict__ nd, float4* __restrict__ tf,
                            double* __restrict__ td) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int nnodes = 2 * n - 1;
  if (x >= nnodes) return;
  const BuildM& m = M[x];
  const int p = pre[x];
  const bool leaf = x >= n - 1;
  double mp[3];
  for (int d = 0; d < 3; ++d) mp[d] = fmax(m.P[d] - m.lo[d], m.hi[d] - m.P[d]);
  const double maxP2 = mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2];
  const int slot = leaf ? (x - (n - 1)) : -1;
  const long long link = leaf ? (long long)~slot : (long long)(p + size[x]);
  SoupNodeD D;
  D.P[0] = m.P[0];
  D.P[1] = m.P[1];
  D.P[2] = m.P[2];
  D.maxP2 = maxP2;
  for (int d = 0; d < 3; ++d) {
    D.N[d] = m.N[d];
    D.Nii[d] = m.Nii[d];
    D.Niii[d] = m.Niii[d];
  }
  D.Nxy_yx = m.Nxy + m.Nyx;
  D.Nyz_zy = m.Nyz + m.Nzy;
  D.Nzx_xz = m.Nzx + m.Nxz;
  D.perm = m.perm;
  for (int k = 0; k < 6; ++k) D.c2[k] = m.c2[k];
  D.link = link;
  nd[p] = D;
  SoupNodeF Fr;
  Fr.a = make_float4((float)D.P[0], (float)D.P[1], (float)D.P[2], (float)maxP2);
  pack_far32(Fr, D.N, D.Nii, D.Nxy_yx, D.Nyz_zy, D.Nzx_xz, D.Niii, D.perm, D.c2, (int)link);
  nf[p] = Fr;
  if (leaf) {
    const int32_t f = sorted_tri[slot];
    double v[9];
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) v[c * 3 + d] = V[(int64_t)F[(int64_t)f * 3 + c] * 3 + d];
    for (int k = 0; k < 9; ++k) td[(int64_t)slot * 9 + k] = v[k];
    tf[(int64_t)slot * 3 + 0] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
    tf[(int64_t)slot * 3 + 1] = make_float4((float)v[4], (float)v[5], (float)v[6], (float)v[7]);
    tf[(int64_t)slot * 3 + 2] = make_float4((float)v[8], tri_screen_slack(v), 0.f, 0.f);
  }
}

// --------------------------------------------------------------- evaluate --
// Mixed-precision warp-coherent walk.  One query per lane.  kStats builds
// an instrumented copy that counts its work into `stats` (see
// gwn_soup_walk_stats); the timed kernel is the kStats = false instance.
template <typename QT, typename WT, bool kStats = false, int kTree = -1>
__global__ void __launch_bounds__(128, 8) soup_eval_mixed_kernel(EvalParams prm, const QT* __restrict__ Q,
                                                              const int32_t* __restrict__ perm,
                                                              int64_t nQ, WT* __restrict__ W,
                                                              int32_t* __restrict__ refine_list,
                                                              unsigned* __restrict__ refine_count,
                                                              unsigned long long* __restrict__ stats = nullptr) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool valid = i < nQ;
  int64_t qi = 0;
  double qx = 0, qy = 0, qz = 0;
  if (valid) soupwalk::read_query(Q, perm, (const int32_t*)nullptr, i, qi, qx, qy, qz);
  __shared__ soupwalk::NearQueue near_q[4];
  float acc;
  double acc64;
  soupwalk::WalkCounters c;
  soupwalk::walk_mixed<kStats, kTree>(prm, valid, qx, qy, qz, acc, acc64, c,
                                      near_q[threadIdx.x >> 5]);
  if (kStats) {
    if ((threadIdx.x & 31) == 0) atomicAdd(&stats[0], c.steps);
    atomicAdd(&stats[1], c.visits);
    atomicAdd(&stats[2], c.far);
    atomicAdd(&stats[3], c.exact32);
    atomicAdd(&stats[4], c.exact64);
    atomicAdd(&stats[5], c.recheck);
  }
  if (!valid) return;
  const double w = soupwalk::mixed_result(acc, acc64);
  __stcs(&W[qi], (WT)w);  // written once, read by no later warp: evict first
  if (fabs(w - 0.5) <= kBand) {
    const unsigned s = atomicAdd(refine_count, 1u);
    refine_list[s] = (int32_t)qi;
  }
}

// Plain FP64 walk (also used, over a list, to re-evaluate threshold queries).
template <typename QT, typename WT>
__global__ void __launch_bounds__(128) soup_eval_fp64_kernel(EvalParams prm, const QT* __restrict__ Q,
                                                             const int32_t* __restrict__ perm,
                                                             const int32_t* __restrict__ list,
                                                             const unsigned* __restrict__ list_count,
                                                             int64_t nQ, WT* __restrict__ W) {
  const int64_t n = list ? (int64_t)*list_count : nQ;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (list && blockIdx.x * (int64_t)blockDim.x >= n) return;  // whole warp idle
  const bool valid = i < n;
  int64_t qi = 0;
  double qx = 0, qy = 0, qz = 0;
  if (valid) soupwalk::read_query(Q, perm, list, i, qi, qx, qy, qz);
  __shared__ soupwalk::Fp64Queue fp64_q[4];
  const double acc = soupwalk::walk_fp64(prm, valid, qx, qy, qz, fp64_q[threadIdx.x >> 5]);
  if (valid) W[qi] = (WT)(acc * kInv4Pi);
}

__global__ void moments_bounded_kernel(const SoupNodeD* __restrict__ nd, int64_t n,
                                       unsigned* __restrict__ unbounded) {
  const int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool bad = false;
  if (x < n) {
    const double* m = nd[x].N;  // N .. c2: the 19 moments after P, maxP2
    for (int k = 0; k < 19; ++k) bad |= !(fabs(m[k]) <= 1e100);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(unbounded, 1u);
}

template <typename WT>
__global__ void fill_zero_kernel(WT* w, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) w[i] = WT(0);
}

}  // namespace

// ------------------------------------------------------------------ build --
void soup_check_moments(gwn_soup_impl& s, cudaStream_t st) {
  s.moments_bounded = true;
  if (s.nnodes == 0) return;
  static_assert(offsetof(SoupNodeD, c2) + 6 * sizeof(double) - offsetof(SoupNodeD, N) ==
                    19 * sizeof(double),
                "the 19 moments are contiguous");
  DevBuf<unsigned> flag(1, st);
  flag.zero(st);
  launch_kernel(moments_bounded_kernel, (unsigned)((s.nnodes + 255) / 256), 256, 0, st,
                (const SoupNodeD*)s.nd.get(), s.nnodes, flag.get());
  unsigned h = 0;
  GWN_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(h), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  s.moments_bounded = h == 0;
}

void soup_build(gwn_soup_impl& s, const double* V, int64_t nV, const int32_t* F, int64_t nF,
                int order, bool host_mode, cudaStream_t st) {
  GWN_REQUIRE(order >= 0 && order <= 2, "order must be 0, 1 or 2");
  GWN_REQUIRE(nF < (int64_t(1) << 30), "at most 2^30 triangles");
  s.order = order;
  s.n_input = nF;
  DeviceStatus status(st, host_mode);
  DevBuf<unsigned long long> cmm(6, st);
  init_minmax(cmm.get(), 3, st);
  DevBuf<unsigned long long> keys((size_t)std::max<int64_t>(nF, 1), st),
      keys_tmp((size_t)std::max<int64_t>(nF, 1), st);
  DevBuf<int32_t> vals((size_t)std::max<int64_t>(nF, 1), st),
      vals_tmp((size_t)std::max<int64_t>(nF, 1), st);
  DevBuf<unsigned> counters(2, st);
  counters.zero(st);
  const unsigned gridF = (unsigned)std::max<int64_t>(1, (nF + 255) / 256);
  if (nF > 0) {
    launch_kernel(tri_keys_kernel, gridF, 256, 0, st, V, nV, F, nF, cmm.get(), 0, keys.get(), vals.get(),
                                           counters.get(), status.ptr());
    launch_kernel(tri_keys_kernel, gridF, 256, 0, st, V, nV, F, nF, cmm.get(), 1, keys.get(), vals.get(),
                                           counters.get(), status.ptr());
    GWN_CUDA(cudaGetLastError());
    radix_sort_pairs<unsigned long long>(keys.get(), vals.get(), keys_tmp.get(), vals_tmp.get(), nF,
                                         0, 64, st);
  }
  unsigned nvalid = 0;
  unsigned long long cmm_h[6];
  GWN_CUDA(cudaMemcpyAsync(&nvalid, counters.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaMemcpyAsync(cmm_h, cmm.get(), sizeof(cmm_h), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  if (host_mode) status.check(st, "soup_build");
  const int n = (int)nvalid;
  s.n = n;
  double lo[3], hi[3], diag2 = 0, cmax = 0;
  for (int d = 0; d < 3; ++d) {
    lo[d] = from_ordered_bits(cmm_h[d]);
    hi[d] = from_ordered_bits(cmm_h[3 + d]);
    if (n == 0) lo[d] = hi[d] = 0;
    s.lo[d] = lo[d];
    s.hi[d] = hi[d];
  }
  if (n == 0) {
    s.nnodes = 0;
    return;
  }
  const int nnodes = 2 * n - 1;
  s.nnodes = nnodes;
  DevBuf<int32_t> left((size_t)std::max(n - 1, 1), st), right((size_t)std::max(n - 1, 1), st);
  DevBuf<int32_t> parent((size_t)nnodes, st), size((size_t)nnodes, st), pre((size_t)nnodes, st),
      depth((size_t)nnodes, st);
  DevBuf<unsigned> flags((size_t)std::max(n - 1, 1), st);
  flags.zero(st);
  DevBuf<BuildM> M((size_t)nnodes, st);
  DevBuf<int32_t> dmax(1, st);
  dmax.zero(st);
  soup_tree_build(V, nV, F, vals.get(), n, lo, hi, left.get(), right.get(), parent.get(), st);
  launch_kernel(bottom_up_kernel, (n + 127) / 128, 128, 0, st, V, F, vals.get(), n, order, left.get(),
                                                    right.get(), parent.get(), M.get(), size.get(),
                                                    flags.get(), dmax.get());
  GWN_CUDA(cudaGetLastError());
  launch_kernel(preorder_kernel, (nnodes + 255) / 256, 256, 0, st, left.get(), parent.get(), size.get(),
                                                        nnodes, 0, pre.get(),
                                                        depth.get(), dmax.get());
  GWN_CUDA(cudaGetLastError());
  s.tri_index.alloc((size_t)n);
  GWN_CUDA(cudaMemcpyAsync(s.tri_index.get(), vals.get(), (size_t)n * sizeof(int32_t),
                           cudaMemcpyDeviceToDevice, st));
  s.nf.alloc((size_t)nnodes);
  // the walk reads records with 256-bit loads
  if (reinterpret_cast<uintptr_t>(s.nf.get()) % 32)
    throw Error(GWN_ERR_INTERNAL, "node records are not 32-byte aligned");
  s.nd.alloc((size_t)nnodes);
  s.tf.alloc((size_t)n * 3);
  s.td.alloc((size_t)n * 9);
  s.snode.alloc((size_t)std::max(n - 1, 1) * 4);
  if (n > 1)
    launch_kernel(search_nodes_kernel, (n - 1 + 255) / 256, 256, 0, st, (const BuildM*)M.get(),
                  (const int32_t*)left.get(), (const int32_t*)right.get(), n, s.snode.get());
  launch_kernel(emit_kernel, (nnodes + 255) / 256, 256, 0, st, M.get(), pre.get(), size.get(), n, V, F,
                                                    vals.get(), s.nf.get(), s.nd.get(), s.tf.get(),
                                                    s.td.get());
  GWN_CUDA(cudaGetLastError());
  int dm = 0;
  BuildM root;
  GWN_CUDA(cudaMemcpyAsync(&dm, dmax.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaMemcpyAsync(&root, M.get(), sizeof(BuildM), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  s.max_depth = dm;
  // The root box bounds every kept vertex; node average points lie inside it.
  for (int d = 0; d < 3; ++d) {
    s.lo[d] = root.lo[d];
    s.hi[d] = root.hi[d];
    const double e = root.hi[d] - root.lo[d];
    diag2 += e * e;
    cmax = fmax(cmax, fmax(fabs(root.lo[d]), fabs(root.hi[d])));
  }
  s.eps = kNearFrac * sqrt(diag2);
  s.cmax = cmax;
  soup_check_moments(s, st);
  s.bytes = s.nf.bytes() + s.nd.bytes() + s.tf.bytes() + s.td.bytes() + s.tri_index.bytes() +
            s.snode.bytes();
}

// ------------------------------------------------------------------- eval --
template <typename QT, typename WT>
static void soup_eval_t(const gwn_soup_impl& s, float beta, const void* Qv, int64_t nQ, void* Wv,
                        int precision, cudaStream_t st) {
  const QT* Q = static_cast<const QT*>(Qv);
  WT* W = static_cast<WT*>(Wv);
  if (nQ == 0) return;
  if (s.nnodes == 0) {
    launch_kernel(fill_zero_kernel<WT>, (unsigned)((nQ + 255) / 256), 256, 0, st, W, nQ);
    GWN_CUDA(cudaGetLastError());
    return;
  }
  EvalParams prm;
  prm.nf = s.nf.get();
  prm.nd = s.nd.get();
  prm.tf = s.tf.get();
  prm.td = s.td.get();
  prm.nnodes = (int)s.nnodes;
  prm.order = s.order;
  prm.beta2f = beta * beta;
  prm.beta2d = (double)beta * (double)beta;
  prm.eps = (float)s.eps;
  prm.cmax = (float)s.cmax;
  prm.status = nullptr;
  prm.ref32 = s.tree == GWN_TREE_REFERENCE;
  prm.fp64_queue = s.moments_bounded;
  QueryOrder qo;
  {
    PhaseTimer ph("order_queries", st);
    order_queries(Qv, sizeof(QT) == 8 ? GWN_F64 : GWN_F32, nQ, s.lo, s.hi, qo, st);
  }
  const int32_t* perm = qo.active ? qo.perm.get() : nullptr;
  const unsigned grid = (unsigned)((nQ + 127) / 128);
  if (precision == GWN_MIXED) {
    DevBuf<int32_t> list((size_t)nQ, st);
    DevBuf<unsigned> count(1, st);
    count.zero(st);
    {
      PhaseTimer ph("walk", st);
      // the tree kind is fixed per launch: the reference tree's instance
      // carries no FP64 re-check code
      auto kernel = prm.ref32 ? soup_eval_mixed_kernel<QT, WT, false, GWN_TREE_REFERENCE>
                              : soup_eval_mixed_kernel<QT, WT, false, GWN_TREE_BINNED>;
      launch_kernel(kernel, grid, 128, 0, st, prm, Q, perm, nQ, W, list.get(), count.get(),
                    (unsigned long long*)nullptr);
    }
    GWN_CUDA(cudaGetLastError());
    {
      PhaseTimer ph("refine", st);
      launch_kernel(soup_eval_fp64_kernel<QT, WT>, grid, 128, 0, st, prm, Q, nullptr, list.get(),
                                                          count.get(), nQ, W);
    }
    GWN_CUDA(cudaGetLastError());
  } else {
    PhaseTimer ph("walk", st);
    launch_kernel(soup_eval_fp64_kernel<QT, WT>, grid, 128, 0, st, prm, Q, perm, nullptr, nullptr, nQ, W);
    GWN_CUDA(cudaGetLastError());
  }
}

void soup_walk_stats(const gwn_soup_impl& s, float beta, const double* Q, int64_t nQ,
                     unsigned long long* out7, cudaStream_t st) {
  for (int k = 0; k < 7; ++k) out7[k] = 0;
  if (nQ == 0 || s.nnodes == 0) return;
  EvalParams prm;
  prm.nf = s.nf.get();
  prm.nd = s.nd.get();
  prm.tf = s.tf.get();
  prm.td = s.td.get();
  prm.nnodes = (int)s.nnodes;
  prm.order = s.order;
  prm.beta2f = beta * beta;
  prm.beta2d = (double)beta * (double)beta;
  prm.eps = (float)s.eps;
  prm.cmax = (float)s.cmax;
  prm.status = nullptr;
  prm.ref32 = s.tree == GWN_TREE_REFERENCE;
  prm.fp64_queue = s.moments_bounded;
  QueryOrder qo;
  order_queries(Q, GWN_F64, nQ, s.lo, s.hi, qo, st);
  DevBuf<double> W((size_t)nQ, st);
  DevBuf<int32_t> list((size_t)nQ, st);
  DevBuf<unsigned> count(1, st);
  DevBuf<unsigned long long> stats(7, st);
  count.zero(st);
  stats.zero(st);
  launch_kernel(soup_eval_mixed_kernel<double, double, true>, (unsigned)((nQ + 127) / 128), 128, 0,
                st, prm, Q, qo.active ? qo.perm.get() : nullptr, nQ, W.get(), list.get(),
                count.get(), stats.get());
  unsigned c = 0;
  GWN_CUDA(cudaMemcpyAsync(out7, stats.get(), 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaMemcpyAsync(&c, count.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  GWN_CUDA(cudaStreamSynchronize(st));
  out7[6] = c;
}

void soup_eval(const gwn_soup_impl& s, float beta, const void* Q, int q_dtype, int64_t nQ, void* W,
               int w_dtype, int precision, cudaStream_t st) {
  const bool qd = q_dtype == GWN_F64, wd = w_dtype == GWN_F64;
  if (qd && wd) soup_eval_t<double, double>(s, beta, Q, nQ, W, precision, st);
  else if (qd) soup_eval_t<double, float>(s, beta, Q, nQ, W, precision, st);
  else if (wd) soup_eval_t<float, double>(s, beta, Q, nQ, W, precision, st);
  else soup_eval_t<float, float>(s, beta, Q, nQ, W, precision, st);
}

}  // namespace gwn
