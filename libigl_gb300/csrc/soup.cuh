// Device layout of a built triangle soup (the state behind gwn_soup).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "gwn_common.cuh"

namespace gwn {

// 96-byte FP32 node record, read by the mixed-precision walk.
//   a: P (average point) xyz, maxPDist2
//   b: N xyz, A_xx     c: A_yy, A_zz, A_xy, A_xz     d: A_yz, K_xxx, K_yyy, K_zzz
//   e: K_xxy, K_xxz, K_xyy, K_yyz     f: K_xzz, K_yzz, K_xyz, link (int bits)
// A and K are the coefficients of the far field's order-1 quadratic and
// order-2 cubic forms in the unit direction (pack_far32 below).
// link >= 0: internal node, index one past its subtree (pre-order);
// link < 0: leaf, triangle slot ~link.
struct __align__(32) SoupNodeF {
  float4 a, b, c, d, e, f;
};
static_assert(sizeof(SoupNodeF) == 96, "96-byte records: a..b, c..d, e..f are 32-byte aligned");

// The far field of FWNFS.h:7195-7251 with q = (x - P)/|x - P|,
// m1 = 1/|x - P|, m2 = m1^2:
//   omega = -m2 q.N
//         + m2 m1 (S - 3 (sum_i q_i^2 Nii + q_x q_y Nxy_yx + ...))          (order 1)
//         + m2 m1^2 (1.5 q.L - 7.5 (sum_i q_i^3 Niii + q_x q_y q_z perm + ...)) (order 2)
// with S = Nxx + Nyy + Nzz and L_i = 3 Niii + the two c2 sums of FWNFS.h:
// 7228-7233.  Since |q| = 1, S = S |q|^2 and q.L = (q.L)|q|^2, so the order-1
// bracket is a quadratic form A(q) and the order-2 bracket a cubic form K(q):
//   omega = m2 (m1 (A(q) + m1 K(q)) - q.N),
// 6 + 10 coefficients in place of the 9 + 10 moments, and about half the
// operations per evaluation.  The coefficients are formed here in FP64 from
// the node's moments and rounded once.
__host__ __device__ inline void pack_far32(SoupNodeF& R, const double N[3], const double Nii[3],
                                           double Nxy_yx, double Nyz_zy, double Nzx_xz,
                                           const double Niii[3], double perm, const double c2[6],
                                           int link) {
  const double S = Nii[0] + Nii[1] + Nii[2];
  const double Lx = 3 * Niii[0] + (c2[3] + c2[4]);
  const double Ly = 3 * Niii[1] + (c2[5] + c2[0]);
  const double Lz = 3 * Niii[2] + (c2[1] + c2[2]);
  R.b = make_float4((float)N[0], (float)N[1], (float)N[2], (float)(S - 3 * Nii[0]));
  R.c = make_float4((float)(S - 3 * Nii[1]), (float)(S - 3 * Nii[2]), (float)(-3 * Nxy_yx),
                    (float)(-3 * Nzx_xz));
  R.d = make_float4((float)(-3 * Nyz_zy), (float)(1.5 * Lx - 7.5 * Niii[0]),
                    (float)(1.5 * Ly - 7.5 * Niii[1]), (float)(1.5 * Lz - 7.5 * Niii[2]));
  R.e = make_float4((float)(1.5 * Ly - 7.5 * c2[0]), (float)(1.5 * Lz - 7.5 * c2[1]),
                    (float)(1.5 * Lx - 7.5 * c2[3]), (float)(1.5 * Lz - 7.5 * c2[2]));
  float lf;
  memcpy(&lf, &link, sizeof(float));
  R.f = make_float4((float)(1.5 * Lx - 7.5 * c2[4]), (float)(1.5 * Ly - 7.5 * c2[5]),
                    (float)(-7.5 * perm), lf);
}

// 192-byte FP64 node record (plain FP64 walk, FP64 re-checks).
struct __align__(16) SoupNodeD {
  double P[3], maxP2;
  double N[3], Nii[3];
  double Nxy_yx, Nyz_zy, Nzx_xz;
  double Niii[3], perm, c2[6];
  long long link;
};

#ifdef __CUDACC__
// Error slack of the FP32 closest-point screen for one triangle (v: three
// FP64 corners; distance.cu): 32 u (|e1|^2 |e2|^2 / |e1 x e2|^2) L + 8 u
// max|v|, u = 2^-24, L the longest edge; infinite for a (near) degenerate one.
__device__ inline float tri_screen_slack(const double* v) {
  double e1[3], e2[3], e3[3], cr[3];
  double l1 = 0, l2 = 0, l3 = 0, vm = 0;
  for (int d = 0; d < 3; ++d) {
    e1[d] = v[3 + d] - v[d];
    e2[d] = v[6 + d] - v[d];
    e3[d] = v[6 + d] - v[3 + d];
    l1 += e1[d] * e1[d];
    l2 += e2[d] * e2[d];
    l3 += e3[d] * e3[d];
    vm = fmax(vm, fmax(fabs(v[d]), fmax(fabs(v[3 + d]), fabs(v[6 + d]))));
  }
  cr[0] = e1[1] * e2[2] - e1[2] * e2[1];
  cr[1] = e1[2] * e2[0] - e1[0] * e2[2];
  cr[2] = e1[0] * e2[1] - e1[1] * e2[0];
  const double den = cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2];
  const double cond = den > 0 ? l1 * l2 / den : INFINITY;
  const double u = 5.9604644775390625e-08;
  if (cond < 1e6) return (float)(32 * u * cond * sqrt(fmax(l1, fmax(l2, l3))) + 8 * u * vm);
  return INFINITY;
}
#endif

struct gwn_soup_impl {
  int device = 0;
  int order = 2;
  // GWN_TREE_REFERENCE: the reference's 4-wide tree (soup_ref.cu), whose
  // open test is the reference's FP32 one; GWN_TREE_BINNED: the binary
  // tree of soup_tree.cu.
  int tree = GWN_TREE_BINNED;
  int64_t ref_nodes = 0;       // nodes of the 4-wide tree (reference numbering)
  DevMem<uint32_t> ref_child;  // 4 lanes per node, the reference's encoding
  int64_t n_input = 0;   // triangles passed in
  int64_t n = 0;         // triangles kept (finite, valid)
  int64_t nnodes = 0;    // 2n-1
  int max_depth = 0;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // bbox of kept vertices
  double eps = 0;        // near-field distance: 1e-3 * bbox diagonal
  double cmax = 0;       // max |coordinate| inside the bbox
  DevMem<SoupNodeF> nf;
  DevMem<SoupNodeD> nd;
  DevMem<float4> tf;     // 3 float4 per slot: a.xyz b.x | b.yz c.xy | c.z
  DevMem<double> td;     // 9 doubles per slot
  DevMem<int32_t> tri_index;  // input triangle id per slot
  // Closest-point search nodes, one per internal node of the binary tree in
  // build order (root 0): 4 float4 = boxes of the two children, rounded
  // outward to FP32, and the children (internal index, or ~slot for a leaf):
  //   {lo_l.xyz, left}, {hi_l.xyz, right}, {lo_r.xyz, 0}, {hi_r.xyz, 0}.
  DevMem<float4> snode;
  // every FP64 moment finite and within 1e100 in magnitude: then no far
  // field at |q - P|^2 >= 1e-100 can overflow, and the plain FP64 walk may
  // queue its far fields (soup_walk.cuh)
  bool moments_bounded = false;
  size_t bytes = 0;
};

// Binary tree over the n triangles vals[0..n) (soup_tree.cu): on return
// vals holds the leaf (slot) order; internal nodes are 0..n-2 (root 0) and
// leaf j is node n-1+j; clo/chi bound the triangles' centroids.  Vertex
// indices outside [0, nV) read vertex 0 (callers report them).
void soup_tree_build(const double* V, int64_t nV, const int32_t* F, int32_t* vals, int n,
                     const double* clo, const double* chi, int32_t* left, int32_t* right,
                     int32_t* parent, cudaStream_t st);

void soup_build(gwn_soup_impl& s, const double* V, int64_t nV, const int32_t* F, int64_t nF,
                int order, bool host_mode, cudaStream_t st);
// The reference's own 4-wide tree and FP32 moments (soup_ref.cu); fills the
// same walk records (slot 0 the root, then every child lane depth-first),
// without the closest-point search nodes.
void soup_build_ref(gwn_soup_impl& s, const double* V, int64_t nV, const int32_t* F, int64_t nF,
                    int order, bool host_mode, cudaStream_t st);
// The binned tree over the triangles of a GWN_TREE_REFERENCE soup (its
// slot-ordered FP64 corners), for the closest-point search; the search
// tree's triangle ids are the reference soup's leaf slots.
void soup_build_search(const gwn_soup_impl& ref, gwn_soup_impl& search, cudaStream_t st);
// Sets s.moments_bounded from the FP64 records (one reduction, one host read).
void soup_check_moments(gwn_soup_impl& s, cudaStream_t st);
// I[q] <- map[I[q]] where I[q] >= 0.
void soup_remap_index(const int32_t* map, int32_t* I, int64_t n, cudaStream_t st);
// Instrumented mixed walk over FP64 device queries: out7 = {warp steps,
// lane visits, far-field evaluations, FP32 exact triangles, FP64 near-field
// triangles, FP64 decision re-checks, threshold re-evaluations}.
void soup_walk_stats(const gwn_soup_impl& s, float beta, const double* Q, int64_t nQ,
                     unsigned long long* out7, cudaStream_t st);
void soup_eval(const gwn_soup_impl& s, float beta, const void* Q, int q_dtype, int64_t nQ,
               void* W, int w_dtype, int precision, cudaStream_t st);
// Closest triangle of each query (distance.cu): squared distance below
// up_sqr_d (else up_sqr_d and I = -1), input triangle index, closest point.
void soup_squared_distance(const gwn_soup_impl& s, const void* Q, int q_dtype, int64_t nQ,
                           double up_sqr_d, double* sqrD, int32_t* I, double* C,
                           cudaStream_t st);

}  // namespace gwn
