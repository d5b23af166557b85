// Device layout of a built triangle soup (the state behind gwn_soup).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

// 96-byte FP32 node record, read by the mixed-precision walk.
//   a: P (average point) xyz, maxPDist2
//   b: N xyz, Nxx          c: Nyy, Nzz, Nxy+Nyx, Nyz+Nzy
//   d: Nzx+Nxz, Nxxx, Nyyy, Nzzz
//   e: 2(Nxyz+Nyzx+Nzxy), 2Nxxy+Nyxx, 2Nxxz+Nzxx, 2Nyyz+Nzyy
//   f: 2Nyyx+Nxyy, 2Nzzx+Nxzz, 2Nzzy+Nyzz, link (int bits)
// link >= 0: internal node, index one past its subtree (pre-order);
// link < 0: leaf, triangle slot ~link.
struct __align__(16) SoupNodeF {
  float4 a, b, c, d, e, f;
};

// 192-byte FP64 node record (plain FP64 walk, FP64 re-checks).
struct __align__(16) SoupNodeD {
  double P[3], maxP2;
  double N[3], Nii[3];
  double Nxy_yx, Nyz_zy, Nzx_xz;
  double Niii[3], perm, c2[6];
  long long link;
};

struct gwn_soup_impl {
  int device = 0;
  int order = 2;
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
