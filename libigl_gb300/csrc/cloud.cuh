// Device layout of a point-cloud expansion (the state behind gwn_cloud).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

// 96-byte FP32 traversal record, 32-byte aligned (read as three 256-bit loads):
//   a: CM xyz, R
//   b: N xyz, Q_xx     c: Q_yy, Q_xy, Q_xz, Q_yz
//   d: K_xxx, K_yyy, K_xxy, K_xxz     e: K_xyy, K_yyz, K_xyz, squared FP64 near-field radius
//   l: skip (one past subtree), first point slot, point count, leaf flag
// N, Q, K: the expansion of the cell in the unit direction u = (CM - q)/r,
// W = (u.N + Q(u)/r + K(u)/r^2) / r^2, with Q and K harmonic (Q_zz and
// K_xzz, K_yzz, K_zzz follow from the others); formed by pack_cloud (below)
// from EC.
struct __align__(32) CloudNodeF {
  float4 a, b, c, d, e;
  int4 l;
};
static_assert(sizeof(CloudNodeF) == 96, "three 32-byte halves per record");

// FP64 traversal record: CM, R, the packed expansion pk (the FP32 record's
// b..e coefficients in FP64: N xyz, Q_xx, Q_yy, Q_xy, Q_xz, Q_yz, K_xxx,
// K_yyy, K_xxy, K_xxz, K_xyy, K_yyz, K_xyz), links as in CloudNodeF.
struct __align__(16) CloudNodeD {
  double cm[3], r;
  double pk[15];
  double pad;
  int4 l;
};

// expansion_eval (fast_winding_number.cpp:174-228) with loc = CM - q = r u,
// |u| = 1, and E1(u,v) = EC[3 + u + 3v], E2(i,u,v) = EC[12 + 9i + u + 3v]:
//   4 pi W = (u.EC[0..2]) / r^2
//          + sum_uv E1(u,v) (delta_uv - 3 u_u u_v) / r^3
//          + sum_iuv E2(i,u,v) (15 u_i u_u u_v - 3 (delta_uv u_i + delta_ui u_v
//                                                  + delta_vi u_u)) / r^4.
// With |u|^2 = 1 the second bracket is the quadratic form
// Q(u) = sum_uv (tr E1 delta_uv - 3 E1(u,v)) u_u u_v and the third the cubic
// form K(u) = 15 sum E2(i,u,v) u_i u_u u_v - 3 (u.w) |u|^2, with
// w_k = sum_j E2(k,j,j) + E2(j,j,k) + E2(j,k,j).  Both are harmonic (their
// Laplacians vanish identically), so Q_zz = -Q_xx - Q_yy and
// K_xzz = -3 K_xxx - K_xyy, K_yzz = -3 K_yyy - K_xxy, K_zzz = -(K_xxz + K_yyz) / 3,
// and the records keep 3 + 5 + 7 coefficients (monomial coefficients,
// 1/(4 pi) folded in), formed in FP64 (the FP64 record) and rounded once (the
// FP32 record).
__host__ __device__ inline void pack_cloud(const double* ec, int num_terms, double* pk) {
  const double s = 1.0 / (4.0 * kPi);
  for (int k = 0; k < 15; ++k) pk[k] = 0;
  for (int d = 0; d < 3; ++d) pk[d] = ec[d] * s;
  if (num_terms > 3) {
    auto E1 = [&](int u, int v) { return ec[3 + u + 3 * v]; };
    const double tr = E1(0, 0) + E1(1, 1) + E1(2, 2);
    pk[3] = (tr - 3 * E1(0, 0)) * s;         // Q_xx
    pk[4] = (tr - 3 * E1(1, 1)) * s;         // Q_yy
    pk[5] = -3 * (E1(0, 1) + E1(1, 0)) * s;  // Q_xy
    pk[6] = -3 * (E1(0, 2) + E1(2, 0)) * s;  // Q_xz
    pk[7] = -3 * (E1(1, 2) + E1(2, 1)) * s;  // Q_yz
  }
  if (num_terms > 12) {
    auto E2 = [&](int i, int u, int v) { return ec[12 + 9 * i + u + 3 * v]; };
    double w[3];
    for (int a = 0; a < 3; ++a) {
      w[a] = 0;
      for (int j = 0; j < 3; ++j) w[a] += E2(a, j, j) + E2(j, j, a) + E2(j, a, j);
    }
    // sum of E2 over the distinct orderings of {a, a, b}
    auto S2 = [&](int a, int b) { return E2(a, a, b) + E2(a, b, a) + E2(b, a, a); };
    pk[8] = (15 * E2(0, 0, 0) - 3 * w[0]) * s;   // K_xxx
    pk[9] = (15 * E2(1, 1, 1) - 3 * w[1]) * s;   // K_yyy
    pk[10] = (15 * S2(0, 1) - 3 * w[1]) * s;     // K_xxy: u_x^2 u_y
    pk[11] = (15 * S2(0, 2) - 3 * w[2]) * s;     // K_xxz
    pk[12] = (15 * S2(1, 0) - 3 * w[0]) * s;     // K_xyy: u_y^2 u_x
    pk[13] = (15 * S2(1, 2) - 3 * w[2]) * s;     // K_yyz
    pk[14] = 15 * (E2(0, 1, 2) + E2(0, 2, 1) + E2(1, 0, 2) + E2(1, 2, 0) + E2(2, 0, 1) +
                   E2(2, 1, 0)) * s;             // K_xyz
  }
}

struct gwn_cloud_impl {
  int device = 0;
  int order = 2;
  int num_terms = 39;
  int64_t n = 0;        // points
  int64_t ncells = 0;   // octree cells (igl ids)
  int64_t nnodes = 0;   // non-empty cells (traversal records)
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  double eps = 0, cmax = 0;
  // per igl cell id (export)
  DevMem<double> CM, R, EC;
  DevMem<double> area;  // sum of A per cell (FP64 near-field radii)
  // traversal (pre-order of non-empty cells)
  DevMem<CloudNodeF> nf;
  DevMem<CloudNodeD> nd;
  // points in slot order (octree perm order): FP32 {P.xyz, 0} {A N .xyz, 0}; FP64 {P, AN}
  DevMem<float4> pf;
  DevMem<double> pd;
  // raw inputs (for the direct beta <= 0 sum)
  DevMem<double> P, AN;
  size_t bytes = 0;
  // drop-in form: traversal layout kept until moments are attached
  DevBuf<int32_t> layout_order, layout_first, layout_count;
  DevBuf<int64_t> layout_skip, layout_start;
  const int32_t* layout_ch = nullptr;
};

struct gwn_octree_impl;

// Precompute on the device from a built octree (P, N, A device pointers).
void cloud_build(gwn_cloud_impl& c, const gwn_octree_impl& t, const double* N, const double* A,
                 int order, cudaStream_t st);
// Drop-in form over caller CSR lists / CH (device copies for the kernels,
// host copies for the pre-order walk; host pointers may be null when only
// the moments are wanted).
void cloud_build_arrays(gwn_cloud_impl& c, const double* P, const double* N, const double* A,
                        int64_t nP, const int64_t* pi_off_d, const int32_t* pi_idx_d,
                        const int32_t* CH_d, int64_t ncells, int order, bool compute_moments,
                        const int64_t* pi_off_h, const int32_t* pi_idx_h, const int32_t* CH_h,
                        cudaStream_t st);
// Attach caller CM/R/EC (device, ncells rows) and emit the walk records.
void cloud_set_moments(gwn_cloud_impl& c, const double* CM, const double* R, const double* EC,
                       cudaStream_t st);
void cloud_emit_arrays(gwn_cloud_impl& c, cudaStream_t st);
void cloud_eval(const gwn_cloud_impl& c, double beta, const void* Q, int q_dtype, int64_t nQ,
                void* W, int w_dtype, int precision, cudaStream_t st);

}  // namespace gwn
