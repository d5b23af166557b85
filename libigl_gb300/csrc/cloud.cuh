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
// K_xzz, K_yzz, K_zzz follow from the others); formed by pack_cloud
// (cloud.cu) from EC.
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
