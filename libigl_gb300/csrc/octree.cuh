// Device octree (the state behind gwn_octree), bit-exact with igl::octree.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

struct gwn_octree_impl {
  int device = 0;
  int64_t n = 0;           // points
  int64_t ncells = 0;      // 1 + 8 * num_internal
  int64_t nindices = 0;    // sum of point-list lengths
  int32_t max_depth = 0;
  // cell arrays in igl id order
  DevMem<double> cn;       // ncells x 3 centres
  DevMem<double> w;        // ncells widths
  DevMem<int32_t> ch;      // ncells x 8 child ids (-1 for leaves)
  DevMem<int64_t> start;   // first position of the cell's points in perm
  DevMem<int32_t> count;   // number of points in the cell
  DevMem<int32_t> depth;   // cell depth (root 0)
  DevMem<int32_t> perm;    // n point ids; every cell's list is a contiguous range
  // input copy (points), kept for the cloud path
  DevMem<double> P;
};

void octree_build(gwn_octree_impl& t, const double* P, int64_t n, bool host_mode, cudaStream_t st);
// pi_offsets (ncells+1) and pi_indices (nindices) written to device memory.
void octree_export_csr(const gwn_octree_impl& t, int64_t* pi_offsets, int32_t* pi_indices,
                       cudaStream_t st);

// k nearest octree points of each query (knn.cu): I is nQ x min(k, n) point
// ids, nearest first, equal distances by index.  Device pointers.
int64_t knn_columns(int64_t n, int64_t k);
void octree_knn(const gwn_octree_impl& tree, const void* Q, int q_dtype, int64_t nQ, int64_t k,
                int32_t* I, cudaStream_t st);

}  // namespace gwn
