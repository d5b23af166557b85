// Internal interfaces between the C-ABI layer (gwn_api.cu) and the kernel
// translation units.  All pointers here are device pointers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

struct ExactArgs {
  const double* V;
  int64_t nV;
  int dim;
  const int32_t* F;
  int64_t nF;
  const void* Q;
  int q_dtype;
  int64_t nQ;
  void* W;
  int w_dtype;
  int precision;
  bool host_mode;
};

void run_exact(const ExactArgs& a, cudaStream_t st);

// No-allocation exact winding number (device pointers, mixed precision,
// triangles); scratch in a static device array of fixed capacity.
int64_t noalloc_max_triangles();
void run_exact_noalloc(const double* V, int64_t nV, const int32_t* F, int64_t nF, const double* Q,
                       int64_t nQ, double* W, unsigned* dev_status, cudaStream_t st);

// igl::signed_distance for 3-D triangles (distance.cu); device pointers;
// synchronizes `st`.
void signed_distance_run(const double* P, int64_t nP, const double* V, int64_t nV,
                         const int32_t* F, int64_t nF, int sign_type, double lower_bound,
                         double upper_bound, double* S, int32_t* I, double* C, double* N,
                         int precision, cudaStream_t st);

}  // namespace gwn
