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

// Eytzinger AABB tree of segments (eytzinger.cu); device pointers.
int64_t eytzinger_slots(int64_t m);
void eytzinger_build(const double* PB1, const double* PB2, int64_t m, int dim, double* B1,
                     double* B2, int32_t* leaf, cudaStream_t st);
// Writes C (slots + 1) and, when I is non-null, I; returns C[slots].
// Synchronizes `st`.
int64_t eytzinger_pairs(const int32_t* E, int64_t nE, const int32_t* leaf, int64_t nb, int32_t* C,
                        int32_t* I, unsigned* status, cudaStream_t st);
void eytzinger_eval(const double* P, int64_t nP, const double* V, int64_t nV, const int32_t* E,
                    int64_t nE, const double* B1, const double* B2, const int32_t* leaf,
                    int64_t nb, const int32_t* I, const int32_t* C, int64_t nI, double* W,
                    int precision, unsigned* status, cudaStream_t st);

}  // namespace gwn
