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

// FP64 all-pairs winding number of the listed queries (W[list[j]] for j <
// *count, read on the device), one block per query; tris64 holds nF
// triangles as 9 doubles (a, b, c).
void exact_refine_listed(const double* tris64, int64_t nF, const double* Q, const int32_t* list,
                         const unsigned* count, double* W, cudaStream_t st);

// No-allocation exact winding number (device pointers, mixed precision,
// triangles); scratch in a static device array of fixed capacity.
int64_t noalloc_max_triangles();
// GWN_STATUS_* bits that gwn_winding_number_noalloc calls without a status
// word of their own recorded on the current device (cleared if `clear`).
unsigned noalloc_sticky_status(bool clear);
void run_exact_noalloc(const double* V, int64_t nV, const int32_t* F, int64_t nF, const double* Q,
                       int64_t nQ, double* W, unsigned* dev_status, cudaStream_t st);

// igl::signed_distance for 3-D triangles (distance.cu); device pointers;
// synchronizes `st`.
void signed_distance_run(const double* P, int64_t nP, const double* V, int64_t nV,
                         const int32_t* F, int64_t nF, int sign_type, double lower_bound,
                         double upper_bound, double* S, int32_t* I, double* C, double* N,
                         int precision, cudaStream_t st);

// Pseudonormals of igl::pseudonormal_test (distance.cu): face, angle-weighted
// vertex and uniform edge normals of a mesh, then per query the sign (+-1,
// into sgn) and normal (N, nullable) at its closest face I and point C.
struct PseudonormalData {
  DevBuf<double> FN, VN, EN;
  DevBuf<int32_t> edge_of;
};
void pseudonormal_precompute(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                             PseudonormalData& d, cudaStream_t st);
void pseudonormal_apply(const PseudonormalData& d, const double* P, int64_t nP, const double* V,
                        const int32_t* F, int64_t nF, const int32_t* I, const double* C,
                        const double* sqrD, double* sgn, double* N, cudaStream_t st);

// igl::swept_volume_signed_distance (swept.cu); device pointers; S holds S0
// on entry.  transforms: nT x 12 row-major (the 3 x 4 [linear | translation]
// rows of each affine transform).  Synchronizes `st`.
void swept_volume_run(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                      const double* transforms_host, int64_t nT, int sign_type, const double* GV,
                      int64_t nG, const int32_t res[3], double h, double isolevel, double* S,
                      int precision, cudaStream_t st);
// igl::flood_fill (swept.cu) over a res[0] x res[1] x res[2] grid (x fastest).
void flood_fill_run(const int32_t res[3], double* S, cudaStream_t st);

// igl::copyleft::cgal::point_areas (point_areas.cu): A (nP) and, when T is
// non-null, T (nP x 3) from the nP x k neighbour lists I; device pointers.
constexpr int kPointAreasMaxK = 128;
static_assert(kPointAreasMaxK == GWN_POINT_AREAS_MAX_K,
              "the kernel's neighbour arrays hold the largest k the ABI accepts");
void point_areas_run(const double* P, int64_t nP, const int32_t* I, int k, const double* N,
                     double* A, double* T, unsigned* status, cudaStream_t st);

// Hierarchical exact winding number of a triangle mesh (hier.cu): the
// caller's V / F stay referenced (device pointers) for the FP64 re-checks.
struct HierTree {
  const double* V = nullptr;
  int64_t nV = 0;
  const int32_t* F = nullptr;
  int64_t nF = 0;
  int n = 0;
  int64_t nnodes = 0, ncap = 0;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, c[3] = {0, 0, 0};
  double eps = 0;
  DevMem<float4> nodes;   // 2 per node
  DevMem<int32_t> capn;   // cap triangles per node
  DevMem<float4> caps;    // 4 per cap triangle
  DevMem<float4> tris;    // 4 per leaf triangle
  DevMem<double> tris64;  // 9 per leaf triangle
  DevMem<double> box64;   // 6 per node (pre-order): the node's FP64 box, lo then hi
  DevMem<double> caps64;  // 9 per cap triangle (absolute FP64 corners)
};
// Out-of-range triangle indices set kStatusBadInput in *status.  With
// per_call, the tree's memory is stream-ordered on `st` (a tree built and
// used inside one call); otherwise it is owned like a handle's.  The build
// ends with work still queued on `st`.
void hier_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, HierTree& h,
                unsigned* status, cudaStream_t st, bool per_call = false);
// W of every query (FP64 device arrays), queued on `st`.  GWN_MIXED: FP32
// caps and leaves with FP64 near terms and threshold re-evaluation;
// GWN_PLAIN_FP64: the reference's walk (a node's cap for a point outside its
// box, WindingNumberTree.h:261-336) with every term in FP64.
void hier_eval(const HierTree& h, const double* Q, int64_t nQ, double* W, cudaStream_t st,
               int precision = GWN_MIXED);

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
