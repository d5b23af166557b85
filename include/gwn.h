/*
 * gwn.h -- C ABI of libgwn.so, the GB300 (sm_103a) generalized winding number
 * library.  Plain pointers and sizes only; every entry point returns a status
 * code (GWN_OK on success) and never throws across the ABI.  The message of
 * the last failure on the calling thread is available from gwn_last_error().
 *
 * Memory kinds: every call that takes arrays takes `mem`:
 *   GWN_HOST   -- pointers are host memory; the call is synchronous (copies in,
 *                 computes on the GPU, copies out, waits).
 *   GWN_DEVICE -- pointers are device memory of the current CUDA device; work
 *                 is enqueued on `stream` (a cudaStream_t, NULL = legacy
 *                 default stream) and the call returns without waiting.
 * Arrays are row-major and contiguous: V[i*3+d], F[f*3+c], Q[i*3+d].
 * A handle (gwn_soup, gwn_octree, gwn_cloud, gwn_wn_aabb) belongs to the
 * device that was current when it was built; a call that runs work on it
 * (evaluation, knn, distance, export through a stream) with another device
 * current is refused with GWN_ERR_INVALID_ARGUMENT.  Arguments are checked
 * on the host before any device work.
 *
 * Precision modes:
 *   GWN_PLAIN_FP64 -- every term, sum and far-field expansion in FP64.
 *   GWN_MIXED      -- FP32 bulk arithmetic; FP64 for (i) exact terms of
 *                     queries within 1e-3 * bbox-diagonal of a primitive
 *                     (for triangle soups: FP64 corner vectors, determinant
 *                     and denominator, the angle itself from FP32 atan2),
 *                     (ii) moment accumulation, (iii) full re-evaluation of
 *                     any query whose FP32 result lies within 1e-3 of 0.5.
 *
 * This header replaces, for C/C++ callers, the libigl entry points cited at
 * each declaration (paths inside the libigl source tree).  The igl::
 * signatures themselves are provided as inline templates over this ABI in
 * include/igl_gb300/.
 */
#ifndef GWN_H
#define GWN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GWN_VERSION 100

enum gwn_status {
  GWN_OK = 0,
  GWN_ERR_INVALID_ARGUMENT = 1,
  GWN_ERR_CUDA = 2,
  GWN_ERR_OUT_OF_MEMORY = 3,
  GWN_ERR_NO_DEVICE = 4,
  GWN_ERR_TIMEOUT = 5, /* a bounded device-side wait gave up */
  GWN_ERR_BUSY = 6,
  GWN_ERR_INTERNAL = 7
};

enum gwn_dtype { GWN_F32 = 0, GWN_F64 = 1 };
enum gwn_precision { GWN_PLAIN_FP64 = 0, GWN_MIXED = 1 };
enum gwn_mem { GWN_HOST = 0, GWN_DEVICE = 1 };
/* Triangle-soup tree (gwn_soup_build_tree):
 *   GWN_TREE_REFERENCE -- the reference's own 4-wide SAH tree (UT_BVH<4>),
 *                         built on the GPU node for node, with its FP32
 *                         moments and FP32 open test: the same tree cut as
 *                         igl::fast_winding_number, so results equal the
 *                         reference's up to its FP32 rounding.
 *   GWN_TREE_BINNED    -- a binary tree of binned splits (triangles x
 *                         squared box diagonal); a different tree cut, so
 *                         results differ from the reference's at the level
 *                         of the approximation (a few 1e-3). */
enum gwn_soup_tree { GWN_TREE_REFERENCE = 0, GWN_TREE_BINNED = 1 };

/* Message of the last failing call on this thread ("" if none). */
const char* gwn_last_error(void);
int gwn_version(void);

/* Device-memory (GWN_DEVICE) calls never synchronize, so failures detected
 * inside kernels (an out-of-range index, a bounded wait that gave up) are
 * recorded in a sticky per-device word.  This call synchronizes the current
 * device, returns the recorded GWN_STATUS_* bits in *flags and clears them if
 * `clear` is non-zero.  Host-memory calls report such failures directly. */
#define GWN_STATUS_WAIT_TIMEOUT 1u
#define GWN_STATUS_BAD_INPUT 2u
int gwn_device_status(unsigned int* flags, int clear);

/* Failure-path testing (no counterpart in the reference, which has asserts
 * only).  The next n launches of a kernel that streams triangles through a
 * bounded bulk-copy ring (the exact path's all-pairs sweeps, in
 * gwn_winding_number and gwn_winding_number_noalloc) initialise one mbarrier
 * for one more arrival than they make, so their first wait runs out of its
 * budget (about 50 ms); each such kernel then makes the missing arrival,
 * waits for its copies in flight, records GWN_STATUS_WAIT_TIMEOUT and
 * returns.  The call reports GWN_ERR_TIMEOUT (host memory) or the status bit
 * (device memory); the device stays usable.  n = 0 cancels. */
int gwn_debug_fail_next_waits(int n);

/* ------------------------------------------------------------------------
 * Exact generalized winding number.
 * Replaces igl::winding_number(V,F,O,W)      include/igl/winding_number.h:35-44
 *   (implementation include/igl/winding_number.cpp:17-56) and, per query,
 *   igl::winding_number(V,F,p)                include/igl/winding_number.h:53-60
 *   (winding_number.cpp:58-89, solid_angle.cpp:5-55, signed_angle.cpp:5-46).
 * dim = 3: V is nV x 3, F is nF x 3 (triangles), O is nO x 3.
 * dim = 2: V is nV x 2, F is nF x 2 (edges),     O is nO x 2.
 * W (nO) receives sum over elements of solid angle / 4pi (or angle / 2pi).
 * With dim = 3, at least 4096 triangles and 1024 queries, both precisions
 * evaluate through the cap hierarchy of gwn_wn_aabb (the reference's own
 * algorithm, winding_number.cpp:40-53; same value up to rounding, built for
 * the call); otherwise every pair is summed.
 * ---------------------------------------------------------------------- */
int gwn_winding_number(const double* V, int64_t nV, int dim, const int32_t* F, int64_t nF,
                       const void* O, int o_dtype, int64_t nO, void* W, int w_dtype,
                       int precision, int mem, void* stream);

/* No-allocation variant of gwn_winding_number (no counterpart in the
 * reference).  For callers that must not allocate device memory during a
 * call: hosts that own every device allocation through their own memory
 * pool and forbid foreign cudaMalloc, or latency-critical loops in which
 * cudaMalloc / cudaFree would synchronize the device.  Device pointers only
 * (V nV x 3, F nF x 3 triangles, O nO x 3, W nO, all float64), mixed
 * precision, work enqueued on `stream`; nothing is allocated: the call's
 * scratch is a static device array inside libgwn sized for
 * GWN_NOALLOC_MAX_TRIANGLES triangles (about 4.2 MB, held by every GPU that
 * loads the library until the process exits); larger nF is rejected with
 * GWN_ERR_INVALID_ARGUMENT.  All calls share that array and leave their
 * contents in it, so calls that overlap on the GPU (on different streams)
 * race; calls on one stream are ordered.  The first call on a device looks up
 * the array's device address and keeps it for the life of the process: make
 * that call before any stream capture, and make no call after a
 * cudaDeviceReset (the kept address would be stale).  V must hold nV > 0
 * vertices whenever nF > 0.  dev_status (optional device pointer, zeroed by
 * the caller) receives GWN_STATUS_* bits for failures found on the device
 * (an index of F outside V, a bounded wait that gave up); with dev_status
 * NULL they are kept in a word of the same static memory, which
 * gwn_device_status reads and clears. */
#define GWN_NOALLOC_MAX_TRIANGLES 65536
int gwn_winding_number_noalloc(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                               const double* O, int64_t nO, double* W, unsigned int* dev_status,
                               void* stream);

/* ------------------------------------------------------------------------
 * Triangle-soup fast winding number (Barnes-Hut over a GPU-built BVH with the
 * HDK order-0/1/2 far field).
 * gwn_soup_build replaces the precompute overload
 *   igl::fast_winding_number(V,F,order,fwn_bvh)  include/igl/fast_winding_number.h:176-181
 *   (fast_winding_number.cpp:380-416; UT_SolidAngle::init,
 *    FastWindingNumberForSoups.h:6543-7133).
 * gwn_soup_eval replaces the evaluate overloads
 *   igl::fast_winding_number(fwn_bvh,accuracy_scale,Q,W)  fast_winding_number.h:189-194
 *   igl::fast_winding_number(fwn_bvh,accuracy_scale,p)    fast_winding_number.h:201-205
 *   (fast_winding_number.cpp:418-455; UT_SolidAngle::computeSolidAngle,
 *    FastWindingNumberForSoups.h:7148-7284).
 * The handle plays the role of struct igl::FastWindingNumberBVH
 *   (fast_winding_number.h:140-147): it owns device copies of V and F.
 * ---------------------------------------------------------------------- */
typedef struct gwn_soup gwn_soup;

typedef struct gwn_soup_stats {
  int64_t num_triangles;   /* triangles kept (non-finite boxes excluded)      */
  int64_t num_nodes;       /* walk records: binary tree nodes, leaves included,
                              or the 4-wide tree's root plus every child lane */
  int64_t device_bytes;    /* device memory held by the handle                 */
  int32_t order;
  int32_t max_depth;       /* binary: longest root-leaf path; 4-wide: depths   */
  int32_t tree;            /* GWN_TREE_REFERENCE or GWN_TREE_BINNED            */
  int32_t reserved;
  int64_t tree_nodes;      /* nodes of the tree (4-wide: the reference's count) */
} gwn_soup_stats;

/* gwn_soup_build_tree builds with the chosen tree (gwn_soup_tree);
 * gwn_soup_build with GWN_SOUP_TREE_DEFAULT. */
#define GWN_SOUP_TREE_DEFAULT GWN_TREE_REFERENCE
int gwn_soup_build_tree(const double* V, int64_t nV, const int32_t* F, int64_t nF, int order,
                        int tree, int mem, void* stream, gwn_soup** out);
int gwn_soup_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, int order,
                   int mem, void* stream, gwn_soup** out);
/* The 4-wide tree of a GWN_TREE_REFERENCE handle as the reference stores it
 * (UT_BVH<4>::Node, FastWindingNumberForSoups.h:4214-4270): *num_nodes
 * nodes in the reference's numbering (depth-first, children in lane order)
 * and, if child is non-null, 4 entries per node: a triangle index, node |
 * 0x80000000 for an internal child, 0xffffffff for an empty lane.  For
 * testing and inspection. */
int gwn_soup_tree_nodes(const gwn_soup* soup, int64_t* num_nodes, uint32_t* child);
int gwn_soup_eval(const gwn_soup* soup, float accuracy_scale, const void* Q, int q_dtype,
                  int64_t nQ, void* W, int w_dtype, int precision, int mem, void* stream);
int gwn_soup_stats_get(const gwn_soup* soup, gwn_soup_stats* out);
/* Work counters of one instrumented mixed-precision evaluation of nQ float64
 * queries (a separate kernel instance; for profiling, no counterpart in the
 * reference): counters[0..6] = warp steps, per-query node visits, far-field
 * evaluations, FP32 exact triangles, FP64 near-field triangles, FP64 decision
 * re-checks, threshold re-evaluations. */
int gwn_soup_walk_stats(const gwn_soup* soup, float accuracy_scale, const double* Q, int64_t nQ,
                        int mem, unsigned long long* counters);
void gwn_soup_free(gwn_soup* soup);

/* Copies the built tree to host memory (for inspection and testing):
 * nodes: num_nodes records of 24 doubles in pre-order,
 *   {P[3], maxPDist2, N[3], Nxx, Nyy, Nzz, Nxy+Nyx, Nyz+Nzy, Nzx+Nxz,
 *    Nxxx, Nyyy, Nzzz, 2(Nxyz+Nyzx+Nzxy), 2Nxxy+Nyxx, 2Nxxz+Nzxx,
 *    2Nyyz+Nzyy, 2Nyyx+Nxyy, 2Nzzx+Nxzz, 2Nzzy+Nyzz, link}
 *   where link (an int64 stored in the last slot's bytes) is >= 0 for an
 *   internal node (index one past its subtree) and ~slot for a leaf;
 * tri_index: num_triangles input-triangle ids, one per leaf slot.
 * Either pointer may be NULL. */
int gwn_soup_export(const gwn_soup* soup, double* nodes, int32_t* tri_index);

/* ------------------------------------------------------------------------
 * Octree over a point cloud, bit-exact with igl::octree.
 * Replaces igl::octree(P,point_indices,CH,CN,W)  include/igl/octree.h:44-50
 *   (include/igl/octree.cpp:5-170).
 * point_indices is exported in CSR form: cell c holds
 *   pi_indices[pi_offsets[c] .. pi_offsets[c+1]).
 * ---------------------------------------------------------------------- */
typedef struct gwn_octree gwn_octree;

int gwn_octree_build(const double* P, int64_t nP, int mem, void* stream, gwn_octree** out);
int gwn_octree_sizes(const gwn_octree* tree, int64_t* num_cells, int64_t* num_indices,
                     int32_t* max_depth);
int gwn_octree_export(const gwn_octree* tree, int64_t* pi_offsets, int32_t* pi_indices,
                      int32_t* CH, double* CN, double* W, int mem, void* stream);
void gwn_octree_free(gwn_octree* tree);

/* ------------------------------------------------------------------------
 * Point-cloud fast winding number (order-2 dipole expansion, Barnes-Hut).
 * gwn_cloud_build replaces the precompute overload
 *   igl::fast_winding_number(P,N,A,point_indices,CH,expansion_order,CM,R,EC)
 *     include/igl/fast_winding_number.h:35-53 (fast_winding_number.cpp:17-124)
 * computing it on the device from an octree handle; gwn_cloud_export returns
 * CM (ncells x 3), R (ncells), EC (ncells x num_terms).
 * gwn_cloud_eval replaces the evaluate overload
 *   igl::fast_winding_number(P,N,A,point_indices,CH,CM,R,EC,Q,beta,WN)
 *     fast_winding_number.h:76-99 (fast_winding_number.cpp:126-311);
 * beta <= 0 selects the direct O(P*Q) sum (fast_winding_number.cpp:300-310).
 * ---------------------------------------------------------------------- */
/* k nearest points: igl::knn(P,V,k,point_indices,CH,CN,W,I)
 *   (include/igl/knn.h, knn.cpp:24-136) over the points the octree was built
 *   from.  I (nQ x min(k, #points), int32, row-major) receives point indices,
 *   nearest first; equal distances are ordered by index (the reference leaves
 *   them to its priority queue).  Distances are the FP64 norm of V(j) - q. */
int gwn_octree_knn(const gwn_octree* tree, const void* Q, int q_dtype, int64_t nQ, int64_t k,
                   int32_t* I, int mem, void* stream);
/* One-shot form: builds the octree of V (nV x 3) and answers the queries P. */
int gwn_knn(const double* P, int64_t nP, const double* V, int64_t nV, int64_t k, int32_t* I,
            int mem, void* stream);

/* Per-point areas of a point cloud: igl::copyleft::cgal::point_areas(P,I,N,A,T)
 *   (include/igl/copyleft/cgal/point_areas.h:40-53, point_areas.cpp:60-160).
 * P, N: nP x 3 points and normals; I: nP x k neighbour indices (e.g. from
 * gwn_knn / gwn_octree_knn), the first normally the point itself.  A (nP)
 * receives each point's Voronoi area in its local Delaunay triangulation
 * (the neighbours whose normal agrees with the first neighbour's, projected
 * on their principal plane); T (nP x 3, optional: NULL skips it) the plane
 * normal turned towards N.  A point with two or fewer agreeing neighbours
 * gets A = 0, T = 0; a non-finite area gives 0.  k <= GWN_POINT_AREAS_MAX_K.
 * The triangulation is computed directly for each point (no CGAL); for four
 * or more cocircular plane points at the point it is not unique, and values
 * there may differ from CGAL's. */
#define GWN_POINT_AREAS_MAX_K 128
int gwn_point_areas(const double* P, int64_t nP, const int32_t* I, int64_t k, const double* N,
                    double* A, double* T, int mem, void* stream);

/* Winding number of an oriented point cloud without areas:
 * igl::copyleft::cgal::fast_winding_number(P,N,Q,expansion_order,beta,WN)
 *   (include/igl/copyleft/cgal/fast_winding_number.h:20-36, .cpp:9-44):
 *   octree of P, its 21 nearest points per point, gwn_point_areas, the
 *   order-`order` expansions and their evaluation at Q (beta as for
 *   gwn_cloud_eval; the reference's short overload uses order 2, beta 2).
 * P, N nP x 3 float64; Q nQ x 3 and W nQ in their dtypes. */
int gwn_cloud_winding_number_points(const double* P, const double* N, int64_t nP, const void* Q,
                                    int q_dtype, int64_t nQ, int order, double beta, void* W,
                                    int w_dtype, int precision, int mem, void* stream);

typedef struct gwn_cloud gwn_cloud;

int gwn_cloud_build(const gwn_octree* tree, const double* P, const double* N, const double* A,
                    int order, int mem, void* stream, gwn_cloud** out);
int gwn_cloud_export(const gwn_cloud* cloud, double* CM, double* R, double* EC, int mem,
                     void* stream);
int gwn_cloud_eval(const gwn_cloud* cloud, double beta, const void* Q, int q_dtype, int64_t nQ,
                   void* W, int w_dtype, int precision, int mem, void* stream);
void gwn_cloud_free(gwn_cloud* cloud);

/* Drop-in forms over caller-held arrays (all host memory, synchronous): the
 * octree / precompute outputs may come from igl::octree or anywhere else.
 * CH has ncells rows of 8 child ids (-1 for leaves). */
int gwn_cloud_precompute_arrays(const double* P, const double* N, const double* A, int64_t nP,
                                const int64_t* pi_offsets, const int32_t* pi_indices,
                                const int32_t* CH, int64_t ncells, int order, double* CM,
                                double* R, double* EC);
int gwn_cloud_eval_arrays(const double* P, const double* N, const double* A, int64_t nP,
                          const int64_t* pi_offsets, const int32_t* pi_indices,
                          const int32_t* CH, int64_t ncells, const double* CM, const double* R,
                          const double* EC, int order, const double* Q, int64_t nQ,
                          double beta, double* W, int precision);

/* ------------------------------------------------------------------------
 * Closest triangle and signed distance (the caller of the winding number
 * that libigl builds on it).
 *
 * gwn_soup_squared_distance: igl::AABB<V,3>::squared_distance(V,F,P,sqrD,I,C)
 * (include/igl/AABB.h:386-397, AABB.cpp:1135-1205) over the triangles of a
 * soup handle: per query the smallest squared distance below up_sqr_d
 * (up_sqr_d and I = -1 if none; pass INFINITY for no bound), the input index
 * of that triangle and the closest point (#Q x 3 float64).  Non-finite
 * queries give up_sqr_d and I = -1.
 *
 * gwn_signed_distance: igl::signed_distance(P,V,F,sign_type,lower_bound,
 * upper_bound,S,I,C,N) (include/igl/signed_distance.h:61-71,
 * signed_distance.cpp:20-137, 372-424) for 3-D triangles.  sign_type takes
 * igl::SignedDistanceType's values.  The sign factor is 1 (UNSIGNED),
 * 1 - 2 W with the exact winding number (WINDING_NUMBER, DEFAULT),
 * 1 - 2 |W| with the soup fast winding number, order 2, accuracy 2
 * (FAST_WINDING_NUMBER; `precision` selects how W is computed), or +-1 from
 * the angle-weighted pseudonormal of the closest feature (PSEUDONORMAL,
 * pseudonormal_test.cpp:16-135), whose normal is written to N (#P x 3,
 * optional: NULL skips it; untouched for the other types).
 * Distances outside the bounds give S = NaN, I = #F + 1, C = 0; an empty F
 * gives S = NaN, I = -1, C = NaN.  The defaults of the reference's
 * bound-less overload are lower_bound = DBL_MIN, upper_bound = DBL_MAX.
 * ---------------------------------------------------------------------- */
enum {
  GWN_SD_PSEUDONORMAL = 0,
  GWN_SD_WINDING_NUMBER = 1,
  GWN_SD_DEFAULT = 2,
  GWN_SD_UNSIGNED = 3,
  GWN_SD_FAST_WINDING_NUMBER = 4
};
int gwn_soup_squared_distance(const gwn_soup* soup, const void* Q, int q_dtype, int64_t nQ,
                              double up_sqr_d, double* sqrD, int32_t* I, double* C, int mem,
                              void* stream);
int gwn_signed_distance(const double* P, int64_t nP, const double* V, int64_t nV,
                        const int32_t* F, int64_t nF, int sign_type, double lower_bound,
                        double upper_bound, double* S, int32_t* I, double* C, double* N,
                        int precision, int mem, void* stream);

/* ------------------------------------------------------------------------
 * Hierarchical exact winding number (igl::WindingNumberAABB,
 * include/igl/WindingNumberAABB.h:23-60 over WindingNumberTree.h:263-350):
 * a tree over the mesh whose nodes carry the cap (fan over the node's
 * boundary edges) that replaces the node's triangles for points outside its
 * box.  The value is the exact winding number's (gwn_winding_number) up to
 * rounding.  gwn_wn_aabb_build copies V (#V x 3 float64) and F (#F x 3
 * int32) to the device; gwn_wn_aabb_eval evaluates Q (#Q x 3 float64) in
 * mixed precision (FP32 terms at least 1e-3 x the mesh diagonal from the
 * query, FP64 nearer, FP64 all-pairs for results within 1e-3 of 0.5).
 * ---------------------------------------------------------------------- */
typedef struct gwn_wn_aabb gwn_wn_aabb;
int gwn_wn_aabb_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, int mem,
                      void* stream, gwn_wn_aabb** out);
int gwn_wn_aabb_eval(const gwn_wn_aabb* tree, const double* Q, int64_t nQ, double* W, int mem,
                     void* stream);
/* The same with a precision: GWN_PLAIN_FP64 walks as the reference does
 * (a node's cap for a point strictly outside the node's box, every term
 * in FP64); GWN_MIXED as gwn_wn_aabb_eval. */
int gwn_wn_aabb_eval_precision(const gwn_wn_aabb* tree, const double* Q, int64_t nQ, double* W,
                               int precision, int mem, void* stream);
void gwn_wn_aabb_free(gwn_wn_aabb* tree);

/* ------------------------------------------------------------------------
 * Swept volumes (the batched caller of the winding number and the signed
 * distance on grids).
 *
 * gwn_swept_volume_signed_distance: igl::swept_volume_signed_distance(V,F,
 * transforms,sign_type,GV,res,h,isolevel,S0,S)
 * (include/igl/swept_volume_signed_distance.h:28-51, .cpp:21-160) for a
 * triangle mesh V (#V x 3), F (#F x 3) under nT rigid motions
 * (transforms: nT x 12 float64, each the row-major 3 x 4 [linear |
 * translation] of the affine transform), over grid points GV (#GV x 3) of a
 * res[0] x res[1] x res[2] grid (x fastest) with spacing h.  S0 (#GV,
 * nullable: all NaN, the reference's second overload) seeds the running
 * minimum; S (#GV) receives it (S may equal S0).  sign_type as for
 * gwn_signed_distance.  A finite isolevel enables the reference's skipping
 * of far and deep points and its final flood fill (#GV must then be
 * res[0] res[1] res[2]).  Synchronizes `stream`.
 *
 * gwn_flood_fill: igl::flood_fill(res,S) (include/igl/flood_fill.h:20-25,
 * .cpp:11-80): NaN entries of S (res[0] x res[1] x res[2], x fastest) take
 * the values of the reference's scan.
 * ---------------------------------------------------------------------- */
int gwn_swept_volume_signed_distance(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                                     const double* transforms, int64_t nT, int sign_type,
                                     const double* GV, int64_t nGV, const int32_t* res, double h,
                                     double isolevel, const double* S0, double* S, int precision,
                                     int mem, void* stream);
int gwn_flood_fill(const int32_t* res, double* S, int mem, void* stream);

/* ------------------------------------------------------------------------
 * 2-D winding numbers over an Eytzinger AABB tree of segments (libigl's
 * hierarchical 2-D path).
 *
 * gwn_eytzinger_slots: the tree's slot count for m primitives,
 * 2^(ceil(log2 m) + 1) (0 for m = 0).
 *
 * gwn_eytzinger_aabb: igl::eytzinger_aabb(PB1,PB2,B1,B2,leaf)
 * (include/igl/eytzinger_aabb.h:24-34, eytzinger_aabb.cpp:16-100).  PB1 / PB2
 * are the m primitives' min / max corners (m x dim float64, dim 1..3); B1 /
 * B2 (slots x dim) receive the node boxes, leaf (slots) the primitive of a
 * leaf, -1 for an internal node, -2 for an empty slot (whose boxes are NaN;
 * the reference leaves them uninitialised).  Median of the box centres
 * along the longest axis as the reference, taken as the order statistics.
 *
 * gwn_eytzinger_winding_number_tree: igl::eytzinger_aabb_winding_number_tree
 * (eytzinger_aabb_winding_number_tree.h:22-35, .cpp:17-118) for segments E
 * (nE x 2 int32) and a tree's leaf array: C (slots + 1) is always written;
 * I (C[slots] entries) only when non-NULL, so a caller sizes I from C and
 * calls again.  Each internal node's pairs list its boundary vertices,
 * positive ones ascending paired with negative ones ascending (the
 * reference's pairing order is an unordered_map's; the sum is the same).
 * Synchronizes `stream`.
 *
 * gwn_eytzinger_winding_number: igl::eytzinger_aabb_winding_number(p,V,E,
 * B1,B2,leaf,I,C,wn) (eytzinger_aabb_winding_number.h:25-44, .cpp:9-125)
 * for nP points P (nP x 2 float64) over V (nV x 2), E, the tree (B1, B2:
 * slots x 2) and its pairs (I: nI entries, C: slots + 1).  GWN_PLAIN_FP64
 * follows the reference's walk and arithmetic; GWN_MIXED walks FP32 boxes
 * with FP32 angles, FP64 for terms within 1e-3 x the root box diagonal and
 * for results within 1e-3 of 0.5.  Indices out of range set
 * GWN_STATUS_BAD_INPUT and are skipped.
 * ---------------------------------------------------------------------- */
int64_t gwn_eytzinger_slots(int64_t m);
int gwn_eytzinger_aabb(const double* PB1, const double* PB2, int64_t m, int dim, double* B1,
                       double* B2, int32_t* leaf, int mem, void* stream);
int gwn_eytzinger_winding_number_tree(const int32_t* E, int64_t nE, const int32_t* leaf,
                                      int64_t slots, int32_t* C, int32_t* I, int mem,
                                      void* stream);
int gwn_eytzinger_winding_number(const double* P, int64_t nP, const double* V, int64_t nV,
                                 const int32_t* E, int64_t nE, const double* B1,
                                 const double* B2, const int32_t* leaf, int64_t slots,
                                 const int32_t* I, int64_t nI, const int32_t* C, double* W,
                                 int precision, int mem, void* stream);

/* ------------------------------------------------------------------------
 * Served evaluation (no counterpart in the reference: libigl evaluates one
 * mesh per call).  A server keeps triangle meshes resident on the device as
 * built soup trees and evaluates requests against them, each request being
 * igl::fast_winding_number(bvh, accuracy_scale, Q, W)
 * (include/igl/fast_winding_number.h:189-194) for its mesh.
 *
 *  - gwn_server_create: hbm_budget_bytes bounds the device bytes of resident
 *    trees; a tree is built when a request first needs it, and the least
 *    recently used trees with no request in flight are evicted to make room.
 *    Builds run on builder threads with their own streams, so batches of
 *    resident meshes keep running while a cold mesh builds; its requests
 *    join a batch once its tree is ready.
 *    max_batch_queries bounds the queries of one batch (each request's
 *    count is padded to a multiple of 32); `slots` batches may be on the
 *    device at once.  A worker thread forms a batch from the pending
 *    requests whenever a slot is free (continuous batching) and runs it as
 *    one captured CUDA graph on that slot's stream.
 *  - gwn_server_add_mesh copies V (#V x 3 double) and F (#F x 3 int32) into
 *    the server; the tree is the one gwn_soup_build makes (`order`).
 *  - gwn_server_submit queues one request; Q (host, #Q x 3, q_dtype) and W
 *    (host, #Q, w_dtype) must stay valid until gwn_server_wait returns for
 *    it.  precision as for gwn_soup_eval.  Results equal gwn_soup_eval's on
 *    the same mesh and queries.
 *  - gwn_server_wait blocks until the request finished (timeout_s < 0 or
 *    above 1e9: no limit; NaN is refused; GWN_ERR_TIMEOUT when it runs out,
 *    the request stays queued),
 *    returns its status, and reports submit-to-result latency in seconds.
 *    Every submitted request must be waited for once.
 *  - gwn_server_destroy finishes every queued request, then frees the
 *    server; no other call on the server may be running or follow.
 * ---------------------------------------------------------------------- */
typedef struct gwn_server gwn_server;

typedef struct gwn_server_stats {
  int64_t requests_done;
  int64_t queries_done;
  int64_t batches;
  int64_t builds;             /* trees built (first use or after eviction) */
  int64_t evictions;
  int64_t resident_meshes;
  int64_t resident_bytes;
  int64_t peak_resident_bytes;
  int64_t budget_bytes;
  int64_t refined;            /* queries re-evaluated in plain FP64 (|W-0.5| <= 1e-3) */
  int64_t pending;            /* submitted, not yet in a batch */
  int64_t kernels_per_batch;  /* kernel nodes of one batch graph */
  double batch_gpu_ms;        /* sum over batches of the graph's device time */
  double walk_gpu_ms;         /* sum over batches of the walk kernel's time */
} gwn_server_stats;

int gwn_server_create(int64_t hbm_budget_bytes, int64_t max_batch_queries, int32_t slots,
                      gwn_server** out);
int gwn_server_add_mesh(gwn_server* server, const double* V, int64_t nV, const int32_t* F,
                        int64_t nF, int order, int64_t* mesh_id);
/* GWN_ERR_BUSY while the mesh has requests queued or in flight. */
int gwn_server_remove_mesh(gwn_server* server, int64_t mesh_id);
int gwn_server_submit(gwn_server* server, int64_t mesh_id, const void* Q, int q_dtype,
                      int64_t nQ, void* W, int w_dtype, float accuracy_scale, int precision,
                      int64_t* request_id);
int gwn_server_wait(gwn_server* server, int64_t request_id, double timeout_s,
                    double* latency_s);
int gwn_server_stats_get(gwn_server* server, gwn_server_stats* out);
int gwn_server_destroy(gwn_server* server);

/* ------------------------------------------------------------------------
 * Per-phase timing (no counterpart in the reference; for benchmarks and
 * profiling).  After gwn_profile_enable(1), every call on this thread records
 * CUDA events around its phases on its stream (e.g. "order_queries", "walk",
 * "refine"); gwn_profile_read waits for the last call's events and returns
 * the phase names ';'-separated and their durations in milliseconds.
 * gwn_profile_enable(2) keeps the phases of every call until the next
 * gwn_profile_enable (so a timed loop can read them once, after it ends);
 * 0 turns recording off.  Each gwn_profile_enable clears what was kept.
 * ---------------------------------------------------------------------- */
int gwn_profile_enable(int on);
int gwn_profile_read(char* names, int names_cap, float* ms, int max_phases, int* num_phases);
/* Number of kernels this library has launched in this process (all threads). */
unsigned long long gwn_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* GWN_H */
