// Device-wide primitives written for this library: exclusive scan of uint32
// and a stable LSD radix sort of (key, int32 value) pairs.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

// out[i] = sum_{j<i} in[i]; returns nothing (total can be read from
// out[n-1] + in[n-1]).  `in` and `out` may alias.  `scratch` (optional,
// scan_scratch_elems(n) elements) replaces the internal allocation, so the
// call can be captured into a graph.
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t st,
                        uint32_t* scratch = nullptr);
int64_t scan_scratch_elems(int64_t n);

// Stable sort of (keys, vals) by bits [begin_bit, end_bit) of the key.  The
// result is left in (keys, vals); tmp buffers must hold n elements.
template <typename K>
void radix_sort_pairs(K* keys, int32_t* vals, K* keys_tmp, int32_t* vals_tmp, int64_t n,
                      int begin_bit, int end_bit, cudaStream_t st);

// Groups n keys (each < nbuckets) by value, ascending, in one counting pass:
// perm[k] is the input index of the k-th element.  The order inside a bucket
// is whatever order the atomics were served in (not stable), which suits
// query ordering for coherence: every walk here gives each query the same
// result whatever its neighbours in the warp.
void bucket_order(const uint32_t* keys, int64_t n, uint32_t nbuckets, int32_t* perm,
                  cudaStream_t st);

// Graph-capturable variant for 32-bit keys: sorts the first min(cap, *n_dev)
// elements (n_dev is device memory, read when the kernels run) with caller
// scratch (radix_sort_scratch_elems(cap)); an even number of 8-bit passes,
// so the result is left in (keys, vals) without a copy.
void radix_sort_scratch_elems(int64_t cap, int64_t* counts_elems, int64_t* scan_elems);
void radix_sort_pairs_devn(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp, int32_t* vals_tmp,
                           int64_t cap, const uint32_t* n_dev, int begin_bit, int end_bit,
                           uint32_t* counts, uint32_t* scan_scratch, cudaStream_t st);

}  // namespace gwn
