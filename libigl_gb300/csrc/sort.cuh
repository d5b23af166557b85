// Device-wide primitives written for this library: exclusive scan of uint32
// and a stable LSD radix sort of (key, int32 value) pairs.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gwn_common.cuh"

namespace gwn {

// out[i] = sum_{j<i} in[i]; returns nothing (total can be read from
// out[n-1] + in[n-1]).  `in` and `out` may alias.
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t st);

// Stable sort of (keys, vals) by bits [begin_bit, end_bit) of the key.  The
// result is left in (keys, vals); tmp buffers must hold n elements.
template <typename K>
void radix_sort_pairs(K* keys, int32_t* vals, K* keys_tmp, int32_t* vals_tmp, int64_t n,
                      int begin_bit, int end_bit, cudaStream_t st);

}  // namespace gwn
