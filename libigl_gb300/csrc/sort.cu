// Exclusive scan and stable LSD radix sort (8-bit digits).
//
// Radix pass = (1) per-tile digit histogram, (2) exclusive scan of the
// digit-major [256 x tiles] count table, (3) stable scatter: each tile
// revisits its elements in rounds of 256 (one per thread, in input order),
// ranks equal digits inside each warp with __match_any_sync, prefixes the
// per-warp counts in shared memory, and writes each element to
// base[digit][tile] + running count + warp prefix + lane rank.
#include <cuda_runtime.h>

#include <algorithm>
#include <utility>

#include "sort.cuh"

namespace gwn {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t& excl) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const uint32_t incl = warp_incl_scan(v);
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < nw ? warp_tot[lane] : 0u;
    t = warp_incl_scan(t);
    if (lane < nw) warp_tot[lane] = t;
  }
  __syncthreads();
  const uint32_t wbase = warp ? warp_tot[warp - 1] : 0u;
  const uint32_t total = warp_tot[nw - 1];
  excl = wbase + incl - v;
  __syncthreads();
  return total;
}

__global__ void scan_partials_kernel(const uint32_t* __restrict__ in, int64_t n,
                                     uint32_t* __restrict__ partials) {
  const int64_t base = blockIdx.x * (int64_t)kScanTile;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
    if (i < n) s += in[i];
  }
  uint32_t ex;
  const uint32_t tot = block_excl_scan(s, ex);
  if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

__global__ void scan_tiles_kernel(const uint32_t* in, uint32_t* out, int64_t n,
                                  const uint32_t* __restrict__ partial_offsets) {
  const int64_t base = blockIdx.x * (int64_t)kScanTile;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
    v[k] = i < n ? in[i] : 0u;
    s += v[k];
  }
  uint32_t ex;
  block_excl_scan(s, ex);
  uint32_t run = ex + (partial_offsets ? partial_offsets[blockIdx.x] : 0u);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
    if (i < n) out[i] = run;
    run += v[k];
  }
}

// ---------------------------------------------------------------- radix ----
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsThreads * kRsRounds;

// n_dev (optional): the element count is min(n, *n_dev), read on the device,
// so that a captured graph can sort batches of varying size.
template <typename K>
__global__ void __launch_bounds__(kRsThreads) rs_hist_kernel(const K* __restrict__ keys,
                                                             int64_t n, int shift,
                                                             uint32_t* __restrict__ counts,
                                                             int ntiles,
                                                             const uint32_t* __restrict__ n_dev) {
  if (n_dev) n = min(n, (int64_t)*n_dev);
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = blockIdx.x * (int64_t)kRsTile;
#pragma unroll 4
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t i = base + (int64_t)r * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

template <typename K>
__global__ void __launch_bounds__(kRsThreads) rs_scatter_kernel(
    const K* __restrict__ kin, const int32_t* __restrict__ vin, K* __restrict__ kout,
    int32_t* __restrict__ vout, int64_t n, int shift, const uint32_t* __restrict__ offsets,
    int ntiles, const uint32_t* __restrict__ n_dev) {
  if (n_dev) n = min(n, (int64_t)*n_dev);
  __shared__ uint32_t s_base[256];
  __shared__ uint32_t s_warp[kRsThreads / 32][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  s_base[tid] = offsets[(int64_t)tid * ntiles + blockIdx.x];
  const uint32_t lt_mask = (1u << lane) - 1u;
  const int64_t base = blockIdx.x * (int64_t)kRsTile;
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t i = base + (int64_t)r * kRsThreads + tid;
    const bool valid = i < n;
    K k = 0;
    int32_t v = 0;
    uint32_t d = 256u;
    if (valid) {
      k = kin[i];
      v = vin[i];
      d = (uint32_t)(k >> shift) & 255u;
    }
#pragma unroll
    for (int w = 0; w < kRsThreads / 32; ++w) s_warp[w][tid] = 0u;
    __syncthreads();
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lt_mask);
    if (valid && rank == 0) s_warp[warp][d] = __popc(peers);
    __syncthreads();
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kRsThreads / 32; ++w) {
      const uint32_t c = s_warp[w][tid];
      s_warp[w][tid] = run;
      run += c;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_base[d] + s_warp[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
    s_base[tid] += run;
  }
}

__global__ void bucket_rank_kernel(const uint32_t* __restrict__ keys, int64_t n,
                                   uint32_t* __restrict__ cnt, uint32_t* __restrict__ rank) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) rank[i] = atomicAdd(&cnt[keys[i]], 1u);
}

__global__ void bucket_place_kernel(const uint32_t* __restrict__ keys, int64_t n,
                                    const uint32_t* __restrict__ off,
                                    const uint32_t* __restrict__ rank, int32_t* __restrict__ perm) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) perm[off[keys[i]] + rank[i]] = (int32_t)i;
}

}  // namespace

void bucket_order(const uint32_t* keys, int64_t n, uint32_t nbuckets, int32_t* perm,
                  cudaStream_t st) {
  if (n <= 0) return;
  GWN_REQUIRE(n < (int64_t(1) << 31), "bucket order: at most 2^31-1 elements");
  DevBuf<uint32_t> cnt((size_t)nbuckets, st), rank((size_t)n, st);
  cnt.zero(st);
  const unsigned grid = (unsigned)((n + 255) / 256);
  launch_kernel(bucket_rank_kernel, grid, 256, 0, st, keys, n, cnt.get(), rank.get());
  exclusive_scan_u32(cnt.get(), cnt.get(), nbuckets, st);
  launch_kernel(bucket_place_kernel, grid, 256, 0, st, keys, n, cnt.get(), rank.get(), perm);
}

int64_t scan_scratch_elems(int64_t n) {
  int64_t total = 0;
  while (n > kScanTile) {
    n = (n + kScanTile - 1) / kScanTile;
    total += n;
  }
  return total;
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t st,
                        uint32_t* scratch) {
  if (n <= 0) return;
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  if (nt == 1) {
    launch_kernel(scan_tiles_kernel, 1, kScanThreads, 0, st, in, out, n, nullptr);
    GWN_CUDA(cudaGetLastError());
    return;
  }
  DevBuf<uint32_t> own;
  uint32_t* partials = scratch;
  if (!partials) {
    own.alloc((size_t)nt, st);
    partials = own.get();
  }
  launch_kernel(scan_partials_kernel, (unsigned)nt, kScanThreads, 0, st, in, n, partials);
  GWN_CUDA(cudaGetLastError());
  exclusive_scan_u32(partials, partials, nt, st, scratch ? scratch + nt : nullptr);
  launch_kernel(scan_tiles_kernel, (unsigned)nt, kScanThreads, 0, st, in, out, n, partials);
  GWN_CUDA(cudaGetLastError());
}

template <typename K>
void radix_sort_pairs(K* keys, int32_t* vals, K* keys_tmp, int32_t* vals_tmp, int64_t n,
                      int begin_bit, int end_bit, cudaStream_t st) {
  if (n <= 1 || end_bit <= begin_bit) return;
  GWN_REQUIRE(n < (int64_t(1) << 32), "radix sort: at most 2^32-1 elements");
  const int ntiles = (int)((n + kRsTile - 1) / kRsTile);
  DevBuf<uint32_t> counts((size_t)ntiles * 256, st);
  K* ka = keys;
  int32_t* va = vals;
  K* kb = keys_tmp;
  int32_t* vb = vals_tmp;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    launch_kernel(rs_hist_kernel<K>, ntiles, kRsThreads, 0, st, ka, n, shift, counts.get(), ntiles,
                  (const uint32_t*)nullptr);
    exclusive_scan_u32(counts.get(), counts.get(), (int64_t)ntiles * 256, st);
    launch_kernel(rs_scatter_kernel<K>, ntiles, kRsThreads, 0, st, ka, va, kb, vb, n, shift,
                  counts.get(), ntiles, (const uint32_t*)nullptr);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    GWN_CUDA(cudaMemcpyAsync(keys, ka, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, st));
    GWN_CUDA(cudaMemcpyAsync(vals, va, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToDevice, st));
  }
}

void radix_sort_scratch_elems(int64_t cap, int64_t* counts_elems, int64_t* scan_elems) {
  const int64_t ntiles = (cap + kRsTile - 1) / kRsTile;
  *counts_elems = ntiles * 256;
  *scan_elems = scan_scratch_elems(ntiles * 256);
}

void radix_sort_pairs_devn(uint32_t* keys, int32_t* vals, uint32_t* keys_tmp, int32_t* vals_tmp,
                           int64_t cap, const uint32_t* n_dev, int begin_bit, int end_bit,
                           uint32_t* counts, uint32_t* scan_scratch, cudaStream_t st) {
  GWN_REQUIRE(((end_bit - begin_bit) / 8) % 2 == 0 && (end_bit - begin_bit) % 8 == 0,
              "radix_sort_pairs_devn: an even number of 8-bit passes");
  if (cap <= 0) return;
  GWN_REQUIRE(cap < (int64_t(1) << 32), "radix sort: at most 2^32-1 elements");
  const int ntiles = (int)((cap + kRsTile - 1) / kRsTile);
  uint32_t* ka = keys;
  int32_t* va = vals;
  uint32_t* kb = keys_tmp;
  int32_t* vb = vals_tmp;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    launch_kernel(rs_hist_kernel<uint32_t>, ntiles, kRsThreads, 0, st, ka, cap, shift, counts,
                  ntiles, n_dev);
    exclusive_scan_u32(counts, counts, (int64_t)ntiles * 256, st, scan_scratch);
    launch_kernel(rs_scatter_kernel<uint32_t>, ntiles, kRsThreads, 0, st, ka, va, kb, vb, cap,
                  shift, counts, ntiles, n_dev);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
}

template void radix_sort_pairs<uint32_t>(uint32_t*, int32_t*, uint32_t*, int32_t*, int64_t, int,
                                         int, cudaStream_t);
template void radix_sort_pairs<unsigned long long>(unsigned long long*, int32_t*,
                                                   unsigned long long*, int32_t*, int64_t, int,
                                                   int, cudaStream_t);

}  // namespace gwn
