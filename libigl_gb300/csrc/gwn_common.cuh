// Shared host/device helpers of libgwn: error plumbing, stream-ordered device
// buffers, and the bulk-copy / mbarrier primitives (inline PTX, sm_103a).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <atomic>

#include "../../include/gwn.h"

namespace gwn {

// ---------------------------------------------------------------- errors ----
struct Error : public std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define GWN_CUDA(call)                                                                  \
  do {                                                                                  \
    cudaError_t _e = (call);                                                            \
    if (_e != cudaSuccess) {                                                            \
      int _code = (_e == cudaErrorMemoryAllocation) ? GWN_ERR_OUT_OF_MEMORY               \
                                                     : GWN_ERR_CUDA;                     \
      throw ::gwn::Error(_code, std::string(#call) + ": " + cudaGetErrorString(_e));     \
    }                                                                                   \
  } while (0)

#define GWN_REQUIRE(cond, msg)                                                          \
  do {                                                                                  \
    if (!(cond)) throw ::gwn::Error(GWN_ERR_INVALID_ARGUMENT, (msg));                   \
  } while (0)

// Run `fn` and convert any exception into a status code + last-error message.
template <typename Fn>
int guarded(const char* where, Fn&& fn) {
  try {
    fn();
    return GWN_OK;
  } catch (const Error& e) {
    set_last_error(std::string(where) + ": " + e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error(std::string(where) + ": host allocation failed");
    return GWN_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_last_error(std::string(where) + ": " + e.what());
    return GWN_ERR_INTERNAL;
  }
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// The library's stream-ordered memory pool on the current device: memory
// freed into it stays reserved for the next call instead of being returned
// to the driver at every synchronization (the default pool's release
// threshold is 0, which makes every call map its buffers again).
cudaMemPool_t device_pool();

// Stream-ordered device buffer (cudaMallocFromPoolAsync on device_pool() /
// cudaFreeAsync).
template <typename T>
class DevBuf {
 public:
  DevBuf() = default;
  DevBuf(size_t n, cudaStream_t s) { alloc(n, s); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { swap(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      swap(o);
    }
    return *this;
  }
  void alloc(size_t n, cudaStream_t s) {
    release();
    stream_ = s;
    n_ = n;
    if (n == 0) return;
    GWN_CUDA(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p_), n * sizeof(T), device_pool(), s));
  }
  void release() {
    if (p_) cudaFreeAsync(p_, stream_);
    p_ = nullptr;
    n_ = 0;
  }
  T* get() const { return p_; }
  size_t size() const { return n_; }
  size_t bytes() const { return n_ * sizeof(T); }
  void zero(cudaStream_t s) {
    if (n_) GWN_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s));
  }
  void upload(const T* h, size_t n, cudaStream_t s) {
    if (n) GWN_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void download(T* h, size_t n, cudaStream_t s) const {
    if (n) GWN_CUDA(cudaMemcpyAsync(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  }

 private:
  void swap(DevBuf& o) {
    std::swap(p_, o.p_);
    std::swap(n_, o.n_);
    std::swap(stream_, o.stream_);
  }
  T* p_ = nullptr;
  size_t n_ = 0;
  cudaStream_t stream_ = nullptr;
};

// Persistent device allocation owned by a handle (cudaMalloc / cudaFree), so
// its lifetime does not depend on any caller stream.  A structure that lives
// for one call only can take its memory stream-ordered instead (ordered()
// before alloc: cudaMallocFromPoolAsync / cudaFreeAsync on that stream), so
// that neither the allocation nor the release synchronizes the device.
template <typename T>
class DevMem {
 public:
  DevMem() = default;
  explicit DevMem(size_t n) { alloc(n); }
  ~DevMem() { release(); }
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  void ordered(cudaStream_t s) {
    release();
    ordered_ = true;
    stream_ = s;
  }
  void alloc(size_t n) {
    release();
    n_ = n;
    if (!n) return;
    if (ordered_)
      GWN_CUDA(cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p_), n * sizeof(T), device_pool(),
                                       stream_));
    else
      GWN_CUDA(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(T)));
  }
  void release() {
    if (p_) {
      if (ordered_)
        cudaFreeAsync(p_, stream_);
      else
        cudaFree(p_);
    }
    p_ = nullptr;
    n_ = 0;
  }
  T* get() const { return p_; }
  size_t size() const { return n_; }
  size_t bytes() const { return n_ * sizeof(T); }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
  bool ordered_ = false;
  cudaStream_t stream_ = nullptr;
};

inline size_t dtype_size(int dt) { return dt == GWN_F64 ? 8 : 4; }

inline void check_dtype(int dt, const char* what) {
  GWN_REQUIRE(dt == GWN_F32 || dt == GWN_F64, std::string(what) + " dtype must be GWN_F32 or GWN_F64");
}
inline void check_precision(int p) {
  GWN_REQUIRE(p == GWN_PLAIN_FP64 || p == GWN_MIXED, "precision must be GWN_PLAIN_FP64 or GWN_MIXED");
}
// Mesh arguments: F (nF rows) indexes V (nV rows).  A non-empty array needs a
// non-null pointer and a non-empty F needs vertices to index, so no kernel
// reads through a null V or clamps indices into an empty one.
inline void check_mesh(const void* V, int64_t nV, const void* F, int64_t nF) {
  GWN_REQUIRE(nV >= 0 && nF >= 0, "sizes must be non-negative");
  GWN_REQUIRE(nV == 0 || V, "V must be non-null when nV > 0");
  GWN_REQUIRE(nF == 0 || F, "F must be non-null when nF > 0");
  GWN_REQUIRE(nF == 0 || nV > 0, "F has elements but V has no vertices");
}
inline void check_mem(int m) {
  GWN_REQUIRE(m == GWN_HOST || m == GWN_DEVICE, "mem must be GWN_HOST or GWN_DEVICE");
}

void ensure_device();
int num_sms();

// Failure-path testing (gwn_debug_fail_next_waits): 1 if the next bounded
// bulk-copy ring launch is to withhold one mbarrier arrival (consumes one
// pending request), else 0.
int take_wait_injection();

// Device-side status word written by kernels (atomicOr of kStatus* bits).
// Host-memory calls get a private word that is read after the call's own
// synchronization.  Device-memory calls never synchronize: they report into
// a sticky per-device word that gwn_device_status() reads and clears.
unsigned int* sticky_status_word();

struct DeviceStatus {
  DevBuf<unsigned int> word;
  bool host_mode;
  DeviceStatus(cudaStream_t s, bool host) : host_mode(host) {
    if (host) {
      word.alloc(1, s);
      word.zero(s);
    }
  }
  unsigned int* ptr() const { return host_mode ? word.get() : sticky_status_word(); }
  // Host mode: synchronizes the stream and raises if a kernel reported a
  // failure.  Device mode: no-op (the sticky word keeps the report).
  void check(cudaStream_t s, const char* where) const;
};

// 64 pinned host words for small device-to-host reads (a copy into pageable
// memory is staged by the driver on every call), one buffer per host thread
// kept for the thread's life: pinning memory costs more than the copies it
// speeds up.  A caller uses the words between its copy and its stream
// synchronization, and calls on one thread do not overlap.
inline unsigned* pinned_words() {
  struct Buf {
    unsigned* p = nullptr;
    ~Buf() {
      if (p) cudaFreeHost(p);
    }
  };
  thread_local Buf b;
  if (!b.p) GWN_CUDA(cudaMallocHost(reinterpret_cast<void**>(&b.p), 64 * sizeof(unsigned)));
  return b.p;
}

// Optional per-phase timing of the calling thread's ABI calls (CUDA events
// recorded on the launch stream).  Off unless gwn_profile_enable(1).
struct PhaseTimer {
  PhaseTimer(const char* name, cudaStream_t st);
  ~PhaseTimer();
  void* rec = nullptr;
};
void profile_begin_call();

// Every kernel of the library is launched through launch_kernel: the launch
// is checked and counted (gwn_launch_count()).
void count_launch();
// Adds n launches (kernels run by a graph launch).
void count_launches(unsigned long long n);
// While alive, launches made by this thread are not counted (graph capture:
// the captured kernels are counted when the graph is launched).
struct LaunchCountPause {
  LaunchCountPause();
  ~LaunchCountPause();
};
#ifdef __CUDACC__
template <typename... KArgs, typename... Args>
inline void launch_kernel(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                          cudaStream_t st, Args&&... args) {
  kernel<<<grid, block, smem, st>>>(std::forward<Args>(args)...);
  GWN_CUDA(cudaGetLastError());
  count_launch();
}
#endif

// Initialise 2*dim ordered-bit slots for atomicMin (first dim) / atomicMax.
void init_minmax(unsigned long long* mm, int dim, cudaStream_t s);

constexpr unsigned kStatusWaitTimeout = 1u;
constexpr unsigned kStatusBadInput = 2u;
constexpr unsigned kStatusInternal = 4u;  // a device-side consistency check failed

// Budget of a bounded mbarrier wait.  A bulk copy of a few KB lands within
// microseconds; a wait gives up once 50 ms of %globaltimer have passed and it
// has polled at least kMinPolls times (so a stale first timer read cannot end
// it early), or after kSpinLimit polls whatever the timer says.
constexpr uint64_t kWaitBudgetNs = 50ull * 1000 * 1000;
constexpr uint32_t kMinPolls = 4096;
constexpr uint32_t kSpinLimit = 1u << 26;

// --------------------------------------------------------- device helpers ----
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared, completion signalled on `bar` (tx bytes).
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait: returns false (and the caller reports a timeout) instead of
// spinning forever; see kWaitBudgetNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t i = 1; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= kMinPolls && (i & 63u) == 0 && globaltimer_ns() - t0 > kWaitBudgetNs) return false;
  }
  return false;
}

// Monotone maps double <-> uint64 so atomicMin/Max on unsigned long long order
// doubles correctly (finite values and infinities).
__device__ __forceinline__ unsigned long long ordered_bits(double x) {
  unsigned long long u = __double_as_longlong(x);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double from_ordered_bits(unsigned long long u) {
  unsigned long long v = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
  double d;
  memcpy(&d, &v, sizeof(d));
  return d;
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}
#endif

constexpr double kPi = 3.1415926535897932384626433832795;

}  // namespace gwn
