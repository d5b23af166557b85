// C-ABI entry points of libgwn.so and the library-wide plumbing (last-error
// string, device status words, host/device staging of arguments).
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "gwn_common.cuh"
#include "gwn_internal.cuh"

namespace gwn {

namespace {
thread_local std::string g_last_error;
std::mutex g_dev_mutex;
std::vector<unsigned int*> g_sticky;  // per device
std::vector<int> g_sms;               // per device
}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }

void ensure_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    throw Error(GWN_ERR_NO_DEVICE, "no CUDA device available");
  }
}

static int current_device() {
  int d = 0;
  GWN_CUDA(cudaGetDevice(&d));
  return d;
}

int num_sms() {
  const int d = current_device();
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if ((int)g_sms.size() <= d) g_sms.resize(d + 1, 0);
  if (!g_sms[d]) GWN_CUDA(cudaDeviceGetAttribute(&g_sms[d], cudaDevAttrMultiProcessorCount, d));
  return g_sms[d];
}

unsigned int* sticky_status_word() {
  const int d = current_device();
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if ((int)g_sticky.size() <= d) g_sticky.resize(d + 1, nullptr);
  if (!g_sticky[d]) {
    GWN_CUDA(cudaMalloc(&g_sticky[d], sizeof(unsigned int)));
    GWN_CUDA(cudaMemset(g_sticky[d], 0, sizeof(unsigned int)));
  }
  return g_sticky[d];
}

static void raise_status(unsigned v, const char* where) {
  if (v & kStatusBadInput)
    throw Error(GWN_ERR_INVALID_ARGUMENT,
                std::string(where) + ": an index is out of range (F or point list)");
  if (v & kStatusWaitTimeout)
    throw Error(GWN_ERR_TIMEOUT, std::string(where) + ": a bounded device wait gave up");
  if (v) throw Error(GWN_ERR_INTERNAL, std::string(where) + ": device status " + std::to_string(v));
}

void DeviceStatus::check(cudaStream_t s, const char* where) const {
  if (!host_mode) return;
  unsigned v = 0;
  GWN_CUDA(cudaMemcpyAsync(&v, word.get(), sizeof(v), cudaMemcpyDeviceToHost, s));
  GWN_CUDA(cudaStreamSynchronize(s));
  raise_status(v, where);
}

__global__ void init_minmax_kernel(unsigned long long* mm, int dim) {
  const int i = threadIdx.x;
  if (i < dim) mm[i] = ~0ull;
  else if (i < 2 * dim) mm[i] = 0ull;
}

void init_minmax(unsigned long long* mm, int dim, cudaStream_t s) {
  init_minmax_kernel<<<1, 32, 0, s>>>(mm, dim);
  GWN_CUDA(cudaGetLastError());
}

// Stages an argument array on the device: host mode copies it in (or out),
// device mode passes the caller's pointer through.
template <typename T>
struct Staged {
  DevBuf<T> buf;
  T* dev = nullptr;
  Staged(const T* p, size_t n, int mem, cudaStream_t s, bool copy_in = true) {
    if (mem == GWN_DEVICE || n == 0) {
      dev = const_cast<T*>(p);
      return;
    }
    buf.alloc(n, s);
    if (copy_in) buf.upload(p, n, s);
    dev = buf.get();
  }
};

struct StagedBytes {
  DevBuf<unsigned char> buf;
  void* dev = nullptr;
  StagedBytes(const void* p, size_t bytes, int mem, cudaStream_t s, bool copy_in = true) {
    if (mem == GWN_DEVICE || bytes == 0) {
      dev = const_cast<void*>(p);
      return;
    }
    buf.alloc(bytes, s);
    if (copy_in)
      GWN_CUDA(cudaMemcpyAsync(buf.get(), p, bytes, cudaMemcpyHostToDevice, s));
    dev = buf.get();
  }
};

}  // namespace gwn

using namespace gwn;

extern "C" {

const char* gwn_last_error(void) { return g_last_error.c_str(); }

int gwn_version(void) { return GWN_VERSION; }

int gwn_device_status(unsigned int* flags, int clear) {
  return guarded("gwn_device_status", [&] {
    ensure_device();
    unsigned int* w = sticky_status_word();
    unsigned v = 0;
    GWN_CUDA(cudaDeviceSynchronize());
    GWN_CUDA(cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost));
    if (clear) GWN_CUDA(cudaMemset(w, 0, sizeof(unsigned int)));
    if (flags) *flags = v;
  });
}

int gwn_winding_number(const double* V, int64_t nV, int dim, const int32_t* F, int64_t nF,
                       const void* O, int o_dtype, int64_t nO, void* W, int w_dtype,
                       int precision, int mem, void* stream) {
  return guarded("gwn_winding_number", [&] {
    GWN_REQUIRE(dim == 2 || dim == 3, "dim must be 2 (edges) or 3 (triangles)");
    GWN_REQUIRE(nV >= 0 && nF >= 0 && nO >= 0, "sizes must be non-negative");
    GWN_REQUIRE(nF == 0 || (V && F), "V and F must be non-null");
    GWN_REQUIRE(nO == 0 || (O && W), "O and W must be non-null");
    GWN_REQUIRE(nO < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    check_dtype(o_dtype, "O");
    check_dtype(w_dtype, "W");
    check_precision(precision);
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    const bool host = mem == GWN_HOST;
    Staged<double> dV(V, (size_t)(nV * dim), mem, st);
    Staged<int32_t> dF(F, (size_t)(nF * dim), mem, st);
    StagedBytes dO(O, (size_t)(nO * dim) * dtype_size(o_dtype), mem, st);
    StagedBytes dW(W, (size_t)nO * dtype_size(w_dtype), mem, st, false);
    ExactArgs a{dV.dev, nV, dim, dF.dev, nF, dO.dev, o_dtype, nO, dW.dev, w_dtype, precision, host};
    run_exact(a, st);
    if (host) {
      if (nO)
        GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nO * dtype_size(w_dtype),
                                 cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

}  // extern "C"
