// C-ABI entry points of libgwn.so and the library-wide plumbing (last-error
// string, device status words, host/device staging of arguments).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gwn_common.cuh"
#include "gwn_internal.cuh"
#include "soup.cuh"
#include "octree.cuh"
#include "cloud.cuh"

namespace gwn {

namespace {
thread_local std::string g_last_error;
std::mutex g_dev_mutex;
std::vector<unsigned int*> g_sticky;  // per device
std::vector<int> g_sms;               // per device
}  // namespace

void set_last_error(const std::string& msg) { g_last_error = msg; }

namespace {
std::atomic<unsigned long long> g_launches{0};
}
static thread_local int t_count_paused = 0;
void count_launch() {
  if (!t_count_paused) g_launches.fetch_add(1, std::memory_order_relaxed);
}
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
LaunchCountPause::LaunchCountPause() { ++t_count_paused; }
LaunchCountPause::~LaunchCountPause() { --t_count_paused; }

namespace {
struct PhaseRec {
  std::string name;
  cudaEvent_t start = nullptr, stop = nullptr;
};
thread_local int g_profile = 0;  // 0 off, 1 per call, 2 accumulate across calls
thread_local std::vector<PhaseRec> g_phases;
void clear_phases() {
  for (auto& p : g_phases) {
    if (p.start) cudaEventDestroy(p.start);
    if (p.stop) cudaEventDestroy(p.stop);
  }
  g_phases.clear();
}
}  // namespace

void profile_begin_call() {
  if (g_profile == 1) clear_phases();
}

PhaseTimer::PhaseTimer(const char* name, cudaStream_t st) {
  if (!g_profile) return;
  g_phases.emplace_back();
  PhaseRec& r = g_phases.back();
  r.name = name;
  cudaEventCreate(&r.start);
  cudaEventCreate(&r.stop);
  cudaEventRecord(r.start, st);
  rec = new std::pair<size_t, cudaStream_t>(g_phases.size() - 1, st);
}

PhaseTimer::~PhaseTimer() {
  if (!rec) return;
  auto* p = static_cast<std::pair<size_t, cudaStream_t>*>(rec);
  if (p->first < g_phases.size()) cudaEventRecord(g_phases[p->first].stop, p->second);
  delete p;
}

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

static std::vector<cudaMemPool_t> g_pools;  // per device
cudaMemPool_t device_pool() {
  const int d = current_device();
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if ((int)g_pools.size() <= d) g_pools.resize(d + 1, nullptr);
  if (!g_pools[d]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = d;
    cudaMemPool_t pool = nullptr;
    GWN_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = ~0ull;
    GWN_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    g_pools[d] = pool;
  }
  return g_pools[d];
}


int num_sms() {
  const int d = current_device();
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if ((int)g_sms.size() <= d) g_sms.resize(d + 1, 0);
  if (!g_sms[d]) GWN_CUDA(cudaDeviceGetAttribute(&g_sms[d], cudaDevAttrMultiProcessorCount, d));
  return g_sms[d];
}

namespace {
std::atomic<int> g_wait_injections{0};
}  // namespace

int take_wait_injection() {
  int n = g_wait_injections.load();
  while (n > 0 && !g_wait_injections.compare_exchange_weak(n, n - 1)) {
  }
  return n > 0 ? 1 : 0;
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
  launch_kernel(init_minmax_kernel, 1, 32, 0, s, mm, dim);
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

struct gwn_soup {
  gwn_soup_impl impl;
  // Closest-point search for a GWN_TREE_REFERENCE handle: the binned tree
  // over the same triangles, built on the first gwn_soup_squared_distance.
  std::mutex search_mu;
  std::unique_ptr<gwn_soup_impl> search;
};
struct gwn_octree {
  gwn_octree_impl impl;
};
struct gwn_cloud {
  gwn_cloud_impl impl;
};
struct gwn_wn_aabb {
  int device = 0;
  DevMem<double> V;
  DevMem<int32_t> F;
  HierTree tree;
};

namespace {
void check_device_of(int dev) {
  int cur = 0;
  GWN_CUDA(cudaGetDevice(&cur));
  GWN_REQUIRE(cur == dev, "handle was built on another CUDA device than the current one");
}
}  // namespace

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
    v |= noalloc_sticky_status(clear != 0);
    if (flags) *flags = v;
  });
}

int gwn_debug_fail_next_waits(int n) {
  return guarded("gwn_debug_fail_next_waits", [&] {
    GWN_REQUIRE(n >= 0, "n must be non-negative");
    g_wait_injections.store(n);
  });
}

int gwn_winding_number(const double* V, int64_t nV, int dim, const int32_t* F, int64_t nF,
                       const void* O, int o_dtype, int64_t nO, void* W, int w_dtype,
                       int precision, int mem, void* stream) {
  return guarded("gwn_winding_number", [&] {
    profile_begin_call();
    GWN_REQUIRE(dim == 2 || dim == 3, "dim must be 2 (edges) or 3 (triangles)");
    GWN_REQUIRE(nV >= 0 && nF >= 0 && nO >= 0, "sizes must be non-negative");
    check_mesh(V, nV, F, nF);
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

int gwn_soup_build_tree(const double* V, int64_t nV, const int32_t* F, int64_t nF, int order,
                        int tree, int mem, void* stream, gwn_soup** out) {
  return guarded("gwn_soup_build", [&] {
    GWN_REQUIRE(out != nullptr, "out must be non-null");
    *out = nullptr;
    check_mesh(V, nV, F, nF);
    GWN_REQUIRE(tree == GWN_TREE_REFERENCE || tree == GWN_TREE_BINNED,
                "tree must be GWN_TREE_REFERENCE or GWN_TREE_BINNED");
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    Staged<double> dV(V, (size_t)nV * 3, mem, st);
    Staged<int32_t> dF(F, (size_t)nF * 3, mem, st);
    gwn_soup* s = new gwn_soup();
    try {
      GWN_CUDA(cudaGetDevice(&s->impl.device));
      if (tree == GWN_TREE_REFERENCE)
        soup_build_ref(s->impl, dV.dev, nV, dF.dev, nF, order, mem == GWN_HOST, st);
      else
        soup_build(s->impl, dV.dev, nV, dF.dev, nF, order, mem == GWN_HOST, st);
      GWN_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      delete s;
      throw;
    }
    *out = s;
  });
}

int gwn_soup_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, int order,
                   int mem, void* stream, gwn_soup** out) {
  return gwn_soup_build_tree(V, nV, F, nF, order, GWN_SOUP_TREE_DEFAULT, mem, stream, out);
}

int gwn_soup_tree_nodes(const gwn_soup* soup, int64_t* num_nodes, uint32_t* child) {
  return guarded("gwn_soup_tree_nodes", [&] {
    GWN_REQUIRE(soup != nullptr, "soup handle is null");
    const gwn_soup_impl& s = soup->impl;
    GWN_REQUIRE(s.tree == GWN_TREE_REFERENCE,
                "the handle was built with GWN_TREE_BINNED (no 4-wide node array)");
    if (num_nodes) *num_nodes = s.ref_nodes;
    if (child && s.ref_nodes)
      GWN_CUDA(cudaMemcpy(child, s.ref_child.get(), s.ref_child.bytes(), cudaMemcpyDeviceToHost));
  });
}

int gwn_soup_eval(const gwn_soup* soup, float accuracy_scale, const void* Q, int q_dtype,
                  int64_t nQ, void* W, int w_dtype, int precision, int mem, void* stream) {
  return guarded("gwn_soup_eval", [&] {
    profile_begin_call();
    GWN_REQUIRE(soup != nullptr, "soup handle is null");
    GWN_REQUIRE(nQ >= 0, "nQ must be non-negative");
    GWN_REQUIRE(nQ == 0 || (Q && W), "Q and W must be non-null");
    GWN_REQUIRE(nQ < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    GWN_REQUIRE(std::isfinite(accuracy_scale), "accuracy_scale must be finite");
    check_dtype(q_dtype, "Q");
    check_dtype(w_dtype, "W");
    check_precision(precision);
    check_mem(mem);
    ensure_device();
    check_device_of(soup->impl.device);
    cudaStream_t st = as_stream(stream);
    StagedBytes dQ(Q, (size_t)nQ * 3 * dtype_size(q_dtype), mem, st);
    StagedBytes dW(W, (size_t)nQ * dtype_size(w_dtype), mem, st, false);
    soup_eval(soup->impl, accuracy_scale, dQ.dev, q_dtype, nQ, dW.dev, w_dtype, precision, st);
    if (mem == GWN_HOST) {
      if (nQ)
        GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nQ * dtype_size(w_dtype),
                                 cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_soup_walk_stats(const gwn_soup* soup, float accuracy_scale, const double* Q, int64_t nQ,
                        int mem, unsigned long long* counters) {
  return guarded("gwn_soup_walk_stats", [&] {
    GWN_REQUIRE(soup && counters, "null argument");
    GWN_REQUIRE(nQ >= 0 && nQ < (int64_t(1) << 31), "0 <= nQ < 2^31");
    GWN_REQUIRE(nQ == 0 || Q, "Q must be non-null");
    GWN_REQUIRE(std::isfinite(accuracy_scale), "accuracy_scale must be finite");
    check_mem(mem);
    ensure_device();
    check_device_of(soup->impl.device);
    cudaStream_t st = nullptr;
    Staged<double> dQ(Q, (size_t)nQ * 3, mem, st);
    soup_walk_stats(soup->impl, accuracy_scale, dQ.dev, nQ, counters, st);
  });
}

int gwn_soup_stats_get(const gwn_soup* soup, gwn_soup_stats* out) {
  return guarded("gwn_soup_stats_get", [&] {
    GWN_REQUIRE(soup && out, "null argument");
    out->num_triangles = soup->impl.n;
    out->num_nodes = soup->impl.nnodes;
    out->tree = soup->impl.tree;
    out->tree_nodes = soup->impl.tree == GWN_TREE_REFERENCE ? soup->impl.ref_nodes
                                                            : soup->impl.nnodes;
    out->device_bytes = (int64_t)soup->impl.bytes;
    out->order = soup->impl.order;
    out->max_depth = soup->impl.max_depth;
  });
}

void gwn_soup_free(gwn_soup* soup) { delete soup; }

int gwn_soup_export(const gwn_soup* soup, double* nodes, int32_t* tri_index) {
  return guarded("gwn_soup_export", [&] {
    GWN_REQUIRE(soup != nullptr, "soup handle is null");
    static_assert(sizeof(SoupNodeD) == 24 * sizeof(double), "node record layout");
    const gwn_soup_impl& s = soup->impl;
    if (nodes && s.nnodes)
      GWN_CUDA(cudaMemcpy(nodes, s.nd.get(), s.nd.bytes(), cudaMemcpyDeviceToHost));
    if (tri_index && s.n)
      GWN_CUDA(cudaMemcpy(tri_index, s.tri_index.get(), s.tri_index.bytes(),
                          cudaMemcpyDeviceToHost));
  });
}


// ------------------------------------------------------------------ octree --
int gwn_octree_build(const double* P, int64_t nP, int mem, void* stream, gwn_octree** out) {
  return guarded("gwn_octree_build", [&] {
    GWN_REQUIRE(out != nullptr, "out must be non-null");
    *out = nullptr;
    GWN_REQUIRE(nP >= 0, "nP must be non-negative");
    GWN_REQUIRE(nP == 0 || P, "P must be non-null");
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    Staged<double> dP(P, (size_t)nP * 3, mem, st);
    gwn_octree* t = new gwn_octree();
    try {
      GWN_CUDA(cudaGetDevice(&t->impl.device));
      octree_build(t->impl, dP.dev, nP, mem == GWN_HOST, st);
      GWN_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      delete t;
      throw;
    }
    *out = t;
  });
}

int gwn_octree_sizes(const gwn_octree* tree, int64_t* num_cells, int64_t* num_indices,
                     int32_t* max_depth) {
  return guarded("gwn_octree_sizes", [&] {
    GWN_REQUIRE(tree != nullptr, "octree handle is null");
    if (num_cells) *num_cells = tree->impl.ncells;
    if (num_indices) *num_indices = tree->impl.nindices;
    if (max_depth) *max_depth = tree->impl.max_depth;
  });
}

int gwn_octree_export(const gwn_octree* tree, int64_t* pi_offsets, int32_t* pi_indices,
                      int32_t* CH, double* CN, double* W, int mem, void* stream) {
  return guarded("gwn_octree_export", [&] {
    GWN_REQUIRE(tree != nullptr, "octree handle is null");
    check_mem(mem);
    check_device_of(tree->impl.device);
    const gwn_octree_impl& t = tree->impl;
    cudaStream_t st = as_stream(stream);
    const size_t nc = (size_t)t.ncells;
    const cudaMemcpyKind kind = mem == GWN_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (pi_offsets || pi_indices) {
      DevBuf<int64_t> off(nc + 1, st);
      DevBuf<int32_t> idx((size_t)std::max<int64_t>(t.nindices, 1), st);
      octree_export_csr(t, off.get(), pi_indices ? idx.get() : nullptr, st);
      if (pi_offsets) GWN_CUDA(cudaMemcpyAsync(pi_offsets, off.get(), (nc + 1) * 8, kind, st));
      if (pi_indices && t.nindices)
        GWN_CUDA(cudaMemcpyAsync(pi_indices, idx.get(), (size_t)t.nindices * 4, kind, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
    if (CH) GWN_CUDA(cudaMemcpyAsync(CH, t.ch.get(), nc * 8 * 4, kind, st));
    if (CN) GWN_CUDA(cudaMemcpyAsync(CN, t.cn.get(), nc * 3 * 8, kind, st));
    if (W) GWN_CUDA(cudaMemcpyAsync(W, t.w.get(), nc * 8, kind, st));
    if (mem == GWN_HOST) GWN_CUDA(cudaStreamSynchronize(st));
  });
}

void gwn_octree_free(gwn_octree* tree) { delete tree; }

// ------------------------------------------------------------------- cloud --
int gwn_cloud_build(const gwn_octree* tree, const double* P, const double* N, const double* A,
                    int order, int mem, void* stream, gwn_cloud** out) {
  return guarded("gwn_cloud_build", [&] {
    GWN_REQUIRE(out != nullptr, "out must be non-null");
    *out = nullptr;
    GWN_REQUIRE(tree != nullptr, "octree handle is null");
    check_mem(mem);
    check_device_of(tree->impl.device);
    const int64_t n = tree->impl.n;
    GWN_REQUIRE(n == 0 || (N && A), "N and A must be non-null");
    (void)P;  // the octree handle holds its own copy of the points
    cudaStream_t st = as_stream(stream);
    Staged<double> dN(N, (size_t)n * 3, mem, st);
    Staged<double> dA(A, (size_t)n, mem, st);
    gwn_cloud* c = new gwn_cloud();
    try {
      c->impl.device = tree->impl.device;
      cloud_build(c->impl, tree->impl, dN.dev, dA.dev, order, st);
      GWN_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}

int gwn_cloud_export(const gwn_cloud* cloud, double* CM, double* R, double* EC, int mem,
                     void* stream) {
  return guarded("gwn_cloud_export", [&] {
    GWN_REQUIRE(cloud != nullptr, "cloud handle is null");
    check_mem(mem);
    check_device_of(cloud->impl.device);
    const gwn_cloud_impl& c = cloud->impl;
    cudaStream_t st = as_stream(stream);
    const cudaMemcpyKind kind = mem == GWN_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    const size_t nc = (size_t)c.ncells;
    if (CM) GWN_CUDA(cudaMemcpyAsync(CM, c.CM.get(), nc * 24, kind, st));
    if (R) GWN_CUDA(cudaMemcpyAsync(R, c.R.get(), nc * 8, kind, st));
    if (EC) GWN_CUDA(cudaMemcpyAsync(EC, c.EC.get(), nc * c.num_terms * 8, kind, st));
    if (mem == GWN_HOST) GWN_CUDA(cudaStreamSynchronize(st));
  });
}

int gwn_cloud_eval(const gwn_cloud* cloud, double beta, const void* Q, int q_dtype, int64_t nQ,
                   void* W, int w_dtype, int precision, int mem, void* stream) {
  return guarded("gwn_cloud_eval", [&] {
    profile_begin_call();
    GWN_REQUIRE(cloud != nullptr, "cloud handle is null");
    GWN_REQUIRE(nQ >= 0 && nQ < (int64_t(1) << 31), "0 <= nQ < 2^31");
    GWN_REQUIRE(nQ == 0 || (Q && W), "Q and W must be non-null");
    check_dtype(q_dtype, "Q");
    check_dtype(w_dtype, "W");
    check_precision(precision);
    check_mem(mem);
    check_device_of(cloud->impl.device);
    cudaStream_t st = as_stream(stream);
    StagedBytes dQ(Q, (size_t)nQ * 3 * dtype_size(q_dtype), mem, st);
    StagedBytes dW(W, (size_t)nQ * dtype_size(w_dtype), mem, st, false);
    cloud_eval(cloud->impl, beta, dQ.dev, q_dtype, nQ, dW.dev, w_dtype, precision, st);
    if (mem == GWN_HOST) {
      if (nQ)
        GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nQ * dtype_size(w_dtype),
                                 cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

void gwn_cloud_free(gwn_cloud* cloud) { delete cloud; }

// The caller's octree arrays (igl::octree's point_indices as CSR, CH): checked
// on the host before anything reaches the device.
static void check_csr(const double* P, const double* N, const double* A, int64_t nP,
                      const int64_t* pi_offsets, const int32_t* pi_indices, const int32_t* CH,
                      int64_t ncells) {
  GWN_REQUIRE(ncells >= 1, "the octree needs at least the root cell");
  GWN_REQUIRE(nP == 0 || (P && N && A), "P, N and A must be non-null");
  GWN_REQUIRE(pi_offsets[0] == 0, "pi_offsets[0] must be 0");
  for (int64_t c = 0; c < ncells; ++c) {
    GWN_REQUIRE(pi_offsets[c + 1] >= pi_offsets[c], "pi_offsets must be non-decreasing");
    if (CH[c * 8] != -1)
      for (int k = 0; k < 8; ++k)
        GWN_REQUIRE(CH[c * 8 + k] > 0 && CH[c * 8 + k] < ncells, "CH child id out of range");
  }
  const int64_t nidx = pi_offsets[ncells];
  GWN_REQUIRE(nidx == 0 || pi_indices, "pi_indices must be non-null");
  for (int64_t j = 0; j < nidx; ++j)
    GWN_REQUIRE(pi_indices[j] >= 0 && pi_indices[j] < nP, "point index out of range");
}

int gwn_cloud_precompute_arrays(const double* P, const double* N, const double* A, int64_t nP,
                                const int64_t* pi_offsets, const int32_t* pi_indices,
                                const int32_t* CH, int64_t ncells, int order, double* CM,
                                double* R, double* EC) {
  return guarded("gwn_cloud_precompute_arrays", [&] {
    GWN_REQUIRE(nP >= 0 && ncells >= 1, "nP >= 0 and ncells >= 1");
    GWN_REQUIRE(pi_offsets && CH && CM && R && EC, "null argument");
    GWN_REQUIRE(order >= 0 && order <= 2, "expansion order must be 0, 1 or 2");
    check_csr(P, N, A, nP, pi_offsets, pi_indices, CH, ncells);
    const int64_t nidx = pi_offsets[ncells];
    ensure_device();
    cudaStream_t st = nullptr;
    Staged<double> dP(P, (size_t)nP * 3, GWN_HOST, st), dN(N, (size_t)nP * 3, GWN_HOST, st),
        dA(A, (size_t)nP, GWN_HOST, st);
    Staged<int64_t> doff(pi_offsets, (size_t)ncells + 1, GWN_HOST, st);
    Staged<int32_t> didx(pi_indices, (size_t)nidx, GWN_HOST, st);
    Staged<int32_t> dch(CH, (size_t)ncells * 8, GWN_HOST, st);
    gwn_cloud_impl c;
    cloud_build_arrays(c, dP.dev, dN.dev, dA.dev, nP, doff.dev, didx.dev, dch.dev, ncells, order,
                       true, nullptr, nullptr, nullptr, st);
    const int nt = c.num_terms;
    GWN_CUDA(cudaMemcpyAsync(CM, c.CM.get(), (size_t)ncells * 24, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaMemcpyAsync(R, c.R.get(), (size_t)ncells * 8, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaMemcpyAsync(EC, c.EC.get(), (size_t)ncells * nt * 8, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
  });
}

int gwn_cloud_eval_arrays(const double* P, const double* N, const double* A, int64_t nP,
                          const int64_t* pi_offsets, const int32_t* pi_indices,
                          const int32_t* CH, int64_t ncells, const double* CM, const double* R,
                          const double* EC, int order, const double* Q, int64_t nQ,
                          double beta, double* W, int precision) {
  return guarded("gwn_cloud_eval_arrays", [&] {
    GWN_REQUIRE(nP >= 0 && ncells >= 1 && nQ >= 0, "sizes");
    GWN_REQUIRE(pi_offsets && CH && CM && R && EC, "null argument");
    GWN_REQUIRE(nQ == 0 || (Q && W), "Q and W must be non-null");
    GWN_REQUIRE(order >= 0 && order <= 2, "expansion order must be 0, 1 or 2");
    check_precision(precision);
    check_csr(P, N, A, nP, pi_offsets, pi_indices, CH, ncells);
    const int64_t nidx = pi_offsets[ncells];
    ensure_device();
    cudaStream_t st = nullptr;
    Staged<double> dP(P, (size_t)nP * 3, GWN_HOST, st), dN(N, (size_t)nP * 3, GWN_HOST, st),
        dA(A, (size_t)nP, GWN_HOST, st);
    Staged<int64_t> doff(pi_offsets, (size_t)ncells + 1, GWN_HOST, st);
    Staged<int32_t> didx(pi_indices, (size_t)nidx, GWN_HOST, st);
    Staged<int32_t> dch(CH, (size_t)ncells * 8, GWN_HOST, st);
    const int nt = order == 0 ? 3 : (order == 1 ? 12 : 39);
    Staged<double> dCM(CM, (size_t)ncells * 3, GWN_HOST, st), dR(R, (size_t)ncells, GWN_HOST, st),
        dEC(EC, (size_t)ncells * nt, GWN_HOST, st);
    gwn_cloud_impl c;
    cloud_build_arrays(c, dP.dev, dN.dev, dA.dev, nP, doff.dev, didx.dev, dch.dev, ncells, order,
                       false, pi_offsets, pi_indices, CH, st);
    cloud_set_moments(c, dCM.dev, dR.dev, dEC.dev, st);
    cloud_emit_arrays(c, st);
    Staged<double> dQ(Q, (size_t)nQ * 3, GWN_HOST, st);
    Staged<double> dW(W, (size_t)nQ, GWN_HOST, st, false);
    cloud_eval(c, beta, dQ.dev, GWN_F64, nQ, dW.dev, GWN_F64, precision, st);
    if (nQ) GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nQ * 8, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
  });
}


// ---------------------------------------------------------------- profile --
int gwn_profile_enable(int on) {
  return guarded("gwn_profile_enable", [&] {
    GWN_REQUIRE(on >= 0 && on <= 2, "on must be 0, 1 or 2");
    g_profile = on;
    clear_phases();
  });
}

int gwn_profile_read(char* names, int names_cap, float* ms, int max_phases, int* num_phases) {
  return guarded("gwn_profile_read", [&] {
    std::string all;
    int n = 0;
    for (auto& p : g_phases) {
      float t = 0.f;
      GWN_CUDA(cudaEventSynchronize(p.stop));
      GWN_CUDA(cudaEventElapsedTime(&t, p.start, p.stop));
      if (n < max_phases && ms) ms[n] = t;
      if (!all.empty()) all += ";";
      all += p.name;
      ++n;
    }
    if (names && names_cap > 0) {
      const size_t k = std::min<size_t>((size_t)names_cap - 1, all.size());
      memcpy(names, all.data(), k);
      names[k] = 0;
    }
    if (num_phases) *num_phases = n;
  });
}


unsigned long long gwn_launch_count(void) { return g_launches.load(); }


int gwn_octree_knn(const gwn_octree* tree, const void* Q, int q_dtype, int64_t nQ, int64_t k,
                   int32_t* I, int mem, void* stream) {
  return guarded("gwn_octree_knn", [&] {
    GWN_REQUIRE(tree != nullptr, "octree handle is null");
    GWN_REQUIRE(nQ >= 0 && k >= 0, "nQ and k must be non-negative");
    const int64_t cols = knn_columns(tree->impl.n, k);
    GWN_REQUIRE(nQ == 0 || cols == 0 || (Q && I), "Q and I must be non-null");
    GWN_REQUIRE(nQ < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    check_dtype(q_dtype, "Q");
    check_mem(mem);
    ensure_device();
    check_device_of(tree->impl.device);
    cudaStream_t st = as_stream(stream);
    StagedBytes dQ(Q, (size_t)nQ * 3 * dtype_size(q_dtype), mem, st);
    Staged<int32_t> dI(I, (size_t)(nQ * cols), mem, st, false);
    octree_knn(tree->impl, dQ.dev, q_dtype, nQ, k, dI.dev, st);
    if (mem == GWN_HOST && nQ * cols) {
      GWN_CUDA(cudaMemcpyAsync(I, dI.dev, (size_t)(nQ * cols) * 4, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_knn(const double* P, int64_t nP, const double* V, int64_t nV, int64_t k, int32_t* I,
            int mem, void* stream) {
  return guarded("gwn_knn", [&] {
    GWN_REQUIRE(nP >= 0 && nV >= 0 && k >= 0, "sizes and k must be non-negative");
    const int64_t cols = knn_columns(nV, k);
    GWN_REQUIRE(nP == 0 || cols == 0 || (P && V && I), "P, V and I must be non-null");
    GWN_REQUIRE(nP < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    check_mem(mem);
    ensure_device();
    if (nP == 0 || cols == 0) return;
    cudaStream_t st = as_stream(stream);
    Staged<double> dV(V, (size_t)nV * 3, mem, st);
    Staged<double> dP(P, (size_t)nP * 3, mem, st);
    Staged<int32_t> dI(I, (size_t)(nP * cols), mem, st, false);
    gwn_octree_impl tree;
    GWN_CUDA(cudaGetDevice(&tree.device));
    octree_build(tree, dV.dev, nV, true, st);
    octree_knn(tree, dP.dev, GWN_F64, nP, k, dI.dev, st);
    if (mem == GWN_HOST)
      GWN_CUDA(cudaMemcpyAsync(I, dI.dev, (size_t)(nP * cols) * 4, cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
  });
}

int gwn_point_areas(const double* P, int64_t nP, const int32_t* I, int64_t k, const double* N,
                    double* A, double* T, int mem, void* stream) {
  return guarded("gwn_point_areas", [&] {
    GWN_REQUIRE(nP >= 0, "nP must be non-negative");
    GWN_REQUIRE(k >= 1 && k <= GWN_POINT_AREAS_MAX_K,
                "k must be in [1, " + std::to_string(GWN_POINT_AREAS_MAX_K) + "]");
    GWN_REQUIRE(nP == 0 || (P && I && N && A), "P, I, N and A must be non-null");
    check_mem(mem);
    ensure_device();
    if (nP == 0) return;
    cudaStream_t st = as_stream(stream);
    Staged<double> dP(P, (size_t)nP * 3, mem, st);
    Staged<int32_t> dI(I, (size_t)(nP * k), mem, st);
    Staged<double> dN(N, (size_t)nP * 3, mem, st);
    Staged<double> dA(A, (size_t)nP, mem, st, false);
    Staged<double> dT(T, T ? (size_t)nP * 3 : 0, mem, st, false);
    DeviceStatus status(st, mem == GWN_HOST);
    point_areas_run(dP.dev, nP, dI.dev, (int)k, dN.dev, dA.dev, T ? dT.dev : nullptr,
                    status.ptr(), st);
    status.check(st, "point_areas");
    if (mem == GWN_HOST) {
      GWN_CUDA(cudaMemcpyAsync(A, dA.dev, (size_t)nP * 8, cudaMemcpyDeviceToHost, st));
      if (T) GWN_CUDA(cudaMemcpyAsync(T, dT.dev, (size_t)nP * 24, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_cloud_winding_number_points(const double* P, const double* N, int64_t nP, const void* Q,
                                    int q_dtype, int64_t nQ, int order, double beta, void* W,
                                    int w_dtype, int precision, int mem, void* stream) {
  return guarded("gwn_cloud_winding_number_points", [&] {
    GWN_REQUIRE(nP >= 0 && nQ >= 0, "sizes must be non-negative");
    GWN_REQUIRE(nP == 0 || (P && N), "P and N must be non-null");
    GWN_REQUIRE(nQ == 0 || (Q && W), "Q and W must be non-null");
    GWN_REQUIRE(nQ < (int64_t(1) << 31) && nP < (int64_t(1) << 31), "at most 2^31-1 points");
    GWN_REQUIRE(order >= 0 && order <= 2, "order must be 0, 1 or 2");
    check_dtype(q_dtype, "Q");
    check_dtype(w_dtype, "W");
    check_precision(precision);
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    StagedBytes dQ(Q, (size_t)nQ * 3 * dtype_size(q_dtype), mem, st);
    StagedBytes dW(W, (size_t)nQ * dtype_size(w_dtype), mem, st, false);
    Staged<double> dP(P, (size_t)nP * 3, mem, st);
    Staged<double> dN(N, (size_t)nP * 3, mem, st);
    // copyleft/cgal/fast_winding_number.cpp:25-43: octree, 21 nearest
    // points, areas, order-`order` expansions, Barnes-Hut evaluation
    gwn_octree_impl tree;
    GWN_CUDA(cudaGetDevice(&tree.device));
    octree_build(tree, dP.dev, nP, true, st);
    const int64_t k = knn_columns(nP, 21);
    DevBuf<int32_t> I((size_t)std::max<int64_t>(nP * k, 1), st);
    DevBuf<double> A((size_t)std::max<int64_t>(nP, 1), st);
    DeviceStatus status(st, true);
    if (nP > 0 && k > 0) {
      octree_knn(tree, dP.dev, GWN_F64, nP, 21, I.get(), st);
      point_areas_run(dP.dev, nP, I.get(), (int)k, dN.dev, A.get(), nullptr, status.ptr(), st);
    }
    status.check(st, "cloud_winding_number_points (areas)");
    gwn_cloud_impl c;
    c.device = tree.device;
    cloud_build(c, tree, dN.dev, A.get(), order, st);
    cloud_eval(c, beta, dQ.dev, q_dtype, nQ, dW.dev, w_dtype, precision, st);
    if (mem == GWN_HOST && nQ)
      GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nQ * dtype_size(w_dtype),
                               cudaMemcpyDeviceToHost, st));
    GWN_CUDA(cudaStreamSynchronize(st));
  });
}

int gwn_soup_squared_distance(const gwn_soup* soup, const void* Q, int q_dtype, int64_t nQ,
                              double up_sqr_d, double* sqrD, int32_t* I, double* C, int mem,
                              void* stream) {
  return guarded("gwn_soup_squared_distance", [&] {
    GWN_REQUIRE(soup != nullptr, "soup handle is null");
    GWN_REQUIRE(nQ >= 0, "nQ must be non-negative");
    GWN_REQUIRE(nQ == 0 || (Q && sqrD && I && C), "Q, sqrD, I and C must be non-null");
    GWN_REQUIRE(nQ < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    check_dtype(q_dtype, "Q");
    check_mem(mem);
    ensure_device();
    check_device_of(soup->impl.device);
    cudaStream_t st = as_stream(stream);
    StagedBytes dQ(Q, (size_t)nQ * 3 * dtype_size(q_dtype), mem, st);
    Staged<double> dD(sqrD, (size_t)nQ, mem, st, false);
    Staged<int32_t> dI(I, (size_t)nQ, mem, st, false);
    Staged<double> dC(C, (size_t)nQ * 3, mem, st, false);
    if (soup->impl.tree == GWN_TREE_REFERENCE) {
      gwn_soup* ms = const_cast<gwn_soup*>(soup);
      {
        std::lock_guard<std::mutex> lk(ms->search_mu);
        if (!ms->search) {
          auto srch = std::make_unique<gwn_soup_impl>();
          srch->device = soup->impl.device;
          soup_build_search(soup->impl, *srch, st);
          ms->search = std::move(srch);
        }
      }
      soup_squared_distance(*soup->search, dQ.dev, q_dtype, nQ, up_sqr_d, dD.dev, dI.dev, dC.dev,
                            st);
      soup_remap_index(soup->impl.tri_index.get(), dI.dev, nQ, st);
    } else {
      soup_squared_distance(soup->impl, dQ.dev, q_dtype, nQ, up_sqr_d, dD.dev, dI.dev, dC.dev,
                            st);
    }
    if (mem == GWN_HOST && nQ) {
      GWN_CUDA(cudaMemcpyAsync(sqrD, dD.dev, (size_t)nQ * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaMemcpyAsync(I, dI.dev, (size_t)nQ * 4, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaMemcpyAsync(C, dC.dev, (size_t)nQ * 24, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_signed_distance(const double* P, int64_t nP, const double* V, int64_t nV,
                        const int32_t* F, int64_t nF, int sign_type, double lower_bound,
                        double upper_bound, double* S, int32_t* I, double* C, double* N,
                        int precision, int mem, void* stream) {
  return guarded("gwn_signed_distance", [&] {
    GWN_REQUIRE(nP >= 0 && nV >= 0 && nF >= 0, "sizes must be non-negative");
    GWN_REQUIRE(nP == 0 || (P && S && I && C), "P, S, I and C must be non-null");
    check_mesh(V, nV, F, nF);
    GWN_REQUIRE(nP < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    GWN_REQUIRE(sign_type >= GWN_SD_PSEUDONORMAL && sign_type <= GWN_SD_FAST_WINDING_NUMBER,
                "sign_type must be one of GWN_SD_*");
    check_precision(precision);
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    Staged<double> dP(P, (size_t)nP * 3, mem, st);
    Staged<double> dV(V, (size_t)nV * 3, mem, st);
    Staged<int32_t> dF(F, (size_t)nF * 3, mem, st);
    Staged<double> dS(S, (size_t)nP, mem, st, false);
    Staged<int32_t> dI(I, (size_t)nP, mem, st, false);
    Staged<double> dC(C, (size_t)nP * 3, mem, st, false);
    const bool want_n = N != nullptr && sign_type == GWN_SD_PSEUDONORMAL;
    Staged<double> dN(want_n ? N : nullptr, want_n ? (size_t)nP * 3 : 0, mem, st, false);
    signed_distance_run(dP.dev, nP, dV.dev, nV, dF.dev, nF, sign_type, lower_bound, upper_bound,
                        dS.dev, dI.dev, dC.dev, want_n ? dN.dev : nullptr, precision, st);
    if (mem == GWN_HOST && nP) {
      GWN_CUDA(cudaMemcpyAsync(S, dS.dev, (size_t)nP * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaMemcpyAsync(I, dI.dev, (size_t)nP * 4, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaMemcpyAsync(C, dC.dev, (size_t)nP * 24, cudaMemcpyDeviceToHost, st));
      if (want_n)
        GWN_CUDA(cudaMemcpyAsync(N, dN.dev, (size_t)nP * 24, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_winding_number_noalloc(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                               const double* O, int64_t nO, double* W, unsigned int* dev_status,
                               void* stream) {
  return guarded("gwn_winding_number_noalloc", [&] {
    GWN_REQUIRE(nV >= 0 && nF >= 0 && nO >= 0, "sizes must be non-negative");
    check_mesh(V, nV, F, nF);
    GWN_REQUIRE(nO == 0 || (O && W), "O and W must be non-null");
    GWN_REQUIRE(nO < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    GWN_REQUIRE(nF <= noalloc_max_triangles(),
                "nF = " + std::to_string(nF) + " exceeds the no-allocation limit of " +
                    std::to_string(noalloc_max_triangles()) + " triangles");
    ensure_device();
    run_exact_noalloc(V, nV, F, nF, static_cast<const double*>(O), nO, W, dev_status,
                      as_stream(stream));
  });
}

int64_t gwn_eytzinger_slots(int64_t m) { return eytzinger_slots(m); }

int gwn_eytzinger_aabb(const double* PB1, const double* PB2, int64_t m, int dim, double* B1,
                       double* B2, int32_t* leaf, int mem, void* stream) {
  return guarded("gwn_eytzinger_aabb", [&] {
    GWN_REQUIRE(m >= 0, "m must be non-negative");
    GWN_REQUIRE(dim >= 1 && dim <= 3, "dim must be 1, 2 or 3");
    GWN_REQUIRE(m < (int64_t(1) << 30), "at most 2^30-1 primitives");
    GWN_REQUIRE(m == 0 || (PB1 && PB2 && B1 && B2 && leaf), "PB1, PB2, B1, B2 and leaf must be non-null");
    check_mem(mem);
    ensure_device();
    if (m == 0) return;
    cudaStream_t st = as_stream(stream);
    const int64_t nb = eytzinger_slots(m);
    Staged<double> dP1(PB1, (size_t)(m * dim), mem, st), dP2(PB2, (size_t)(m * dim), mem, st);
    Staged<double> dB1(B1, (size_t)(nb * dim), mem, st, false), dB2(B2, (size_t)(nb * dim), mem, st, false);
    Staged<int32_t> dL(leaf, (size_t)nb, mem, st, false);
    eytzinger_build(dP1.dev, dP2.dev, m, dim, dB1.dev, dB2.dev, dL.dev, st);
    if (mem == GWN_HOST) {
      GWN_CUDA(cudaMemcpyAsync(B1, dB1.dev, (size_t)(nb * dim) * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaMemcpyAsync(B2, dB2.dev, (size_t)(nb * dim) * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaMemcpyAsync(leaf, dL.dev, (size_t)nb * 4, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_eytzinger_winding_number_tree(const int32_t* E, int64_t nE, const int32_t* leaf,
                                      int64_t slots, int32_t* C, int32_t* I, int mem,
                                      void* stream) {
  return guarded("gwn_eytzinger_winding_number_tree", [&] {
    GWN_REQUIRE(nE >= 0 && slots >= 0, "sizes must be non-negative");
    GWN_REQUIRE(C != nullptr, "C must be non-null");
    GWN_REQUIRE(slots == 0 || leaf, "leaf must be non-null");
    GWN_REQUIRE(nE == 0 || E, "E must be non-null");
    GWN_REQUIRE(nE < (int64_t(1) << 30) && slots <= (int64_t(1) << 31),
                "at most 2^30-1 segments and 2^31 slots");
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    DeviceStatus status(st, true);
    Staged<int32_t> dE(E, (size_t)nE * 2, mem, st), dL(leaf, (size_t)slots, mem, st);
    Staged<int32_t> dC(C, (size_t)slots + 1, mem, st, false);
    // the pair count is known only after the first pass: host-mode I is
    // staged after it
    int64_t total = eytzinger_pairs(dE.dev, nE, dL.dev, slots, dC.dev, nullptr, status.ptr(), st);
    if (I && total > 0) {
      Staged<int32_t> dI(I, (size_t)total, mem, st, false);
      eytzinger_pairs(dE.dev, nE, dL.dev, slots, dC.dev, dI.dev, status.ptr(), st);
      if (mem == GWN_HOST)
        GWN_CUDA(cudaMemcpyAsync(I, dI.dev, (size_t)total * 4, cudaMemcpyDeviceToHost, st));
    }
    if (mem == GWN_HOST)
      GWN_CUDA(cudaMemcpyAsync(C, dC.dev, (size_t)(slots + 1) * 4, cudaMemcpyDeviceToHost, st));
    status.check(st, "eytzinger_winding_number_tree");
  });
}

int gwn_eytzinger_winding_number(const double* P, int64_t nP, const double* V, int64_t nV,
                                 const int32_t* E, int64_t nE, const double* B1,
                                 const double* B2, const int32_t* leaf, int64_t slots,
                                 const int32_t* I, int64_t nI, const int32_t* C, double* W,
                                 int precision, int mem, void* stream) {
  return guarded("gwn_eytzinger_winding_number", [&] {
    profile_begin_call();
    GWN_REQUIRE(nP >= 0 && nV >= 0 && nE >= 0 && slots >= 0 && nI >= 0,
                "sizes must be non-negative");
    GWN_REQUIRE(nP == 0 || (P && W), "P and W must be non-null");
    GWN_REQUIRE(slots == 0 || (B1 && B2 && leaf && C), "B1, B2, leaf and C must be non-null");
    GWN_REQUIRE(nE == 0 || E, "E must be non-null");
    GWN_REQUIRE(nV == 0 || V, "V must be non-null");
    GWN_REQUIRE(nI == 0 || I, "I must be non-null");
    GWN_REQUIRE(slots == 0 || (slots >= 2 && (slots & (slots - 1)) == 0),
                "slots must be 0 or a power of two");
    GWN_REQUIRE(nP < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    check_precision(precision);
    check_mem(mem);
    ensure_device();
    if (nP == 0) return;
    cudaStream_t st = as_stream(stream);
    DeviceStatus status(st, mem == GWN_HOST);
    Staged<double> dP(P, (size_t)nP * 2, mem, st), dV(V, (size_t)nV * 2, mem, st);
    Staged<int32_t> dE(E, (size_t)nE * 2, mem, st);
    Staged<double> dB1(B1, (size_t)slots * 2, mem, st), dB2(B2, (size_t)slots * 2, mem, st);
    Staged<int32_t> dL(leaf, (size_t)slots, mem, st), dI(I, (size_t)nI, mem, st);
    Staged<int32_t> dC(C, slots ? (size_t)slots + 1 : 0, mem, st);
    Staged<double> dW(W, (size_t)nP, mem, st, false);
    eytzinger_eval(dP.dev, nP, dV.dev, nV, dE.dev, nE, dB1.dev, dB2.dev, dL.dev, slots, dI.dev,
                   dC.dev, nI, dW.dev, precision, status.ptr(), st);
    if (mem == GWN_HOST) {
      GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nP * 8, cudaMemcpyDeviceToHost, st));
      status.check(st, "eytzinger_winding_number");
    }
  });
}

int gwn_swept_volume_signed_distance(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                                     const double* transforms, int64_t nT, int sign_type,
                                     const double* GV, int64_t nGV, const int32_t* res, double h,
                                     double isolevel, const double* S0, double* S, int precision,
                                     int mem, void* stream) {
  return guarded("gwn_swept_volume_signed_distance", [&] {
    profile_begin_call();
    GWN_REQUIRE(nV >= 0 && nF >= 0 && nT >= 0 && nGV >= 0, "sizes must be non-negative");
    check_mesh(V, nV, F, nF);
    GWN_REQUIRE(nT == 0 || transforms, "transforms must be non-null");
    GWN_REQUIRE(nGV == 0 || (GV && S), "GV and S must be non-null");
    GWN_REQUIRE(res != nullptr, "res must be non-null");
    GWN_REQUIRE(nGV < (int64_t(1) << 31), "at most 2^31-1 grid points");
    GWN_REQUIRE(sign_type >= GWN_SD_PSEUDONORMAL && sign_type <= GWN_SD_FAST_WINDING_NUMBER,
                "sign_type must be one of GWN_SD_*");
    if (std::isfinite(isolevel))
      GWN_REQUIRE(res[0] >= 0 && res[1] >= 0 && res[2] >= 0 &&
                      (int64_t)res[0] * res[1] * res[2] == nGV,
                  "with a finite isolevel #GV must equal res[0]*res[1]*res[2]");
    check_precision(precision);
    check_mem(mem);
    ensure_device();
    if (nGV == 0) return;
    cudaStream_t st = as_stream(stream);
    Staged<double> dV(V, (size_t)nV * 3, mem, st), dGV(GV, (size_t)nGV * 3, mem, st);
    Staged<int32_t> dF(F, (size_t)nF * 3, mem, st);
    Staged<double> dS(S, (size_t)nGV, mem, st, false);
    if (S0) {
      if (mem == GWN_HOST)
        GWN_CUDA(cudaMemcpyAsync(dS.dev, S0, (size_t)nGV * 8, cudaMemcpyHostToDevice, st));
      else if (S0 != S)
        GWN_CUDA(cudaMemcpyAsync(dS.dev, S0, (size_t)nGV * 8, cudaMemcpyDeviceToDevice, st));
    } else {
      GWN_CUDA(cudaMemsetAsync(dS.dev, 0xff, (size_t)nGV * 8, st));  // NaN
    }
    std::vector<double> T((size_t)nT * 12);
    if (nT) {
      if (mem == GWN_HOST) {
        std::copy(transforms, transforms + nT * 12, T.begin());
      } else {
        GWN_CUDA(cudaMemcpyAsync(T.data(), transforms, T.size() * 8, cudaMemcpyDeviceToHost, st));
        GWN_CUDA(cudaStreamSynchronize(st));
      }
    }
    const int32_t r3[3] = {res[0], res[1], res[2]};
    swept_volume_run(dV.dev, nV, dF.dev, nF, T.data(), nT, sign_type, dGV.dev, nGV, r3, h,
                     isolevel, dS.dev, precision, st);
    if (mem == GWN_HOST) {
      GWN_CUDA(cudaMemcpyAsync(S, dS.dev, (size_t)nGV * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_flood_fill(const int32_t* res, double* S, int mem, void* stream) {
  return guarded("gwn_flood_fill", [&] {
    GWN_REQUIRE(res != nullptr, "res must be non-null");
    GWN_REQUIRE(res[0] >= 0 && res[1] >= 0 && res[2] >= 0, "res must be non-negative");
    const int64_t n = (int64_t)res[0] * res[1] * res[2];
    GWN_REQUIRE(n == 0 || S, "S must be non-null");
    GWN_REQUIRE(n < (int64_t(1) << 40), "grid too large");
    check_mem(mem);
    ensure_device();
    if (n == 0) return;
    cudaStream_t st = as_stream(stream);
    Staged<double> dS(S, (size_t)n, mem, st);
    const int32_t r3[3] = {res[0], res[1], res[2]};
    flood_fill_run(r3, dS.dev, st);
    if (mem == GWN_HOST) {
      GWN_CUDA(cudaMemcpyAsync(S, dS.dev, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

int gwn_wn_aabb_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, int mem,
                      void* stream, gwn_wn_aabb** out) {
  return guarded("gwn_wn_aabb_build", [&] {
    GWN_REQUIRE(out != nullptr, "out must be non-null");
    *out = nullptr;
    GWN_REQUIRE(nV >= 0 && nF >= 0, "sizes must be non-negative");
    check_mesh(V, nV, F, nF);
    check_mem(mem);
    ensure_device();
    cudaStream_t st = as_stream(stream);
    auto h = std::make_unique<gwn_wn_aabb>();
    GWN_CUDA(cudaGetDevice(&h->device));
    h->V.alloc((size_t)std::max<int64_t>(nV, 1) * 3);
    h->F.alloc((size_t)std::max<int64_t>(nF, 1) * 3);
    const cudaMemcpyKind kind = mem == GWN_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (nV) GWN_CUDA(cudaMemcpyAsync(h->V.get(), V, (size_t)nV * 24, kind, st));
    if (nF) GWN_CUDA(cudaMemcpyAsync(h->F.get(), F, (size_t)nF * 12, kind, st));
    DeviceStatus status(st, true);
    hier_build(h->V.get(), nV, h->F.get(), nF, h->tree, status.ptr(), st);
    status.check(st, "wn_aabb_build");
    *out = h.release();
  });
}

int gwn_wn_aabb_eval(const gwn_wn_aabb* tree, const double* Q, int64_t nQ, double* W, int mem,
                     void* stream) {
  return gwn_wn_aabb_eval_precision(tree, Q, nQ, W, GWN_MIXED, mem, stream);
}

int gwn_wn_aabb_eval_precision(const gwn_wn_aabb* tree, const double* Q, int64_t nQ, double* W,
                               int precision, int mem, void* stream) {
  return guarded("gwn_wn_aabb_eval", [&] {
    check_precision(precision);
    profile_begin_call();
    GWN_REQUIRE(tree != nullptr, "tree handle is null");
    GWN_REQUIRE(nQ >= 0, "nQ must be non-negative");
    GWN_REQUIRE(nQ == 0 || (Q && W), "Q and W must be non-null");
    GWN_REQUIRE(nQ < (int64_t(1) << 31), "at most 2^31-1 queries per call");
    check_mem(mem);
    ensure_device();
    check_device_of(tree->device);
    if (nQ == 0) return;
    cudaStream_t st = as_stream(stream);
    Staged<double> dQ(Q, (size_t)nQ * 3, mem, st);
    Staged<double> dW(W, (size_t)nQ, mem, st, false);
    hier_eval(tree->tree, dQ.dev, nQ, dW.dev, st, precision);
    if (mem == GWN_HOST) {
      GWN_CUDA(cudaMemcpyAsync(W, dW.dev, (size_t)nQ * 8, cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
    }
  });
}

void gwn_wn_aabb_free(gwn_wn_aabb* tree) { delete tree; }

}  // extern "C"
