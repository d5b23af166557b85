// Served winding-number queries: many triangle meshes kept resident on the
// device as built soup trees, requests against them batched continuously and
// evaluated in one launch sequence per batch, replayed from a CUDA graph.
//
// libigl has no serving layer.  Each request computes what
// igl::fast_winding_number(bvh, accuracy_scale, Q, W)
// (include/igl/fast_winding_number.cpp:418-455) computes for its mesh, the
// tree being the one igl::fast_winding_number(V, F, order, bvh) (:380-416)
// stands for (built here as gwn_soup_build builds it: GWN_SOUP_TREE_DEFAULT,
// the reference's own tree).
//
//  admission  a mesh is built on the device the first time a request needs
//             it; resident trees are limited to an HBM budget, and the least
//             recently used trees with no request in flight are evicted to
//             make room;
//  batching   a worker thread forms a batch from the pending requests (FIFO,
//             up to a query capacity and 256 requests) whenever one of the
//             batch slots is free, so requests that arrive while others are
//             on the device join the next batch, and consecutive batches
//             overlap on the device (one stream per slot);
//  one launch per batch, for meshes of any mix of sizes:
//     desc     copy the batch descriptor (per request: tree pointers, beta,
//              query box, offsets) from pinned host memory;
//     stage    copy the queries from the pinned host stage into the device
//              (FP64) and give each a 32-bit key: request index (8 bits),
//              padding flag, 21-bit Morton code in its mesh's box; each
//              request's queries are padded to a multiple of 32 so that a
//              warp never spans two requests;
//     sort     stable radix sort of the keys (4 passes, batch size read on
//              the device);
//     walk     persistent warps take 32-query chunks from an atomic counter
//              and run the mixed-precision (or plain FP64) warp-coherent
//              walk of the chunk's mesh; results near 0.5 are listed;
//     refine   listed queries re-evaluated by the plain FP64 walk, one
//              thread each;
//     out      results (FP64, request-major) to pinned host memory.
//  The sequence is captured once per slot into a CUDA graph: every kernel
//  reads the batch size from the descriptor, so the graph is replayed
//  unchanged for every batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bh_common.cuh"
#include "gwn_common.cuh"
#include "soup.cuh"
#include "soup_walk.cuh"
#include "sort.cuh"

namespace gwn {
namespace {

using soupwalk::EvalParams;

constexpr int kMaxReqs = 256;  // the request index occupies 8 key bits
constexpr int kBuilders = 4;   // tree builder threads (and streams) per server

struct __align__(16) ServeReq {
  EvalParams prm;     // the request's tree and beta
  float lo[3], inv[3];  // Morton box of the mesh
  int64_t q_byte_off;   // queries: byte offset in the host stage
  int64_t out_off;      // first result / device query index (dense)
  int32_t aoff;         // first key position (multiple of 32)
  int32_t nq;
  int32_t q_f64;
  int32_t precision;
};

struct __align__(16) ServeHeader {
  uint32_t nreq;
  uint32_t n_aligned;  // key positions in use (sum of padded request sizes)
  uint32_t nq_total;   // dense query count
  uint32_t status;
};

static_assert(sizeof(ServeReq) % 16 == 0, "ServeReq must be a whole number of 16-byte words");

constexpr size_t kDescBytes = sizeof(ServeHeader) + kMaxReqs * sizeof(ServeReq);

// counters: [0] walk chunk counter, [1] refine list length
__global__ void serve_desc_kernel(const uint4* hdesc, uint4* __restrict__ ddesc,
                                  unsigned* __restrict__ counters) {
  const volatile ServeHeader* h = reinterpret_cast<const volatile ServeHeader*>(hdesc);
  const uint32_t nreq = min(h->nreq, (uint32_t)kMaxReqs);
  const int words = (int)((sizeof(ServeHeader) + nreq * sizeof(ServeReq)) / 16);
  const volatile uint4* src = hdesc;
  for (int i = threadIdx.x; i < words; i += blockDim.x) {
    uint4 v;
    v.x = src[i].x;
    v.y = src[i].y;
    v.z = src[i].z;
    v.w = src[i].w;
    ddesc[i] = v;
  }
  if (threadIdx.x < 4) counters[threadIdx.x] = 0u;
}

__device__ __forceinline__ uint32_t morton_cell7(double v, float lo, float inv) {
  const float t = ((float)v - lo) * inv * 128.f;
  const int c = (int)t;  // NaN -> 0
  return (uint32_t)min(max(c, 0), 127);
}

__global__ void __launch_bounds__(256) serve_stage_kernel(const ServeHeader* __restrict__ dh,
                                                          const ServeReq* __restrict__ dreq,
                                                          const unsigned char* hstage,
                                                          double* __restrict__ dq,
                                                          uint32_t* __restrict__ keys,
                                                          int32_t* __restrict__ vals) {
  const uint32_t na = dh->n_aligned;
  const int nreq = (int)dh->nreq;
  for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x) {
    int lo = 0, hi = nreq - 1;  // last request with aoff <= a
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (dreq[mid].aoff <= (int)a) lo = mid;
      else hi = mid - 1;
    }
    const ServeReq& R = dreq[lo];
    const int j = (int)a - R.aoff;
    uint32_t key = (uint32_t)lo << 24;
    if (j < R.nq) {
      double x, y, z;
      if (R.q_f64) {
        const volatile double* p =
            reinterpret_cast<const volatile double*>(hstage + R.q_byte_off) + 3 * (int64_t)j;
        x = p[0];
        y = p[1];
        z = p[2];
      } else {
        const volatile float* p =
            reinterpret_cast<const volatile float*>(hstage + R.q_byte_off) + 3 * (int64_t)j;
        x = (double)p[0];
        y = (double)p[1];
        z = (double)p[2];
      }
      double* d = dq + 3 * (R.out_off + j);
      d[0] = x;
      d[1] = y;
      d[2] = z;
      key |= spread10(morton_cell7(x, R.lo[0], R.inv[0])) |
             (spread10(morton_cell7(y, R.lo[1], R.inv[1])) << 1) |
             (spread10(morton_cell7(z, R.lo[2], R.inv[2])) << 2);
    } else {
      key |= 1u << 23;  // padding lanes sort after the request's queries
    }
    keys[a] = key;
    vals[a] = (int32_t)a;
  }
}

// 8 blocks per SM (64 registers): saturated 6.2e8 -> 7.0e8 queries/s against
// the 5 that the registers of the mixed and FP64 walks together would give.
__global__ void __launch_bounds__(128, 8) serve_walk_kernel(ServeHeader* __restrict__ dh,
                                                         const ServeReq* __restrict__ dreq,
                                                         const double* __restrict__ dq,
                                                         const uint32_t* __restrict__ keys,
                                                         const int32_t* __restrict__ vals,
                                                         double* __restrict__ dW,
                                                         int2* __restrict__ refine,
                                                         unsigned* __restrict__ counters) {
  // a warp walks either precision at a time: the two queues share memory
  __shared__ union WarpQueue {
    soupwalk::NearQueue near;
    soupwalk::Fp64Queue fp64;
  } warp_q[4];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t na = dh->n_aligned;
  const int nreq = (int)dh->nreq;
  const int64_t nq_total = (int64_t)dh->nq_total;
  for (;;) {
    unsigned chunk = 0;
    if (lane == 0) chunk = atomicAdd(&counters[0], 1u);
    chunk = __shfl_sync(full, chunk, 0);
    const uint32_t p = chunk * 32u + (uint32_t)lane;
    if (chunk * 32u >= na) break;
    const uint32_t key = keys[p];
    const int r_lane = (int)(key >> 24);
    const int r = __shfl_sync(full, r_lane, 0);
    if (r >= nreq) {  // corrupt keys: report, skip the chunk (r is warp-uniform)
      if (lane == 0) atomicOr(&dh->status, kStatusBadInput);
      continue;
    }
    const ServeReq& R = dreq[r];
    const int j = vals[p] - R.aoff;
    // Padded request sizes keep every chunk inside one request; a lane that
    // disagrees would mean a corrupt batch: it is reported and skipped.
    bool valid = j >= 0 && j < R.nq && R.out_off + j < nq_total;
    if (r_lane != r) {
      valid = false;
      atomicOr(&dh->status, kStatusBadInput);
    }
    double qx = 0, qy = 0, qz = 0;
    if (valid) {
      const double* q = dq + 3 * (R.out_off + j);
      qx = q[0];
      qy = q[1];
      qz = q[2];
    }
    const EvalParams prm = R.prm;
    double w;
    if (R.precision == GWN_MIXED) {
      float acc;
      double acc64;
      soupwalk::WalkCounters c;
      // every served tree is of the default kind (the builder below)
      soupwalk::walk_mixed<false, GWN_SOUP_TREE_DEFAULT>(prm, valid, qx, qy, qz, acc, acc64, c,
                                                         warp_q[threadIdx.x >> 5].near);
      w = soupwalk::mixed_result(acc, acc64);
      if (valid && fabs(w - 0.5) <= soupwalk::kBand) {
        const unsigned s = atomicAdd(&counters[1], 1u);
        refine[s] = make_int2(r, j);
      }
    } else {
      w = soupwalk::walk_fp64(prm, valid, qx, qy, qz, warp_q[threadIdx.x >> 5].fp64) *
          soupwalk::kInv4Pi;
    }
    if (valid) dW[R.out_off + j] = w;
  }
}

__global__ void __launch_bounds__(128) serve_refine_kernel(const ServeReq* __restrict__ dreq,
                                                           const double* __restrict__ dq,
                                                           const int2* __restrict__ refine,
                                                           const unsigned* __restrict__ counters,
                                                           double* __restrict__ dW) {
  const unsigned n = counters[1];
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int2 e = refine[i];
    const ServeReq& R = dreq[e.x];
    const double* q = dq + 3 * (R.out_off + e.y);
    dW[R.out_off + e.y] = soupwalk::walk_fp64_lane(R.prm, q[0], q[1], q[2]) * soupwalk::kInv4Pi;
  }
}

__global__ void __launch_bounds__(256) serve_out_kernel(const ServeHeader* __restrict__ dh,
                                                        const double* __restrict__ dW,
                                                        const unsigned* __restrict__ counters,
                                                        double* hout, unsigned* hinfo) {
  const uint32_t n = dh->nq_total;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    hout[i] = dW[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    hinfo[0] = counters[1];
    hinfo[1] = dh->status;
  }
}

// A small fork-join pool for the host-side copies of a batch (queries into
// the pinned stage, results out to the callers' arrays): run(n, f) calls
// f(0..n-1) on the pool threads and the calling thread, and returns when all
// calls have returned.
class CopyPool {
 public:
  explicit CopyPool(int threads) {
    for (int i = 0; i < threads; ++i) th_.emplace_back([this] { loop(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(int n, const std::function<void(int)>& f) {
    if (n <= 0) return;
    std::unique_lock<std::mutex> lk(mu_);
    job_ = &f;
    njobs_ = n;
    next_ = 0;
    finished_ = 0;
    ++gen_;
    cv_.notify_all();
    work(lk);
    done_.wait(lk, [&] { return finished_ == njobs_; });
    job_ = nullptr;
  }

 private:
  void work(std::unique_lock<std::mutex>& lk) {
    while (job_ && next_ < njobs_) {
      const int i = next_++;
      const std::function<void(int)>* f = job_;
      lk.unlock();
      (*f)(i);
      lk.lock();
      if (++finished_ == njobs_) done_.notify_all();
    }
  }
  void loop() {
    std::unique_lock<std::mutex> lk(mu_);
    uint64_t seen = 0;
    for (;;) {
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      work(lk);
    }
  }
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int njobs_ = 0, next_ = 0, finished_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Pieces of at most kCopyPiece queries per copy task.
constexpr int64_t kCopyPiece = 1 << 16;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Pinned, device-mapped host buffer.
struct HostMapped {
  void* h = nullptr;
  void* d = nullptr;
  size_t bytes = 0;
  void alloc(size_t n) {
    bytes = n;
    GWN_CUDA(cudaHostAlloc(&h, n, cudaHostAllocMapped | cudaHostAllocPortable));
    GWN_CUDA(cudaHostGetDevicePointer(&d, h, 0));
  }
  ~HostMapped() {
    if (h) cudaFreeHost(h);
  }
};

}  // namespace
}  // namespace gwn

using namespace gwn;

struct SrvMesh {
  int64_t id = 0;
  std::vector<double> V;
  std::vector<int32_t> F;
  int order = 2;
  std::unique_ptr<gwn_soup_impl> res;
  size_t bytes = 0;       // resident bytes (estimate until the first build)
  uint64_t last_use = 0;
  int pending = 0;        // submitted, not yet in a batch
  int inflight = 0;       // in a batch on the device
  bool building = false;  // queued for, or being built by, the builder thread
  int64_t reserved = 0;   // bytes of the budget held for it while it builds
};

struct SrvReq {
  int64_t id = 0;
  SrvMesh* mesh = nullptr;
  const void* Q = nullptr;
  int q_dtype = GWN_F32;
  int64_t nq = 0;
  void* W = nullptr;
  int w_dtype = GWN_F32;
  float beta = 2.f;
  int precision = GWN_MIXED;
  double t_submit = 0, t_done = 0;
  bool done = false;
  int status = GWN_OK;
  std::string err;
};

struct SrvSlot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev_start = nullptr, ev_done = nullptr, ev_walk0 = nullptr, ev_walk1 = nullptr;
  HostMapped hdesc, hstage, hout, hinfo;
  DevMem<unsigned char> ddesc;
  DevMem<double> dq, dW;
  DevMem<uint32_t> keys, keys_tmp, counts, scan, counters;
  DevMem<int32_t> vals, vals_tmp;
  DevMem<int2> refine;
  cudaGraphExec_t exec = nullptr;
  int64_t kernels = 0;
  bool busy = false;
  std::vector<SrvReq*> reqs;
  std::vector<int64_t> out_off;
};

struct gwn_server {
  int device = 0;
  int64_t budget = 0;
  int64_t cap = 0;  // key positions per batch (multiple of 32)
  int max_reqs = kMaxReqs;
  std::vector<std::unique_ptr<SrvSlot>> slots;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false, stop_builder = false;
  std::thread worker;
  // Tree builds run on their own thread and stream: the worker keeps
  // completing and launching batches while a mesh builds, and a request
  // whose mesh is building waits in `pending` while later ones go ahead.
  std::vector<std::thread> builders;  // kBuilders threads, one stream each
  std::vector<cudaStream_t> build_streams;
  std::condition_variable cv_build;
  std::deque<SrvMesh*> build_q;
  int building = 0;       // meshes queued or being built
  uint64_t events = 0;    // bumped by submissions and finished builds

  int64_t next_mesh = 1, next_req = 1;
  uint64_t tick = 0;
  std::unordered_map<int64_t, std::unique_ptr<SrvMesh>> meshes;
  std::unordered_map<int64_t, std::unique_ptr<SrvReq>> reqs;
  std::deque<SrvReq*> pending;

  gwn_server_stats stats{};
  int64_t resident_bytes = 0;
  std::unique_ptr<CopyPool> pool;
  std::vector<std::pair<int, int64_t>> pieces;  // (request, first query) of the batch being copied

  ~gwn_server();
  void capture(SrvSlot& s);
  void run();
  void finish(SrvSlot& s, std::unique_lock<std::mutex>& lk);
  bool form_and_launch(SrvSlot& s, std::unique_lock<std::mutex>& lk);
  int admit(SrvMesh* m, bool room_may_free, int& code, std::string& err);
  void build_loop(cudaStream_t st);
  void evict(SrvMesh* m);
  void complete(SrvReq* r, int status, const std::string& err);
};

// A resident tree's device bytes, bounded before its build: at most 2n-1
// walk records of 96 + 192 bytes, 124 bytes per triangle, and for the
// 4-wide tree at most n-1 nodes of 16 bytes (the binary tree: 2 search
// records of 16 bytes per node instead).
static int64_t estimate_bytes(int64_t nF) {
  const int64_t recs = std::max<int64_t>(1, 2 * nF - 1);
  const int64_t tree = GWN_SOUP_TREE_DEFAULT == GWN_TREE_REFERENCE
                           ? std::max<int64_t>(1, nF - 1) * 16
                           : recs * (int64_t)(2 * sizeof(float4));
  return recs * (int64_t)(sizeof(SoupNodeF) + sizeof(SoupNodeD)) + tree +
         nF * (int64_t)(3 * sizeof(float4) + 9 * sizeof(double) + sizeof(int32_t));
}

void gwn_server::capture(SrvSlot& s) {
  LaunchCountPause pause;
  ServeHeader* dh = reinterpret_cast<ServeHeader*>(s.ddesc.get());
  const ServeReq* dreq = reinterpret_cast<const ServeReq*>(s.ddesc.get() + sizeof(ServeHeader));
  const int sms = num_sms();
  int walk_blocks = 0;
  GWN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&walk_blocks, serve_walk_kernel, 128, 0));
  walk_blocks = std::max(1, walk_blocks) * sms;
  GWN_CUDA(cudaStreamBeginCapture(s.st, cudaStreamCaptureModeThreadLocal));
  cudaGraph_t g = nullptr;
  try {
    launch_kernel(serve_desc_kernel, 1, 256, 0, s.st, (const uint4*)s.hdesc.d,
                  (uint4*)s.ddesc.get(), s.counters.get());
    launch_kernel(serve_stage_kernel, sms * 8, 256, 0, s.st, (const ServeHeader*)dh, dreq,
                  (const unsigned char*)s.hstage.d, s.dq.get(), s.keys.get(), s.vals.get());
    radix_sort_pairs_devn(s.keys.get(), s.vals.get(), s.keys_tmp.get(), s.vals_tmp.get(), cap,
                          &dh->n_aligned, 0, 32, s.counts.get(), s.scan.get(), s.st);
    GWN_CUDA(cudaEventRecordWithFlags(s.ev_walk0, s.st, cudaEventRecordExternal));
    launch_kernel(serve_walk_kernel, walk_blocks, 128, 0, s.st, dh, dreq,
                  (const double*)s.dq.get(), (const uint32_t*)s.keys.get(),
                  (const int32_t*)s.vals.get(), s.dW.get(), s.refine.get(), s.counters.get());
    GWN_CUDA(cudaEventRecordWithFlags(s.ev_walk1, s.st, cudaEventRecordExternal));
    launch_kernel(serve_refine_kernel, sms * 4, 128, 0, s.st, dreq, (const double*)s.dq.get(),
                  (const int2*)s.refine.get(), (const unsigned*)s.counters.get(), s.dW.get());
    launch_kernel(serve_out_kernel, sms * 4, 256, 0, s.st, (const ServeHeader*)dh,
                  (const double*)s.dW.get(), (const unsigned*)s.counters.get(),
                  (double*)s.hout.d, (unsigned*)s.hinfo.d);
  } catch (...) {
    cudaStreamEndCapture(s.st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  GWN_CUDA(cudaStreamEndCapture(s.st, &g));
  size_t nn = 0;
  cudaError_t e = cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (e == cudaSuccess && nn) e = cudaGraphGetNodes(g, nodes.data(), &nn);
  s.kernels = 0;
  for (size_t i = 0; e == cudaSuccess && i < nn; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
      ++s.kernels;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s.exec, g, 0);
  cudaGraphDestroy(g);
  GWN_CUDA(e);
}

void gwn_server::complete(SrvReq* r, int status, const std::string& err) {
  r->status = status;
  r->err = err;
  r->t_done = now_s();
  r->done = true;
}

void gwn_server::evict(SrvMesh* m) {
  resident_bytes -= (int64_t)m->bytes;
  m->res.reset();
  ++stats.evictions;
}

// Make mesh m resident.  Returns 0 (resident), 1 (its tree is queued or
// building), 3 (room is held by batches in flight or by other builds) or 2
// (cannot be served; code and err say why).  Called with the lock held; a
// build is queued for the builder thread with its bytes reserved, never run
// here.  room_may_free: some batch or build still holds budget that will
// come free.
int gwn_server::admit(SrvMesh* m, bool room_may_free, int& code, std::string& err) {
  if (m->res) return 0;
  if (m->building) return 1;
  const int64_t need = estimate_bytes((int64_t)m->F.size() / 3);
  if (need > budget) {
    code = GWN_ERR_OUT_OF_MEMORY;
    err = "mesh " + std::to_string(m->id) + " needs about " + std::to_string(need) +
          " device bytes, more than the budget of " + std::to_string(budget);
    return 2;
  }
  while (resident_bytes + need > budget) {
    SrvMesh* victim = nullptr;
    for (auto& kv : meshes) {
      SrvMesh* c = kv.second.get();
      if (c->res && c->inflight == 0 && c != m && (!victim || c->last_use < victim->last_use))
        victim = c;
    }
    if (!victim) {
      if (room_may_free || building > 0) return 3;
      code = GWN_ERR_OUT_OF_MEMORY;
      err = "mesh " + std::to_string(m->id) + " does not fit in the HBM budget";
      return 2;
    }
    evict(victim);
  }
  m->building = true;
  m->reserved = need;
  resident_bytes += need;
  stats.peak_resident_bytes = std::max<int64_t>(stats.peak_resident_bytes, resident_bytes);
  ++building;
  build_q.push_back(m);
  cv_build.notify_one();
  return 1;
}

// A builder thread: one tree at a time on its own stream, the lock
// released while it builds (small trees are latency-bound, so several
// builders overlap on the device).  A failed build completes the mesh's
// pending requests with the error.
void gwn_server::build_loop(cudaStream_t build_st) {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    cv_build.wait(lk, [&] { return stop_builder || !build_q.empty(); });
    if (build_q.empty()) {
      if (stop_builder) return;
      continue;
    }
    SrvMesh* m = build_q.front();
    build_q.pop_front();
    lk.unlock();
    std::unique_ptr<gwn_soup_impl> res(new gwn_soup_impl());
    int rc = GWN_OK;
    std::string err;
    try {
      const int64_t nF = (int64_t)m->F.size() / 3, nV = (int64_t)m->V.size() / 3;
      DevBuf<double> dV((size_t)nV * 3, build_st);
      DevBuf<int32_t> dF((size_t)nF * 3, build_st);
      dV.upload(m->V.data(), (size_t)nV * 3, build_st);
      dF.upload(m->F.data(), (size_t)nF * 3, build_st);
      res->device = device;
      if (GWN_SOUP_TREE_DEFAULT == GWN_TREE_REFERENCE)
        soup_build_ref(*res, dV.get(), nV, dF.get(), nF, m->order, true, build_st);
      else
        soup_build(*res, dV.get(), nV, dF.get(), nF, m->order, true, build_st);
      GWN_CUDA(cudaStreamSynchronize(build_st));
    } catch (const Error& e) {
      rc = e.code;
      err = std::string("building mesh ") + std::to_string(m->id) + ": " + e.what();
    } catch (const std::exception& e) {
      rc = GWN_ERR_INTERNAL;
      err = std::string("building mesh ") + std::to_string(m->id) + ": " + e.what();
    }
    lk.lock();
    resident_bytes -= m->reserved;
    m->reserved = 0;
    m->building = false;
    --building;
    if (rc == GWN_OK) {
      m->bytes = res->bytes;
      m->res = std::move(res);
      resident_bytes += (int64_t)m->bytes;
      stats.peak_resident_bytes = std::max<int64_t>(stats.peak_resident_bytes, resident_bytes);
      ++stats.builds;
    } else {
      for (auto it = pending.begin(); it != pending.end();) {
        if ((*it)->mesh == m) {
          m->pending--;
          complete(*it, rc, err);
          it = pending.erase(it);
        } else {
          ++it;
        }
      }
      cv_done.notify_all();
    }
    ++events;
    cv_work.notify_all();
  }
}

bool gwn_server::form_and_launch(SrvSlot& s, std::unique_lock<std::mutex>& lk) {
  std::vector<SrvReq*> take;
  int64_t aligned = 0;
  bool any_busy = false;
  for (auto& o : slots) any_busy |= o->busy;
  // In submission order, every request whose tree is resident joins the
  // batch; one whose tree is building (or waits for room) stays pending
  // without holding back the requests behind it.
  for (auto it = pending.begin(); it != pending.end() && (int)take.size() < max_reqs;) {
    SrvReq* r = *it;
    const int64_t al = (r->nq + 31) / 32 * 32;
    if (aligned + al > cap) break;
    std::string err;
    int code = GWN_ERR_OUT_OF_MEMORY;
    const int a = admit(r->mesh, any_busy || !take.empty(), code, err);
    if (a == 1) {
      ++it;
      continue;
    }
    // no room yet: launch what there is and admit this one when batches
    // finish (no later request may overtake it for the room)
    if (a == 3) break;
    it = pending.erase(it);
    r->mesh->pending--;
    if (a == 2) {
      complete(r, code, err);
      cv_done.notify_all();
      continue;
    }
    r->mesh->inflight++;
    r->mesh->last_use = ++tick;
    take.push_back(r);
    aligned += al;
  }
  if (take.empty()) return false;
  lk.unlock();
  // descriptor + host stage
  ServeHeader* hh = reinterpret_cast<ServeHeader*>(s.hdesc.h);
  ServeReq* hr = reinterpret_cast<ServeReq*>((unsigned char*)s.hdesc.h + sizeof(ServeHeader));
  unsigned char* stage = static_cast<unsigned char*>(s.hstage.h);
  int64_t boff = 0, dense = 0;
  int32_t aoff = 0;
  s.out_off.resize(take.size());
  for (size_t i = 0; i < take.size(); ++i) {
    SrvReq* r = take[i];
    const gwn_soup_impl& t = *r->mesh->res;
    ServeReq d;
    std::memset(&d, 0, sizeof(d));
    d.prm.nf = t.nf.get();
    d.prm.nd = t.nd.get();
    d.prm.tf = t.tf.get();
    d.prm.td = t.td.get();
    d.prm.nnodes = (int)t.nnodes;
    d.prm.order = t.order;
    d.prm.beta2f = r->beta * r->beta;
    d.prm.beta2d = (double)r->beta * (double)r->beta;
    d.prm.eps = (float)t.eps;
    d.prm.cmax = (float)t.cmax;
    d.prm.status = nullptr;
    d.prm.ref32 = t.tree == GWN_TREE_REFERENCE;
    d.prm.fp64_queue = t.moments_bounded;
    for (int k = 0; k < 3; ++k) {
      // the query box: the mesh box grown by a quarter on each side
      const double e = std::max(t.hi[k] - t.lo[k], 1e-30);
      d.lo[k] = (float)(t.lo[k] - 0.25 * e);
      d.inv[k] = (float)(1.0 / (1.5 * e));
    }
    d.q_byte_off = boff;
    d.out_off = dense;
    d.aoff = aoff;
    d.nq = (int32_t)r->nq;
    d.q_f64 = r->q_dtype == GWN_F64;
    d.precision = r->precision;
    hr[i] = d;
    const size_t qb = (size_t)r->nq * 3 * dtype_size(r->q_dtype);
    boff += (int64_t)((qb + 15) / 16 * 16);
    s.out_off[i] = dense;
    dense += r->nq;
    aoff += (int32_t)((r->nq + 31) / 32 * 32);
  }
  pieces.clear();
  for (size_t i = 0; i < take.size(); ++i)
    for (int64_t k = 0; k < take[i]->nq; k += kCopyPiece) pieces.emplace_back((int)i, k);
  pool->run((int)pieces.size(), [&](int t) {
    const SrvReq* r = take[(size_t)pieces[t].first];
    const ServeReq& d = hr[pieces[t].first];
    const int64_t k0 = pieces[t].second, n = std::min(kCopyPiece, r->nq - k0);
    const size_t qs = 3 * dtype_size(r->q_dtype);
    std::memcpy(stage + d.q_byte_off + k0 * qs,
                static_cast<const unsigned char*>(r->Q) + k0 * qs, (size_t)n * qs);
  });
  hh->nreq = (uint32_t)take.size();
  hh->n_aligned = (uint32_t)aoff;
  hh->nq_total = (uint32_t)dense;
  hh->status = 0;
  std::atomic_thread_fence(std::memory_order_seq_cst);
  cudaError_t e = cudaEventRecord(s.ev_start, s.st);
  if (e == cudaSuccess) e = cudaGraphLaunch(s.exec, s.st);
  if (e == cudaSuccess) e = cudaEventRecord(s.ev_done, s.st);
  lk.lock();
  s.reqs = std::move(take);
  if (e != cudaSuccess) {
    for (SrvReq* r : s.reqs) {
      r->mesh->inflight--;
      complete(r, GWN_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
    }
    s.reqs.clear();
    cv_done.notify_all();
    return true;
  }
  count_launches((unsigned long long)s.kernels);
  s.busy = true;
  ++stats.batches;
  return true;
}

void gwn_server::finish(SrvSlot& s, std::unique_lock<std::mutex>& lk) {
  lk.unlock();
  std::atomic_thread_fence(std::memory_order_seq_cst);
  const double* hout = static_cast<const double*>(s.hout.h);
  const unsigned* info = static_cast<const unsigned*>(s.hinfo.h);
  const unsigned refined = info[0], dstatus = info[1];
  float ms = 0.f, wms = 0.f;
  cudaEventElapsedTime(&ms, s.ev_start, s.ev_done);
  cudaEventElapsedTime(&wms, s.ev_walk0, s.ev_walk1);
  int64_t nq = 0;
  pieces.clear();
  for (size_t i = 0; i < s.reqs.size(); ++i) {
    for (int64_t k = 0; k < s.reqs[i]->nq; k += kCopyPiece) pieces.emplace_back((int)i, k);
    nq += s.reqs[i]->nq;
  }
  pool->run((int)pieces.size(), [&](int t) {
    SrvReq* r = s.reqs[(size_t)pieces[t].first];
    const int64_t k0 = pieces[t].second, n = std::min(kCopyPiece, r->nq - k0);
    const double* src = hout + s.out_off[(size_t)pieces[t].first] + k0;
    if (r->w_dtype == GWN_F64) {
      std::memcpy(static_cast<double*>(r->W) + k0, src, (size_t)n * sizeof(double));
    } else {
      float* w = static_cast<float*>(r->W) + k0;
      for (int64_t k = 0; k < n; ++k) w[k] = (float)src[k];
    }
  });
  lk.lock();
  for (SrvReq* r : s.reqs) {
    r->mesh->inflight--;
    if (dstatus)
      complete(r, GWN_ERR_INTERNAL, "a served batch reported an inconsistent descriptor");
    else
      complete(r, GWN_OK, "");
  }
  stats.requests_done += (int64_t)s.reqs.size();
  stats.queries_done += nq;
  stats.refined += refined;
  stats.batch_gpu_ms += ms;
  stats.walk_gpu_ms += wms;
  s.reqs.clear();
  s.busy = false;
  cv_done.notify_all();
}

void gwn_server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    const uint64_t seen = events;
    bool progressed = false, any_busy = false;
    for (auto& sp : slots) {
      SrvSlot& s = *sp;
      if (!s.busy) continue;
      const cudaError_t e = cudaEventQuery(s.ev_done);
      if (e == cudaSuccess) {
        finish(s, lk);
        progressed = true;
      } else if (e != cudaErrorNotReady) {
        for (SrvReq* r : s.reqs) {
          r->mesh->inflight--;
          complete(r, GWN_ERR_CUDA, std::string("served batch: ") + cudaGetErrorString(e));
        }
        s.reqs.clear();
        s.busy = false;
        cv_done.notify_all();
        progressed = true;
      } else {
        any_busy = true;
      }
    }
    if (!pending.empty()) {
      for (auto& sp : slots) {
        if (sp->busy) continue;
        if (form_and_launch(*sp, lk)) {
          progressed = true;
          any_busy = true;
        }
        break;
      }
    }
    if (stop && pending.empty() && building == 0) {
      bool busy = false;
      for (auto& sp : slots) busy |= sp->busy;
      if (!busy) break;
    }
    if (!progressed) {
      if (any_busy)
        cv_work.wait_for(lk, std::chrono::microseconds(20));
      else  // until a submission, a finished build or stop
        cv_work.wait_for(lk, std::chrono::milliseconds(50),
                         [&] { return stop || events != seen; });
    }
  }
}

gwn_server::~gwn_server() {
  {
    std::lock_guard<std::mutex> g(mu);
    stop = true;
  }
  cv_work.notify_all();
  if (worker.joinable()) worker.join();  // the builder serves it until it ends
  {
    std::lock_guard<std::mutex> g(mu);
    stop_builder = true;
  }
  cv_build.notify_all();
  for (auto& b : builders)
    if (b.joinable()) b.join();
  for (cudaStream_t bs : build_streams) cudaStreamDestroy(bs);
  for (auto& sp : slots) {
    if (sp->exec) cudaGraphExecDestroy(sp->exec);
    if (sp->ev_start) cudaEventDestroy(sp->ev_start);
    if (sp->ev_done) cudaEventDestroy(sp->ev_done);
    if (sp->ev_walk0) cudaEventDestroy(sp->ev_walk0);
    if (sp->ev_walk1) cudaEventDestroy(sp->ev_walk1);
    if (sp->st) cudaStreamDestroy(sp->st);
  }
}

extern "C" {

int gwn_server_create(int64_t hbm_budget_bytes, int64_t max_batch_queries, int32_t slots,
                      gwn_server** out) {
  return guarded("gwn_server_create", [&] {
    GWN_REQUIRE(out != nullptr, "out must be non-null");
    *out = nullptr;
    GWN_REQUIRE(hbm_budget_bytes > 0, "hbm_budget_bytes must be positive");
    GWN_REQUIRE(max_batch_queries >= 32 && max_batch_queries <= (int64_t(1) << 28),
                "max_batch_queries must be in [32, 2^28]");
    GWN_REQUIRE(slots >= 1 && slots <= 8, "slots must be in [1, 8]");
    ensure_device();
    std::unique_ptr<gwn_server> S(new gwn_server());
    GWN_CUDA(cudaGetDevice(&S->device));
    S->budget = hbm_budget_bytes;
    S->cap = max_batch_queries / 32 * 32;
    S->stats.budget_bytes = hbm_budget_bytes;
    {
      const unsigned hc = std::thread::hardware_concurrency();
      S->pool.reset(new CopyPool((int)std::min(7u, std::max(1u, hc / 2))));
    }
    int64_t counts_n = 0, scan_n = 0;
    radix_sort_scratch_elems(S->cap, &counts_n, &scan_n);
    for (int i = 0; i < slots; ++i) {
      std::unique_ptr<SrvSlot> s(new SrvSlot());
      GWN_CUDA(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
      GWN_CUDA(cudaEventCreate(&s->ev_start));
      GWN_CUDA(cudaEventCreate(&s->ev_done));
      GWN_CUDA(cudaEventCreate(&s->ev_walk0));
      GWN_CUDA(cudaEventCreate(&s->ev_walk1));
      s->hdesc.alloc(kDescBytes);
      std::memset(s->hdesc.h, 0, kDescBytes);
      // room for every request's queries in FP64, each rounded up to 16 bytes
      s->hstage.alloc((size_t)S->cap * 24 + (size_t)kMaxReqs * 16);
      s->hout.alloc((size_t)S->cap * sizeof(double));
      s->hinfo.alloc(16);
      s->ddesc.alloc(kDescBytes);
      s->dq.alloc((size_t)S->cap * 3);
      s->dW.alloc((size_t)S->cap);
      s->keys.alloc((size_t)S->cap);
      s->keys_tmp.alloc((size_t)S->cap);
      s->vals.alloc((size_t)S->cap);
      s->vals_tmp.alloc((size_t)S->cap);
      s->counts.alloc((size_t)counts_n);
      s->scan.alloc((size_t)std::max<int64_t>(scan_n, 1));
      s->counters.alloc(4);
      s->refine.alloc((size_t)S->cap);
      S->capture(*s);
      S->slots.push_back(std::move(s));
    }
    gwn_server* raw = S.get();
    S->worker = std::thread([raw] { raw->run(); });
    for (int b = 0; b < kBuilders; ++b) {
      cudaStream_t bs = nullptr;
      GWN_CUDA(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
      S->build_streams.push_back(bs);
      S->builders.emplace_back([raw, bs] { raw->build_loop(bs); });
    }
    *out = S.release();
  });
}

int gwn_server_add_mesh(gwn_server* S, const double* V, int64_t nV, const int32_t* F, int64_t nF,
                        int order, int64_t* mesh_id) {
  return guarded("gwn_server_add_mesh", [&] {
    GWN_REQUIRE(S != nullptr && mesh_id != nullptr, "server and mesh_id must be non-null");
    GWN_REQUIRE(nV >= 0 && nF >= 0, "sizes must be non-negative");
    check_mesh(V, nV, F, nF);
    GWN_REQUIRE(nF < (int64_t(1) << 30), "at most 2^30 triangles");
    GWN_REQUIRE(order >= 0 && order <= 2, "order must be 0, 1 or 2");
    for (int64_t i = 0; i < nF * 3; ++i)
      GWN_REQUIRE(F[i] >= 0 && F[i] < nV, "F holds a vertex index outside [0, nV)");
    std::unique_ptr<SrvMesh> m(new SrvMesh());
    m->V.assign(V, V + nV * 3);
    m->F.assign(F, F + nF * 3);
    m->order = order;
    m->bytes = (size_t)estimate_bytes(nF);
    std::lock_guard<std::mutex> g(S->mu);
    m->id = S->next_mesh++;
    *mesh_id = m->id;
    S->meshes[m->id] = std::move(m);
  });
}

int gwn_server_remove_mesh(gwn_server* S, int64_t mesh_id) {
  return guarded("gwn_server_remove_mesh", [&] {
    GWN_REQUIRE(S != nullptr, "server is null");
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->meshes.find(mesh_id);
    GWN_REQUIRE(it != S->meshes.end(), "unknown mesh id");
    SrvMesh* m = it->second.get();
    if (m->pending || m->inflight || m->building)
      throw Error(GWN_ERR_BUSY, "mesh has requests pending or in flight, or is building");
    if (m->res) {
      S->resident_bytes -= (int64_t)m->bytes;
      m->res.reset();
    }
    S->meshes.erase(it);
  });
}

int gwn_server_submit(gwn_server* S, int64_t mesh_id, const void* Q, int q_dtype, int64_t nQ,
                      void* W, int w_dtype, float accuracy_scale, int precision,
                      int64_t* request_id) {
  return guarded("gwn_server_submit", [&] {
    GWN_REQUIRE(S != nullptr && request_id != nullptr, "server and request_id must be non-null");
    GWN_REQUIRE(nQ >= 0, "nQ must be non-negative");
    GWN_REQUIRE(nQ == 0 || (Q && W), "Q and W must be non-null");
    GWN_REQUIRE(std::isfinite(accuracy_scale), "accuracy_scale must be finite");
    GWN_REQUIRE((nQ + 31) / 32 * 32 <= S->cap,
                "nQ = " + std::to_string(nQ) + " exceeds the batch capacity of " +
                    std::to_string(S->cap) + " queries");
    check_dtype(q_dtype, "Q");
    check_dtype(w_dtype, "W");
    check_precision(precision);
    std::unique_ptr<SrvReq> r(new SrvReq());
    r->Q = Q;
    r->q_dtype = q_dtype;
    r->nq = nQ;
    r->W = W;
    r->w_dtype = w_dtype;
    r->beta = accuracy_scale;
    r->precision = precision;
    r->t_submit = now_s();
    {
      std::lock_guard<std::mutex> g(S->mu);
      auto it = S->meshes.find(mesh_id);
      GWN_REQUIRE(it != S->meshes.end(), "unknown mesh id");
      r->mesh = it->second.get();
      r->id = S->next_req++;
      *request_id = r->id;
      SrvReq* raw = r.get();
      S->reqs[r->id] = std::move(r);
      if (raw->nq == 0 || raw->mesh->F.empty()) {
        // nothing to evaluate: no triangles give W = 0 (the reference's
        // empty tree returns 0 for every query)
        if (raw->nq) {
          if (w_dtype == GWN_F64) std::memset(W, 0, (size_t)nQ * sizeof(double));
          else std::memset(W, 0, (size_t)nQ * sizeof(float));
        }
        S->complete(raw, GWN_OK, "");
        ++S->stats.requests_done;
        S->cv_done.notify_all();
        return;
      }
      raw->mesh->pending++;
      S->pending.push_back(raw);
      ++S->events;
    }
    S->cv_work.notify_one();
  });
}

int gwn_server_wait(gwn_server* S, int64_t request_id, double timeout_s, double* latency_s) {
  if (!S) {
    set_last_error("gwn_server_wait: server is null");
    return GWN_ERR_INVALID_ARGUMENT;
  }
  if (std::isnan(timeout_s)) {  // a NaN duration has no meaning for wait_for
    set_last_error("gwn_server_wait: timeout_s is NaN");
    return GWN_ERR_INVALID_ARGUMENT;
  }
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(request_id);
  if (it == S->reqs.end()) {
    set_last_error("gwn_server_wait: unknown request id");
    return GWN_ERR_INVALID_ARGUMENT;
  }
  SrvReq* r = it->second.get();
  const auto pred = [&] { return r->done; };
  if (timeout_s < 0 || timeout_s > 1e9) {  // no limit (1e9 s: past any clock's range use)
    S->cv_done.wait(lk, pred);
  } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
    set_last_error("gwn_server_wait: request not finished within the timeout");
    return GWN_ERR_TIMEOUT;
  }
  if (latency_s) *latency_s = r->t_done - r->t_submit;
  const int st = r->status;
  if (st != GWN_OK) set_last_error("gwn_server_wait: " + r->err);
  S->reqs.erase(it);
  return st;
}

int gwn_server_stats_get(gwn_server* S, gwn_server_stats* out) {
  return guarded("gwn_server_stats_get", [&] {
    GWN_REQUIRE(S != nullptr && out != nullptr, "server and out must be non-null");
    std::lock_guard<std::mutex> g(S->mu);
    *out = S->stats;
    out->resident_bytes = S->resident_bytes;
    int64_t rm = 0;
    for (auto& kv : S->meshes) rm += kv.second->res ? 1 : 0;
    out->resident_meshes = rm;
    out->pending = (int64_t)S->pending.size();
    out->kernels_per_batch = S->slots.empty() ? 0 : S->slots[0]->kernels;
  });
}

int gwn_server_destroy(gwn_server* S) {
  return guarded("gwn_server_destroy", [&] { delete S; });
}

}  // extern "C"
