// igl::swept_volume_signed_distance (include/igl/swept_volume_signed_distance.cpp:21-160)
// and igl::flood_fill (include/igl/flood_fill.cpp:11-80) on the GPU.
//
// Swept volume.  The reference loops over the transforms, and for each over
// the grid: a point already deeper than isolevel - sqrt(3) h is skipped, the
// point is carried into the mesh's frame by the inverse of the rigid motion,
// ((g - t) L), points outside the mesh box grown by isolevel + sqrt(3) h are
// skipped, and the closest triangle below (isolevel + sqrt(3) h)^2 gives
// s sqrt(d2) (s from the sign type), kept as the running minimum.  Here the
// transforms go through in chunks of up to 16: an activation kernel takes
// every grid point not yet below the skip level (the running minimum only
// decreases, so such a point is skipped by the whole chunk) with every
// transform of the chunk, applies the box rule and compacts the surviving
// (point, transform) pairs; the library's bounded closest-triangle search
// runs on that batch, the pairs closer than the bound are compacted again
// and signed (exact winding number: the cap hierarchy of hier.cu in mixed
// precision, all pairs in FP64; soup fast winding number; or pseudonormal),
// and their values land in a per-chunk table.  A last kernel replays the
// chunk's transforms in order for every point with the reference's skip
// rule and running minimum, so values the reference would not have computed
// are ignored and the result is the reference's.  The mesh's search tree,
// soup tree, cap hierarchy and pseudonormals are built once.
//
// Flood fill.  The reference scans the grid once (x fastest) and fills each
// unsigned (NaN) cell from the signed cells around it.  Its result, read off
// the scan: a NaN cell takes the next signed value to its right on its row,
// or the row's last signed value; a row with no signed cell takes the first
// signed value of the next row of its sheet that has one, or of the last
// such row; a sheet with no signed cell takes the first signed value (scan
// order) of the next sheet that has one, or of the last such sheet; a grid
// with no signed cell stays NaN.  Three small kernels compute the row, sheet
// and grid levels of that rule and one kernel writes the cells.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "gwn_internal.cuh"
#include "soup.cuh"

namespace gwn {
namespace {

constexpr double kNaN = __builtin_nan("");

__global__ void mesh_box_kernel(const double* __restrict__ V, int64_t nV,
                                unsigned long long* __restrict__ mm) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nV;
       i += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) {
      lo[d] = fmin(lo[d], V[i * 3 + d]);
      hi[d] = fmax(hi[d], V[i * 3 + d]);
    }
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&mm[d], ordered_bits(lo[d]));
      atomicMax(&mm[3 + d], ordered_bits(hi[d]));
    }
  }
}

struct SweepParams {
  bool finite_iso;
  double skip_below;  // isolevel - sqrt(3) h
  double ext;         // box growth
};

// Transforms go through in chunks of K.  For a chunk: every grid point not
// already deeper than the skip level (the running minimum only decreases,
// so such a point is skipped by every transform of the chunk) and every
// transform k of the chunk: the inverse motion ((g - t) L, products and sums
// unfused in the reference's order) and the box test; surviving (point,
// transform) pairs are compacted into Q / gidx / kidx (batch order:
// arbitrary).
__global__ void activate_chunk_kernel(const double* __restrict__ GV, int64_t nG,
                                      const double* __restrict__ S,
                                      const double* __restrict__ T, int K, SweepParams sp,
                                      const unsigned long long* __restrict__ mm,
                                      double* __restrict__ Q, int32_t* __restrict__ gidx,
                                      int32_t* __restrict__ kidx, unsigned* __restrict__ cnt) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nG) return;
  const double sg = S[g];
  if (sp.finite_iso && sg == sg && sg < sp.skip_below) return;
  const double x = GV[g * 3], y = GV[g * 3 + 1], z = GV[g * 3 + 2];
  double lo[3], hi[3];
  for (int j = 0; j < 3; ++j) {
    lo[j] = __dsub_rn(from_ordered_bits(mm[j]), sp.ext);
    hi[j] = __dadd_rn(from_ordered_bits(mm[3 + j]), sp.ext);
  }
  for (int k = 0; k < K; ++k) {
    const double* A = T + 12 * k;
    const double d0 = __dsub_rn(x, A[3]), d1 = __dsub_rn(y, A[7]), d2 = __dsub_rn(z, A[11]);
    double gv[3];
    bool inside = true;
    for (int j = 0; j < 3; ++j) {
      gv[j] = __dadd_rn(__dadd_rn(__dmul_rn(d0, A[j]), __dmul_rn(d1, A[4 + j])),
                        __dmul_rn(d2, A[8 + j]));
      inside &= lo[j] <= gv[j] && gv[j] <= hi[j];
    }
    if (sp.finite_iso && !inside) continue;
    const unsigned i = atomicAdd(cnt, 1u);
    Q[(int64_t)i * 3] = gv[0];
    Q[(int64_t)i * 3 + 1] = gv[1];
    Q[(int64_t)i * 3 + 2] = gv[2];
    gidx[i] = (int32_t)g;
    kidx[i] = k;
  }
}

// The batch's pairs closer than the bound (the only ones the reference
// signs), compacted with their distance, closest face and point.
__global__ void select_kernel(int64_t n, const double* __restrict__ Q,
                              const int32_t* __restrict__ gidx, const int32_t* __restrict__ kidx,
                              const double* __restrict__ sqrD, const int32_t* __restrict__ I,
                              const double* __restrict__ C, double min_sqrd,
                              double* __restrict__ Q2, int32_t* __restrict__ g2,
                              int32_t* __restrict__ k2, double* __restrict__ d2,
                              int32_t* __restrict__ I2, double* __restrict__ C2,
                              unsigned* __restrict__ cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n || !(sqrD[i] < min_sqrd)) return;
  const int64_t j = atomicAdd(cnt, 1u);
  for (int c = 0; c < 3; ++c) {
    Q2[j * 3 + c] = Q[i * 3 + c];
    C2[j * 3 + c] = C[i * 3 + c];
  }
  g2[j] = gidx[i];
  k2[j] = kidx[i];
  d2[j] = sqrD[i];
  I2[j] = I[i];
}

// SD[k nG + g] = s sqrt(d2) for the pairs closer than the bound (s from the
// sign mode: 1, 1 - 2 W, 1 - 2 |W|, or the pseudonormal sign W).
__global__ void scatter_sd_kernel(int64_t n, const int32_t* __restrict__ gidx,
                                  const int32_t* __restrict__ kidx,
                                  const double* __restrict__ sqrD,
                                  const double* __restrict__ W, int mode, double min_sqrd,
                                  int64_t nG, double* __restrict__ SD) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d2 = sqrD[i];
  if (!(d2 < min_sqrd)) return;
  double s = 1.0;
  if (mode == 1) s = 1.0 - 2.0 * W[i];
  else if (mode == 2) s = 1.0 - 2.0 * fabs(W[i]);
  else if (mode == 3) s = W[i];
  SD[(int64_t)kidx[i] * nG + gidx[i]] = s * sqrt(d2);
}

// The reference's loop over the chunk's transforms for every grid point, in
// order: stop at the skip level, else S = min(S, value) where the transform
// produced one (std::min's operand order; a NaN S takes the value).
__global__ void update_chunk_kernel(int64_t nG, int K, const double* __restrict__ SD,
                                    SweepParams sp, double* __restrict__ S) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nG) return;
  double cur = S[g];
  for (int k = 0; k < K; ++k) {
    if (sp.finite_iso && cur == cur && cur < sp.skip_below) break;
    const double v = SD[(int64_t)k * nG + g];
    if (v == v) cur = cur == cur ? (v < cur ? v : cur) : v;
  }
  S[g] = cur;
}

// ------------------------------------------------------------ flood fill --
// One warp per row: cells with a signed value to their right take the next
// one (right-to-left sweep in 32-cell segments), the cells after the row's
// last signed cell take that value.  rowfirst = the row's first signed value
// (NaN for a row without one).
__global__ void ff_rows_kernel(double* __restrict__ S, int64_t X, int64_t rows,
                               double* __restrict__ rowfirst) {
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  double* row = S + r * X;
  double carry = kNaN;  // next signed value right of the current segment
  double last = kNaN;   // the row's last signed value
  int64_t last_x = -1;
  for (int64_t base = ((X - 1) / 32) * 32; base >= 0; base -= 32) {
    const int64_t x = base + lane;
    const double v = x < X ? row[x] : kNaN;
    const bool sgn = v == v;
    const unsigned m = __ballot_sync(0xffffffffu, sgn);
    if (last_x < 0 && m) {
      const int hi = 31 - __clz(m);
      last = __shfl_sync(0xffffffffu, v, hi);
      last_x = base + hi;
    }
    // next signed lane strictly to the right of this lane, within the segment
    const unsigned right = lane == 31 ? 0u : (m & (0xffffffffu << (lane + 1)));
    const double cand = __shfl_sync(0xffffffffu, v, right ? __ffs(right) - 1 : lane);
    const double nxt = right ? cand : carry;
    if (x < X && !sgn && nxt == nxt) row[x] = nxt;
    if (m) carry = __shfl_sync(0xffffffffu, v, __ffs(m) - 1);
  }
  if (last_x >= 0)
    for (int64_t x = last_x + 1 + lane; x < X; x += 32) row[x] = last;
  if (lane == 0) rowfirst[r] = carry;
}

// One thread per sheet: rows without a signed cell take the first value of
// the next row with one, else of the last row with one; sheetfirst = the
// sheet's first signed value in scan order.
__global__ void ff_sheets_kernel(const double* __restrict__ rowfirst, int64_t Y, int64_t Z,
                                 double* __restrict__ rowfill, double* __restrict__ sheetfirst) {
  const int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (z >= Z) return;
  const double* rf = rowfirst + z * Y;
  double* fill = rowfill + z * Y;
  double next = kNaN;
  for (int64_t y = Y - 1; y >= 0; --y) {
    const double v = rf[y];
    if (v == v) next = v;
    else fill[y] = next;
  }
  sheetfirst[z] = next;
  double lastv = kNaN;
  for (int64_t y = 0; y < Y; ++y) {
    const double v = rf[y];
    if (v == v) lastv = v;
    else if (!(fill[y] == fill[y])) fill[y] = lastv;
  }
}

// One thread: sheets without a signed cell take the first value of the next
// sheet with one, else of the last sheet with one.
__global__ void ff_grid_kernel(const double* __restrict__ sheetfirst, int64_t Z,
                               double* __restrict__ sheetfill) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double next = kNaN;
  for (int64_t z = Z - 1; z >= 0; --z) {
    const double v = sheetfirst[z];
    if (v == v) next = v;
    else sheetfill[z] = next;
  }
  double lastv = kNaN;
  for (int64_t z = 0; z < Z; ++z) {
    const double v = sheetfirst[z];
    if (v == v) lastv = v;
    else if (!(sheetfill[z] == sheetfill[z])) sheetfill[z] = lastv;
  }
}

__global__ void ff_cells_kernel(double* __restrict__ S, int64_t X, int64_t Y, int64_t n,
                                const double* __restrict__ rowfirst,
                                const double* __restrict__ rowfill,
                                const double* __restrict__ sheetfirst,
                                const double* __restrict__ sheetfill) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t r = i / X, z = r / Y;
  if (rowfirst[r] == rowfirst[r]) return;  // the row kernel filled it
  S[i] = sheetfirst[z] == sheetfirst[z] ? rowfill[r] : sheetfill[z];
}

}  // namespace

void flood_fill_run(const int32_t res[3], double* S, cudaStream_t st) {
  const int64_t X = res[0], Y = res[1], Z = res[2];
  if (X <= 0 || Y <= 0 || Z <= 0) return;
  const int64_t rows = Y * Z, n = X * rows;
  DevBuf<double> rowfirst((size_t)rows, st), rowfill((size_t)rows, st), sheetfirst((size_t)Z, st),
      sheetfill((size_t)Z, st);
  GWN_CUDA(cudaMemsetAsync(rowfill.get(), 0xff, rowfill.bytes(), st));  // NaN
  GWN_CUDA(cudaMemsetAsync(sheetfill.get(), 0xff, sheetfill.bytes(), st));
  launch_kernel(ff_rows_kernel, (unsigned)((rows * 32 + 255) / 256), 256, 0, st, S, X, rows,
                rowfirst.get());
  launch_kernel(ff_sheets_kernel, (unsigned)((Z + 127) / 128), 128, 0, st,
                (const double*)rowfirst.get(), Y, Z, rowfill.get(), sheetfirst.get());
  launch_kernel(ff_grid_kernel, 1, 32, 0, st, (const double*)sheetfirst.get(), Z,
                sheetfill.get());
  launch_kernel(ff_cells_kernel, (unsigned)((n + 255) / 256), 256, 0, st, S, X, Y, n,
                (const double*)rowfirst.get(), (const double*)rowfill.get(),
                (const double*)sheetfirst.get(), (const double*)sheetfill.get());
}

void swept_volume_run(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                      const double* transforms_host, int64_t nT, int sign_type, const double* GV,
                      int64_t nG, const int32_t res[3], double h, double isolevel, double* S,
                      int precision, cudaStream_t st) {
  const bool finite_iso = std::isfinite(isolevel);
  // swept_volume_signed_distance.cpp:47-54, 110-114
  const double iso = finite_iso ? isolevel : INFINITY;
  const double ext = (finite_iso ? iso : 0.0) + std::sqrt(3.0) * h;
  const double min_sqrd = finite_iso ? std::pow(std::sqrt(3.) * h + iso, 2) : INFINITY;
  const SweepParams sp{finite_iso, iso - std::sqrt(3.0) * h, ext};
  if (nG > 0 && nF > 0 && nT > 0) {
    DevBuf<unsigned long long> mm(6, st);
    init_minmax(mm.get(), 3, st);
    launch_kernel(mesh_box_kernel, (unsigned)std::max<int64_t>(1, std::min<int64_t>((nV + 255) / 256, 1024)),
                  256, 0, st, V, nV, mm.get());
    gwn_soup_impl tree;
    PseudonormalData pn;
    HierTree hier;
    const bool use_hier = (sign_type == GWN_SD_WINDING_NUMBER || sign_type == GWN_SD_DEFAULT) &&
                          precision == GWN_MIXED;
    {
      PhaseTimer ph("build", st);
      soup_build(tree, V, nV, F, nF, 2, true, st);
      if (sign_type == GWN_SD_PSEUDONORMAL) pseudonormal_precompute(V, nV, F, nF, pn, st);
      if (use_hier) hier_build(V, nV, F, nF, hier, sticky_status_word(), st, true);
    }
    // up to 16 transforms per chunk, about 8M (point, transform) slots
    const int K = (int)std::max<int64_t>(1, std::min<int64_t>(16, (int64_t(8) << 20) / nG));
    const int64_t cap = nG * K;
    GWN_REQUIRE(cap < (int64_t(1) << 31), "too many grid points");
    DevBuf<double> Tdev((size_t)nT * 12, st);
    Tdev.upload(transforms_host, (size_t)nT * 12, st);
    DevBuf<double> Q((size_t)cap * 3, st), sqrD((size_t)cap, st), C((size_t)cap * 3, st),
        W((size_t)cap, st), Q2((size_t)cap * 3, st), d2((size_t)cap, st), C2((size_t)cap * 3, st),
        SD((size_t)cap, st);
    DevBuf<int32_t> gidx((size_t)cap, st), kidx((size_t)cap, st), I((size_t)cap, st),
        g2((size_t)cap, st), k2((size_t)cap, st), I2((size_t)cap, st);
    DevBuf<unsigned> cnt(2, st);
    auto read_count = [&](int which) {
      unsigned v = 0;
      GWN_CUDA(cudaMemcpyAsync(&v, cnt.get() + which, sizeof(v), cudaMemcpyDeviceToHost, st));
      GWN_CUDA(cudaStreamSynchronize(st));
      return v;
    };
    int mode = 0;
    if (sign_type == GWN_SD_WINDING_NUMBER || sign_type == GWN_SD_DEFAULT) mode = 1;
    else if (sign_type == GWN_SD_FAST_WINDING_NUMBER) mode = 2;
    else if (sign_type == GWN_SD_PSEUDONORMAL) mode = 3;
    const unsigned grid = (unsigned)((nG + 255) / 256);
    auto blocks = [](int64_t n) { return (unsigned)std::max<int64_t>(1, (n + 255) / 256); };
    for (int64_t t0 = 0; t0 < nT; t0 += K) {
      const int Kc = (int)std::min<int64_t>(K, nT - t0);
      cnt.zero(st);
      GWN_CUDA(cudaMemsetAsync(SD.get(), 0xff, (size_t)nG * Kc * sizeof(double), st));  // NaN
      {
        PhaseTimer ph("activate", st);
        launch_kernel(activate_chunk_kernel, grid, 256, 0, st, GV, nG, (const double*)S,
                      (const double*)(Tdev.get() + t0 * 12), Kc, sp,
                      (const unsigned long long*)mm.get(), Q.get(), gidx.get(), kidx.get(),
                      cnt.get());
      }
      const unsigned n = read_count(0);
      if (n > 0) {
        soup_squared_distance(tree, Q.get(), GWN_F64, n, min_sqrd, sqrD.get(), I.get(), C.get(),
                              st);
        if (mode == 0) {
          launch_kernel(scatter_sd_kernel, blocks(n), 256, 0, st, (int64_t)n,
                        (const int32_t*)gidx.get(), (const int32_t*)kidx.get(),
                        (const double*)sqrD.get(), (const double*)nullptr, mode, min_sqrd, nG,
                        SD.get());
        } else {
          launch_kernel(select_kernel, blocks(n), 256, 0, st, (int64_t)n, (const double*)Q.get(),
                        (const int32_t*)gidx.get(), (const int32_t*)kidx.get(),
                        (const double*)sqrD.get(), (const int32_t*)I.get(),
                        (const double*)C.get(), min_sqrd, Q2.get(), g2.get(), k2.get(), d2.get(),
                        I2.get(), C2.get(), cnt.get() + 1);
          const unsigned m = read_count(1);
          if (m > 0) {
            if (mode == 1 && use_hier) {
              hier_eval(hier, Q2.get(), m, W.get(), st);
            } else if (mode == 1) {
              ExactArgs a{V, nV, 3, F, nF, Q2.get(), GWN_F64, (int64_t)m, W.get(), GWN_F64,
                          precision, false};
              run_exact(a, st);
            } else if (mode == 2) {
              soup_eval(tree, 2.0f, Q2.get(), GWN_F64, m, W.get(), GWN_F64, precision, st);
            } else {
              PhaseTimer ph("pseudonormal", st);
              pseudonormal_apply(pn, Q2.get(), m, V, F, nF, I2.get(), C2.get(), d2.get(),
                                 W.get(), nullptr, st);
            }
            launch_kernel(scatter_sd_kernel, blocks(m), 256, 0, st, (int64_t)m,
                          (const int32_t*)g2.get(), (const int32_t*)k2.get(),
                          (const double*)d2.get(), (const double*)W.get(), mode, min_sqrd, nG,
                          SD.get());
          }
        }
      }
      PhaseTimer ph("update", st);
      launch_kernel(update_chunk_kernel, grid, 256, 0, st, nG, Kc, (const double*)SD.get(), sp, S);
    }
  }
  if (finite_iso) {
    PhaseTimer ph("flood_fill", st);
    flood_fill_run(res, S, st);
  }
  GWN_CUDA(cudaStreamSynchronize(st));
}

}  // namespace gwn
