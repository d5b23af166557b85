// Per-point Voronoi areas of a point cloud from its k nearest neighbours:
// igl::copyleft::cgal::point_areas(P,I,N,A,T)
// (include/igl/copyleft/cgal/point_areas.cpp:60-160), the step that gives the
// point-cloud winding number its areas A from a raw scan
// (copyleft/cgal/fast_winding_number.cpp:30-38).
//
// A warp takes 32 points: their kept neighbours' mean and scatter matrix
// point by point (lane j holds neighbours j, j + 32, ...), the 3 x 3
// eigenproblems lane by lane (one point each), then point by point the
// plane and the triangulation.  GB300 runs FP64 far slower than FP32, so
// the hull's orientation tests run in FP32 with an error bound and fall
// back to FP64 only where the sign is not certain.  Per point, as the
// reference:
//   * the neighbours I(i,:) whose normal has a positive dot product with the
//     first neighbour's normal are kept, in order (no filter for k = 1);
//     two or fewer kept: A = 0, T = 0;
//   * their mean and principal directions: the reference takes the SVD of
//     the centred neighbours; here the eigenvectors of their 3 x 3 scatter
//     matrix (cyclic Jacobi, FP64), the same right singular vectors up to
//     sign.  T = the least direction, turned towards N(i); the kept points'
//     coordinates along the two largest are the plane (the reference's
//     scores U S, up to signs that move no distance);
//   * the Delaunay triangles of the plane points that have the first kept
//     point (vertex 0) as a corner.  The reference triangulates everything
//     with CGAL and keeps those; here they come directly: inverting the
//     other points about vertex 0 (q -> q / |q|^2) maps the circle through
//     vertex 0, a and b to the line through the images of a and b and its
//     inside to the side away from vertex 0, so triangle (0, a, b) has an
//     empty circumcircle exactly when (a', b') is an edge of the convex hull
//     of the images with vertex 0 strictly on the hull's side.  Each lane
//     finds its point's hull successor (one gift-wrapping step, then a check
//     that no image lies right of the edge).  Coinciding points are counted
//     once, as CGAL keeps the first of equal points;
//   * each such triangle adds the reference's share of its area to vertex 0
//     (the circumcentric split for an acute triangle, half or a quarter of
//     it when obtuse at vertex 0 or elsewhere), summed in FP64; a non-finite
//     sum gives 0.
// Neighbours are summed in a fixed warp order, so results are deterministic.
// In degenerate configurations (four or more cocircular plane points at
// vertex 0) the triangulation is not unique and CGAL's depends on its
// insertion order; results there may differ.
#include <cuda_runtime.h>

#include <cmath>

#include "gwn_common.cuh"
#include "gwn_internal.cuh"

namespace gwn {
namespace {

constexpr int kWarps = 4;  // points per CTA

struct PaShared {
  double p[kPointAreasMaxK][3];  // kept neighbours, in order
  double u[kPointAreasMaxK], w[kPointAreasMaxK];    // plane coordinates
  double su[kPointAreasMaxK], sw[kPointAreasMaxK];  // images under inversion about vertex 0
  float fu[kPointAreasMaxK], fw[kPointAreasMaxK];   // the images rounded to FP32
  unsigned char ok[kPointAreasMaxK];                // image usable (distinct, not vertex 0)
};

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Eigen-decomposition of the symmetric 3 x 3 matrix a (cyclic Jacobi);
// returns eigenvalues d and eigenvectors as the columns of v, sorted by
// decreasing eigenvalue.
__device__ void sym3_eigen(double a[3][3], double d[3], double v[3][3]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) v[r][c] = r == c ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 32; ++sweep) {
    const double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    const double scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
    if (off == 0.0 || off <= 1e-300 + scale * 1e-17) break;
    for (int p = 0; p < 2; ++p) {
      for (int q = p + 1; q < 3; ++q) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {  // a <- a J
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {  // a <- J^T a
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {  // v <- v J
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
    }
  }
  for (int k = 0; k < 3; ++k) d[k] = a[k][k];
  // sort descending (three elements)
  for (int x = 0; x < 2; ++x)
    for (int y = 0; y < 2 - x; ++y)
      if (d[y] < d[y + 1]) {
        const double t = d[y];
        d[y] = d[y + 1];
        d[y + 1] = t;
        for (int r = 0; r < 3; ++r) {
          const double tv = v[r][y];
          v[r][y] = v[r][y + 1];
          v[r][y + 1] = tv;
        }
      }
}

// The reference's share of triangle (X, Y, Z) for vertex X
// (point_areas.cpp:122-150), plane coordinates: side lengths x, y, z opposite
// X, Y, Z, the cosines by the law of cosines (the same numerators, so the
// same obtuse-angle cases), barycentric weights of the circumcentre
// x cos X : y cos Y : z cos Z, Heron's area in the reference's form.  One
// division serves the three cosines and one the weights (the FP64 pipe is
// this kernel's bound), where the reference divides six times.
__device__ double voronoi_share(double xx, double xy, double yx, double yy, double zx,
                                double zy) {
  const double ax = yx - zx, ay = yy - zy, bx = xx - zx, by = xy - zy;
  const double cx = yx - xx, cy = yy - xy;
  const double x = sqrt(ax * ax + ay * ay), y = sqrt(bx * bx + by * by),
               z = sqrt(cx * cx + cy * cy);
  const double inv = 1.0 / (2 * x * y * z);  // cos X = (z^2 + y^2 - x^2) / (2 y z), ...
  const double cosX = (z * z + y * y - x * x) * (x * inv);
  const double cosY = (z * z + x * x - y * y) * (y * inv);
  const double cosZ = (x * x + y * y - z * z) * (z * inv);
  const double full = 0.25 * sqrt((x + (y + z)) * (z - (x - y)) * (z + (x - y)) * (x + (y - z)));
  if (cosX < 0) return 0.5 * full;
  if (cosY < 0 || cosZ < 0) return 0.25 * full;
  const double b1 = y * cosY, b2 = z * cosZ;
  return 0.5 * full * ((b1 + b2) / (x * cosX + b1 + b2));
}

// orientation of (b - a) x (c - a): > 0 when c is left of a -> b
__device__ __forceinline__ double orient(double ax, double ay, double bx, double by, double cx,
                                         double cy) {
  return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

// Kept neighbours of point i into S.p (the reference's normal filter);
// returns their number (-1 when an index lies outside P).  Warp-uniform.
__device__ int gather_kept(const double* __restrict__ P, int64_t nP, const int32_t* __restrict__ row,
                           int k, const double* __restrict__ N, PaShared& S) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int32_t i0 = row[0];
  if (i0 < 0 || i0 >= nP) return -1;
  const double n0x = N[(int64_t)i0 * 3], n0y = N[(int64_t)i0 * 3 + 1], n0z = N[(int64_t)i0 * 3 + 2];
  int m = 0;
  bool any_bad = false;
  for (int j0 = 0; j0 < k; j0 += 32) {
    const int j = j0 + lane;
    const int32_t idx = j < k ? row[j] : -1;
    const bool bad = j < k && (idx < 0 || idx >= nP);
    bool keep = j < k && !bad;
    if (keep && k > 1) {
      const double* nj = N + (int64_t)idx * 3;
      keep = n0x * nj[0] + n0y * nj[1] + n0z * nj[2] > 0;
    }
    any_bad |= __any_sync(full, bad);
    const unsigned b = __ballot_sync(full, keep);
    if (keep) {
      const int pos = m + __popc(b & lt);
      for (int d = 0; d < 3; ++d) S.p[pos][d] = P[(int64_t)idx * 3 + d];
    }
    m += __popc(b);
  }
  __syncwarp();
  return any_bad ? -1 : m;
}

// Sign of orient(a, b, c) for the images: FP32 when its error bound
// (input rounding of the FP64 images and the FP32 operations, a generous
// 16 u) leaves the sign certain, else FP64.
__device__ __forceinline__ int orient_sign(const PaShared& S, int a, int b, int c) {
  const float ax = S.fu[a], ay = S.fw[a], bx = S.fu[b], by = S.fw[b], cx = S.fu[c], cy = S.fw[c];
  const float o = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
  const float bound = 9.6e-7f * ((fabsf(bx) + fabsf(ax)) * (fabsf(cy) + fabsf(ay)) +
                                 (fabsf(by) + fabsf(ay)) * (fabsf(cx) + fabsf(ax)));
  if (o > bound) return 1;
  if (o < -bound) return -1;
  const double od = orient(S.su[a], S.sw[a], S.su[b], S.sw[b], S.su[c], S.sw[c]);
  return od > 0 ? 1 : (od < 0 ? -1 : 0);
}

__global__ void __launch_bounds__(32 * kWarps) point_areas_kernel(
    const double* __restrict__ P, int64_t nP, const int32_t* __restrict__ I, int k,
    const double* __restrict__ N, double* __restrict__ A, double* __restrict__ T,
    unsigned* __restrict__ status) {
  __shared__ PaShared sh_all[kWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  PaShared& S = sh_all[wib];
  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  for (int64_t base = ((int64_t)blockIdx.x * kWarps + wib) * 32; base < nP; base += nwarps * 32) {
    const int np = (int)(nP - base < 32 ? nP - base : 32);
    // ---- stage A, point by point: kept count, mean and scatter matrix;
    // lane t keeps point base + t's
    int my_m = 0;
    double my_mean[3] = {0, 0, 0}, my_c[6] = {0, 0, 0, 0, 0, 0};
    for (int t = 0; t < np; ++t) {
      const int m = gather_kept(P, nP, I + (base + t) * k, k, N, S);
      if (m <= 2) {
        if (lane == t) my_m = m;
        __syncwarp();
        continue;
      }
      double s0 = 0, s1 = 0, s2 = 0;
      for (int j = lane; j < m; j += 32) {
        s0 += S.p[j][0];
        s1 += S.p[j][1];
        s2 += S.p[j][2];
      }
      const double mean[3] = {warp_sum(s0) / m, warp_sum(s1) / m, warp_sum(s2) / m};
      double c[6] = {0, 0, 0, 0, 0, 0};
      for (int j = lane; j < m; j += 32) {
        const double x = S.p[j][0] - mean[0], y = S.p[j][1] - mean[1], z = S.p[j][2] - mean[2];
        c[0] += x * x;
        c[1] += x * y;
        c[2] += x * z;
        c[3] += y * y;
        c[4] += y * z;
        c[5] += z * z;
      }
      for (int q = 0; q < 6; ++q) c[q] = warp_sum(c[q]);
      if (lane == t) {
        my_m = m;
        for (int d = 0; d < 3; ++d) my_mean[d] = mean[d];
        for (int q = 0; q < 6; ++q) my_c[q] = c[q];
      }
      __syncwarp();
    }
    // ---- stage B, lane per point: principal directions, T, A for the
    // degenerate cases
    double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (lane < np && my_m > 2) {
      double a[3][3] = {{my_c[0], my_c[1], my_c[2]},
                        {my_c[1], my_c[3], my_c[4]},
                        {my_c[2], my_c[4], my_c[5]}};
      double ev[3];
      sym3_eigen(a, ev, V);
    }
    if (lane < np) {
      const int64_t i = base + lane;
      if (my_m < 0) atomicOr(status, kStatusBadInput);
      if (my_m <= 2) A[i] = 0.0;
      if (T) {
        double t[3] = {0, 0, 0};
        if (my_m > 2) {
          const double* ni = N + i * 3;
          t[0] = V[0][2];
          t[1] = V[1][2];
          t[2] = V[2][2];
          if (t[0] * ni[0] + t[1] * ni[1] + t[2] * ni[2] < 0)
            for (int d = 0; d < 3; ++d) t[d] = -t[d];
        }
        for (int d = 0; d < 3; ++d) T[i * 3 + d] = t[d];
      }
    }
    // ---- stage C, point by point: plane, Delaunay star, area
    for (int t = 0; t < np; ++t) {
      const int m = __shfl_sync(0xffffffffu, my_m, t);
      if (m <= 2) continue;
      double mean[3], e1[3], e2[3];
      for (int d = 0; d < 3; ++d) {
        mean[d] = __shfl_sync(0xffffffffu, my_mean[d], t);
        e1[d] = __shfl_sync(0xffffffffu, V[d][0], t);
        e2[d] = __shfl_sync(0xffffffffu, V[d][1], t);
      }
      gather_kept(P, nP, I + (base + t) * k, k, N, S);
      for (int j = lane; j < m; j += 32) {
        const double x = S.p[j][0] - mean[0], y = S.p[j][1] - mean[1], z = S.p[j][2] - mean[2];
        S.u[j] = x * e1[0] + y * e1[1] + z * e1[2];
        S.w[j] = x * e2[0] + y * e2[1] + z * e2[2];
      }
      __syncwarp();
      const double u0 = S.u[0], w0 = S.w[0];
      const long long bu0 = __double_as_longlong(u0), bw0 = __double_as_longlong(w0);
      // images about vertex 0; a point equal to vertex 0 or to an earlier
      // point is left out (CGAL keeps the first of equal points)
      for (int j = lane; j < m; j += 32) {
        const long long bu = __double_as_longlong(S.u[j]), bw = __double_as_longlong(S.w[j]);
        bool ok = j > 0 && !(bu == bu0 && bw == bw0);
        for (int l = 1; ok && l < j; ++l)
          if (__double_as_longlong(S.u[l]) == bu && __double_as_longlong(S.w[l]) == bw) ok = false;
        const double qx = S.u[j] - u0, qy = S.w[j] - w0;
        const double inv = ok ? 1.0 / (qx * qx + qy * qy) : 0.0;
        S.ok[j] = ok ? 1 : 0;
        S.su[j] = qx * inv;
        S.sw[j] = qy * inv;
        S.fu[j] = (float)(qx * inv);
        S.fw[j] = (float)(qy * inv);
      }
      __syncwarp();
      double acc = 0.0;
      for (int j = lane; j < m; j += 32) {
        if (!S.ok[j]) continue;
        int c = -1;
        for (int l = 1; l < m; ++l) {  // most clockwise image seen from j
          if (l == j || !S.ok[l]) continue;
          if (c < 0) {
            c = l;
            continue;
          }
          const int o = orient_sign(S, j, c, l);
          if (o < 0) {
            c = l;
          } else if (o == 0) {  // collinear: the farther one
            const double dc = (S.su[c] - S.su[j]) * (S.su[c] - S.su[j]) +
                              (S.sw[c] - S.sw[j]) * (S.sw[c] - S.sw[j]);
            const double dl = (S.su[l] - S.su[j]) * (S.su[l] - S.su[j]) +
                              (S.sw[l] - S.sw[j]) * (S.sw[l] - S.sw[j]);
            if (dl > dc) c = l;
          }
        }
        if (c < 0) continue;
        bool edge = true;  // no image strictly right of j -> c
        for (int l = 1; edge && l < m; ++l)
          if (S.ok[l] && l != j && l != c && orient_sign(S, j, c, l) < 0) edge = false;
        if (!edge) continue;
        // vertex 0 (the origin of the images) strictly left of j -> c
        const double o0 = orient(S.su[j], S.sw[j], S.su[c], S.sw[c], 0.0, 0.0);
        if (!(o0 > 0)) continue;
        acc += voronoi_share(u0, w0, S.u[j], S.w[j], S.u[c], S.w[c]);
      }
      const double area = warp_sum(acc);
      if (lane == 0) A[base + t] = isfinite(area) ? area : 0.0;
      __syncwarp();
    }
  }
}

}  // namespace

void point_areas_run(const double* P, int64_t nP, const int32_t* I, int k, const double* N,
                     double* A, double* T, unsigned* status, cudaStream_t st) {
  if (nP == 0) return;
  const int64_t blocks =
      std::min<int64_t>((nP + 32 * kWarps - 1) / (32 * kWarps), (int64_t)num_sms() * 16);
  launch_kernel(point_areas_kernel, (unsigned)blocks, 32 * kWarps, 0, st, P, nP, I, k, N, A, T,
                status);
}

}  // namespace gwn
