// CPU restatement of igl::copyleft::cgal::point_areas
// (include/igl/copyleft/cgal/point_areas.cpp:60-160).  TEST INFRASTRUCTURE
// ONLY: the checker of the GPU kernel (libgwn never uses it).
//
// CGAL is not available, so this restatement takes the reference's steps
// with independent methods of its own, different from the GPU's:
//   * the kept neighbours (positive dot product of normals with the first
//     neighbour's normal; none filtered for k = 1), A = 0 for two or fewer;
//   * the SVD of the centred neighbours by one-sided Jacobi rotations (the
//     method of Eigen's JacobiSVD, which the reference calls), plane = the
//     coordinates along the two largest right singular vectors (U S);
//     T = the least one, turned towards N(i);
//   * the Delaunay triangulation by brute force: every triangle of three
//     distinct, non-collinear plane points whose circumcircle holds no other
//     point strictly inside (points equal to an earlier one dropped, as
//     CGAL keeps the first of equal points);
//   * for each such triangle through the first kept point, the reference's
//     area share (point_areas.cpp:122-150), summed in triangle order; a
//     non-finite sum gives 0.
// O(m^3) per point: for tests on modest clouds.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

void jacobi_svd_v(std::vector<double>& X, int m, double V[3][3], double sv[3]) {
  // X: m x 3 row-major, orthogonalised in place (columns become U S)
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) V[r][c] = r == c ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double a = 0, b = 0, g = 0;
        for (int i = 0; i < m; ++i) {
          a += X[i * 3 + p] * X[i * 3 + p];
          b += X[i * 3 + q] * X[i * 3 + q];
          g += X[i * 3 + p] * X[i * 3 + q];
        }
        if (std::fabs(g) <= 1e-15 * std::sqrt(a * b) || g == 0) continue;
        rotated = true;
        const double zeta = (b - a) / (2 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
        const double c = 1 / std::sqrt(1 + t * t), s = c * t;
        for (int i = 0; i < m; ++i) {
          const double xp = X[i * 3 + p], xq = X[i * 3 + q];
          X[i * 3 + p] = c * xp - s * xq;
          X[i * 3 + q] = s * xp + c * xq;
        }
        for (int r = 0; r < 3; ++r) {
          const double vp = V[r][p], vq = V[r][q];
          V[r][p] = c * vp - s * vq;
          V[r][q] = s * vp + c * vq;
        }
      }
    if (!rotated) break;
  }
  int order[3] = {0, 1, 2};
  double n[3];
  for (int c = 0; c < 3; ++c) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += X[i * 3 + c] * X[i * 3 + c];
    n[c] = std::sqrt(s);
  }
  std::sort(order, order + 3, [&](int a, int b) { return n[a] > n[b]; });
  double V2[3][3];
  std::vector<double> X2((size_t)m * 3);
  for (int c = 0; c < 3; ++c) {
    sv[c] = n[order[c]];
    for (int r = 0; r < 3; ++r) V2[r][c] = V[r][order[c]];
    for (int i = 0; i < m; ++i) X2[(size_t)i * 3 + c] = X[(size_t)i * 3 + order[c]];
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) V[r][c] = V2[r][c];
  X.swap(X2);
}

double share(const double* X, const double* Y, const double* Z) {
  const double x = std::hypot(Y[0] - Z[0], Y[1] - Z[1]);
  const double y = std::hypot(X[0] - Z[0], X[1] - Z[1]);
  const double z = std::hypot(Y[0] - X[0], Y[1] - X[1]);
  const double cosX = (z * z + y * y - x * x) / (2 * y * z);
  const double cosY = (z * z + x * x - y * y) / (2 * x * z);
  const double cosZ = (x * x + y * y - z * z) / (2 * y * x);
  double b[3] = {x * cosX, y * cosY, z * cosZ};
  const double bs = b[0] + b[1] + b[2];
  for (double& v : b) v /= bs;
  const double full = 0.25 * std::sqrt((x + (y + z)) * (z - (x - y)) * (z + (x - y)) * (x + (y - z)));
  if (cosX < 0) return 0.5 * full;
  if (cosY < 0 || cosZ < 0) return 0.25 * full;
  return (b[1] * full + b[2] * full) / 2;
}

// > 0 when d is strictly inside the circle through a, b, c (any orientation)
double incircle(const double* a, const double* b, const double* c, const double* d) {
  const double adx = a[0] - d[0], ady = a[1] - d[1], bdx = b[0] - d[0], bdy = b[1] - d[1];
  const double cdx = c[0] - d[0], cdy = c[1] - d[1];
  const double det = (adx * adx + ady * ady) * (bdx * cdy - cdx * bdy) -
                     (bdx * bdx + bdy * bdy) * (adx * cdy - cdx * ady) +
                     (cdx * cdx + cdy * cdy) * (adx * bdy - bdx * ady);
  const double orient = (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]);
  return orient > 0 ? det : -det;
}

void one_point(const double* P, int64_t nP, const int32_t* I, int k, const double* N, int64_t i,
               double* A, double* T) {
  const int32_t* row = I + i * k;
  std::vector<int> kept;
  for (int j = 0; j < k; ++j) {
    const int32_t idx = row[j];
    if (idx < 0 || idx >= nP) {
      A[i] = 0;
      if (T) T[i * 3] = T[i * 3 + 1] = T[i * 3 + 2] = 0;
      return;
    }
    if (k > 1) {
      const double* n0 = N + (int64_t)row[0] * 3;
      const double* nj = N + (int64_t)idx * 3;
      if (!(n0[0] * nj[0] + n0[1] * nj[1] + n0[2] * nj[2] > 0)) continue;
    }
    kept.push_back(idx);
  }
  const int m = (int)kept.size();
  if (T) T[i * 3] = T[i * 3 + 1] = T[i * 3 + 2] = 0;
  if (m <= 2) {
    A[i] = 0;
    return;
  }
  double mean[3] = {0, 0, 0};
  for (int j = 0; j < m; ++j)
    for (int d = 0; d < 3; ++d) mean[d] += P[(int64_t)kept[j] * 3 + d];
  for (double& v : mean) v /= m;
  std::vector<double> X((size_t)m * 3);
  for (int j = 0; j < m; ++j)
    for (int d = 0; d < 3; ++d) X[(size_t)j * 3 + d] = P[(int64_t)kept[j] * 3 + d] - mean[d];
  double V[3][3], sv[3];
  jacobi_svd_v(X, m, V, sv);
  if (T) {
    double t[3] = {V[0][2], V[1][2], V[2][2]};
    const double* ni = N + i * 3;
    if (t[0] * ni[0] + t[1] * ni[1] + t[2] * ni[2] < 0)
      for (double& v : t) v = -v;
    for (int d = 0; d < 3; ++d) T[i * 3 + d] = t[d];
  }
  std::vector<std::array<double, 2>> pl;
  std::vector<int> id;  // distinct plane points (first of equal ones)
  for (int j = 0; j < m; ++j) {
    const std::array<double, 2> p = {X[(size_t)j * 3], X[(size_t)j * 3 + 1]};
    bool dup = false;
    for (const auto& q : pl) dup |= (q[0] == p[0] && q[1] == p[1]);
    if (dup) continue;
    pl.push_back(p);
    id.push_back(j);
  }
  double acc = 0;
  if (!pl.empty() && id[0] == 0) {
    const int n = (int)pl.size();
    for (int b = 1; b < n; ++b)
      for (int c = b + 1; c < n; ++c) {
        const double* pa = pl[0].data();
        const double* pb = pl[b].data();
        const double* pc = pl[c].data();
        const double o = (pb[0] - pa[0]) * (pc[1] - pa[1]) - (pb[1] - pa[1]) * (pc[0] - pa[0]);
        if (o == 0) continue;
        bool empty = true;
        for (int d = 1; empty && d < n; ++d)
          if (d != b && d != c && incircle(pa, pb, pc, pl[d].data()) > 0) empty = false;
        if (empty) acc += share(pa, pb, pc);
      }
  }
  A[i] = std::isfinite(acc) ? acc : 0.0;
}

}  // namespace

extern "C" {

// Rows 0 .. nI-1 of I are points 0 .. nI-1 of P (nP points in all).
void oracle_point_areas(const double* P, int64_t nP, int64_t nI, const int32_t* I, int k,
                        const double* N, double* A, double* T, int nthreads) {
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::thread::hardware_concurrency();
  if (nt == 0) nt = 8;
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([=] {
      for (int64_t i = t; i < nI; i += nt) one_point(P, nP, I, k, N, i, A, T);
    });
  for (auto& th : pool) th.join();
}

}  // extern "C"
