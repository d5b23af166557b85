// CPU oracle: closest point on a triangle mesh (the distance half of
// igl::signed_distance).
//
// TEST INFRASTRUCTURE ONLY (see gwn_oracle.cpp): only tests/ and bench.py's
// CPU baseline load it; libgwn.so never does.
//
// Brute force over every triangle in index order instead of the reference's
// AABB tree (include/igl/AABB.cpp:1135-1205): the minimum squared distance is
// the same; in a tie the reference keeps the first triangle its traversal
// reaches (set_min's strict '<', AABB.cpp:787-802), brute force keeps the
// lowest index.  The per-triangle closest point is Ericson's region test
// (Real-Time Collision Detection, 5.1.5) as restated in
// include/igl/point_simplex_squared_distance.cpp:40-112, with the squared
// distance taken from the closest point (:124).
#include <cmath>
#include <cstdint>
#include <limits>
#include <thread>
#include <vector>

namespace {

struct P3 {
  double x, y, z;
};
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 axpy(P3 a, double s, P3 d) { return {a.x + s * d.x, a.y + s * d.y, a.z + s * d.z}; }

// Closest point to p on triangle (a, b, c), by Voronoi region.
P3 closest_on_triangle(P3 p, P3 a, P3 b, P3 c) {
  const P3 ab = sub(b, a), ac = sub(c, a), ap = sub(p, a);
  const double d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return a;  // vertex region a
  const P3 bp = sub(p, b);
  const double d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return b;  // vertex region b
  const double vc = d1 * d4 - d3 * d2;
  const bool a_is_b = a.x == b.x && a.y == b.y && a.z == b.z;
  if (!a_is_b && vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {  // edge ab
    const double v = d1 / (d1 - d3);
    return axpy(a, v, ab);
  }
  const P3 cp = sub(p, c);
  const double d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return c;  // vertex region c
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {  // edge ac
    const double w = d2 / (d2 - d6);
    return axpy(a, w, ac);
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {  // edge bc
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    return axpy(b, w, sub(c, b));
  }
  const double denom = 1.0 / (va + vb + vc);  // face interior
  const double v = vb * denom, w = vc * denom;
  return axpy(axpy(a, v, ab), w, ac);
}

unsigned threads(int requested) {
  if (requested > 0) return (unsigned)requested;
  const unsigned hw = std::thread::hardware_concurrency();
  return hw ? hw : 8u;
}

}  // namespace

extern "C" {

// For each query: the smallest squared distance to any triangle below
// up_sqr_d (sqrD = up_sqr_d and I = -1 when there is none), the triangle
// index and the closest point.
int oracle_squared_distance(const double* V, const int32_t* F, int64_t nF, const double* P,
                            int64_t nP, double up_sqr_d, double* sqrD, int32_t* I, double* C,
                            int nthreads) {
  const unsigned nt = threads(nthreads);
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t) {
    pool.emplace_back([=] {
      for (int64_t q = t; q < nP; q += nt) {
        const P3 p{P[q * 3], P[q * 3 + 1], P[q * 3 + 2]};
        double best = up_sqr_d;
        int32_t bi = -1;
        P3 bc{0, 0, 0};
        for (int64_t f = 0; f < nF; ++f) {
          const double* a = V + (int64_t)F[f * 3] * 3;
          const double* b = V + (int64_t)F[f * 3 + 1] * 3;
          const double* c = V + (int64_t)F[f * 3 + 2] * 3;
          const P3 cp = closest_on_triangle(p, {a[0], a[1], a[2]}, {b[0], b[1], b[2]},
                                            {c[0], c[1], c[2]});
          const P3 d = sub(p, cp);
          const double d2 = dot(d, d);
          if (d2 < best) {
            best = d2;
            bi = (int32_t)f;
            bc = cp;
          }
        }
        sqrD[q] = best;
        I[q] = bi;
        C[q * 3] = bc.x;
        C[q * 3 + 1] = bc.y;
        C[q * 3 + 2] = bc.z;
      }
    });
  }
  for (auto& th : pool) th.join();
  return 0;
}

// Closest point and squared distance for one (point, triangle) pair.
double oracle_point_triangle(const double* p, const double* a, const double* b,
                             const double* c, double* closest) {
  const P3 cp = closest_on_triangle({p[0], p[1], p[2]}, {a[0], a[1], a[2]}, {b[0], b[1], b[2]},
                                    {c[0], c[1], c[2]});
  closest[0] = cp.x;
  closest[1] = cp.y;
  closest[2] = cp.z;
  const P3 d = sub({p[0], p[1], p[2]}, cp);
  return dot(d, d);
}

}  // extern "C"
