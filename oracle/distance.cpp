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
#include <algorithm>
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

// Pseudonormal signs (signed_distance.cpp:69-76, 118-124): per_face_normals
// (per_face_normals.cpp:17-30), corner angles (internal_angles.cpp:15-38),
// per_vertex_normals with angle weights and per_edge_normals with uniform
// weights (sums in face order, then normalised), and pseudonormal_test
// (pseudonormal_test.cpp:16-135) at each query's closest face I and point C.
// sgn[p] = +-1, N[p] = the normal used.
int oracle_pseudonormal(const double* V, int64_t nV, const int32_t* F, int64_t nF, const double* P,
                        int64_t nP, const int32_t* I, const double* C, double* sgn, double* N) {
  auto vr = [&](int64_t f, int c) {
    const double* p = V + (int64_t)F[f * 3 + c] * 3;
    return P3{p[0], p[1], p[2]};
  };
  auto nrm = [](P3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); };
  std::vector<P3> FN((size_t)nF), VN((size_t)nV, P3{0, 0, 0});
  for (int64_t f = 0; f < nF; ++f) {
    const P3 a = vr(f, 0), v1 = sub(vr(f, 1), a), v2 = sub(vr(f, 2), a);
    P3 n{v1.y * v2.z - v1.z * v2.y, v1.z * v2.x - v1.x * v2.z, v1.x * v2.y - v1.y * v2.x};
    const double r = nrm(n);
    FN[(size_t)f] = r == 0 ? P3{0, 0, 0} : P3{n.x / r, n.y / r, n.z / r};
  }
  // vertex normals, angle weights, in (face, corner) order
  for (int64_t f = 0; f < nF; ++f)
    for (int j = 0; j < 3; ++j) {
      const P3 x = vr(f, (j + 2) % 3), y = vr(f, j), z = vr(f, (j + 1) % 3);
      const P3 v1 = sub(x, y), v2 = sub(z, y);
      const double n1 = nrm(v1), n2 = nrm(v2);
      const P3 u1{v1.x / n1, v1.y / n1, v1.z / n1}, u2{v2.x / n2, v2.y / n2, v2.z / n2};
      const double w = 2.0 * std::atan(nrm(P3{u1.x - u2.x, u1.y - u2.y, u1.z - u2.z}) /
                                       nrm(P3{u1.x + u2.x, u1.y + u2.y, u1.z + u2.z}));
      P3& acc = VN[(size_t)F[f * 3 + j]];
      acc.x += w * FN[(size_t)f].x;
      acc.y += w * FN[(size_t)f].y;
      acc.z += w * FN[(size_t)f].z;
    }
  for (auto& v : VN) {
    const double r = nrm(v);
    if (r > 0) v = {v.x / r, v.y / r, v.z / r};
  }
  // edge normals: undirected edge of (face, corner) = the edge opposite it
  std::vector<std::pair<uint64_t, int64_t>> ek((size_t)nF * 3);
  for (int64_t f = 0; f < nF; ++f)
    for (int c = 0; c < 3; ++c) {
      const uint64_t a = (uint32_t)F[f * 3 + (c + 1) % 3], b = (uint32_t)F[f * 3 + (c + 2) % 3];
      ek[(size_t)(f * 3 + c)] = {(std::min(a, b) << 32) | std::max(a, b), f * 3 + c};
    }
  std::vector<std::pair<uint64_t, int64_t>> sorted = ek;
  std::stable_sort(sorted.begin(), sorted.end(),
                   [](const auto& x, const auto& y) { return x.first < y.first; });
  std::vector<int64_t> edge_of((size_t)nF * 3);
  std::vector<P3> EN;
  for (size_t i = 0; i < sorted.size();) {
    size_t j = i;
    P3 acc{0, 0, 0};
    for (; j < sorted.size() && sorted[j].first == sorted[i].first; ++j) {
      const P3 fn = FN[(size_t)(sorted[j].second / 3)];
      acc.x += fn.x;
      acc.y += fn.y;
      acc.z += fn.z;
      edge_of[(size_t)sorted[j].second] = (int64_t)EN.size();
    }
    const double r = nrm(acc);
    EN.push_back(r > 0 ? P3{acc.x / r, acc.y / r, acc.z / r} : acc);
    i = j;
  }
  for (int64_t p = 0; p < nP; ++p) {
    const int64_t f = I[p];
    if (f < 0 || f >= nF) {
      sgn[p] = 1.0;
      N[p * 3] = N[p * 3 + 1] = N[p * 3 + 2] = 0.0;
      continue;
    }
    const P3 q{P[p * 3], P[p * 3 + 1], P[p * 3 + 2]}, c{C[p * 3], C[p * 3 + 1], C[p * 3 + 2]};
    const P3 A = vr(f, 0), B = vr(f, 1), Cc = vr(f, 2);
    double l[3] = {nrm(sub(B, Cc)), nrm(sub(Cc, A)), nrm(sub(A, B))};
    std::sort(l, l + 3, [](double x, double y) { return x > y; });
    const double area =
        2.0 * 0.25 * std::sqrt((l[0] + (l[1] + l[2])) * (l[2] - (l[0] - l[1])) *
                               (l[2] + (l[0] - l[1])) * (l[0] + (l[1] - l[2])));
    P3 n = FN[(size_t)f];
    bool found = false;
    if (area > 1e-4) {
      const P3 v0 = sub(B, A), v1 = sub(Cc, A), v2 = sub(c, A);
      const double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0),
                   d21 = dot(v2, v1);
      const double den = d00 * d11 - d01 * d01;
      const double b1 = (d11 * d20 - d01 * d21) / den, b2 = (d00 * d21 - d01 * d20) / den;
      const double b[3] = {1.0 - (b1 + b2), b1, b2};
      const int type = (b[0] <= 1e-12) + (b[1] <= 1e-12) + (b[2] <= 1e-12);
      if (type == 2) {
        for (int x = 0; x < 3; ++x)
          if (b[x] > 1e-12) {
            n = VN[(size_t)F[f * 3 + x]];
            break;
          }
      } else if (type == 1) {
        for (int x = 0; x < 3; ++x)
          if (b[x] <= 1e-12) {
            n = EN[(size_t)edge_of[(size_t)(f * 3 + x)]];
            break;
          }
      }
    } else {
      for (int v = 0; v < 3 && !found; ++v)
        if (nrm(sub(c, vr(f, v))) < 1e-12) {
          n = VN[(size_t)F[f * 3 + v]];
          found = true;
        }
      for (int e = 0; e < 3 && !found; ++e) {
        const P3 S = vr(f, (e + 1) % 3), D = vr(f, (e + 2) % 3);
        const P3 dms = sub(D, S), smp = sub(S, c);
        const double t = -(dms.x * smp.x + dms.y * smp.y + dms.z * smp.z) / dot(dms, dms);
        double sq;
        if (t < 0) sq = dot(sub(c, S), sub(c, S));
        else if (t > 1) sq = dot(sub(c, D), sub(c, D));
        else {
          const P3 pp{(1 - t) * S.x + t * D.x, (1 - t) * S.y + t * D.y, (1 - t) * S.z + t * D.z};
          sq = dot(sub(c, pp), sub(c, pp));
        }
        if (std::sqrt(sq) < 1e-12) {
          n = EN[(size_t)edge_of[(size_t)(f * 3 + e)]];
          found = true;
        }
      }
    }
    sgn[p] = dot(sub(q, c), n) >= 0 ? 1.0 : -1.0;
    N[p * 3] = n.x;
    N[p * 3 + 1] = n.y;
    N[p * 3 + 2] = n.z;
  }
  return 0;
}

}  // extern "C"
