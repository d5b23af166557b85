// CPU restatement of igl::AABB<V,3> for triangles: build and the
// closest-triangle query, used as the timed CPU baseline of the signed
// distance (and cross-checked against the brute force of distance.cpp).
//
// TEST INFRASTRUCTURE ONLY (see gwn_oracle.cpp).
//
// Build, include/igl/AABB.cpp:810-960: barycentres; for every axis the rank
// of each barycentre in a sort of that axis; a node's box bounds its
// triangles' vertices; a node of one triangle is a leaf; otherwise split at
// the median rank along the box's longest axis (nth_element on the ranks,
// ranks <= median go left).  Query, AABB.cpp:1135-1205: look into a child
// whose box contains the point, then into the children in order of their
// exterior distance while that distance is below the best so far; leaves use
// Ericson's closest point (point_simplex_squared_distance.cpp:40-124) and a
// strictly smaller distance wins (set_min, AABB.cpp:787-802).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

namespace {

struct Box {
  double lo[3] = {std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity(),
                  std::numeric_limits<double>::infinity()};
  double hi[3] = {-std::numeric_limits<double>::infinity(),
                  -std::numeric_limits<double>::infinity(),
                  -std::numeric_limits<double>::infinity()};
  void extend(const double* p) {
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], p[d]);
      hi[d] = std::max(hi[d], p[d]);
    }
  }
  bool contains(const double* p) const {
    for (int d = 0; d < 3; ++d)
      if (!(p[d] >= lo[d] && p[d] <= hi[d])) return false;
    return true;
  }
  double exterior2(const double* p) const {
    double s = 0;
    for (int d = 0; d < 3; ++d) {
      double e = 0;
      if (p[d] < lo[d]) e = lo[d] - p[d];
      else if (p[d] > hi[d]) e = p[d] - hi[d];
      s += e * e;
    }
    return s;
  }
};

struct Node {
  Box box;
  int left = -1, right = -1, prim = -1;
};

struct Tree {
  const double* V;
  const int32_t* F;
  std::vector<Node> nodes;
  std::vector<int> rank;  // nF x 3
  int build(std::vector<int> I) {
    const int id = (int)nodes.size();
    nodes.emplace_back();
    Box b;
    for (int f : I)
      for (int c = 0; c < 3; ++c) b.extend(V + (int64_t)F[(int64_t)f * 3 + c] * 3);
    nodes[id].box = b;
    if (I.size() == 1) {
      nodes[id].prim = I[0];
      return id;
    }
    int max_d = 0;
    double best = -1;
    for (int d = 0; d < 3; ++d) {
      const double e = b.hi[d] - b.lo[d];
      if (e > best) {
        best = e;
        max_d = d;
      }
    }
    std::vector<int> r(I.size());
    for (size_t i = 0; i < I.size(); ++i) r[i] = rank[(size_t)I[i] * 3 + max_d];
    std::vector<int> tmp = r;
    const size_t n = (tmp.size() - 1) / 2;
    std::nth_element(tmp.begin(), tmp.begin() + n, tmp.end());
    const int med = tmp[n];
    std::vector<int> L, R;
    L.reserve((I.size() + 1) / 2);
    R.reserve(I.size() / 2);
    for (size_t i = 0; i < I.size(); ++i) (r[i] <= med ? L : R).push_back(I[i]);
    if (!L.empty()) {
      const int l = build(std::move(L));
      nodes[id].left = l;
    }
    if (!R.empty()) {
      const int rr = build(std::move(R));
      nodes[id].right = rr;
    }
    return id;
  }
};

inline void sub3(const double* a, const double* b, double* o) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}
inline double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

void closest(const double* p, const double* a, const double* b, const double* c, double* out) {
  double ab[3], ac[3], ap[3], bp[3], cp[3];
  sub3(b, a, ab);
  sub3(c, a, ac);
  sub3(p, a, ap);
  const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  auto set = [&](const double* s) { out[0] = s[0]; out[1] = s[1]; out[2] = s[2]; };
  auto lerp = [&](const double* s, double t, const double* d) {
    out[0] = s[0] + t * d[0]; out[1] = s[1] + t * d[1]; out[2] = s[2] + t * d[2];
  };
  if (d1 <= 0.0 && d2 <= 0.0) return set(a);
  sub3(p, b, bp);
  const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return set(b);
  const double vc = d1 * d4 - d3 * d2;
  const bool a_is_b = a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
  if (!a_is_b && vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return lerp(a, d1 / (d1 - d3), ab);
  sub3(p, c, cp);
  const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return set(c);
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return lerp(a, d2 / (d2 - d6), ac);
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
    double bc[3];
    sub3(c, b, bc);
    return lerp(b, (d4 - d3) / ((d4 - d3) + (d5 - d6)), bc);
  }
  const double denom = 1.0 / (va + vb + vc);
  const double v = vb * denom, w = vc * denom;
  double t[3];
  lerp(a, v, ab);
  t[0] = out[0]; t[1] = out[1]; t[2] = out[2];
  lerp(t, w, ac);
}

double query(const Tree& T, int id, const double* p, double up, int& i, double* c) {
  const Node& n = T.nodes[id];
  double sqr_d = up;
  if (n.prim >= 0) {
    const int f = n.prim;
    double cc[3];
    closest(p, T.V + (int64_t)T.F[(int64_t)f * 3] * 3, T.V + (int64_t)T.F[(int64_t)f * 3 + 1] * 3,
            T.V + (int64_t)T.F[(int64_t)f * 3 + 2] * 3, cc);
    double d[3];
    sub3(p, cc, d);
    const double d2 = dot3(d, d);
    if (d2 < sqr_d) {
      sqr_d = d2;
      i = f;
      c[0] = cc[0]; c[1] = cc[1]; c[2] = cc[2];
    }
    return sqr_d;
  }
  bool looked_l = false, looked_r = false;
  auto look = [&](int child, bool& flag) {
    int ic = -1;
    double cc[3] = {c[0], c[1], c[2]};
    const double d2 = query(T, child, p, sqr_d, ic, cc);
    if (d2 < sqr_d) {
      sqr_d = d2;
      i = ic;
      c[0] = cc[0]; c[1] = cc[1]; c[2] = cc[2];
    }
    flag = true;
  };
  if (n.left >= 0 && T.nodes[n.left].box.contains(p)) look(n.left, looked_l);
  if (n.right >= 0 && T.nodes[n.right].box.contains(p)) look(n.right, looked_r);
  const double dl = n.left >= 0 ? T.nodes[n.left].box.exterior2(p)
                                : std::numeric_limits<double>::infinity();
  const double dr = n.right >= 0 ? T.nodes[n.right].box.exterior2(p)
                                 : std::numeric_limits<double>::infinity();
  if (dl < dr) {
    if (!looked_l && n.left >= 0 && dl < sqr_d) look(n.left, looked_l);
    if (!looked_r && n.right >= 0 && dr < sqr_d) look(n.right, looked_r);
  } else {
    if (!looked_r && n.right >= 0 && dr < sqr_d) look(n.right, looked_r);
    if (!looked_l && n.left >= 0 && dl < sqr_d) look(n.left, looked_l);
  }
  return sqr_d;
}

}  // namespace

extern "C" {

void* oracle_aabb_build(const double* V, const int32_t* F, int64_t nF) {
  Tree* T = new Tree();
  T->V = V;
  T->F = F;
  if (nF == 0) return T;
  std::vector<double> bc((size_t)nF * 3);
  for (int64_t f = 0; f < nF; ++f)
    for (int d = 0; d < 3; ++d) {
      double s = 0;
      for (int c = 0; c < 3; ++c) s += V[(int64_t)F[f * 3 + c] * 3 + d];
      bc[(size_t)f * 3 + d] = s / 3.0;
    }
  T->rank.assign((size_t)nF * 3, 0);
  std::vector<int> idx((size_t)nF);
  for (int d = 0; d < 3; ++d) {
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return bc[(size_t)a * 3 + d] < bc[(size_t)b * 3 + d]; });
    for (int64_t r = 0; r < nF; ++r) T->rank[(size_t)idx[(size_t)r] * 3 + d] = (int)r;
  }
  std::vector<int> all((size_t)nF);
  std::iota(all.begin(), all.end(), 0);
  T->nodes.reserve((size_t)nF * 2);
  T->build(std::move(all));
  return T;
}

void oracle_aabb_free(void* h) { delete static_cast<Tree*>(h); }

// sqrD / I / C per query as AABB::squared_distance(V,F,p,0,up_sqr_d,i,c);
// nthreads host threads, interleaved queries.
void oracle_aabb_squared_distance(void* h, const double* P, int64_t nP, double up_sqr_d,
                                  double* sqrD, int32_t* I, double* C, int nthreads) {
  const Tree* T = static_cast<const Tree*>(h);
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::thread::hardware_concurrency();
  if (!nt) nt = 8;
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([=] {
      for (int64_t q = t; q < nP; q += nt) {
        int i = -1;
        double c[3] = {0, 0, 0};
        const double d2 = T->nodes.empty() ? up_sqr_d : query(*T, 0, P + q * 3, up_sqr_d, i, c);
        sqrD[q] = d2;
        I[q] = i;
        C[q * 3] = c[0];
        C[q * 3 + 1] = c[1];
        C[q * 3 + 2] = c[2];
      }
    });
  for (auto& th : pool) th.join();
}

}  // extern "C"
