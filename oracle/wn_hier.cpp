// CPU restatement of the reference's hierarchical exact winding number
// (TEST INFRASTRUCTURE ONLY: CPU baseline and checker; not used by libgwn.so).
//
// igl::winding_number(V,F,O,W) for triangles (include/igl/winding_number.cpp:
// 40-53) builds a WindingNumberAABB hierarchy and evaluates each query with
// it, in igl::parallel_for(..., 10000):
//   * set_mesh (WindingNumberTree.h:166-200): merge exactly duplicate
//     vertices (remove_duplicate_vertices, eps 0), then cap = triangle fan of
//     the exterior (boundary) edges (exterior_edges.cpp:44-99,
//     triangle_fan.cpp:15-47, apex chosen with rand());
//   * grow (WindingNumberAABB.h:149-247): stop at <= 100 faces or when the
//     cap is not smaller than the face set; otherwise split at the median of
//     the face barycentres along the longest bbox axis (<= goes left), stop if
//     one side is empty, recurse;
//   * query (WindingNumberTree.h:261-336): inside the node's bbox (inclusive)
//     recurse into children or sum every face; outside, sum the cap when it
//     has fewer faces, else every face.  Per-face terms are solid_angle.cpp.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <thread>
#include <tuple>
#include <vector>

namespace {

const double kPi = 3.1415926535897932384626433832795;

double solid_angle(const double* A, const double* B, const double* C, const double* P) {
  double v[3][3];
  for (int d = 0; d < 3; ++d) {
    v[0][d] = A[d] - P[d];
    v[1][d] = B[d] - P[d];
    v[2][d] = C[d] - P[d];
  }
  double vl[3];
  for (int r = 0; r < 3; ++r)
    vl[r] = std::sqrt(v[r][0] * v[r][0] + (v[r][1] * v[r][1] + v[r][2] * v[r][2]));
  const double det = v[0][0] * v[1][1] * v[2][2] + v[1][0] * v[2][1] * v[0][2] +
                     v[2][0] * v[0][1] * v[1][2] - v[2][0] * v[1][1] * v[0][2] -
                     v[1][0] * v[0][1] * v[2][2] - v[0][0] * v[2][1] * v[1][2];
  double dp0 = v[1][0] * v[2][0];
  dp0 += v[1][1] * v[2][1];
  dp0 += v[1][2] * v[2][2];
  double dp1 = v[2][0] * v[0][0];
  dp1 += v[2][1] * v[0][1];
  dp1 += v[2][2] * v[0][2];
  double dp2 = v[0][0] * v[1][0];
  dp2 += v[0][1] * v[1][1];
  dp2 += v[0][2] * v[1][2];
  return std::atan2(det, vl[0] * vl[1] * vl[2] + dp0 * vl[0] + dp1 * vl[1] + dp2 * vl[2]) /
         (2. * kPi);
}

using Tri = std::array<int32_t, 3>;

// exterior_edges.cpp:44-99: signed count of each undirected edge over the
// oriented facets; an edge with non-zero count is emitted |count| times,
// oriented by the sign, in lexicographic order of the sorted edge.
std::vector<std::pair<int32_t, int32_t>> exterior_edges(const std::vector<Tri>& F) {
  std::map<std::pair<int32_t, int32_t>, int> cnt;
  for (const Tri& f : F) {
    const int32_t e[3][2] = {{f[1], f[2]}, {f[2], f[0]}, {f[0], f[1]}};
    for (auto& ed : e) {
      if (ed[0] <= ed[1]) cnt[{ed[0], ed[1]}] += 1;
      else cnt[{ed[1], ed[0]}] -= 1;
    }
  }
  std::vector<std::pair<int32_t, int32_t>> E;
  for (auto& kv : cnt) {
    const int c = kv.second;
    if (c == 0) continue;
    const auto ij = c < 0 ? std::make_pair(kv.first.second, kv.first.first) : kv.first;
    for (int k = 0; k < std::abs(c); ++k) E.push_back(ij);
  }
  return E;
}

std::vector<Tri> triangle_fan(const std::vector<std::pair<int32_t, int32_t>>& E) {
  std::vector<Tri> cap;
  if (E.empty()) return cap;
  const int32_t s = E[(size_t)(std::rand() % (int)E.size())].first;
  for (auto& e : E) {
    if (e.first == s || e.second == s) continue;
    cap.push_back({s, e.first, e.second});
  }
  return cap;
}

// median.cpp:16-35, with its two nth_element calls.
double median(std::vector<double> v) {
  const size_t n = v.size() / 2;
  std::nth_element(v.begin(), v.begin() + n, v.end());
  if (v.size() % 2 == 0) {
    std::nth_element(v.begin(), v.begin() + n - 1, v.end());
    return 0.5 * (v[n] + v[n - 1]);
  }
  return v[n];
}

struct Node {
  std::vector<Tri> F, cap;
  double mn[3], mx[3];
  std::vector<std::unique_ptr<Node>> children;
};

struct Hier {
  std::vector<double> SV;  // merged vertices, 3 per vertex

  const double* v(int32_t i) const { return &SV[(size_t)i * 3]; }

  void init_node(Node& nd) {
    for (int d = 0; d < 3; ++d) {
      nd.mn[d] = INFINITY;
      nd.mx[d] = -INFINITY;
    }
    for (const Tri& f : nd.F)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) {
          const double x = v(f[c])[d];
          nd.mn[d] = x < nd.mn[d] ? x : nd.mn[d];
          nd.mx[d] = x > nd.mx[d] ? x : nd.mx[d];
        }
  }

  void grow(Node& nd) {
    if ((int64_t)nd.F.size() <= 100 || ((int64_t)nd.cap.size() - 2) >= (int64_t)nd.F.size()) return;
    int ax = -1;
    double len = -INFINITY;
    for (int d = 0; d < 3; ++d)
      if (nd.mx[d] - nd.mn[d] > len) {
        len = nd.mx[d] - nd.mn[d];
        ax = d;
      }
    std::vector<double> bc(nd.F.size());
    for (size_t i = 0; i < nd.F.size(); ++i) {
      const Tri& f = nd.F[i];
      bc[i] = (v(f[0])[ax] + v(f[1])[ax] + v(f[2])[ax]) / 3.0;
    }
    const double split = median(bc);
    std::vector<Tri> L, R;
    for (size_t i = 0; i < nd.F.size(); ++i) (bc[i] <= split ? L : R).push_back(nd.F[i]);
    if (L.empty() || R.empty()) return;
    for (auto* part : {&L, &R}) {
      auto c = std::make_unique<Node>();
      c->F = std::move(*part);
      c->cap = triangle_fan(exterior_edges(c->F));
      init_node(*c);
      grow(*c);
      nd.children.push_back(std::move(c));
    }
  }

  static bool inside(const Node& nd, const double* p) {
    for (int d = 0; d < 3; ++d)
      if (p[d] < nd.mn[d] || p[d] > nd.mx[d]) return false;
    return true;
  }

  double sum(const std::vector<Tri>& F, const double* p) const {
    double w = 0;
    for (const Tri& f : F) w += solid_angle(v(f[0]), v(f[1]), v(f[2]), p);
    return w;
  }

  double query(const Node& nd, const double* p) const {
    if (inside(nd, p)) {
      if (!nd.children.empty()) {
        double s = 0;
        for (auto& c : nd.children) s += query(*c, p);
        return s;
      }
      return sum(nd.F, p);
    }
    if (((int64_t)nd.cap.size() - 2) < (int64_t)nd.F.size()) return sum(nd.cap, p);
    return sum(nd.F, p);
  }

  Node root;

  void build(const double* V, int64_t nV, const int32_t* F, int64_t nF) {
    // remove_duplicate_vertices(eps = 0): unique rows, faces remapped
    std::vector<int64_t> order((size_t)nV);
    for (int64_t i = 0; i < nV; ++i) order[(size_t)i] = i;
    auto row = [&](int64_t i) { return std::make_tuple(V[i * 3], V[i * 3 + 1], V[i * 3 + 2]); };
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return row(a) < row(b); });
    std::vector<int32_t> map((size_t)nV);
    SV.clear();
    for (size_t k = 0; k < order.size(); ++k) {
      if (k == 0 || row(order[k]) != row(order[k - 1])) {
        const int64_t i = order[k];
        SV.insert(SV.end(), {V[i * 3], V[i * 3 + 1], V[i * 3 + 2]});
      }
      map[(size_t)order[k]] = (int32_t)(SV.size() / 3 - 1);
    }
    root.F.resize((size_t)nF);
    for (int64_t f = 0; f < nF; ++f)
      root.F[(size_t)f] = {map[(size_t)F[f * 3]], map[(size_t)F[f * 3 + 1]], map[(size_t)F[f * 3 + 2]]};
    root.cap = triangle_fan(exterior_edges(root.F));
    init_node(root);
    grow(root);
  }
};

}  // namespace

extern "C" {

int oracle_winding_number_hier(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                               const double* O, int64_t nO, double* W, int nthreads) {
  Hier h;
  h.build(V, nV, F, nF);
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : 0;
  if (!nt) {
    if (const char* s = std::getenv("IGL_NUM_THREADS")) nt = (unsigned)std::max(0, std::atoi(s));
    if (!nt) nt = std::thread::hardware_concurrency();
    if (!nt) nt = 8;
  }
  auto one = [&](int64_t o) { W[o] = h.query(h.root, O + o * 3); };
  if (nO < 10000 || nt <= 1) {
    for (int64_t o = 0; o < nO; ++o) one(o);
    return 0;
  }
  const int64_t slice = std::max<int64_t>((int64_t)std::llround((nO + 1) / (double)nt), 1);
  std::vector<std::thread> pool;
  int64_t i1 = 0, i2 = std::min<int64_t>(slice, nO);
  unsigned t = 0;
  for (; t + 1 < nt && i1 < nO; ++t) {
    pool.emplace_back([=, &one] { for (int64_t k = i1; k < i2; ++k) one(k); });
    i1 = i2;
    i2 = std::min<int64_t>(i2 + slice, nO);
  }
  if (i1 < nO) pool.emplace_back([=, &one] { for (int64_t k = i1; k < nO; ++k) one(k); });
  for (auto& th : pool) th.join();
  return 0;
}

}  // extern "C"
