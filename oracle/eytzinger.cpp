// CPU restatement of libigl's Eytzinger-AABB 2-D winding number:
//   eytzinger_aabb                      include/igl/eytzinger_aabb.cpp:16-100
//   eytzinger_aabb_winding_number_tree  include/igl/eytzinger_aabb_winding_number_tree.cpp:17-118
//   eytzinger_aabb_winding_number       include/igl/eytzinger_aabb_winding_number.cpp:9-125
//
// TEST INFRASTRUCTURE ONLY (see gwn_oracle.cpp): the checker of the GPU
// kernels and the timed CPU baseline, never part of the product.
//
// Tree.  Slots 2^(ceil(log2 m)+1); a node's box is the min / max of its
// primitives' boxes; one primitive makes a leaf; otherwise the primitives are
// split at the median of their box centres along the box's longest axis
// (first axis on a tie): centres below go left, above go right (in list
// order), then the centres equal to the median, in list order, each to the
// smaller side (right on a tie).  The reference takes the median with
// igl::median (median.cpp:14-35): std::nth_element at n/2 and, for an even
// count, again at n/2-1 over the same array, then 0.5*(v[n/2] + v[n/2-1]).
// median_mode 0 restates exactly that (libstdc++'s nth_element, as a gcc
// build of the reference uses); median_mode 1 takes the two order statistics
// (the GPU's rule).  On inputs with distinct centre coordinates the two
// agree; the second nth_element call may leave a value other than the n/2-th
// order statistic at v[n/2] when centres repeat.
//
// Pair lists.  For each internal node, every vertex's net count over the
// subtree's segments (+1 per segment start, -1 per end); the vertices with a
// positive count (repeated count times) are paired in order with the negative
// ones.  The reference walks an unordered_map, so its pairing order is
// unspecified; canonical = 1 sorts both lists by vertex index (the GPU's
// order).  Any pairing gives the same winding number up to rounding: a box
// that excludes the query subtends less than pi, so the sum of the pairs'
// angles equals the sum of the subtree's segment angles.
//
// Evaluation.  Depth-first from the root with an explicit stack (push left,
// push right, pop): a leaf adds its segment's angle; a box that excludes p
// adds the node's pairs; otherwise both children are pushed.  The angle is
// atan2(cross, dot) of (V[a]-p, V[b]-p) divided by 2*pi, per term.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <functional>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

constexpr double kPi = 3.1415926535897932384626433832795;

double median_ref(std::vector<double> v) {
  const size_t n = v.size() / 2;
  std::nth_element(v.begin(), v.begin() + n, v.end());
  if (v.size() % 2 == 0) {
    std::nth_element(v.begin(), v.begin() + n - 1, v.end());
    return 0.5 * (v[n] + v[n - 1]);
  }
  return v[n];
}

double median_exact(std::vector<double> v) {
  std::sort(v.begin(), v.end());
  const size_t n = v.size() / 2;
  if (v.size() % 2 == 0) return 0.5 * (v[n] + v[n - 1]);
  return v[n];
}

inline double seg_angle(const double* V, int a, int b, double px, double py) {
  const double v0x = V[2 * (int64_t)a] - px, v0y = V[2 * (int64_t)a + 1] - py;
  const double v1x = V[2 * (int64_t)b] - px, v1y = V[2 * (int64_t)b + 1] - py;
  return std::atan2(v0x * v1y - v0y * v1x, v0x * v1x + v0y * v1y);
}

}  // namespace

extern "C" {

// Number of slots for m primitives (0 for m == 0).
int64_t oracle_eytzinger_slots(int64_t m) {
  if (m <= 0) return 0;
  return int64_t(1) << ((int)std::ceil(std::log2((double)m)) + 1);
}

// B1, B2: slots x dim (empty slots left as NaN); leaf: slots.
void oracle_eytzinger_aabb(const double* PB1, const double* PB2, int64_t m, int dim,
                           int median_mode, double* B1, double* B2, int32_t* leaf) {
  const int64_t nb = oracle_eytzinger_slots(m);
  for (int64_t i = 0; i < nb; ++i) {
    leaf[i] = -2;
    for (int d = 0; d < dim; ++d) B1[i * dim + d] = B2[i * dim + d] = NAN;
  }
  if (m == 0) return;
  std::vector<double> PBC((size_t)m * dim);
  for (int64_t i = 0; i < m * dim; ++i) PBC[(size_t)i] = (PB1[i] + PB2[i]) / 2;
  std::function<void(int64_t, const std::vector<int>&)> rec = [&](int64_t i,
                                                                  const std::vector<int>& I) {
    if (I.empty()) return;
    for (int d = 0; d < dim; ++d) {
      double lo = PB1[(int64_t)I[0] * dim + d], hi = PB2[(int64_t)I[0] * dim + d];
      for (int e : I) {
        lo = std::min(lo, PB1[(int64_t)e * dim + d]);
        hi = std::max(hi, PB2[(int64_t)e * dim + d]);
      }
      B1[i * dim + d] = lo;
      B2[i * dim + d] = hi;
    }
    if (I.size() == 1) {
      leaf[i] = I[0];
      return;
    }
    leaf[i] = -1;
    int dir = 0;
    double best = B2[i * dim] - B1[i * dim];
    for (int d = 1; d < dim; ++d) {
      const double e = B2[i * dim + d] - B1[i * dim + d];
      if (e > best) {
        best = e;
        dir = d;
      }
    }
    std::vector<double> Z(I.size());
    for (size_t j = 0; j < I.size(); ++j) Z[j] = PBC[(size_t)I[j] * dim + dir];
    const double split = median_mode == 0 ? median_ref(Z) : median_exact(Z);
    std::vector<int> left, right;
    left.reserve(I.size() / 2 + 1);
    right.reserve(I.size() / 2 + 1);
    for (size_t j = 0; j < I.size(); ++j) {
      if (Z[j] < split) left.push_back(I[j]);
      else if (Z[j] > split) right.push_back(I[j]);
    }
    for (size_t j = 0; j < I.size(); ++j)
      if (Z[j] == split) (left.size() < right.size() ? left : right).push_back(I[j]);
    rec(2 * i + 1, left);
    rec(2 * i + 2, right);
  };
  std::vector<int> all((size_t)m);
  for (int64_t i = 0; i < m; ++i) all[(size_t)i] = (int)i;
  rec(0, all);
}

// C: nb + 1 entries; I (C[nb] entries) written when non-null.
void oracle_eytzinger_wn_tree(const int32_t* E, const int32_t* leaf, int64_t nb, int canonical,
                              int32_t* C, int32_t* I) {
  std::vector<std::vector<int>> vI((size_t)nb);
  for (int64_t r = 0; r < nb; ++r) {
    if (leaf[r] != -1) continue;
    std::unordered_map<int, int> count;
    std::vector<int64_t> stack{r};
    while (!stack.empty()) {
      const int64_t i = stack.back();
      stack.pop_back();
      if (leaf[i] >= 0) {
        count[E[2 * (int64_t)leaf[i]]] += 1;
        count[E[2 * (int64_t)leaf[i] + 1]] -= 1;
      } else {
        stack.push_back(2 * i + 2);
        stack.push_back(2 * i + 1);
      }
    }
    std::vector<int> pos, neg;
    for (const auto& kv : count)
      for (int c = 0; c < std::abs(kv.second); ++c) (kv.second > 0 ? pos : neg).push_back(kv.first);
    if (canonical) {
      std::sort(pos.begin(), pos.end());
      std::sort(neg.begin(), neg.end());
    }
    for (size_t k = 0; k < pos.size() && k < neg.size(); ++k) {
      vI[(size_t)r].push_back(pos[k]);
      vI[(size_t)r].push_back(neg[k]);
    }
  }
  C[0] = 0;
  for (int64_t r = 0; r < nb; ++r) C[r + 1] = C[r] + (int32_t)vI[(size_t)r].size();
  if (I)
    for (int64_t r = 0; r < nb; ++r)
      std::copy(vI[(size_t)r].begin(), vI[(size_t)r].end(), I + C[r]);
}

// W per query point (P: nP x 2), nthreads host threads over interleaved
// queries.
void oracle_eytzinger_wn(const double* P, int64_t nP, const double* V, const int32_t* E,
                         const double* B1, const double* B2, const int32_t* leaf, int64_t nb,
                         const int32_t* I, const int32_t* C, double* W, int nthreads) {
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::thread::hardware_concurrency();
  if (!nt) nt = 8;
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([=] {
      std::vector<int64_t> stack;
      for (int64_t q = t; q < nP; q += nt) {
        const double px = P[2 * q], py = P[2 * q + 1];
        double wn = 0;
        if (nb > 0) {
          stack.assign(1, 0);
          while (!stack.empty()) {
            const int64_t r = stack.back();
            stack.pop_back();
            if (leaf[r] >= 0) {
              const int e = leaf[r];
              wn += seg_angle(V, E[2 * (int64_t)e], E[2 * (int64_t)e + 1], px, py) / (2.0 * kPi);
              continue;
            }
            if (px < B1[2 * r] || px > B2[2 * r] || py < B1[2 * r + 1] || py > B2[2 * r + 1]) {
              for (int i = C[r]; i < C[r + 1]; i += 2)
                wn += seg_angle(V, I[i], I[i + 1], px, py) / (2.0 * kPi);
              continue;
            }
            stack.push_back(2 * r + 1);
            stack.push_back(2 * r + 2);
          }
        }
        W[q] = wn;
      }
    });
  for (auto& th : pool) th.join();
}

// Direct sum over all segments with the same per-term formula (the value the
// hierarchy reproduces).
void oracle_segments_wn(const double* P, int64_t nP, const double* V, const int32_t* E,
                        int64_t nE, double* W) {
  for (int64_t q = 0; q < nP; ++q) {
    double wn = 0;
    for (int64_t e = 0; e < nE; ++e)
      wn += seg_angle(V, E[2 * e], E[2 * e + 1], P[2 * q], P[2 * q + 1]) / (2.0 * kPi);
    W[q] = wn;
  }
}

}  // extern "C"
