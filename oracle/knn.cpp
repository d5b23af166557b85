// CPU restatement of igl::knn (include/igl/knn.cpp:24-136) over octree
// arrays (CSR point_indices, CH, CN, W as igl::octree gives them).
//
// TEST INFRASTRUCTURE ONLY (see gwn_oracle.cpp).
//
// The reference's best-first search: one std::priority_queue of point ids
// (< #V) and cell ids (+ #V), ordered by distance (points: the norm of
// V(j) - p; cells: the distance to the cube of half-width W around CN, the
// reference's distance_to_cube, :56-70); pop until k points came out.  When
// #V <= k all points are sorted by distance (:41-51; igl::sort ascending,
// ties by index).  A leaf pushes only the first point of its list (:121-125),
// so duplicates beyond the first are never returned; where the reference's
// loop would then pop an empty queue (fewer reachable points than k), the
// row is filled with -1.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <queue>
#include <thread>
#include <vector>

extern "C" {

int oracle_knn(const double* P, int64_t nP, const double* V, int64_t nV, int64_t k,
               const int64_t* pi_off, const int32_t* pi_idx, const int32_t* CH,
               const double* CN, const double* W, int32_t* I, int nthreads) {
  const int64_t cols = std::min(nV, k);
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::thread::hardware_concurrency();
  if (!nt) nt = 8;
  std::vector<std::thread> pool;
  for (unsigned th = 0; th < nt; ++th)
    pool.emplace_back([=] {
      for (int64_t i = th; i < nP; i += nt) {
        const double* p = P + i * 3;
        auto pdist = [&](int64_t j) {
          const double dx = V[j * 3] - p[0], dy = V[j * 3 + 1] - p[1], dz = V[j * 3 + 2] - p[2];
          return std::sqrt(dx * dx + dy * dy + dz * dz);
        };
        if (nV <= k) {
          std::vector<int> idx((size_t)nV);
          std::iota(idx.begin(), idx.end(), 0);
          std::stable_sort(idx.begin(), idx.end(),
                           [&](int a, int b) { return pdist(a) < pdist(b); });
          for (int64_t j = 0; j < nV; ++j) I[i * cols + j] = idx[(size_t)j];
          continue;
        }
        auto cdist = [&](int64_t c) {  // distance_to_cube(point, CN(c), W(c))
          double s = 0;
          for (int d = 0; d < 3; ++d) {
            const double t = (p[d] - CN[c * 3 + d]) / W[c];
            const double e = std::max(std::abs(t) - 1.0, 0.0);
            s += e * e;
          }
          return W[c] * std::sqrt(s);
        };
        auto dist = [&](int64_t x) { return x < nV ? pdist(x) : cdist(x - nV); };
        auto cmp = [&](int64_t a, int64_t b) { return dist(a) > dist(b); };
        std::priority_queue<int64_t, std::vector<int64_t>, decltype(cmp)> q(cmp);
        q.push(nV);
        int64_t found = 0;
        while (found < k) {
          if (q.empty()) {  // fewer reachable points than k (duplicates): -1
            for (; found < k; ++found) I[i * cols + found] = -1;
            break;
          }
          const int64_t x = q.top();
          q.pop();
          if (x < nV) {
            I[i * cols + found++] = (int32_t)x;
          } else {
            const int64_t c = x - nV;
            if (CH[c * 8] == -1) {
              if (pi_off[c + 1] > pi_off[c]) q.push(pi_idx[pi_off[c]]);
            } else {
              for (int j = 0; j < 8; ++j) q.push(CH[c * 8 + j] + nV);
            }
          }
        }
      }
    });
  for (auto& t : pool) t.join();
  return 0;
}

}  // extern "C"
