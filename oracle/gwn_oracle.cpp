// CPU oracle for the generalized-winding-number path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++ over raw arrays,
// the FP64 algorithms of libigl's winding-number path so that the CUDA library
// can be checked against them.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline / reference arm may load it.  The product library
// (libgwn.so) never links or calls anything in this directory.
//
// Every function cites the reference file:line it follows (paths relative to
// the libigl source tree).  Where the reference relies on Eigen expression
// evaluation order that cannot be reproduced without Eigen, the order chosen
// here is stated; such differences are at the rounding level only.
//
// Arrays are row-major: V[i*3+d], F[f*3+c], P[i*3+d], EC[c*39+k].

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

namespace {

const double kPi = 3.1415926535897932384626433832795;  // include/igl/PI.h

// ---------------------------------------------------------------------------
// Host threading: static slicing over std::thread, the scheme of
// include/igl/parallel_for.h:122-204 (slice = round((n+1)/nthreads), serial
// below min_parallel) with the thread count rule of
// include/igl/default_num_threads.cpp:14-66 (IGL_NUM_THREADS, then hardware).
// ---------------------------------------------------------------------------
unsigned oracle_threads(int requested) {
  if (requested > 0) return (unsigned)requested;
  if (const char* s = std::getenv("IGL_NUM_THREADS")) {
    int v = std::atoi(s);
    if (v > 0) return (unsigned)v;
  }
  unsigned hw = std::thread::hardware_concurrency();
  return hw ? hw : 8u;
}

template <typename Fn>
void static_parallel_for(int64_t n, Fn fn, int64_t min_parallel, int requested) {
  if (n <= 0) return;
  const unsigned nt = oracle_threads(requested);
  if (n < min_parallel || nt <= 1) {
    for (int64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  int64_t slice = std::max<int64_t>((int64_t)std::llround((n + 1) / (double)nt), 1);
  std::vector<std::thread> pool;
  int64_t i1 = 0, i2 = std::min<int64_t>(slice, n);
  unsigned t = 0;
  for (; t + 1 < nt && i1 < n; ++t) {
    pool.emplace_back([=, &fn] { for (int64_t k = i1; k < i2; ++k) fn(k); });
    i1 = i2;
    i2 = std::min<int64_t>(i2 + slice, n);
  }
  if (i1 < n) pool.emplace_back([=, &fn] { for (int64_t k = i1; k < n; ++k) fn(k); });
  for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// X3: solid angle of one triangle / 4pi, include/igl/solid_angle.cpp:16-54.
// Corner vectors v_i = corner_i - p (:21-26); row norms (:27, evaluated here
// as x*x + (y*y + z*z), Eigen's unrolled 3-term reduction); determinant in
// the 6-term order of :30-36; pairwise dots of :38-47; atan2 / (2 pi) (:50-54).
// ---------------------------------------------------------------------------
inline double solid_angle(const double* A, const double* B, const double* C,
                          const double* P) {
  double v[3][3];
  for (int d = 0; d < 3; ++d) {
    v[0][d] = A[d] - P[d];
    v[1][d] = B[d] - P[d];
    v[2][d] = C[d] - P[d];
  }
  double vl[3];
  for (int r = 0; r < 3; ++r)
    vl[r] = std::sqrt(v[r][0] * v[r][0] + (v[r][1] * v[r][1] + v[r][2] * v[r][2]));
  const double detf = v[0][0] * v[1][1] * v[2][2] + v[1][0] * v[2][1] * v[0][2] +
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
  return std::atan2(detf, vl[0] * vl[1] * vl[2] + dp0 * vl[0] + dp1 * vl[1] + dp2 * vl[2]) /
         (2. * kPi);
}

// X4: 2D signed angle / 2pi of edge (A,B) seen from P,
// include/igl/signed_angle.cpp:14-45.
inline double signed_angle(const double* A, const double* B, const double* P) {
  double a[2], b[2], al = 0, bl = 0;
  for (int i = 0; i < 2; ++i) {
    a[i] = P[i] - A[i];
    b[i] = P[i] - B[i];
    al += a[i] * a[i];
    bl += b[i] * b[i];
  }
  al = std::sqrt(al);
  bl = std::sqrt(bl);
  for (int i = 0; i < 2; ++i) {
    if (al != 0) a[i] /= al;
    if (bl != 0) b[i] /= bl;
  }
  return -std::atan2(b[0] * a[1] - b[1] * a[0], b[0] * a[0] + b[1] * a[1]) / (2. * kPi);
}

// ---------------------------------------------------------------------------
// Octree (O1), include/igl/octree.cpp:5-170, restated with an explicit stack
// so that degenerate inputs (duplicate points recurse to MAX_DEPTH = 30000,
// :16, :98) do not overflow the call stack.  The stack pops cells in the
// same depth-first pre-order as the recursive helper (children 0..7 in
// order), so child ids m..m+7 are handed out in the same order (:100-131).
// ---------------------------------------------------------------------------
struct Octree {
  std::vector<std::vector<int32_t>> pi;
  std::vector<int32_t> ch;   // ncells * 8
  std::vector<double> cn;    // ncells * 3
  std::vector<double> w;     // ncells
};

void build_octree(const double* P, int64_t n, Octree& o) {
  const int MAX_DEPTH = 30000;
  o.pi.clear();
  o.ch.clear();
  o.cn.clear();
  o.w.clear();
  {
    std::vector<int32_t> all((size_t)n);
    for (int64_t i = 0; i < n; ++i) all[(size_t)i] = (int32_t)i;
    o.pi.emplace_back(std::move(all));
  }
  for (int k = 0; k < 8; ++k) o.ch.push_back(-1);
  // Root cube from the points' AABB (:142-153).  An empty cloud has no AABB
  // in the reference (Eigen min/max of zero rows); the root is then given
  // centre 0 and width 0 here.
  double mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
  if (n > 0) {
    for (int d = 0; d < 3; ++d) mn[d] = mx[d] = P[d];
    for (int64_t i = 1; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
        mn[d] = std::min(mn[d], P[i * 3 + d]);
        mx[d] = std::max(mx[d], P[i * 3 + d]);
      }
  }
  double width = mx[0] - mn[0];
  for (int d = 1; d < 3; ++d) width = std::max(width, mx[d] - mn[d]);
  for (int d = 0; d < 3; ++d) o.cn.push_back((mn[d] + mx[d]) / 2.0);
  o.w.push_back(width);
  int32_t m = 1;

  struct Item { int32_t index; int depth; };
  std::vector<Item> stack;
  stack.push_back({0, 0});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    const int32_t index = it.index;
    if (!(o.pi[(size_t)index].size() > 1 && it.depth < MAX_DEPTH)) continue;
    for (int k = 0; k < 8; ++k) o.ch[(size_t)index * 8 + k] = m + k;
    const double h = o.w[(size_t)index] / 2;
    const double c[3] = {o.cn[(size_t)index * 3 + 0], o.cn[(size_t)index * 3 + 1],
                         o.cn[(size_t)index * 3 + 2]};
    const double hh = h / 2;  // translate_center(curr_center, h/2, i), :104-113
    for (int i = 0; i < 8; ++i) {
      for (int k = 0; k < 8; ++k) o.ch.push_back(-1);
      o.pi.emplace_back();
      // :59-81: x positive for odd i, y positive for i in {2,3,6,7}, z for i>3
      const double cx = (i % 2) ? hh : -hh;
      const double cy = (i == 2 || i == 3 || i == 6 || i == 7) ? hh : -hh;
      const double cz = (i > 3) ? hh : -hh;
      o.cn.push_back(c[0] + cx);
      o.cn.push_back(c[1] + cy);
      o.cn.push_back(c[2] + cz);
      o.w.push_back(h);
    }
    // Stable split into octants, bits x=1,y=2,z=4 via >= centre (:32-53, :117-122)
    const std::vector<int32_t>& mine = o.pi[(size_t)index];
    for (size_t j = 0; j < mine.size(); ++j) {
      const int32_t p = mine[j];
      int oct = 0;
      if (P[(size_t)p * 3 + 0] >= c[0]) oct += 1;
      if (P[(size_t)p * 3 + 1] >= c[1]) oct += 2;
      if (P[(size_t)p * 3 + 2] >= c[2]) oct += 4;
      o.pi[(size_t)(m + oct)].push_back(p);
    }
    const int32_t first = m;
    m += 8;
    for (int i = 7; i >= 0; --i) stack.push_back({first + i, it.depth + 1});
  }
}

// ---------------------------------------------------------------------------
// Cloud precompute (C1), src/.../fast_winding_number.cpp:17-124, over one
// cell list.  CM = area-weighted mass centre (:57-75, NaN for an empty cell),
// EC[0:3] = sum A n (:64), R = max |p - CM| (:80-88), EC[3:12] column-major
// A (p-CM) n^T (:92-97), EC[12+9k:21+9k] column-major 0.5 (p-CM)_k A (p-CM) n^T
// (:100-107).  Products are associated as ((0.5*p_k) * ((A*p_u) * n_v)).
// ---------------------------------------------------------------------------
struct CloudArrays {
  const double* P;
  const double* N;
  const double* A;
  const int64_t* pi_off;
  const int32_t* pi_idx;
  const int32_t* CH;
  int64_t ncells;
};

void precompute_cell(const CloudArrays& c, int64_t index, int num_terms, double* CM,
                     double* R, double* EC) {
  double mc[3] = {0, 0, 0}, ze[3] = {0, 0, 0}, area = 0.0;
  const int64_t b = c.pi_off[index], e = c.pi_off[index + 1];
  for (int64_t j = b; j < e; ++j) {
    const int64_t p = c.pi_idx[j];
    const double a = c.A[p];
    area += a;
    for (int d = 0; d < 3; ++d) {
      mc[d] += a * c.P[p * 3 + d];
      ze[d] += a * c.N[p * 3 + d];
    }
  }
  if (e > b) {
    for (int d = 0; d < 3; ++d) mc[d] = mc[d] / area;
  } else {
    for (int d = 0; d < 3; ++d) mc[d] = std::numeric_limits<double>::quiet_NaN();
  }
  double* ec = EC + index * num_terms;
  for (int k = 0; k < num_terms; ++k) ec[k] = 0.0;
  for (int d = 0; d < 3; ++d) {
    CM[index * 3 + d] = mc[d];
    ec[d] = ze[d];
  }
  double max_norm = 0;
  for (int64_t j = b; j < e; ++j) {
    const int64_t p = c.pi_idx[j];
    const double a = c.A[p];
    double pt[3];
    for (int d = 0; d < 3; ++d) pt[d] = c.P[p * 3 + d] - mc[d];
    const double nrm = std::sqrt(pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]);
    if (nrm > max_norm) max_norm = nrm;
    if (num_terms >= 12) {
      for (int v = 0; v < 3; ++v)
        for (int u = 0; u < 3; ++u) ec[3 + u + 3 * v] += (a * pt[u]) * c.N[p * 3 + v];
    }
    if (num_terms == 39) {
      for (int k = 0; k < 3; ++k) {
        const double s = 0.5 * pt[k];
        for (int v = 0; v < 3; ++v)
          for (int u = 0; u < 3; ++u)
            ec[12 + 9 * k + u + 3 * v] += s * ((a * pt[u]) * c.N[p * 3 + v]);
      }
    }
  }
  R[index] = max_norm;
}

// Cloud evaluation (C2), fast_winding_number.cpp:126-311.
struct CloudEval {
  CloudArrays c;
  const double* CM;
  const double* R;
  const double* EC;
  int num_terms;
  double beta;
};

const double kPi4 = 4.0 * kPi;  // :149

// direct_eval, :159-172: 0.5 when the point coincides with the query.
inline double direct_eval(const double loc[3], const double an[3]) {
  const double ln = std::sqrt(loc[0] * loc[0] + loc[1] * loc[1] + loc[2] * loc[2]);
  if (ln == 0) return 0.5;
  return (loc[0] * an[0] + loc[1] * an[1] + loc[2] * an[2]) / (kPi4 * (ln * ln * ln));
}

// expansion_eval, :174-228.
inline double expansion_eval(const double loc[3], const double* ec, int num_terms) {
  double wn = direct_eval(loc, ec);
  const double r = std::sqrt(loc[0] * loc[0] + loc[1] * loc[1] + loc[2] * loc[2]);
  if (num_terms > 3) {
    const double r3 = kPi4 * r * r * r;
    const double r5 = r3 * r * r;
    const double d = 1.0 / r3;
    const double s = -3.0 / r5;
    double acc = 0;
    for (int v = 0; v < 3; ++v)
      for (int u = 0; u < 3; ++u) {
        double sd = (loc[u] * loc[v]) * s;
        if (u == v) sd += d;
        acc += sd * ec[3 + u + 3 * v];
      }
    wn += acc;
    if (num_terms > 12) {
      const double r7 = r5 * r * r;
      for (int i = 0; i < 3; ++i) {
        double acc3 = 0;
        for (int v = 0; v < 3; ++v)
          for (int u = 0; u < 3; ++u) {
            double rcd = 0;
            if (u == v) rcd += loc[i];
            if (u == i) rcd += loc[v];
            if (v == i) rcd += loc[u];
            const double ltl = loc[u] * (loc[v] / r7);
            const double td = 15.0 * loc[i] * ltl + s * rcd;
            acc3 += td * ec[12 + i * 9 + u + 3 * v];
          }
        wn += acc3;
      }
    }
  }
  return wn;
}

inline double leaf_direct(const CloudEval& E, int64_t index, const double q[3]) {
  double wn = 0;
  for (int64_t j = E.c.pi_off[index]; j < E.c.pi_off[index + 1]; ++j) {
    const int64_t p = E.c.pi_idx[j];
    double loc[3], an[3];
    for (int d = 0; d < 3; ++d) {
      loc[d] = E.c.P[p * 3 + d] - q[d];
      an[d] = E.c.N[p * 3 + d] * E.c.A[p];
    }
    wn += direct_eval(loc, an);
  }
  return wn;
}

// Level-synchronous near-list descent of helper (:233-292).  The result is
// s_0 + (s_1 + (... + s_L)), s_l summed in list order, as the recursion does.
double cloud_query(const CloudEval& E, const double q[3]) {
  std::vector<int32_t> near{0}, next;
  std::vector<double> level_sums;
  while (!near.empty()) {
    double wn = 0;
    next.clear();
    for (int32_t index : near) {
      if (E.c.CH[(int64_t)index * 8] == -1) {
        wn += leaf_direct(E, index, q);
      } else {
        for (int ch = 0; ch < 8; ++ch) {
          const int32_t ci = E.c.CH[(int64_t)index * 8 + ch];
          if (E.c.pi_off[ci + 1] - E.c.pi_off[ci] > 0) {
            double loc[3];
            for (int d = 0; d < 3; ++d) loc[d] = E.CM[(int64_t)ci * 3 + d] - q[d];
            const double nrm = std::sqrt(loc[0] * loc[0] + loc[1] * loc[1] + loc[2] * loc[2]);
            if (nrm > E.beta * E.R[ci]) {
              if (E.c.CH[(int64_t)ci * 8] == -1)
                wn += leaf_direct(E, ci, q);
              else
                wn += expansion_eval(loc, E.EC + (int64_t)ci * E.num_terms, E.num_terms);
            } else {
              next.push_back(ci);
            }
          }
        }
      }
    }
    level_sums.push_back(wn);
    std::swap(near, next);
  }
  double acc = 0;
  for (size_t l = level_sums.size(); l-- > 0;) acc = level_sums[l] + acc;
  return acc;
}

}  // namespace

extern "C" {

// Exact winding number by brute force: X1/X2, winding_number.cpp:61-93 per
// query, over the whole face list.  dim = 3 (triangles, solid_angle) or
// dim = 2 (edges, signed_angle).  The reference's hierarchical dispatch
// (winding_number.cpp:40-53) returns the same value up to rounding.
int oracle_winding_number(const double* V, int64_t nV, const int32_t* F, int64_t nF,
                          int dim, const double* O, int64_t nO, double* W,
                          int nthreads) {
  (void)nV;
  if (dim != 2 && dim != 3) return 1;
  static_parallel_for(
      nO,
      [&](int64_t o) {
        double w = 0;
        const double* p = O + o * dim;
        for (int64_t f = 0; f < nF; ++f) {
          if (dim == 3)
            w += solid_angle(V + (int64_t)F[f * 3 + 0] * 3, V + (int64_t)F[f * 3 + 1] * 3,
                             V + (int64_t)F[f * 3 + 2] * 3, p);
          else
            w += signed_angle(V + (int64_t)F[f * 2 + 0] * 2, V + (int64_t)F[f * 2 + 1] * 2,
                              p);
        }
        W[o] = w;
      },
      10000, nthreads);
  return 0;
}

// Single-triangle term, exposed so tests can probe edge cases directly.
double oracle_solid_angle(const double* A, const double* B, const double* C,
                          const double* P) {
  return solid_angle(A, B, C, P);
}

// Octree: build into an opaque handle, query sizes, export CSR + arrays.
void* oracle_octree_build(const double* P, int64_t n) {
  Octree* o = new Octree();
  build_octree(P, n, *o);
  return o;
}
void oracle_octree_sizes(void* h, int64_t* ncells, int64_t* nindices) {
  Octree* o = (Octree*)h;
  *ncells = (int64_t)o->pi.size();
  int64_t t = 0;
  for (auto& v : o->pi) t += (int64_t)v.size();
  *nindices = t;
}
void oracle_octree_export(void* h, int64_t* pi_off, int32_t* pi_idx, int32_t* CH,
                          double* CN, double* W) {
  Octree* o = (Octree*)h;
  int64_t t = 0;
  for (size_t c = 0; c < o->pi.size(); ++c) {
    pi_off[c] = t;
    for (int32_t p : o->pi[c]) pi_idx[t++] = p;
  }
  pi_off[o->pi.size()] = t;
  std::memcpy(CH, o->ch.data(), o->ch.size() * sizeof(int32_t));
  std::memcpy(CN, o->cn.data(), o->cn.size() * sizeof(double));
  std::memcpy(W, o->w.data(), o->w.size() * sizeof(double));
}
void oracle_octree_free(void* h) { delete (Octree*)h; }

// Cloud precompute over ncells cells (rows >= ncells of the reference's
// 8*ncells-row outputs are not produced here).
int oracle_cloud_precompute(const double* P, const double* N, const double* A,
                            const int64_t* pi_off, const int32_t* pi_idx,
                            const int32_t* CH, int64_t ncells, int order, double* CM,
                            double* R, double* EC, int nthreads) {
  if (order < 0 || order > 2) return 1;
  const int num_terms = order == 0 ? 3 : (order == 1 ? 12 : 39);
  CloudArrays c{P, N, A, pi_off, pi_idx, CH, ncells};
  static_parallel_for(
      ncells, [&](int64_t i) { precompute_cell(c, i, num_terms, CM, R, EC); }, 1024,
      nthreads);
  return 0;
}

// Cloud evaluation.  beta > 0: Barnes-Hut (:294-299); beta <= 0: direct sum
// over all points (:300-310).
int oracle_cloud_eval(const double* P, const double* N, const double* A, int64_t nP,
                      const int64_t* pi_off, const int32_t* pi_idx, const int32_t* CH,
                      int64_t ncells, const double* CM, const double* R,
                      const double* EC, int order, const double* Q, int64_t nQ,
                      double beta, double* W, int nthreads) {
  if (order < 0 || order > 2) return 1;
  const int num_terms = order == 0 ? 3 : (order == 1 ? 12 : 39);
  CloudEval E{{P, N, A, pi_off, pi_idx, CH, ncells}, CM, R, EC, num_terms, beta};
  if (beta > 0) {
    static_parallel_for(nQ, [&](int64_t i) { W[i] = cloud_query(E, Q + i * 3); }, 1000,
                        nthreads);
  } else {
    static_parallel_for(
        nQ,
        [&](int64_t i) {
          double wn = 0;
          for (int64_t j = 0; j < nP; ++j) {
            double loc[3], an[3];
            for (int d = 0; d < 3; ++d) {
              loc[d] = P[j * 3 + d] - Q[i * 3 + d];
              an[d] = N[j * 3 + d] * A[j];
            }
            wn += direct_eval(loc, an);
          }
          W[i] = wn;
        },
        1000, nthreads);
  }
  return 0;
}

int oracle_num_threads(int requested) { return (int)oracle_threads(requested); }

}  // extern "C"
