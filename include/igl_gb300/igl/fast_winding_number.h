// Drop-in replacement for include/igl/fast_winding_number.h (libigl) running
// on the GPU through libgwn's C ABI.  Same overloads and argument meaning:
//   point cloud: precompute (P,N,A,point_indices,CH,order -> CM,R,EC),
//                evaluate (.., CM,R,EC,Q,beta -> WN), one-shot (P,N,A,Q[,order,beta]);
//   triangle soup: FastWindingNumberBVH precompute (V,F,order), evaluate
//                (bvh, accuracy_scale, Q or p), one-shot (V,F,Q).
// As in the reference, CM/R/EC come back with 8 * #cells rows (the reference
// sizes them by CH.size(), fast_winding_number.cpp:34); rows >= #cells hold
// CM = NaN, R = 0, EC = 0 here.
// Precision: the point-cloud path runs in plain FP64 (the reference's
// precision); the soup path runs the mixed FP32/FP64 walk (the reference's
// soup path is FP32).  Override with IGL_GB300_FWN_CLOUD_PRECISION /
// IGL_GB300_FWN_SOUP_PRECISION (GWN_PLAIN_FP64 or GWN_MIXED).
#ifndef IGL_FAST_WINDING_NUMBER
#define IGL_FAST_WINDING_NUMBER

#include <cmath>
#include <limits>
#include <utility>
#include <vector>

#include "gwn_dropin_detail.h"

#ifndef IGL_GB300_FWN_CLOUD_PRECISION
#  define IGL_GB300_FWN_CLOUD_PRECISION GWN_PLAIN_FP64
#endif
#ifndef IGL_GB300_FWN_SOUP_PRECISION
#  define IGL_GB300_FWN_SOUP_PRECISION GWN_MIXED
#endif

namespace igl {
namespace gwn_detail {

template <typename Index, typename DerivedCH>
void csr_of(const std::vector<std::vector<Index>>& point_indices,
            const Eigen::MatrixBase<DerivedCH>& CH, std::vector<int64_t>& off,
            std::vector<int32_t>& idx, std::vector<int32_t>& ch) {
  const size_t nc = point_indices.size();
  off.assign(nc + 1, 0);
  for (size_t c = 0; c < nc; ++c) off[c + 1] = off[c] + (int64_t)point_indices[c].size();
  idx.resize((size_t)off[nc]);
  for (size_t c = 0; c < nc; ++c)
    for (size_t j = 0; j < point_indices[c].size(); ++j)
      idx[(size_t)off[c] + j] = (int32_t)point_indices[c][j];
  ch.resize(nc * 8);
  for (size_t c = 0; c < nc; ++c)
    for (int k = 0; k < 8; ++k) ch[c * 8 + k] = (int32_t)CH((Eigen::Index)c, k);
}

inline int num_terms(int order) { return order == 0 ? 3 : (order == 1 ? 12 : 39); }

}  // namespace gwn_detail

// ---------------------------------------------------------------- cloud --
/// Expansion precompute.  (include/igl/fast_winding_number.h:35-53)
template <typename DerivedP, typename DerivedA, typename DerivedN, typename Index,
          typename DerivedCH, typename DerivedCM, typename DerivedR, typename DerivedEC>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                const Eigen::MatrixBase<DerivedN>& N,
                                const Eigen::MatrixBase<DerivedA>& A,
                                const std::vector<std::vector<Index>>& point_indices,
                                const Eigen::MatrixBase<DerivedCH>& CH, const int expansion_order,
                                Eigen::PlainObjectBase<DerivedCM>& CM,
                                Eigen::PlainObjectBase<DerivedR>& R,
                                Eigen::PlainObjectBase<DerivedEC>& EC) {
  std::vector<int64_t> off;
  std::vector<int32_t> idx, ch;
  gwn_detail::csr_of(point_indices, CH, off, idx, ch);
  const int64_t nc = (int64_t)point_indices.size();
  const int nt = gwn_detail::num_terms(expansion_order);
  const std::vector<double> p = gwn_detail::rows_f64(P), n = gwn_detail::rows_f64(N);
  std::vector<double> a((size_t)A.size());
  for (Eigen::Index i = 0; i < A.size(); ++i) a[(size_t)i] = (double)A(i);
  std::vector<double> cm((size_t)nc * 3), r((size_t)nc), ec((size_t)nc * nt);
  gwn_detail::check(gwn_cloud_precompute_arrays(p.data(), n.data(), a.data(), (int64_t)P.rows(),
                                                off.data(), idx.data(), ch.data(), nc,
                                                expansion_order, cm.data(), r.data(), ec.data()));
  const Eigen::Index m = CH.size();
  CM.resize(m, 3);
  R.resize(m, 1);
  EC.resize(m, nt);
  for (Eigen::Index i = 0; i < m; ++i) {
    const bool in = i < nc;
    for (int d = 0; d < 3; ++d)
      CM(i, d) = in ? cm[(size_t)i * 3 + d] : std::numeric_limits<double>::quiet_NaN();
    R(i) = in ? r[(size_t)i] : 0.0;
    for (int k = 0; k < nt; ++k) EC(i, k) = in ? ec[(size_t)i * nt + k] : 0.0;
  }
}

/// Barnes-Hut evaluation.  (include/igl/fast_winding_number.h:76-99)
template <typename DerivedP, typename DerivedA, typename DerivedN, typename Index,
          typename DerivedCH, typename DerivedCM, typename DerivedR, typename DerivedEC,
          typename DerivedQ, typename BetaType, typename DerivedWN>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                const Eigen::MatrixBase<DerivedN>& N,
                                const Eigen::MatrixBase<DerivedA>& A,
                                const std::vector<std::vector<Index>>& point_indices,
                                const Eigen::MatrixBase<DerivedCH>& CH,
                                const Eigen::MatrixBase<DerivedCM>& CM,
                                const Eigen::MatrixBase<DerivedR>& R,
                                const Eigen::MatrixBase<DerivedEC>& EC,
                                const Eigen::MatrixBase<DerivedQ>& Q, const BetaType beta,
                                Eigen::PlainObjectBase<DerivedWN>& WN) {
  std::vector<int64_t> off;
  std::vector<int32_t> idx, ch;
  gwn_detail::csr_of(point_indices, CH, off, idx, ch);
  const int64_t nc = (int64_t)point_indices.size();
  const int nt = (int)EC.cols();
  const int order = nt == 3 ? 0 : (nt == 12 ? 1 : 2);
  const std::vector<double> p = gwn_detail::rows_f64(P), n = gwn_detail::rows_f64(N),
                            q = gwn_detail::rows_f64(Q);
  std::vector<double> a((size_t)A.size());
  for (Eigen::Index i = 0; i < A.size(); ++i) a[(size_t)i] = (double)A(i);
  std::vector<double> cm((size_t)nc * 3), r((size_t)nc), ec((size_t)nc * nt);
  for (int64_t i = 0; i < nc; ++i) {
    for (int d = 0; d < 3; ++d) cm[(size_t)i * 3 + d] = (double)CM(i, d);
    r[(size_t)i] = (double)R(i);
    for (int k = 0; k < nt; ++k) ec[(size_t)i * nt + k] = (double)EC(i, k);
  }
  std::vector<double> w((size_t)Q.rows());
  gwn_detail::check(gwn_cloud_eval_arrays(p.data(), n.data(), a.data(), (int64_t)P.rows(),
                                          off.data(), idx.data(), ch.data(), nc, cm.data(),
                                          r.data(), ec.data(), order, q.data(), (int64_t)Q.rows(),
                                          (double)beta, w.data(), IGL_GB300_FWN_CLOUD_PRECISION));
  WN.resize(Q.rows(), 1);
  for (Eigen::Index i = 0; i < Q.rows(); ++i) WN(i) = (typename DerivedWN::Scalar)w[(size_t)i];
}

/// One shot: octree, precompute, evaluate (all on the device).
/// (include/igl/fast_winding_number.h:104-131)
template <typename DerivedP, typename DerivedA, typename DerivedN, typename DerivedQ,
          typename BetaType, typename DerivedWN>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                const Eigen::MatrixBase<DerivedN>& N,
                                const Eigen::MatrixBase<DerivedA>& A,
                                const Eigen::MatrixBase<DerivedQ>& Q, const int expansion_order,
                                const BetaType beta, Eigen::PlainObjectBase<DerivedWN>& WN) {
  const std::vector<double> p = gwn_detail::rows_f64(P), n = gwn_detail::rows_f64(N),
                            q = gwn_detail::rows_f64(Q);
  std::vector<double> a((size_t)A.size());
  for (Eigen::Index i = 0; i < A.size(); ++i) a[(size_t)i] = (double)A(i);
  gwn_octree* tree = nullptr;
  gwn_detail::check(gwn_octree_build(p.data(), (int64_t)P.rows(), GWN_HOST, nullptr, &tree));
  gwn_cloud* cloud = nullptr;
  const int rc = gwn_cloud_build(tree, p.data(), n.data(), a.data(), expansion_order, GWN_HOST,
                                 nullptr, &cloud);
  gwn_octree_free(tree);
  gwn_detail::check(rc);
  std::vector<double> w((size_t)Q.rows());
  const int rc2 = gwn_cloud_eval(cloud, (double)beta, q.data(), GWN_F64, (int64_t)Q.rows(),
                                 w.data(), GWN_F64, IGL_GB300_FWN_CLOUD_PRECISION, GWN_HOST,
                                 nullptr);
  gwn_cloud_free(cloud);
  gwn_detail::check(rc2);
  WN.resize(Q.rows(), 1);
  for (Eigen::Index i = 0; i < Q.rows(); ++i) WN(i) = (typename DerivedWN::Scalar)w[(size_t)i];
}

template <typename DerivedP, typename DerivedA, typename DerivedN, typename DerivedQ,
          typename DerivedWN>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                const Eigen::MatrixBase<DerivedN>& N,
                                const Eigen::MatrixBase<DerivedA>& A,
                                const Eigen::MatrixBase<DerivedQ>& Q,
                                Eigen::PlainObjectBase<DerivedWN>& WN) {
  fast_winding_number(P, N, A, Q, 2, 2.0, WN);
}

// ----------------------------------------------------------------- soup --
/// Device-resident soup tree + moments (replaces the reference's struct of
/// the same name, include/igl/fast_winding_number.h:140-147).  Owns a
/// gwn_soup handle; movable, not copyable.
struct FastWindingNumberBVH {
  gwn_soup* handle = nullptr;
  FastWindingNumberBVH() = default;
  FastWindingNumberBVH(const FastWindingNumberBVH&) = delete;
  FastWindingNumberBVH& operator=(const FastWindingNumberBVH&) = delete;
  FastWindingNumberBVH(FastWindingNumberBVH&& o) noexcept : handle(o.handle) { o.handle = nullptr; }
  FastWindingNumberBVH& operator=(FastWindingNumberBVH&& o) noexcept {
    std::swap(handle, o.handle);
    return *this;
  }
  ~FastWindingNumberBVH() {
    if (handle) gwn_soup_free(handle);
  }
};

/// Soup precompute.  (include/igl/fast_winding_number.h:176-181)
template <typename DerivedV, typename DerivedF>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedV>& V,
                                const Eigen::MatrixBase<DerivedF>& F, const int order,
                                FastWindingNumberBVH& fwn_bvh) {
  const std::vector<double> v = gwn_detail::rows_f64(V);
  const std::vector<int32_t> f = gwn_detail::rows_i32(F);
  if (fwn_bvh.handle) {
    gwn_soup_free(fwn_bvh.handle);
    fwn_bvh.handle = nullptr;
  }
  gwn_detail::check(gwn_soup_build(v.data(), (int64_t)V.rows(), f.data(), (int64_t)F.rows(),
                                   order, GWN_HOST, nullptr, &fwn_bvh.handle));
}

/// Soup evaluation of every row of Q.  (include/igl/fast_winding_number.h:189-194)
template <typename DerivedQ, typename DerivedW>
inline void fast_winding_number(const FastWindingNumberBVH& fwn_bvh, const float accuracy_scale,
                                const Eigen::MatrixBase<DerivedQ>& Q,
                                Eigen::PlainObjectBase<DerivedW>& W) {
  const std::vector<double> q = gwn_detail::rows_f64(Q);
  std::vector<double> w((size_t)Q.rows());
  gwn_detail::check(gwn_soup_eval(fwn_bvh.handle, accuracy_scale, q.data(), GWN_F64,
                                  (int64_t)Q.rows(), w.data(), GWN_F64,
                                  IGL_GB300_FWN_SOUP_PRECISION, GWN_HOST, nullptr));
  W.resize(Q.rows(), 1);
  for (Eigen::Index i = 0; i < Q.rows(); ++i) W(i) = (typename DerivedW::Scalar)w[(size_t)i];
}

/// Soup evaluation of one point.  (include/igl/fast_winding_number.h:201-205)
template <typename Derivedp>
inline typename Derivedp::Scalar fast_winding_number(const FastWindingNumberBVH& fwn_bvh,
                                                     const float accuracy_scale,
                                                     const Eigen::MatrixBase<Derivedp>& p) {
  double q[3] = {(double)p(0, 0), (double)p(0, 1), (double)p(0, 2)}, w = 0;
  gwn_detail::check(gwn_soup_eval(fwn_bvh.handle, accuracy_scale, q, GWN_F64, 1, &w, GWN_F64,
                                  IGL_GB300_FWN_SOUP_PRECISION, GWN_HOST, nullptr));
  return (typename Derivedp::Scalar)w;
}

/// Soup one shot with order 2 and accuracy_scale 2.  (include/igl/fast_winding_number.h:157-163)
template <typename DerivedV, typename DerivedF, typename DerivedQ, typename DerivedW>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedV>& V,
                                const Eigen::MatrixBase<DerivedF>& F,
                                const Eigen::MatrixBase<DerivedQ>& Q,
                                Eigen::PlainObjectBase<DerivedW>& W) {
  FastWindingNumberBVH bvh;
  fast_winding_number(V, F, 2, bvh);
  fast_winding_number(bvh, 2.0f, Q, W);
}

}  // namespace igl

#endif
