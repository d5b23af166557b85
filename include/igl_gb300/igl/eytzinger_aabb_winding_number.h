// Drop-in replacement for include/igl/eytzinger_aabb_winding_number.h
// (libigl) running on the GPU through libgwn's C ABI
// (gwn_eytzinger_winding_number).
//
// The segment overload keeps the reference's signature (one point p, wn
// out) and its arithmetic (plain FP64).  Each such call copies the tree to
// the device, so for many points use the batched overload below (P: #P x 2,
// W: #P), which takes GWN_MIXED or GWN_PLAIN_FP64.  The overload taking a
// std::function primitive (a host callback per leaf) has no GPU form and is
// not provided.
#ifndef IGL_EYTZINGER_AABB_WINDING_NUMBER_H
#define IGL_EYTZINGER_AABB_WINDING_NUMBER_H

#include <vector>

#include "gwn_dropin_detail.h"

namespace igl {
namespace gwn_detail {

template <typename DerivedP, typename DerivedV, typename DerivedE, typename DerivedB,
          typename Derivedleaf, typename DerivedI, typename DerivedC>
std::vector<double> eytzinger_wn(const Eigen::MatrixBase<DerivedP>& P,
                                 const Eigen::MatrixBase<DerivedV>& V,
                                 const Eigen::MatrixBase<DerivedE>& E,
                                 const Eigen::MatrixBase<DerivedB>& B1,
                                 const Eigen::MatrixBase<DerivedB>& B2,
                                 const Eigen::MatrixBase<Derivedleaf>& leaf,
                                 const Eigen::MatrixBase<DerivedI>& I,
                                 const Eigen::MatrixBase<DerivedC>& C, int precision) {
  const std::vector<double> p = rows_f64(P), v = rows_f64(V), b1 = rows_f64(B1),
                            b2 = rows_f64(B2);
  const std::vector<int32_t> e = rows_i32(E), lf = rows_i32(leaf), ii = rows_i32(I),
                             cc = rows_i32(C);
  std::vector<double> w((size_t)P.rows());
  check(gwn_eytzinger_winding_number(p.data(), (int64_t)P.rows(), v.data(), (int64_t)V.rows(),
                                     e.data(), (int64_t)E.rows(), b1.data(), b2.data(), lf.data(),
                                     (int64_t)lf.size(), ii.data(), (int64_t)ii.size(), cc.data(),
                                     w.data(), precision, GWN_HOST, nullptr));
  return w;
}

}  // namespace gwn_detail

/// Winding number of one point with respect to the segments E of V
/// (include/igl/eytzinger_aabb_winding_number.h), plain FP64.
template <typename Derivedp, typename DerivedV, typename DerivedE, typename DerivedB,
          typename Derivedleaf, typename DerivedI, typename DerivedC>
inline void eytzinger_aabb_winding_number(const Eigen::MatrixBase<Derivedp>& p,
                                          const Eigen::MatrixBase<DerivedV>& V,
                                          const Eigen::MatrixBase<DerivedE>& E,
                                          const Eigen::MatrixBase<DerivedB>& B1,
                                          const Eigen::MatrixBase<DerivedB>& B2,
                                          const Eigen::MatrixBase<Derivedleaf>& leaf,
                                          const Eigen::MatrixBase<DerivedI>& I,
                                          const Eigen::MatrixBase<DerivedC>& C,
                                          typename DerivedV::Scalar& wn) {
  wn = (typename DerivedV::Scalar)gwn_detail::eytzinger_wn(p, V, E, B1, B2, leaf, I, C,
                                                          GWN_PLAIN_FP64)[0];
}

/// Batched form: W(i) = the winding number of row i of P (#P x 2).
template <typename DerivedP, typename DerivedV, typename DerivedE, typename DerivedB,
          typename Derivedleaf, typename DerivedI, typename DerivedC, typename DerivedW>
inline void eytzinger_aabb_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                          const Eigen::MatrixBase<DerivedV>& V,
                                          const Eigen::MatrixBase<DerivedE>& E,
                                          const Eigen::MatrixBase<DerivedB>& B1,
                                          const Eigen::MatrixBase<DerivedB>& B2,
                                          const Eigen::MatrixBase<Derivedleaf>& leaf,
                                          const Eigen::MatrixBase<DerivedI>& I,
                                          const Eigen::MatrixBase<DerivedC>& C,
                                          Eigen::PlainObjectBase<DerivedW>& W,
                                          int precision = GWN_MIXED) {
  const std::vector<double> w = gwn_detail::eytzinger_wn(P, V, E, B1, B2, leaf, I, C, precision);
  W.resize(P.rows(), 1);
  for (Eigen::Index i = 0; i < P.rows(); ++i) W(i) = (typename DerivedW::Scalar)w[(size_t)i];
}

}  // namespace igl

#endif
