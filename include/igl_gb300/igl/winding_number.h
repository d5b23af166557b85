// Drop-in replacement for include/igl/winding_number.h (libigl) running on the
// GPU through libgwn's C ABI (gwn_winding_number).  Same signatures, same
// argument meaning; for 3-D meshes of at least 4096 triangles and 1024
// points the GPU walks the reference's cap hierarchy (winding_number.cpp:
// 40-53), otherwise it sums every element's solid angle (the same value up
// to rounding).
//
// Precision: plain FP64, as the reference (set IGL_GB300_WINDING_MIXED to use
// the mixed FP32/FP64 path).
#ifndef IGL_WINDING_NUMBER_H
#define IGL_WINDING_NUMBER_H

#include "gwn_dropin_detail.h"

#ifndef IGL_GB300_WINDING_PRECISION
#  ifdef IGL_GB300_WINDING_MIXED
#    define IGL_GB300_WINDING_PRECISION GWN_MIXED
#  else
#    define IGL_GB300_WINDING_PRECISION GWN_PLAIN_FP64
#  endif
#endif

namespace igl {

/// Generalized winding number of each row of O w.r.t. (V,F): F.cols()==3
/// triangles in 3D, F.cols()==2 edges in 2D.  (include/igl/winding_number.h:35-44)
template <typename DerivedV, typename DerivedF, typename DerivedO, typename DerivedW>
inline void winding_number(const Eigen::MatrixBase<DerivedV>& V,
                           const Eigen::MatrixBase<DerivedF>& F,
                           const Eigen::MatrixBase<DerivedO>& O,
                           Eigen::PlainObjectBase<DerivedW>& W) {
  W.resize(O.rows(), 1);
  const int dim = (int)F.cols();
  const std::vector<double> v = gwn_detail::rows_f64(V);
  const std::vector<int32_t> f = gwn_detail::rows_i32(F);
  const std::vector<double> o = gwn_detail::rows_f64(O);
  std::vector<double> w((size_t)O.rows());
  gwn_detail::check(gwn_winding_number(v.data(), (int64_t)V.rows(), dim, f.data(),
                                       (int64_t)F.rows(), o.data(), GWN_F64, (int64_t)O.rows(),
                                       w.data(), GWN_F64, IGL_GB300_WINDING_PRECISION, GWN_HOST,
                                       nullptr));
  for (Eigen::Index i = 0; i < O.rows(); ++i) W(i) = (typename DerivedW::Scalar)w[(size_t)i];
}

/// Winding number of a single point p.  (include/igl/winding_number.h:53-60)
template <typename DerivedV, typename DerivedF, typename Derivedp>
inline typename DerivedV::Scalar winding_number(const Eigen::MatrixBase<DerivedV>& V,
                                                const Eigen::MatrixBase<DerivedF>& F,
                                                const Eigen::MatrixBase<Derivedp>& p) {
  const int dim = (int)F.cols();
  const std::vector<double> v = gwn_detail::rows_f64(V);
  const std::vector<int32_t> f = gwn_detail::rows_i32(F);
  double q[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) q[d] = (double)p(d);
  double w = 0;
  gwn_detail::check(gwn_winding_number(v.data(), (int64_t)V.rows(), dim, f.data(),
                                       (int64_t)F.rows(), q, GWN_F64, 1, &w, GWN_F64,
                                       IGL_GB300_WINDING_PRECISION, GWN_HOST, nullptr));
  return (typename DerivedV::Scalar)w;
}

}  // namespace igl

#endif
