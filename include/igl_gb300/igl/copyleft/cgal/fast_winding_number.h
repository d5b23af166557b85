// Drop-in replacement for include/igl/copyleft/cgal/fast_winding_number.h
// (libigl) running on the GPU through libgwn's C ABI
// (gwn_cloud_winding_number_points): the winding number of an oriented
// point cloud whose areas are estimated from its 21 nearest points
// (octree, knn, point_areas, precompute, evaluate on the device).
//
// Precision: plain FP64, as the reference (define IGL_GB300_WINDING_MIXED
// for the mixed FP32/FP64 walk).
#ifndef IGL_COPYLEFT_CGAL_FAST_WINDING_NUMBER_H
#define IGL_COPYLEFT_CGAL_FAST_WINDING_NUMBER_H

#include <vector>

#include "../../gwn_dropin_detail.h"

#ifndef IGL_GB300_CLOUD_PRECISION
#  ifdef IGL_GB300_WINDING_MIXED
#    define IGL_GB300_CLOUD_PRECISION GWN_MIXED
#  else
#    define IGL_GB300_CLOUD_PRECISION GWN_PLAIN_FP64
#  endif
#endif

namespace igl {
namespace copyleft {
namespace cgal {

/// (include/igl/copyleft/cgal/fast_winding_number.h:20-30)
template <typename DerivedP, typename DerivedN, typename DerivedQ, typename BetaType,
          typename DerivedWN>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                const Eigen::MatrixBase<DerivedN>& N,
                                const Eigen::MatrixBase<DerivedQ>& Q, const int expansion_order,
                                const BetaType beta, Eigen::PlainObjectBase<DerivedWN>& WN) {
  const std::vector<double> p = gwn_detail::rows_f64(P);
  const std::vector<double> n = gwn_detail::rows_f64(N);
  const std::vector<double> q = gwn_detail::rows_f64(Q);
  std::vector<double> w((size_t)Q.rows());
  gwn_detail::check(gwn_cloud_winding_number_points(
      p.data(), n.data(), (int64_t)P.rows(), q.data(), GWN_F64, (int64_t)Q.rows(),
      expansion_order, (double)beta, w.data(), GWN_F64, IGL_GB300_CLOUD_PRECISION, GWN_HOST,
      nullptr));
  WN.resize(Q.rows(), 1);
  for (Eigen::Index i = 0; i < Q.rows(); ++i) WN(i) = (typename DerivedWN::Scalar)w[(size_t)i];
}

/// Order 2, beta 2 (include/igl/copyleft/cgal/fast_winding_number.h:31-36)
template <typename DerivedP, typename DerivedN, typename DerivedQ, typename DerivedWN>
inline void fast_winding_number(const Eigen::MatrixBase<DerivedP>& P,
                                const Eigen::MatrixBase<DerivedN>& N,
                                const Eigen::MatrixBase<DerivedQ>& Q,
                                Eigen::PlainObjectBase<DerivedWN>& WN) {
  fast_winding_number(P, N, Q, 2, 2.0, WN);
}

}  // namespace cgal
}  // namespace copyleft
}  // namespace igl

#endif
