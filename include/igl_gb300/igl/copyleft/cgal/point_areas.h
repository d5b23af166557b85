// Drop-in replacement for include/igl/copyleft/cgal/point_areas.h (libigl)
// running on the GPU through libgwn's C ABI (gwn_point_areas): the two
// igl::copyleft::cgal::point_areas overloads, without CGAL.
//
// Same arguments and outputs: A (#P) the estimated Voronoi area of each
// point from its neighbour list I (#P x k, k <= GWN_POINT_AREAS_MAX_K), T
// (#P x 3) the tangent-plane normal.  The local Delaunay triangulation is
// computed directly per point; for four or more cocircular plane points at
// a point it is not unique, and values there may differ from CGAL's.
#ifndef IGL_COPYLEFT_CGAL_POINT_AREAS_H
#define IGL_COPYLEFT_CGAL_POINT_AREAS_H

#include <vector>

#include "../../gwn_dropin_detail.h"

namespace igl {
namespace copyleft {
namespace cgal {

/// Areas and tangent-plane normals (include/igl/copyleft/cgal/point_areas.h:40-46).
template <typename DerivedP, typename DerivedI, typename DerivedN, typename DerivedA,
          typename DerivedT>
inline void point_areas(const Eigen::MatrixBase<DerivedP>& P, const Eigen::MatrixBase<DerivedI>& I,
                        const Eigen::MatrixBase<DerivedN>& N, Eigen::PlainObjectBase<DerivedA>& A,
                        Eigen::PlainObjectBase<DerivedT>& T) {
  const std::vector<double> p = gwn_detail::rows_f64(P);
  const std::vector<int32_t> idx = gwn_detail::rows_i32(I);
  const std::vector<double> n = gwn_detail::rows_f64(N);
  std::vector<double> a((size_t)P.rows()), t((size_t)P.rows() * 3);
  gwn_detail::check(gwn_point_areas(p.data(), (int64_t)P.rows(), idx.data(), (int64_t)I.cols(),
                                    n.data(), a.data(), t.data(), GWN_HOST, nullptr));
  A.resize(P.rows(), 1);
  T.resize(P.rows(), 3);
  for (Eigen::Index i = 0; i < P.rows(); ++i) {
    A(i) = (typename DerivedA::Scalar)a[(size_t)i];
    for (int d = 0; d < 3; ++d) T(i, d) = (typename DerivedT::Scalar)t[(size_t)i * 3 + d];
  }
}

/// Areas only (include/igl/copyleft/cgal/point_areas.h:47-53).
template <typename DerivedP, typename DerivedI, typename DerivedN, typename DerivedA>
inline void point_areas(const Eigen::MatrixBase<DerivedP>& P, const Eigen::MatrixBase<DerivedI>& I,
                        const Eigen::MatrixBase<DerivedN>& N, Eigen::PlainObjectBase<DerivedA>& A) {
  const std::vector<double> p = gwn_detail::rows_f64(P);
  const std::vector<int32_t> idx = gwn_detail::rows_i32(I);
  const std::vector<double> n = gwn_detail::rows_f64(N);
  std::vector<double> a((size_t)P.rows());
  gwn_detail::check(gwn_point_areas(p.data(), (int64_t)P.rows(), idx.data(), (int64_t)I.cols(),
                                    n.data(), a.data(), nullptr, GWN_HOST, nullptr));
  A.resize(P.rows(), 1);
  for (Eigen::Index i = 0; i < P.rows(); ++i) A(i) = (typename DerivedA::Scalar)a[(size_t)i];
}

}  // namespace cgal
}  // namespace copyleft
}  // namespace igl

#endif
