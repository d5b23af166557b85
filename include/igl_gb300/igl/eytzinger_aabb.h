// Drop-in replacement for include/igl/eytzinger_aabb.h (libigl) running on
// the GPU through libgwn's C ABI (gwn_eytzinger_aabb).
//
// Same arguments and outputs: B1 / B2 (#B x dim node boxes) and leaf (#B:
// the primitive of a leaf, -1 internal, -2 empty) for #B =
// 2^(ceil(log2 #P) + 1) slots.  The split rule is the reference's (median
// box centre along the longest axis, equal centres to the smaller side);
// the median is taken as the order statistics, which is what igl::median
// returns on distinct centre coordinates.  Empty slots' boxes are NaN (the
// reference leaves them uninitialised).
#ifndef IGL_EYTZINGER_AABB_H
#define IGL_EYTZINGER_AABB_H

#include <vector>

#include "gwn_dropin_detail.h"

namespace igl {

/// Eytzinger AABB tree over primitive boxes (include/igl/eytzinger_aabb.h).
template <typename DerivedPB, typename DerivedB, typename Derivedleaf>
inline void eytzinger_aabb(const Eigen::MatrixBase<DerivedPB>& PB1,
                           const Eigen::MatrixBase<DerivedPB>& PB2,
                           Eigen::PlainObjectBase<DerivedB>& B1,
                           Eigen::PlainObjectBase<DerivedB>& B2,
                           Eigen::PlainObjectBase<Derivedleaf>& leaf) {
  const int64_t m = (int64_t)PB1.rows();
  const int dim = (int)PB1.cols();
  const int64_t nb = gwn_eytzinger_slots(m);
  B1.resize(nb, dim);
  B2.resize(nb, dim);
  leaf.resize(nb, 1);
  if (m == 0) return;
  const std::vector<double> p1 = gwn_detail::rows_f64(PB1), p2 = gwn_detail::rows_f64(PB2);
  std::vector<double> b1((size_t)(nb * dim)), b2((size_t)(nb * dim));
  std::vector<int32_t> lf((size_t)nb);
  gwn_detail::check(gwn_eytzinger_aabb(p1.data(), p2.data(), m, dim, b1.data(), b2.data(),
                                       lf.data(), GWN_HOST, nullptr));
  for (int64_t i = 0; i < nb; ++i) {
    leaf(i) = (typename Derivedleaf::Scalar)lf[(size_t)i];
    for (int d = 0; d < dim; ++d) {
      B1(i, d) = (typename DerivedB::Scalar)b1[(size_t)(i * dim + d)];
      B2(i, d) = (typename DerivedB::Scalar)b2[(size_t)(i * dim + d)];
    }
  }
}

}  // namespace igl

#endif
