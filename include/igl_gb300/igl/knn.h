// Drop-in replacement for include/igl/knn.h (libigl) running on the GPU
// through libgwn's C ABI (gwn_knn): the two igl::knn overloads (knn.h).
//
// Same arguments and output (I: #P x min(k, #V) point indices, nearest
// first).  The octree arguments are accepted for signature compatibility;
// the GPU builds its own (identical) octree of V.  Equal distances are
// ordered by index; a leaf offers only its first point, as in the
// reference (knn.cpp:121-125).
#ifndef IGL_KNN_H
#define IGL_KNN_H

#include <vector>

#include "gwn_dropin_detail.h"

namespace igl {

/// k nearest points of V for each row of P (include/igl/knn.h).
template <typename DerivedP, typename DerivedV, typename IndexType, typename DerivedCH,
          typename DerivedCN, typename DerivedW, typename DerivedI>
inline void knn(const Eigen::MatrixBase<DerivedP>& P, const Eigen::MatrixBase<DerivedV>& V,
                size_t k, const std::vector<std::vector<IndexType>>& point_indices,
                const Eigen::MatrixBase<DerivedCH>& CH, const Eigen::MatrixBase<DerivedCN>& CN,
                const Eigen::MatrixBase<DerivedW>& W, Eigen::PlainObjectBase<DerivedI>& I) {
  (void)point_indices;
  (void)CH;
  (void)CN;
  (void)W;
  const std::vector<double> p = gwn_detail::rows_f64(P);
  const std::vector<double> v = gwn_detail::rows_f64(V);
  const int64_t cols = (int64_t)V.rows() < (int64_t)k ? (int64_t)V.rows() : (int64_t)k;
  std::vector<int32_t> idx((size_t)(P.rows() * cols));
  gwn_detail::check(gwn_knn(p.data(), (int64_t)P.rows(), v.data(), (int64_t)V.rows(),
                            (int64_t)k, idx.data(), GWN_HOST, nullptr));
  I.resize(P.rows(), cols);
  for (Eigen::Index i = 0; i < P.rows(); ++i)
    for (int64_t j = 0; j < cols; ++j)
      I(i, j) = (typename DerivedI::Scalar)idx[(size_t)(i * cols + j)];
}

/// knn of the points against themselves (include/igl/knn.h).
template <typename DerivedP, typename IndexType, typename DerivedCH, typename DerivedCN,
          typename DerivedW, typename DerivedI>
inline void knn(const Eigen::MatrixBase<DerivedP>& P, size_t k,
                const std::vector<std::vector<IndexType>>& point_indices,
                const Eigen::MatrixBase<DerivedCH>& CH, const Eigen::MatrixBase<DerivedCN>& CN,
                const Eigen::MatrixBase<DerivedW>& W, Eigen::PlainObjectBase<DerivedI>& I) {
  knn(P, P, k, point_indices, CH, CN, W, I);
}

}  // namespace igl

#endif
