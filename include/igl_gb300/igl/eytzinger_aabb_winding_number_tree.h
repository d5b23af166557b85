// Drop-in replacement for include/igl/eytzinger_aabb_winding_number_tree.h
// (libigl) running on the GPU through libgwn's C ABI
// (gwn_eytzinger_winding_number_tree).
//
// Same arguments and outputs: for each internal node, the boundary vertices
// of its segments as (positive, negative) pairs in I, node r's pairs in
// I[C(r) : C(r+1)-1].  Positive vertices ascending are paired with negative
// vertices ascending; the reference pairs in unordered_map order.  Any
// pairing gives the same winding number up to rounding.
#ifndef IGL_EYTZINGER_AABB_WINDING_NUMBER_TREE_H
#define IGL_EYTZINGER_AABB_WINDING_NUMBER_TREE_H

#include <vector>

#include "gwn_dropin_detail.h"

namespace igl {

/// Pair lists of an Eytzinger AABB tree of segments
/// (include/igl/eytzinger_aabb_winding_number_tree.h).
template <typename DerivedE, typename Derivedleaf, typename DerivedI, typename DerivedC>
inline void eytzinger_aabb_winding_number_tree(const Eigen::MatrixBase<DerivedE>& E,
                                               const Eigen::MatrixBase<Derivedleaf>& leaf,
                                               Eigen::PlainObjectBase<DerivedI>& I,
                                               Eigen::PlainObjectBase<DerivedC>& C) {
  const std::vector<int32_t> e = gwn_detail::rows_i32(E), lf = gwn_detail::rows_i32(leaf);
  const int64_t nb = (int64_t)lf.size();
  std::vector<int32_t> c((size_t)nb + 1);
  gwn_detail::check(gwn_eytzinger_winding_number_tree(e.data(), (int64_t)E.rows(), lf.data(), nb,
                                                      c.data(), nullptr, GWN_HOST, nullptr));
  std::vector<int32_t> pairs((size_t)c[(size_t)nb]);
  if (!pairs.empty())
    gwn_detail::check(gwn_eytzinger_winding_number_tree(e.data(), (int64_t)E.rows(), lf.data(),
                                                        nb, c.data(), pairs.data(), GWN_HOST,
                                                        nullptr));
  C.resize(nb + 1, 1);
  for (int64_t r = 0; r <= nb; ++r) C(r) = (typename DerivedC::Scalar)c[(size_t)r];
  I.resize((Eigen::Index)pairs.size(), 1);
  for (size_t i = 0; i < pairs.size(); ++i) I((Eigen::Index)i) = (typename DerivedI::Scalar)pairs[i];
}

}  // namespace igl

#endif
