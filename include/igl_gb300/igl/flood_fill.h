// Drop-in replacement for include/igl/flood_fill.h (libigl) running on the
// GPU through libgwn's C ABI (gwn_flood_fill): the NaN entries of S
// (res(0) x res(1) x res(2), x fastest) take the values the reference's scan
// gives them.
#ifndef IGL_FLOOD_FILL_H
#define IGL_FLOOD_FILL_H

#include <vector>

#include "gwn_dropin_detail.h"

namespace igl {

/// Flood fill of a grid of values with NaN gaps (include/igl/flood_fill.h).
template <typename Derivedres, typename DerivedS>
inline void flood_fill(const Eigen::MatrixBase<Derivedres>& res,
                       Eigen::PlainObjectBase<DerivedS>& S) {
  const int32_t r[3] = {(int32_t)res(0), (int32_t)res(1), (int32_t)res(2)};
  std::vector<double> s((size_t)S.size());
  for (Eigen::Index i = 0; i < S.size(); ++i) s[(size_t)i] = (double)S(i);
  gwn_detail::check(gwn_flood_fill(r, s.data(), GWN_HOST, nullptr));
  for (Eigen::Index i = 0; i < S.size(); ++i) S(i) = (typename DerivedS::Scalar)s[(size_t)i];
}

}  // namespace igl

#endif
