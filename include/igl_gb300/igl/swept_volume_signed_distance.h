// Drop-in replacement for include/igl/swept_volume_signed_distance.h
// (libigl) running on the GPU through libgwn's C ABI
// (gwn_swept_volume_signed_distance): both overloads, same arguments and
// output.  Each transform is passed as the top 3 x 4 of its matrix.
#ifndef IGL_SWEPT_VOLUME_SIGNED_DISTANCE_H
#define IGL_SWEPT_VOLUME_SIGNED_DISTANCE_H

#include <Eigen/Geometry>
#include <vector>

#include "gwn_dropin_detail.h"
#include "signed_distance.h"

namespace igl {

/// Signed distance at grid points to the volume swept by a mesh under rigid
/// motions, seeded with S0 (include/igl/swept_volume_signed_distance.h).
template <typename DerivedV, typename DerivedF, typename TScalar, typename TAlloc,
          typename DerivedGV, typename Derivedres, typename DerivedS0, typename DerivedS>
inline void swept_volume_signed_distance(
    const Eigen::MatrixBase<DerivedV>& V, const Eigen::MatrixBase<DerivedF>& F,
    const std::vector<Eigen::Transform<TScalar, 3, Eigen::Affine>, TAlloc>& transforms,
    const SignedDistanceType sign_type, const Eigen::MatrixBase<DerivedGV>& GV,
    const Eigen::MatrixBase<Derivedres>& res, const typename DerivedGV::Scalar h,
    const typename DerivedGV::Scalar isolevel, const Eigen::MatrixBase<DerivedS0>& S0,
    Eigen::PlainObjectBase<DerivedS>& S) {
  const std::vector<double> v = gwn_detail::rows_f64(V), gv = gwn_detail::rows_f64(GV);
  const std::vector<int32_t> f = gwn_detail::rows_i32(F);
  std::vector<double> T(transforms.size() * 12);
  for (size_t t = 0; t < transforms.size(); ++t)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) T[t * 12 + (size_t)(i * 4 + j)] = (double)transforms[t](i, j);
  const int32_t r[3] = {(int32_t)res(0), (int32_t)res(1), (int32_t)res(2)};
  std::vector<double> s0((size_t)GV.rows()), s((size_t)GV.rows());
  for (Eigen::Index i = 0; i < GV.rows(); ++i) s0[(size_t)i] = (double)S0(i);
  gwn_detail::check(gwn_swept_volume_signed_distance(
      v.data(), (int64_t)V.rows(), f.data(), (int64_t)F.rows(), T.data(),
      (int64_t)transforms.size(), (int)sign_type, gv.data(), (int64_t)GV.rows(), r, (double)h,
      (double)isolevel, s0.data(), s.data(),
      sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER ? GWN_MIXED : GWN_PLAIN_FP64,
      GWN_HOST, nullptr));
  S.resize(GV.rows(), 1);
  for (Eigen::Index i = 0; i < GV.rows(); ++i) S(i) = (typename DerivedS::Scalar)s[(size_t)i];
}

/// Same, starting from an all-NaN S (include/igl/swept_volume_signed_distance.h).
template <typename DerivedV, typename DerivedF, typename TScalar, typename TAlloc,
          typename DerivedGV, typename Derivedres, typename DerivedS>
inline void swept_volume_signed_distance(
    const Eigen::MatrixBase<DerivedV>& V, const Eigen::MatrixBase<DerivedF>& F,
    const std::vector<Eigen::Transform<TScalar, 3, Eigen::Affine>, TAlloc>& transforms,
    const SignedDistanceType sign_type, const Eigen::MatrixBase<DerivedGV>& GV,
    const Eigen::MatrixBase<Derivedres>& res, const typename DerivedGV::Scalar h,
    const typename DerivedGV::Scalar isolevel, Eigen::PlainObjectBase<DerivedS>& S) {
  const std::vector<double> v = gwn_detail::rows_f64(V), gv = gwn_detail::rows_f64(GV);
  const std::vector<int32_t> f = gwn_detail::rows_i32(F);
  std::vector<double> T(transforms.size() * 12);
  for (size_t t = 0; t < transforms.size(); ++t)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 4; ++j) T[t * 12 + (size_t)(i * 4 + j)] = (double)transforms[t](i, j);
  const int32_t r[3] = {(int32_t)res(0), (int32_t)res(1), (int32_t)res(2)};
  std::vector<double> s((size_t)GV.rows());
  gwn_detail::check(gwn_swept_volume_signed_distance(
      v.data(), (int64_t)V.rows(), f.data(), (int64_t)F.rows(), T.data(),
      (int64_t)transforms.size(), (int)sign_type, gv.data(), (int64_t)GV.rows(), r, (double)h,
      (double)isolevel, nullptr, s.data(),
      sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER ? GWN_MIXED : GWN_PLAIN_FP64,
      GWN_HOST, nullptr));
  S.resize(GV.rows(), 1);
  for (Eigen::Index i = 0; i < GV.rows(); ++i) S(i) = (typename DerivedS::Scalar)s[(size_t)i];
}

}  // namespace igl

#endif
