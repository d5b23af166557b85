// Drop-in replacement for the main entry points of include/igl/signed_distance.h
// (libigl) running on the GPU through libgwn's C ABI (gwn_signed_distance):
// the SignedDistanceType enum and the two igl::signed_distance(P,V,F,...)
// overloads (signed_distance.h:20-31, 61-90) for 3-D triangle meshes.
//
// Same argument meaning and outputs (S #P, I #P, C #P x 3, N #P x 3 for the
// pseudonormal type).  2-D inputs throw std::runtime_error.  The sign's
// winding number is plain FP64 for WINDING_NUMBER / DEFAULT (as the
// reference) and mixed precision for FAST_WINDING_NUMBER (the reference's is
// FP32); define IGL_GB300_SD_FWN_PRECISION to change the latter.  The other
// functions of libigl's signed_distance.h (the per-point and tree-taking
// helpers) are not declared here.
#ifndef IGL_SIGNED_DISTANCE_H
#define IGL_SIGNED_DISTANCE_H

#include <limits>
#include <stdexcept>

#include "gwn_dropin_detail.h"

#ifndef IGL_GB300_SD_FWN_PRECISION
#  define IGL_GB300_SD_FWN_PRECISION GWN_MIXED
#endif

namespace igl {

enum SignedDistanceType {
  SIGNED_DISTANCE_TYPE_PSEUDONORMAL = 0,
  SIGNED_DISTANCE_TYPE_WINDING_NUMBER = 1,
  SIGNED_DISTANCE_TYPE_DEFAULT = 2,
  SIGNED_DISTANCE_TYPE_UNSIGNED = 3,
  SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER = 4,
  NUM_SIGNED_DISTANCE_TYPE = 5
};

/// Signed distance of each row of P to the triangle mesh (V,F), with the
/// distance bounds of the reference (signed_distance.h:61-71).
template <typename DerivedP, typename DerivedV, typename DerivedF, typename DerivedS,
          typename DerivedI, typename DerivedC, typename DerivedN>
inline void signed_distance(const Eigen::MatrixBase<DerivedP>& P,
                            const Eigen::MatrixBase<DerivedV>& V,
                            const Eigen::MatrixBase<DerivedF>& F,
                            const SignedDistanceType sign_type,
                            const typename DerivedV::Scalar lower_bound,
                            const typename DerivedV::Scalar upper_bound,
                            Eigen::PlainObjectBase<DerivedS>& S,
                            Eigen::PlainObjectBase<DerivedI>& I,
                            Eigen::PlainObjectBase<DerivedC>& C,
                            Eigen::PlainObjectBase<DerivedN>& N) {
  if (P.cols() != 3 || V.cols() != 3 || (F.rows() > 0 && F.cols() != 3))
    throw std::runtime_error("igl::signed_distance (GPU drop-in): 3-D triangle meshes only");
  const std::vector<double> p = gwn_detail::rows_f64(P);
  const std::vector<double> v = gwn_detail::rows_f64(V);
  const std::vector<int32_t> f = gwn_detail::rows_i32(F);
  const int64_t n = (int64_t)P.rows();
  std::vector<double> s((size_t)n), c((size_t)n * 3), nn;
  const bool want_n = sign_type == SIGNED_DISTANCE_TYPE_PSEUDONORMAL;
  if (want_n) nn.resize((size_t)n * 3);
  std::vector<int32_t> idx((size_t)n);
  const int precision = sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER
                            ? IGL_GB300_SD_FWN_PRECISION
                            : GWN_PLAIN_FP64;
  gwn_detail::check(gwn_signed_distance(p.data(), n, v.data(), (int64_t)V.rows(), f.data(),
                                        (int64_t)F.rows(), (int)sign_type, (double)lower_bound,
                                        (double)upper_bound, s.data(), idx.data(), c.data(),
                                        want_n ? nn.data() : nullptr, precision, GWN_HOST,
                                        nullptr));
  S.resize(n, 1);
  I.resize(n, 1);
  C.resize(n, 3);
  if (want_n) N.resize(n, 3);
  for (int64_t i = 0; i < n; ++i) {
    S(i) = (typename DerivedS::Scalar)s[(size_t)i];
    I(i) = (typename DerivedI::Scalar)idx[(size_t)i];
    for (int d = 0; d < 3; ++d) C(i, d) = (typename DerivedC::Scalar)c[(size_t)i * 3 + d];
    if (want_n)
      for (int d = 0; d < 3; ++d) N(i, d) = (typename DerivedN::Scalar)nn[(size_t)i * 3 + d];
  }
}

/// The bound-less overload (signed_distance.h:81-90): lower = numeric_limits
/// min, upper = numeric_limits max, as the reference (signed_distance.cpp:426-440).
template <typename DerivedP, typename DerivedV, typename DerivedF, typename DerivedS,
          typename DerivedI, typename DerivedC, typename DerivedN>
inline void signed_distance(const Eigen::MatrixBase<DerivedP>& P,
                            const Eigen::MatrixBase<DerivedV>& V,
                            const Eigen::MatrixBase<DerivedF>& F,
                            const SignedDistanceType sign_type,
                            Eigen::PlainObjectBase<DerivedS>& S,
                            Eigen::PlainObjectBase<DerivedI>& I,
                            Eigen::PlainObjectBase<DerivedC>& C,
                            Eigen::PlainObjectBase<DerivedN>& N) {
  typedef typename DerivedV::Scalar Scalar;
  signed_distance(P, V, F, sign_type, std::numeric_limits<Scalar>::min(),
                  std::numeric_limits<Scalar>::max(), S, I, C, N);
}

}  // namespace igl

#endif
