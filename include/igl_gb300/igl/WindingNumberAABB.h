// Drop-in replacement for include/igl/WindingNumberAABB.h (libigl) running
// on the GPU through libgwn's C ABI (gwn_wn_aabb_*): the hierarchy of
// boundary caps over a triangle mesh and its exact winding number.
//
// set_mesh / grow / winding_number(p) as in the reference (the tree is built
// by grow(), or at the first evaluation), plus a batched
// winding_number(Q, W).  Evaluation is plain FP64 as in the reference (the
// same walk: a node's cap for a point outside its box); define
// IGL_GB300_WINDING_MIXED for the mixed FP32/FP64 walk (see gwn.h).  The
// value is the exact winding number's up to rounding.  The reference's split
// methods and approximate WindingNumberMethod modes are not provided.
#ifndef IGL_WINDINGNUMBERAABB_H
#define IGL_WINDINGNUMBERAABB_H

#include <vector>

#include "gwn_dropin_detail.h"

#ifndef IGL_GB300_WINDING_PRECISION
#  ifdef IGL_GB300_WINDING_MIXED
#    define IGL_GB300_WINDING_PRECISION GWN_MIXED
#  else
#    define IGL_GB300_WINDING_PRECISION GWN_PLAIN_FP64
#  endif
#endif

namespace igl {

template <typename Scalar, typename Index>
class WindingNumberAABB {
 public:
  using Point = Eigen::Matrix<Scalar, 1, 3>;

  WindingNumberAABB() = default;
  template <typename DerivedV, typename DerivedF>
  WindingNumberAABB(const Eigen::MatrixBase<DerivedV>& V, const Eigen::MatrixBase<DerivedF>& F) {
    set_mesh(V, F);
  }
  WindingNumberAABB(const WindingNumberAABB& o) : v_(o.v_), f_(o.f_) {}
  WindingNumberAABB& operator=(const WindingNumberAABB& o) {
    if (this != &o) {
      release();
      v_ = o.v_;
      f_ = o.f_;
    }
    return *this;
  }
  ~WindingNumberAABB() { release(); }

  /// Initialise the hierarchy to a mesh (V #V x 3, F #F x 3).
  template <typename DerivedV, typename DerivedF>
  void set_mesh(const Eigen::MatrixBase<DerivedV>& V, const Eigen::MatrixBase<DerivedF>& F) {
    release();
    v_ = gwn_detail::rows_f64(V);
    f_ = gwn_detail::rows_i32(F);
  }
  /// Build the tree.
  void grow() const {
    if (h_) return;
    gwn_detail::check(gwn_wn_aabb_build(v_.data(), (int64_t)(v_.size() / 3), f_.data(),
                                        (int64_t)(f_.size() / 3), GWN_HOST, nullptr, &h_));
  }
  /// Winding number of one point.
  template <typename Derivedp>
  Scalar winding_number(const Eigen::MatrixBase<Derivedp>& p) const {
    grow();
    const double q[3] = {(double)p(0), (double)p(1), (double)p(2)};
    double w = 0;
    gwn_detail::check(
        gwn_wn_aabb_eval_precision(h_, q, 1, &w, IGL_GB300_WINDING_PRECISION, GWN_HOST, nullptr));
    return (Scalar)w;
  }
  /// Winding numbers of the rows of Q (#Q x 3) into W.
  template <typename DerivedQ, typename DerivedW>
  void winding_number(const Eigen::MatrixBase<DerivedQ>& Q,
                      Eigen::PlainObjectBase<DerivedW>& W) const {
    grow();
    const std::vector<double> q = gwn_detail::rows_f64(Q);
    std::vector<double> w((size_t)Q.rows());
    gwn_detail::check(gwn_wn_aabb_eval_precision(h_, q.data(), (int64_t)Q.rows(), w.data(),
                                                 IGL_GB300_WINDING_PRECISION, GWN_HOST, nullptr));
    W.resize(Q.rows(), 1);
    for (Eigen::Index i = 0; i < Q.rows(); ++i) W(i) = (typename DerivedW::Scalar)w[(size_t)i];
  }

 private:
  void release() {
    if (h_) gwn_wn_aabb_free(h_);
    h_ = nullptr;
  }
  std::vector<double> v_;
  std::vector<int32_t> f_;
  mutable gwn_wn_aabb* h_ = nullptr;
};

}  // namespace igl

#endif
