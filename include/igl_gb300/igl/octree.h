// Drop-in replacement for include/igl/octree.h (libigl): the octree is built
// on the GPU (gwn_octree_build) and is bit-exact with the reference's
// (same point_indices, CH, CN, W).
#ifndef IGL_OCTREE
#define IGL_OCTREE

#include <vector>

#include "gwn_dropin_detail.h"

namespace igl {

/// (include/igl/octree.h:44-50)
template <typename DerivedP, typename IndexType, typename DerivedCH, typename DerivedCN,
          typename DerivedW>
inline void octree(const Eigen::MatrixBase<DerivedP>& P,
                   std::vector<std::vector<IndexType>>& point_indices,
                   Eigen::PlainObjectBase<DerivedCH>& CH, Eigen::PlainObjectBase<DerivedCN>& CN,
                   Eigen::PlainObjectBase<DerivedW>& W) {
  const std::vector<double> p = gwn_detail::rows_f64(P);
  gwn_octree* t = nullptr;
  gwn_detail::check(gwn_octree_build(p.data(), (int64_t)P.rows(), GWN_HOST, nullptr, &t));
  int64_t nc = 0, ni = 0;
  int32_t md = 0;
  gwn_octree_sizes(t, &nc, &ni, &md);
  std::vector<int64_t> off((size_t)nc + 1);
  std::vector<int32_t> idx((size_t)ni + 1), ch((size_t)nc * 8);
  std::vector<double> cn((size_t)nc * 3), w((size_t)nc);
  const int rc = gwn_octree_export(t, off.data(), idx.data(), ch.data(), cn.data(), w.data(),
                                   GWN_HOST, nullptr);
  gwn_octree_free(t);
  gwn_detail::check(rc);
  // the reference appends to whatever point_indices holds (octree.cpp:136-139);
  // callers pass it empty
  point_indices.clear();
  point_indices.resize((size_t)nc);
  for (int64_t c = 0; c < nc; ++c)
    point_indices[(size_t)c].assign(idx.begin() + off[(size_t)c], idx.begin() + off[(size_t)c + 1]);
  CH.resize(nc, 8);
  CN.resize(nc, 3);
  W.resize(nc, 1);
  for (int64_t c = 0; c < nc; ++c) {
    for (int k = 0; k < 8; ++k) CH(c, k) = ch[(size_t)c * 8 + k];
    for (int d = 0; d < 3; ++d) CN(c, d) = cn[(size_t)c * 3 + d];
    W(c) = w[(size_t)c];
  }
}

}  // namespace igl

#endif
