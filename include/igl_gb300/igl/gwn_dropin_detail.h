// Helpers shared by the igl:: drop-in headers in this directory: marshal
// Eigen inputs of any scalar type and storage order to the contiguous
// row-major buffers libgwn's C ABI takes, and raise on ABI errors.
#ifndef IGL_GB300_GWN_DROPIN_DETAIL_H
#define IGL_GB300_GWN_DROPIN_DETAIL_H

#include <Eigen/Core>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../gwn.h"

namespace igl {
namespace gwn_detail {

inline void check(int rc) {
  if (rc != GWN_OK) throw std::runtime_error(std::string("libgwn: ") + gwn_last_error());
}

template <typename Derived>
std::vector<double> rows_f64(const Eigen::MatrixBase<Derived>& M) {
  std::vector<double> out((size_t)M.rows() * (size_t)M.cols());
  for (Eigen::Index i = 0; i < M.rows(); ++i)
    for (Eigen::Index j = 0; j < M.cols(); ++j)
      out[(size_t)i * (size_t)M.cols() + (size_t)j] = (double)M(i, j);
  return out;
}

template <typename Derived>
std::vector<int32_t> rows_i32(const Eigen::MatrixBase<Derived>& M) {
  std::vector<int32_t> out((size_t)M.rows() * (size_t)M.cols());
  for (Eigen::Index i = 0; i < M.rows(); ++i)
    for (Eigen::Index j = 0; j < M.cols(); ++j)
      out[(size_t)i * (size_t)M.cols() + (size_t)j] = (int32_t)M(i, j);
  return out;
}

}  // namespace gwn_detail
}  // namespace igl

#endif
