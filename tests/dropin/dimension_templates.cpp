// Compile-only counterpart of the reference's "signed_distance:
// dimension-templates" case (tests/include/igl/signed_distance.cpp:77-120):
// the drop-in igl::signed_distance overloads instantiate with dynamic and
// fixed-column matrix types for a single triangle.  Its 3-D half only: the
// drop-in refuses 2-D inputs at run time.  Nothing here is run.
#include <limits>

#include <Eigen/Core>
#include <igl/signed_distance.h>

void dimension_templates() {
  Eigen::MatrixXd VX3(3, 3);
  VX3.set({0, 0, 0, 1, 0, 0, 0, 1, 0});
  Eigen::MatrixXi F(1, 3);
  F.set({0, 1, 2});
  Eigen::MatrixX3d V3(3, 3);
  V3.set({0, 0, 0, 1, 0, 0, 0, 1, 0});
  Eigen::MatrixX3i F3(1, 3);
  F3.set({0, 1, 2});
  const Eigen::MatrixXd PX3 = VX3;
  const Eigen::MatrixX3d P3 = V3;
  Eigen::VectorXd S;
  Eigen::VectorXi I;
  Eigen::MatrixXd C, N;
  Eigen::MatrixX3d C3, N3;
  const igl::SignedDistanceType type = igl::SIGNED_DISTANCE_TYPE_DEFAULT;
  const double lower_bound = std::numeric_limits<double>::min();
  const double upper_bound = std::numeric_limits<double>::max();
  igl::signed_distance(P3, V3, F3, type, lower_bound, upper_bound, S, I, C3, N3);
  igl::signed_distance(PX3, VX3, F, type, lower_bound, upper_bound, S, I, C, N);
  igl::signed_distance(P3, V3, F3, type, S, I, C3, N3);
  igl::signed_distance(PX3, VX3, F, type, S, I, C, N);
}
