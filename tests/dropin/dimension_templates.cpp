// Compile-only counterpart of the reference's "signed_distance:
// dimension-templates" case (tests/include/igl/signed_distance.cpp:77-120):
// the drop-in igl::signed_distance overloads instantiate with dynamic and
// fixed-column matrix types for a single triangle.  Its 3-D half only: the
// drop-in refuses 2-D inputs at run time.  Below it, the winding-number
// overloads with float and fixed-column types.  Nothing here is run.
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

// The winding-number overloads with float and fixed-column types (the
// reference instantiates them for float and double matrices,
// winding_number.cpp and fast_winding_number.cpp's template lists).
#include <igl/fast_winding_number.h>
#include <igl/winding_number.h>

void scalar_and_column_templates() {
  Eigen::MatrixX3d V(4, 3);
  V.set({0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1});
  Eigen::MatrixX3i F(4, 3);
  F.set({0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3});
  Eigen::MatrixX3d Q(1, 3);
  Q.set({0.1, 0.1, 0.1});
  Eigen::VectorXd W;
  igl::winding_number(V, F, Q, W);
  Eigen::RowVector3d p(1, 3);
  p.set({0.1, 0.1, 0.1});
  (void)igl::winding_number(V, F, p);

  Eigen::MatrixXf Vf(4, 3);
  Vf.set({0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1});
  Eigen::MatrixXi Fi(4, 3);
  Fi.set({0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3});
  Eigen::MatrixXf Qf(1, 3);
  Qf.set({0.1f, 0.1f, 0.1f});
  Eigen::VectorXf Wf;
  igl::fast_winding_number(Vf, Fi, Qf, Wf);
  igl::FastWindingNumberBVH bvh;
  igl::fast_winding_number(Vf, Fi, 2, bvh);
  igl::fast_winding_number(bvh, 2.0f, Qf, Wf);
  Eigen::RowVector3f pf(1, 3);
  pf.set({0.1f, 0.1f, 0.1f});
  (void)igl::fast_winding_number(bvh, 2.0f, pf);
}
