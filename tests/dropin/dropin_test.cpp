// The reference's own hot-path tests, written against the igl:: drop-in
// headers (include/igl_gb300/igl/*.h) and run on the GPU through libgwn.so:
//   tests/include/igl/fast_winding_number.cpp:17-53  one_point_cloud (1e-15)
//   tests/include/igl/signed_distance.cpp:4-42       single tet (FWN sign)
// plus the octree and exact winding number on the same data.  Prints
// "name value" lines that the Python test compares with the CPU oracle.
#include <cmath>
#include <limits>
#include <cstdio>
#include <vector>

#include <Eigen/Core>
#include <igl/fast_winding_number.h>
#include <igl/eytzinger_aabb.h>
#include <igl/eytzinger_aabb_winding_number.h>
#include <igl/eytzinger_aabb_winding_number_tree.h>
#include <igl/WindingNumberAABB.h>
#include <igl/flood_fill.h>
#include <igl/knn.h>
#include <igl/octree.h>
#include <igl/signed_distance.h>
#include <igl/swept_volume_signed_distance.h>
#include <igl/winding_number.h>
#include <igl/copyleft/cgal/fast_winding_number.h>
#include <igl/copyleft/cgal/point_areas.h>

static int failures = 0;
static void check_near(const char* what, double a, double b, double tol) {
  const bool ok = std::fabs(a - b) <= tol;
  if (!ok) ++failures;
  std::printf("%s %.17g %.17g %s\n", what, a, b, ok ? "ok" : "FAIL");
}

int main() {
  // one_point_cloud
  Eigen::MatrixXd P(1, 3);
  P.set({0.1, 0.2, 0.3});
  Eigen::MatrixXd N(1, 3);
  const double nn = std::sqrt(16.0 + 25.0 + 36.0);
  N.set({4 / nn, 5 / nn, 6 / nn});
  Eigen::VectorXd A(1);
  A(0) = 0.7;
  std::vector<std::vector<int>> O_PI;
  Eigen::MatrixXi O_CH;
  Eigen::MatrixXd O_CN;
  Eigen::VectorXd O_W;
  igl::octree(P, O_PI, O_CH, O_CN, O_W);
  Eigen::MatrixXd O_CM;
  Eigen::VectorXd O_R;
  Eigen::MatrixXd O_EC;
  igl::fast_winding_number(P, N, A, O_PI, O_CH, 2, O_CM, O_R, O_EC);
  Eigen::MatrixXd Q(4, 3);
  Q.set({0, 0, 0, 4, -3, 2, -1, 1, 3, 0, 5, -2});
  Eigen::VectorXd WiP;
  igl::fast_winding_number(P, N, A, O_PI, O_CH, O_CM, O_R, O_EC, Q, 2, WiP);
  const double cached[4] = {0.38779369004261133, -0.00041235296362485, -0.00362978253577090,
                            -0.00041235296362485};
  for (int i = 0; i < 4; ++i) check_near("one_point_cloud", WiP(i), cached[i], 1e-15);
  std::printf("octree_cells %ld rows_of_EC %ld\n", (long)O_CH.rows(), (long)O_EC.rows());

  // single tet (signed_distance.cpp:4-42): (.5,.5,.5) is outside
  Eigen::MatrixXd V(4, 3);
  V.set({0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1});
  Eigen::MatrixXi F(4, 3);
  F.set({0, 1, 3, 0, 2, 1, 0, 3, 2, 1, 2, 3});
  Eigen::MatrixXd T(2, 3);
  T.set({0.5, 0.5, 0.5, 0.1, 0.1, 0.1});
  igl::FastWindingNumberBVH bvh;
  igl::fast_winding_number(V, F, 2, bvh);
  Eigen::VectorXd Ws;
  igl::fast_winding_number(bvh, 2.0f, T, Ws);
  check_near("tet_soup_outside", Ws(0), 0.0, 1e-6);
  check_near("tet_soup_inside", Ws(1), 1.0, 1e-6);
  Eigen::RowVector3d p;
  p(0, 0) = 0.1;
  p(0, 1) = 0.1;
  p(0, 2) = 0.1;
  check_near("tet_soup_point", igl::fast_winding_number(bvh, 2.0f, p), 1.0, 1e-6);
  Eigen::VectorXd We;
  igl::winding_number(V, F, T, We);
  check_near("tet_exact_outside", We(0), 0.0, 1e-15);
  check_near("tet_exact_inside", We(1), 1.0, 1e-15);
  check_near("tet_exact_point", igl::winding_number(V, F, p), 1.0, 1e-15);
  Eigen::VectorXd W1;
  igl::fast_winding_number(V, F, T, W1);
  check_near("tet_soup_oneshot", W1(1), 1.0, 1e-6);
  // cloud one shot from the tet's face centroids
  Eigen::VectorXd Wc;
  igl::fast_winding_number(P, N, A, Q, Wc);
  for (int i = 0; i < 4; ++i) check_near("one_point_cloud_oneshot", Wc(i), cached[i], 1e-15);
  // signed_distance single tet (tests/include/igl/signed_distance.cpp:4-42):
  // every provided sign type gives sqrt(1/12) at (.5,.5,.5)
  {
    Eigen::MatrixXd Pq(1, 3);
    Pq.set({0.5, 0.5, 0.5});
    const igl::SignedDistanceType types[5] = {
        igl::SIGNED_DISTANCE_TYPE_PSEUDONORMAL, igl::SIGNED_DISTANCE_TYPE_WINDING_NUMBER,
        igl::SIGNED_DISTANCE_TYPE_DEFAULT, igl::SIGNED_DISTANCE_TYPE_UNSIGNED,
        igl::SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER};
    for (const auto type : types) {
      Eigen::VectorXd S;
      Eigen::VectorXi I;
      Eigen::MatrixXd Cc, Nn;
      igl::signed_distance(Pq, V, F, type, S, I, Cc, Nn);
      const double tol = type == igl::SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER ? 1e-7 : 1e-15;
      check_near("signed_distance_tet", S(0), std::sqrt(1.0 / 12.0), tol);
    }
  }
  // knn (tests/include/igl/knn.cpp:8-73), unit-cube corners
  {
    Eigen::MatrixXd Vc(8, 3);
    Vc.set({0, 0, 1, 0, 1, 0, 0, 1, 1, 0, 0, 0, 1, 0, 0, 1, 1, 0, 1, 1, 1, 1, 0, 1});
    Eigen::MatrixXd Pc(3, 3);
    Pc.set({0, 0, 0.6, 0.3, 0.1, 0.2, 0.7, 0.6, 0});
    std::vector<std::vector<int>> pi;
    Eigen::MatrixXi ch;
    Eigen::MatrixXd cn;
    Eigen::VectorXd w;
    igl::octree(Vc, pi, ch, cn, w);
    Eigen::MatrixXi I;
    igl::knn(Pc, Vc, 3, pi, ch, cn, w, I);
    const int answer[9] = {0, 3, 2, 3, 4, 0, 5, 4, 1};
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) check_near("knn_unit_cube", I(r, c), answer[r * 3 + c], 0.0);
  }
  // 2-D Eytzinger AABB winding number: unit square, counter-clockwise
  {
    Eigen::MatrixXd V2(4, 2);
    V2.set({0, 0, 1, 0, 1, 1, 0, 1});
    Eigen::MatrixXi E2(4, 2);
    E2.set({0, 1, 1, 2, 2, 3, 3, 0});
    Eigen::MatrixXd PB1(4, 2), PB2(4, 2);
    for (int e = 0; e < 4; ++e)
      for (int d = 0; d < 2; ++d) {
        const double a = V2(E2(e, 0), d), b = V2(E2(e, 1), d);
        PB1(e, d) = a < b ? a : b;
        PB2(e, d) = a < b ? b : a;
      }
    Eigen::MatrixXd B1, B2;
    Eigen::VectorXi leaf, I, C;
    igl::eytzinger_aabb(PB1, PB2, B1, B2, leaf);
    check_near("eytzinger_slots", (double)leaf.rows(), 8, 0);
    igl::eytzinger_aabb_winding_number_tree(E2, leaf, I, C);
    check_near("eytzinger_C_rows", (double)C.rows(), 9, 0);
    Eigen::MatrixXd p(1, 2);
    p.set({0.5, 0.5});
    double wn = 0;
    igl::eytzinger_aabb_winding_number(p, V2, E2, B1, B2, leaf, I, C, wn);
    check_near("eytzinger_wn_inside", wn, 1.0, 1e-15);
    Eigen::MatrixXd Pq(3, 2);
    Pq.set({0.5, 0.5, 2, 0.5, 0.25, 0.75});
    Eigen::VectorXd Wq;
    igl::eytzinger_aabb_winding_number(Pq, V2, E2, B1, B2, leaf, I, C, Wq);
    check_near("eytzinger_wn_batch0", Wq(0), 1.0, 1e-6);
    check_near("eytzinger_wn_batch1", Wq(1), 0.0, 1e-6);
    check_near("eytzinger_wn_batch2", Wq(2), 1.0, 1e-6);
  }
  // flood fill: one signed cell fills a 3 x 2 x 2 grid
  {
    Eigen::VectorXd S(12);
    for (int i = 0; i < 12; ++i) S(i) = std::nan("");
    S(7) = 0.75;
    Eigen::Matrix<int, 1, 3> res;
    res.set({3, 2, 2});
    igl::flood_fill(res, S);
    for (int i = 0; i < 12; ++i) check_near("flood_fill", S(i), 0.75, 0.0);
  }
  // swept volume of the unit tet under the identity and a unit shift in x:
  // unsigned distances 2 below the first copy's bottom face and sqrt(4.005)
  // from the shifted copy's vertex (2, 0, 0)
  {
    Eigen::MatrixXd Vt(4, 3);
    Vt.set({0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1});
    Eigen::MatrixXi Ft(4, 3);
    Ft.set({0, 2, 1, 0, 3, 2, 0, 1, 3, 1, 2, 3});
    std::vector<Eigen::Affine3d> Ts(2);
    Ts[1](0, 3) = 1.0;
    Eigen::MatrixXd GVt(2, 3);
    GVt.set({0.1, 0.1, -2.0, 4.0, 0.05, 0.05});
    Eigen::Matrix<int, 1, 3> res;
    res.set({2, 1, 1});
    Eigen::VectorXd St;
    igl::swept_volume_signed_distance(Vt, Ft, Ts, igl::SIGNED_DISTANCE_TYPE_UNSIGNED, GVt, res,
                                      0.1, std::numeric_limits<double>::infinity(), St);
    check_near("swept_below", St(0), 2.0, 1e-12);
    check_near("swept_vertex", St(1), std::sqrt(4.005), 1e-12);
  }
  // WindingNumberAABB: unit tet, outward
  {
    Eigen::MatrixXd Vt(4, 3);
    Vt.set({0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1});
    Eigen::MatrixXi Ft(4, 3);
    Ft.set({0, 2, 1, 0, 3, 2, 0, 1, 3, 1, 2, 3});
    igl::WindingNumberAABB<double, int> hier;
    hier.set_mesh(Vt, Ft);
    hier.grow();
    Eigen::RowVector3d pin, pout;
    pin.set({0.1, 0.1, 0.1});
    pout.set({2, 2, 2});
    check_near("wn_aabb_inside", hier.winding_number(pin), 1.0, 1e-6);
    check_near("wn_aabb_outside", hier.winding_number(pout), 0.0, 1e-6);
  }
  // copyleft::cgal::point_areas on a 7 x 7 hexagonal patch: the centre point
  // owns its hexagonal Voronoi cell, (sqrt(3)/2) h^2; then the point-cloud
  // winding number of the CGAL module from points and normals alone
  {
    const double h = 0.1;
    Eigen::MatrixXd Ph(49, 3), Nh(49, 3);
    int c = 0, centre = 0;
    for (int j = -3; j <= 3; ++j)
      for (int i = -3; i <= 3; ++i, ++c) {
        Ph(c, 0) = h * (i + 0.5 * (j & 1));
        Ph(c, 1) = h * j * std::sqrt(3.0) / 2;
        Ph(c, 2) = 1e-7 * ((c * 37) % 11);  // tiny relief: no exact cocircularity
        Nh(c, 0) = 0;
        Nh(c, 1) = 0;
        Nh(c, 2) = 1;
        if (i == 0 && j == 0) centre = c;
      }
    std::vector<std::vector<int>> PIh;
    Eigen::MatrixXi CHh;
    Eigen::MatrixXd CNh;
    Eigen::VectorXd Wh;
    igl::octree(Ph, PIh, CHh, CNh, Wh);
    Eigen::MatrixXi Ih;
    igl::knn(Ph, 13, PIh, CHh, CNh, Wh, Ih);
    Eigen::VectorXd Ah;
    Eigen::MatrixXd Th;
    igl::copyleft::cgal::point_areas(Ph, Ih, Nh, Ah, Th);
    check_near("point_areas_hex", Ah(centre), std::sqrt(3.0) / 2 * h * h, 1e-6);
    check_near("point_areas_normal", Th(centre, 2), 1.0, 1e-6);
    Eigen::MatrixXd Qh(1, 3);
    Qh.set({0.0, 0.0, 5.0});
    Eigen::VectorXd WNh;
    igl::copyleft::cgal::fast_winding_number(Ph, Nh, Qh, WNh);
    check_near("cgal_fwn_far", WNh(0), 0.0, 1e-2);
  }
  std::printf("failures %d\n", failures);
  return failures ? 1 : 0;
}
