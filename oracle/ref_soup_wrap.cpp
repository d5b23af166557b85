// Thin C wrapper around the libigl reference's own triangle-soup fast winding
// number (the vendored HDK UT_SolidAngle in
// include/igl/FastWindingNumberForSoups.h), compiled from the reference tree
// where it lies by oracle/build_ref.sh into oracle/_ref/ (never committed).
//
// TEST INFRASTRUCTURE ONLY: used in this container to pin the oracle and to
// generate the committed golden fixtures under tests/golden/.  The calls
// below follow include/igl/fast_winding_number.cpp:383-415 (precompute: V and
// F copied to float / row-major int, init(order)) and :421-437 (evaluate:
// query cast to float, computeSolidAngle(q, accuracy_scale) / (4 pi), in
// igl::parallel_for(..., 1000)).
// The tree lives in a private member of UT_SolidAngle; this test-only
// wrapper opens it up to export the reference's own node array.
#define private public
#include <igl/FastWindingNumberForSoups.h>
#undef private
#include <igl/parallel_for.h>

#include <cstdint>
#include <vector>

namespace hdk = igl::FastWindingNumber::HDK_Sample;

struct RefSoup {
  hdk::UT_SolidAngle<float, float> sa;
  std::vector<hdk::UT_Vector3T<float>> U;
  std::vector<int> F;
};

extern "C" {

void* ref_soup_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, int order) {
  RefSoup* s = new RefSoup();
  s->U.resize((size_t)nV);
  for (int64_t i = 0; i < nV; ++i)
    for (int j = 0; j < 3; ++j) s->U[(size_t)i][j] = (float)V[i * 3 + j];
  s->F.resize((size_t)nF * 3);
  for (int64_t f = 0; f < nF * 3; ++f) s->F[(size_t)f] = F[f];
  s->sa.clear();
  s->sa.init((int)nF, s->F.data(), (int)nV, s->U.data(), order);
  return s;
}

void ref_soup_eval(void* h, float accuracy_scale, const double* Q, int64_t nQ, double* W) {
  RefSoup* s = (RefSoup*)h;
  igl::parallel_for(
      (int)nQ,
      [&](int p) {
        hdk::UT_Vector3T<float> q;
        q[0] = (float)Q[(int64_t)p * 3 + 0];
        q[1] = (float)Q[(int64_t)p * 3 + 1];
        q[2] = (float)Q[(int64_t)p * 3 + 2];
        W[p] = s->sa.computeSolidAngle(q, accuracy_scale) / (4.0 * 3.1415926535897932384626433832795);
      },
      1000);
}

// The reference's UT_BVH<4> nodes: returns the node count and, when `child`
// is non-null, writes 4 entries per node (an item index, node | 2^31 for an
// internal child, or ~0 for an empty lane), in the reference's node order.
int64_t ref_soup_tree(void* h, uint32_t* child) {
  RefSoup* s = (RefSoup*)h;
  const auto& tree = s->sa.myTree;
  const int64_t n = (int64_t)tree.getNumNodes();
  if (child) {
    const auto* nodes = tree.getNodes();
    for (int64_t i = 0; i < n; ++i)
      for (int c = 0; c < 4; ++c) child[i * 4 + c] = (uint32_t)nodes[i].child[c];
  }
  return n;
}

void ref_soup_free(void* h) { delete (RefSoup*)h; }

}  // extern "C"
