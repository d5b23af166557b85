// Host-side probe of the walk records' packed far-field coefficients (TEST
// ONLY): reads moment records from stdin, writes what pack_far32 (soup.cuh)
// and pack_cloud (cloud.cuh) make of them, so that tests/test_packed_forms.py
// can evaluate the packed forms against the reference's own formulas.
//
// stdin:  "soup n" then n lines of 19 moments (N[3], Nii[3], Nxy_yx, Nyz_zy,
//         Nzx_xz, Niii[3], perm, c2[6]); "cloud n" then n lines of 39 EC terms.
// stdout: per soup record the 19 packed FP32 coefficients (b.xyzw c.xyzw
//         d.xyzw e.xyzw f.xyz); per cloud record the 15 packed FP64 ones.
#include <cstdio>
#include <cstring>

#include "cloud.cuh"
#include "soup.cuh"

int main() {
  char kind[16];
  long n = 0;
  while (std::scanf("%15s %ld", kind, &n) == 2) {
    for (long r = 0; r < n; ++r) {
      if (std::strcmp(kind, "soup") == 0) {
        double m[19];
        for (double& v : m)
          if (std::scanf("%lf", &v) != 1) return 1;
        gwn::SoupNodeF R;
        gwn::pack_far32(R, m, m + 3, m[6], m[7], m[8], m + 9, m[12], m + 13, 0);
        const float out[19] = {R.b.x, R.b.y, R.b.z, R.b.w, R.c.x, R.c.y, R.c.z, R.c.w, R.d.x, R.d.y,
                               R.d.z, R.d.w, R.e.x, R.e.y, R.e.z, R.e.w, R.f.x, R.f.y, R.f.z};
        for (float v : out) std::printf("%.9e ", (double)v);
        std::printf("\n");
      } else {
        double ec[39], pk[15];
        for (double& v : ec)
          if (std::scanf("%lf", &v) != 1) return 1;
        gwn::pack_cloud(ec, 39, pk);
        for (double v : pk) std::printf("%.17e ", v);
        std::printf("\n");
      }
    }
  }
  return 0;
}
