// CPU restatement of igl::flood_fill (include/igl/flood_fill.cpp:11-80), the
// last step of igl::swept_volume_signed_distance.
//
// TEST INFRASTRUCTURE ONLY (see gwn_oracle.cpp).
//
// One scan over the grid, x fastest: an unsigned (NaN) cell takes the value
// carried in `s`; at each signed cell, the cells of its row back to the
// previous signed cell of the row, the rows of its sheet back to the previous
// row with a signed cell, and the sheets back to the previous sheet with a
// signed cell all take its value.  At the start of a row (sheet) `s` is the
// first cell of the previous row (sheet).
#include <cmath>
#include <cstdint>

extern "C" {

void oracle_flood_fill(const int32_t* res, double* S) {
  const int64_t X = res[0], Y = res[1], Z = res[2];
  auto at = [&](int64_t x, int64_t y, int64_t z) -> double& { return S[x + X * (y + Y * z)]; };
  auto flood = [&](int64_t xi, int64_t yi, int64_t zi, int64_t sxi, int64_t syi, int64_t szi,
                   double s) {
    for (int64_t bx = xi; sxi < --bx;) at(bx, yi, zi) = s;
    for (int64_t by = yi; syi < --by;)
      for (int64_t x = 0; x < X; ++x) at(x, by, zi) = s;
    for (int64_t bz = zi; szi < --bz;)
      for (int64_t y = 0; y < Y; ++y)
        for (int64_t x = 0; x < X; ++x) at(x, y, bz) = s;
  };
  int64_t szi = -1;
  double s = NAN;
  for (int64_t zi = 0; zi < Z; ++zi) {
    int64_t syi = -1;
    if (zi != 0) s = at(0, 0, zi - 1);
    for (int64_t yi = 0; yi < Y; ++yi) {
      int64_t sxi = -1;
      if (yi != 0) s = at(0, yi - 1, zi);
      for (int64_t xi = 0; xi < X; ++xi) {
        double& c = at(xi, yi, zi);
        if (c != c) {
          if (s == s) c = s;
          continue;
        }
        s = c;
        flood(xi, yi, zi, sxi, syi, szi, s);
        sxi = xi;
        syi = yi;
        szi = zi;
      }
    }
  }
}

}  // extern "C"
