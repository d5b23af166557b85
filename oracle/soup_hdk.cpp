// CPU restatement of the reference's triangle-soup fast winding number
// (TEST INFRASTRUCTURE ONLY: the CPU baseline / reference arm and a checker;
// libgwn.so never uses it).
//
// Follows the HDK sample vendored as include/igl/FastWindingNumberForSoups.h,
// used by igl::fast_winding_number (include/igl/fast_winding_number.cpp:
// 383-437), in single precision exactly as the reference instantiates it
// (UT_SolidAngle<float,float>):
//   * triangle boxes, then a 4-wide BVH built top-down with the BOX_AREA
//     heuristic (UT_BVH<4>::init / initNode, FWNFS.h:4581-4634, 4918-5047):
//     <= 4 boxes fill one node; otherwise multiSplit (FWNFS.h:5249-5346)
//     repeatedly splits the sub-range with the largest area x count;
//     split (FWNFS.h:5350-5800): 2 boxes trivially, <= 6 boxes by trying
//     every 2-partition, <= 32 by sorting centres along the longest axis
//     and sweeping, otherwise 16 equal spans along the longest axis with at
//     least 1/16 of the boxes on each side (falling back to an nth-element
//     split), boxes with a NaN/Inf bound excluded (FWNFS.h:4536-4616);
//   * per-node child-lane moments by a post-order pass (item/post,
//     FWNFS.h:6668-7118);
//   * computeSolidAngle (FWNFS.h:7148-7284): per node all child lanes are
//     tested and approximated, descending where |q-P|^2 <= maxP^2 beta^2 or
//     the approximation is not finite; leaves use UTsignedSolidAngleTri.
// Float division by a scalar is a multiply by its reciprocal, as in
// UT_FixedVector::operator/ (FWNFS.h:3437-3452).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

using uint = unsigned int;
constexpr uint kEmpty = ~0u;
constexpr uint kInternal = 1u << 31;
constexpr int kSpans = 16;
constexpr int kMinFraction = 16;

struct Box {
  float lo[3], hi[3];
  void init() {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::numeric_limits<float>::max();
      hi[a] = -std::numeric_limits<float>::max();
    }
  }
  void combine(const Box& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = lo[a] < b.lo[a] ? lo[a] : b.lo[a];
      hi[a] = hi[a] > b.hi[a] ? hi[a] : b.hi[a];
    }
  }
  float half_area() const {
    const float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
    return d0 * d1 + d1 * d2 + d2 * d0;
  }
  float centre2(int a) const { return lo[a] + hi[a]; }  // twice the centre
};

struct Node {
  uint child[4];
};

struct Builder {
  const Box* boxes;
  std::vector<Node> nodes;

  void split(const Box& all, uint* idx, uint n, uint*& mid, Box sub[2]) {
    if (n == 2) {
      sub[0] = boxes[idx[0]];
      sub[1] = boxes[idx[1]];
      mid = idx + 1;
      return;
    }
    if (n <= 6) {  // every partition with box 0 on side 0
      Box lb[6];
      for (uint b = 0; b < n; ++b) lb[b] = boxes[idx[b]];
      const uint lim = 1u << (n - 1);
      uint best = ~0u;
      float best_h = 0;
      for (uint bits = 1; bits < lim; ++bits) {
        Box s[2];
        s[0] = lb[0];
        s[1].init();
        uint cnt[2] = {1, 0};
        for (uint b = 0; b + 1 < n; ++b) {
          const uint d = (bits >> b) & 1u;
          s[d].combine(lb[b + 1]);
          ++cnt[d];
        }
        const float h = s[0].half_area() * cnt[0] + s[1].half_area() * cnt[1];
        if (best == ~0u || h < best_h) {
          best = bits;
          best_h = h;
          sub[0] = s[0];
          sub[1] = s[1];
        }
      }
      uint rest[5];
      for (uint b = 0; b + 1 < n; ++b) rest[b] = idx[b + 1];
      uint* out = idx + 1;
      for (uint b = 0; b + 1 < n; ++b)
        if (!((best >> b) & 1u)) *out++ = rest[b];
      mid = out;
      for (uint b = 0; b + 1 < n; ++b)
        if ((best >> b) & 1u) *out++ = rest[b];
      return;
    }
    int axis = 0;
    float axis_len = all.hi[0] - all.lo[0];
    for (int a = 1; a < 3; ++a) {
      const float l = all.hi[a] - all.lo[a];
      if (l > axis_len) {
        axis = a;
        axis_len = l;
      }
    }
    if (!(axis_len > 0.f)) {  // single point or NaN: arbitrary split
      mid = idx + n / 2;
      sub[0] = all;
      sub[1] = all;
      return;
    }
    if (n <= 2 * (uint)kSpans) {  // stable sort by centre, then sweep
      std::vector<uint> ord(n);
      for (uint i = 0; i < n; ++i) ord[i] = i;
      std::stable_sort(ord.begin(), ord.end(), [&](uint a, uint b) {
        return boxes[idx[a]].centre2(axis) < boxes[idx[b]].centre2(axis);
      });
      std::vector<uint> sorted(n);
      for (uint i = 0; i < n; ++i) sorted[i] = idx[ord[i]];
      std::copy(sorted.begin(), sorted.end(), idx);
      const uint ns = n - 1;
      std::vector<Box> L(ns), R(ns);
      Box acc = boxes[idx[0]];
      L[0] = acc;
      for (uint i = 1; i < ns; ++i) {
        acc.combine(boxes[idx[i]]);
        L[i] = acc;
      }
      // The right-hand accumulation starts from element ns-1, so the last
      // element's box never enters the right boxes (FWNFS.h:5560-5565);
      // kept as written so the tree matches the reference's.
      acc = boxes[idx[ns - 1]];
      R[ns - 1] = acc;
      for (uint i = ns - 1; i > 0; --i) {
        acc.combine(boxes[idx[i]]);
        R[i - 1] = acc;
      }
      uint best = 0;
      float best_h = L[0].half_area() + R[0].half_area() * (n - 1);
      for (uint s = 1; s < ns; ++s) {
        const float h = L[s].half_area() * (s + 1) + R[s].half_area() * (n - (s + 1));
        if (h < best_h) {
          best = s;
          best_h = h;
        }
      }
      mid = idx + best + 1;
      sub[0] = L[best];
      sub[1] = R[best];
      return;
    }
    // 16 spans along the axis
    const float axis_min2 = 2.0f * all.lo[axis];
    const float scale = ((1.0f / 2.0f) * kSpans) / axis_len;
    Box span[kSpans];
    uint cnt[kSpans];
    for (int i = 0; i < kSpans; ++i) {
      span[i].init();
      cnt[i] = 0;
    }
    for (uint i = 0; i < n; ++i) {
      const Box& b = boxes[idx[i]];
      int si = (int)((b.centre2(axis) - axis_min2) * scale);
      si = si < 0 ? 0 : (si > kSpans - 1 ? kSpans - 1 : si);
      ++cnt[si];
      span[si].combine(b);
    }
    Box L[kSpans - 1], R[kSpans - 1];
    uint lc[kSpans - 1];
    Box acc = span[0];
    L[0] = acc;
    for (int i = 1; i < kSpans - 1; ++i) {
      acc.combine(span[i]);
      L[i] = acc;
    }
    acc = span[kSpans - 1];
    R[kSpans - 2] = acc;
    for (int i = kSpans - 2; i > 0; --i) {
      acc.combine(span[i]);
      R[i - 1] = acc;
    }
    uint run = cnt[0];
    lc[0] = run;
    for (int i = 1; i < kSpans - 1; ++i) {
      run += cnt[i];
      lc[i] = run;
    }
    const uint min_count = n / kMinFraction;
    const uint max_count = (uint)(((uint64_t)(kMinFraction - 1) * n) / kMinFraction);
    float smallest = std::numeric_limits<float>::infinity();
    int si = -1;
    for (int i = 0; i < kSpans - 1; ++i) {
      if (lc[i] < min_count || lc[i] > max_count) continue;
      const float h = lc[i] * L[i].half_area() + (n - lc[i]) * R[i].half_area();
      if (h < smallest) {
        smallest = h;
        si = i;
      }
    }
    uint* end = idx + n;
    if (si == -1) {
      uint* nth;
      if (lc[0] > max_count) nth = idx + max_count;
      else if (lc[kSpans - 2] < min_count) nth = idx + min_count;
      else nth = idx + n / 2;
      nth_element(idx, end, axis, nth);
      mid = nth;
      Box lb = boxes[idx[0]];
      for (uint* p = idx + 1; p < nth; ++p) lb.combine(boxes[*p]);
      Box rb = boxes[nth[0]];
      for (uint* p = nth + 1; p < end; ++p) rb.combine(boxes[*p]);
      sub[0] = lb;
      sub[1] = rb;
      return;
    }
    const float pivot2 = axis_min2 + (si + 1) * axis_len / (kSpans / 2.0f);
    uint *ps, *pe;
    partition(idx, end, axis, pivot2, ps, pe);
    mid = idx + lc[si];
    if (mid >= ps && mid <= pe) {
      sub[0] = L[si];
      sub[1] = R[si];
      return;
    }
    mid = mid < ps ? ps : pe;
    if (mid == idx) ++mid;
    else if (mid == end) --mid;
    Box lb = boxes[idx[0]];
    for (uint* p = idx + 1; p < mid; ++p) lb.combine(boxes[*p]);
    Box rb = boxes[mid[0]];
    for (uint* p = mid + 1; p < end; ++p) rb.combine(boxes[*p]);
    sub[0] = lb;
    sub[1] = rb;
  }

  // three-way partition around pivot2 (less | equal | greater), FWNFS.h:5903-5944
  void partition(uint* idx, const uint* end, int axis, float pivot2, uint*& ps, uint*& pe) {
    uint* s = idx;
    uint* e = idx;
    for (uint* p = idx; p != end; ++p) {
      const float v = boxes[*p].centre2(axis);
      if (v < pivot2) {
        if (p != s) {
          if (s == e) {
            std::swap(*p, *s);
          } else {
            const uint t = *p;
            *p = *e;
            *e = *s;
            *s = t;
          }
        }
        ++s;
        ++e;
      } else if (v == pivot2) {
        if (p != e) std::swap(*p, *e);
        ++e;
      }
    }
    ps = s;
    pe = e;
  }

  // median-of-three quickselect on centres, FWNFS.h:5847-5900
  void nth_element(uint* idx, uint* end, int axis, uint* nth) {
    while (true) {
      float pv[3] = {boxes[idx[0]].centre2(axis), boxes[idx[(end - idx) / 2]].centre2(axis),
                     boxes[*(end - 1)].centre2(axis)};
      if (pv[0] < pv[1]) std::swap(pv[0], pv[1]);
      if (pv[0] < pv[2]) std::swap(pv[0], pv[2]);
      if (pv[1] < pv[2]) std::swap(pv[1], pv[2]);
      uint *ps, *pe;
      partition(idx, end, axis, pv[1], ps, pe);
      if (nth < ps) end = ps;
      else if (nth < pe) return;
      else idx = pe;
      if (end <= idx + 1) return;
    }
  }

  void multi_split(const Box& all, uint* idx, uint n, uint* sub_idx[5], Box sub[4]) {
    sub_idx[0] = idx;
    sub_idx[2] = idx + n;
    split(all, idx, n, sub_idx[1], sub);
    float area[4];
    area[0] = sub[0].half_area();
    area[1] = sub[1].half_area();
    for (uint ns = 2; ns < 4; ++ns) {
      uint choice = ~0u;
      float best = 0;
      for (uint i = 0; i < ns; ++i) {
        const uint c = (uint)(sub_idx[i + 1] - sub_idx[i]);
        if (c > 1) {
          const float h = area[i] * c;
          if (choice == ~0u || h > best) {
            choice = i;
            best = h;
          }
        }
      }
      uint* s = sub_idx[choice];
      uint* e = sub_idx[choice + 1];
      for (uint i = ns; i > choice; --i) sub_idx[i + 1] = sub_idx[i];
      for (uint i = ns - 1; i > choice; --i) sub[i + 1] = sub[i];
      for (uint i = ns - 1; i > choice; --i) area[i + 1] = area[i];
      Box pair[2];
      split(sub[choice], s, (uint)(e - s), sub_idx[choice + 1], pair);
      sub[choice] = pair[0];
      sub[choice + 1] = pair[1];
      area[choice] = sub[choice].half_area();
      area[choice + 1] = sub[choice + 1].half_area();
    }
  }

  void init_node(uint node_index, const Box& all, uint* idx, uint n) {
    if (n <= 4) {
      for (uint i = 0; i < 4; ++i) nodes[node_index].child[i] = i < n ? idx[i] : kEmpty;
      return;
    }
    uint* sub_idx[5];
    Box sub[4];
    multi_split(all, idx, n, sub_idx, sub);
    for (uint i = 0; i < 4; ++i)
      if (sub_idx[i + 1] - sub_idx[i] == 1) nodes[node_index].child[i] = sub_idx[i][0];
    for (uint i = 0; i < 4; ++i) {
      const uint c = (uint)(sub_idx[i + 1] - sub_idx[i]);
      if (c != 1) {
        const uint ni = (uint)nodes.size();
        nodes[node_index].child[i] = ni | kInternal;
        nodes.push_back(Node{});
        init_node(ni, sub[i], sub_idx[i], c);
      }
    }
  }
};

bool box_bad(const Box& b) {
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(b.lo[a]) || !std::isfinite(b.hi[a])) return true;
  return false;
}

using V3 = float[3];

struct Lanes {  // BoxData: one lane per child
  float maxP2[4], P[3][4], N[3][4];
  float Nii[3][4], Nxy_yx[4], Nyz_zy[4], Nzx_xz[4];
  float Niii[3][4], perm[4], c2[6][4];
};

struct Local {
  Box box;
  float P[3], areaP[3], N[3], area;
  float Nii[3], Nxy, Nyx, Nyz, Nzy, Nzx, Nxz;
  float Niii[3], perm, c2[6];
};

struct Soup {
  std::vector<float> U;  // float vertex copies (fast_winding_number.cpp:392-399)
  std::vector<int> F;
  std::vector<Box> tri_boxes;
  std::vector<Node> nodes;
  std::vector<Lanes> data;
  int order = 2;

  const float* vtx(int i) const { return &U[(size_t)i * 3]; }

  void item(uint t, Local& L) const {
    const float* a = vtx(F[t * 3]);
    const float* b = vtx(F[t * 3 + 1]);
    const float* c = vtx(F[t * 3 + 2]);
    float ab[3], ac[3];
    for (int d = 0; d < 3; ++d) {
      ab[d] = b[d] - a[d];
      ac[d] = c[d] - a[d];
    }
    L.box = tri_boxes[t];
    const float cr[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2],
                         ab[0] * ac[1] - ab[1] * ac[0]};
    for (int d = 0; d < 3; ++d) L.N[d] = 0.5f * cr[d];
    const float area2 = L.N[0] * L.N[0] + L.N[1] * L.N[1] + L.N[2] * L.N[2];
    const float area = std::sqrt(area2);
    const float third = 1.0f / 3.0f;
    for (int d = 0; d < 3; ++d) {
      L.P[d] = ((a[d] + b[d]) + c[d]) * third;
      L.areaP[d] = L.P[d] * area;
      L.Nii[d] = 0;
      L.Niii[d] = 0;
    }
    L.area = area;
    L.Nxy = L.Nyx = L.Nyz = L.Nzy = L.Nzx = L.Nxz = 0;
    L.perm = 0;
    for (float& x : L.c2) x = 0;
    if (order < 2 || area == 0) return;
    const float inv = 1.0f / area;
    const float n[3] = {L.N[0] * inv, L.N[1] * inv, L.N[2] * inv};
    const float* v[3] = {a, b, c};
    int o[3][3];
    for (int ax = 0; ax < 3; ++ax) {
      int* oo = o[ax];
      oo[0] = 0, oo[1] = 1, oo[2] = 2;
      if (a[ax] > b[ax]) std::swap(oo[0], oo[1]);
      if (v[oo[0]][ax] > c[ax]) std::swap(oo[0], oo[2]);
      if (v[oo[1]][ax] > v[oo[2]][ax]) std::swap(oo[1], oo[2]);
    }
    const float dx = v[o[0][2]][0] - v[o[0][0]][0];
    const float dy = v[o[1][2]][1] - v[o[1][0]][1];
    const float dz = v[o[2][2]][2] - v[o[2][0]][2];
    float xx = 0, xy = 0, yy = 0, yz = 0, zz = 0, zx = 0;
    auto integ = [&](const float* A, const float* B, const float* Cc, float* ii, float* ij, float* ik,
                     int i) {
      float oab[3], oac[3], ocb[3];
      for (int d = 0; d < 3; ++d) {
        oab[d] = B[d] - A[d];
        oac[d] = Cc[d] - A[d];
        ocb[d] = B[d] - Cc[d];
      }
      const float t = oab[i] / oac[i];
      const int j = (i == 2) ? 0 : i + 1, k = (j == 2) ? 0 : j + 1;
      const float jd = t * oac[j] - oab[j], kd = t * oac[k] - oab[k];
      const float xa[3] = {jd * oab[k] - kd * oab[j], kd * oab[i], jd * oab[i]};
      const float xc[3] = {jd * ocb[k] - kd * ocb[j], kd * ocb[i], jd * ocb[i]};
      const float sa = std::sqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
      const float sc = std::sqrt(xc[0] * xc[0] + xc[1] * xc[1] + xc[2] * xc[2]);
      const float Pai = A[i] - L.P[i], Pci = Cc[i] - L.P[i];
      const float ia = sa * (0.5f * Pai * Pai + float(2.0 / 3.0) * Pai * oab[i] + 0.25f * oab[i] * oab[i]);
      const float ic = sc * (0.5f * Pci * Pci + float(2.0 / 3.0) * Pci * ocb[i] + 0.25f * ocb[i] * ocb[i]);
      *ii = ia + ic;
      const int jks[2] = {j, k};
      const float df[2] = {jd, kd};
      float* outs[2] = {ij, ik};
      for (int s = 0; s < 2; ++s) {
        if (!outs[s]) continue;
        const int jk = jks[s];
        const float mid = B[jk] + 0.5f * df[s];
        const float am = mid - A[jk], cm = mid - Cc[jk];
        const float Paj = A[jk] - L.P[jk], Pcj = Cc[jk] - L.P[jk];
        const float ija = sa * (0.5f * Pai * Paj + float(1.0 / 3.0) * Pai * am +
                                float(1.0 / 3.0) * Paj * oab[i] + 0.25f * oab[i] * am);
        const float ijc = sc * (0.5f * Pci * Pcj + float(1.0 / 3.0) * Pci * cm +
                                float(1.0 / 3.0) * Pcj * ocb[i] + 0.25f * ocb[i] * cm);
        *outs[s] = ija + ijc;
      }
    };
    if (dx > 0)
      integ(v[o[0][0]], v[o[0][1]], v[o[0][2]], &xx, (dx >= dy && dy > 0) ? &xy : nullptr,
            (dx >= dz && dz > 0) ? &zx : nullptr, 0);
    if (dy > 0)
      integ(v[o[1][0]], v[o[1][1]], v[o[1][2]], &yy, (dy >= dz && dz > 0) ? &yz : nullptr,
            (dx < dy && dx > 0) ? &xy : nullptr, 1);
    if (dz > 0)
      integ(v[o[2][0]], v[o[2][1]], v[o[2][2]], &zz, (dx < dz && dx > 0) ? &zx : nullptr,
            (dy < dz && dy > 0) ? &yz : nullptr, 2);
    L.Niii[0] = xx * n[0];
    L.Niii[1] = yy * n[1];
    L.Niii[2] = zz * n[2];
    L.perm = 2 * (n[0] * yz + n[1] * zx + n[2] * xy);
    const float Nxxy = n[0] * xy, Nxxz = n[0] * zx, Nyyz = n[1] * yz, Nyyx = n[1] * xy,
                Nzzx = n[2] * zx, Nzzy = n[2] * yz;
    L.c2[0] = 2 * Nxxy + n[1] * xx;
    L.c2[1] = 2 * Nxxz + n[2] * xx;
    L.c2[2] = 2 * Nyyz + n[2] * yy;
    L.c2[3] = 2 * Nyyx + n[0] * yy;
    L.c2[4] = 2 * Nzzx + n[0] * zz;
    L.c2[5] = 2 * Nzzy + n[1] * zz;
  }

  // post-order moments of node `ni` (FWNFS.h:6892-7118); returns its data
  void build_node(uint ni, Local& out) {
    Local ch[4];
    int nch = 0;
    for (int s = 0; s < 4; ++s) {
      const uint c = nodes[ni].child[s];
      if (c == kEmpty) break;
      if (c & kInternal) build_node(c & ~kInternal, ch[s]);
      else item(c, ch[s]);
      ++nch;
    }
    Lanes& D = data[ni];
    std::memset(&D, 0, sizeof(D));
    float N[3], areaP[3], area = ch[0].area;
    for (int d = 0; d < 3; ++d) {
      N[d] = ch[0].N[d];
      areaP[d] = ch[0].areaP[d];
      D.N[d][0] = ch[0].N[d];
      D.P[d][0] = ch[0].P[d];
    }
    for (int i = 1; i < nch; ++i) {
      for (int d = 0; d < 3; ++d) {
        N[d] += ch[i].N[d];
        D.N[d][i] = ch[i].N[d];
        areaP[d] += ch[i].areaP[d];
        D.P[d][i] = ch[i].P[d];
      }
      area += ch[i].area;
    }
    for (int d = 0; d < 3; ++d) {
      out.N[d] = N[d];
      out.areaP[d] = areaP[d];
    }
    out.area = area;
    Box box = ch[0].box;
    for (int i = 1; i < nch; ++i) box.combine(ch[i].box);
    if (area > 0) {
      const float inv = 1.0f / area;
      for (int d = 0; d < 3; ++d) out.P[d] = areaP[d] * inv;
    } else {
      for (int d = 0; d < 3; ++d) out.P[d] = 0.5f * (box.lo[d] + box.hi[d]);
    }
    out.box = box;
    for (int i = 0; i < nch; ++i) {
      float m2 = 0;
      for (int d = 0; d < 3; ++d) {
        const float a = ch[i].P[d] - ch[i].box.lo[d], b = ch[i].box.hi[d] - ch[i].P[d];
        const float mx = a > b ? a : b;
        m2 = d == 0 ? mx * mx : m2 + mx * mx;
      }
      D.maxP2[i] = m2;
    }
    for (int i = nch; i < 4; ++i) D.maxP2[i] = std::numeric_limits<float>::infinity();
    if (order < 1) return;
    for (int d = 0; d < 3; ++d) out.Nii[d] = ch[0].Nii[d];
    out.Nxy = out.Nyx = out.Nyz = out.Nzy = out.Nzx = out.Nxz = 0;
    for (int d = 0; d < 3; ++d) out.Niii[d] = ch[0].Niii[d];
    out.perm = ch[0].perm;
    for (int k = 0; k < 6; ++k) out.c2[k] = ch[0].c2[k];
    for (int i = 1; i < nch; ++i) {
      for (int d = 0; d < 3; ++d) {
        out.Nii[d] += ch[i].Nii[d];
        out.Niii[d] += ch[i].Niii[d];
      }
      out.perm += ch[i].perm;
      for (int k = 0; k < 6; ++k) out.c2[k] += ch[i].c2[k];
    }
    for (int i = 0; i < nch; ++i) {
      for (int d = 0; d < 3; ++d) D.Nii[d][i] = ch[i].Nii[d];
      D.Nxy_yx[i] = ch[i].Nxy + ch[i].Nyx;
      D.Nyz_zy[i] = ch[i].Nyz + ch[i].Nzy;
      D.Nzx_xz[i] = ch[i].Nzx + ch[i].Nxz;
      for (int d = 0; d < 3; ++d) D.Niii[d][i] = ch[i].Niii[d];
      D.perm[i] = ch[i].perm;
      for (int k = 0; k < 6; ++k) D.c2[k][i] = ch[i].c2[k];
    }
    for (int i = 0; i < nch; ++i) {
      const Local& C = ch[i];
      const float dx = C.P[0] - out.P[0], dy = C.P[1] - out.P[1], dz = C.P[2] - out.P[2];
      const float* n = C.N;
      out.Nii[0] += n[0] * dx;
      out.Nii[1] += n[1] * dy;
      out.Nii[2] += n[2] * dz;
      const float Nxy = C.Nxy + n[0] * dy, Nyx = C.Nyx + n[1] * dx, Nyz = C.Nyz + n[1] * dz,
                  Nzy = C.Nzy + n[2] * dy, Nzx = C.Nzx + n[2] * dx, Nxz = C.Nxz + n[0] * dz;
      out.Nxy += Nxy, out.Nyx += Nyx, out.Nyz += Nyz, out.Nzy += Nzy, out.Nzx += Nzx, out.Nxz += Nxz;
      if (order >= 2) {
        const float dd[3] = {dx, dy, dz};
        for (int d = 0; d < 3; ++d) out.Niii[d] += 2.0f * dd[d] * C.Nii[d] + dd[d] * dd[d] * n[d];
        out.perm += (dx * (Nyz + Nzy) + dy * (Nzx + Nxz) + dz * (Nxy + Nyx));
        out.c2[0] += 2 * (dy * C.Nii[0] + dx * C.Nxy + n[0] * dx * dy) + 2 * C.Nyx * dx + n[1] * dx * dx;
        out.c2[1] += 2 * (dz * C.Nii[0] + dx * C.Nxz + n[0] * dx * dz) + 2 * C.Nzx * dx + n[2] * dx * dx;
        out.c2[2] += 2 * (dz * C.Nii[1] + dy * C.Nyz + n[1] * dy * dz) + 2 * C.Nzy * dy + n[2] * dy * dy;
        out.c2[3] += 2 * (dx * C.Nii[1] + dy * C.Nyx + n[1] * dy * dx) + 2 * C.Nxy * dy + n[0] * dy * dy;
        out.c2[4] += 2 * (dx * C.Nii[2] + dz * C.Nzx + n[2] * dz * dx) + 2 * C.Nxz * dz + n[0] * dz * dz;
        out.c2[5] += 2 * (dy * C.Nii[2] + dz * C.Nzy + n[2] * dz * dy) + 2 * C.Nyz * dz + n[1] * dz * dz;
      }
    }
  }

  void build(const double* V, int64_t nV, const int32_t* Fi, int64_t nF, int ord) {
    order = ord;
    U.resize((size_t)nV * 3);
    for (int64_t i = 0; i < nV * 3; ++i) U[(size_t)i] = (float)V[i];
    F.assign(Fi, Fi + nF * 3);
    tri_boxes.resize((size_t)nF);
    for (int64_t t = 0; t < nF; ++t) {
      Box& b = tri_boxes[(size_t)t];
      const float* p0 = vtx(F[t * 3]);
      for (int a = 0; a < 3; ++a) b.lo[a] = b.hi[a] = p0[a];
      // enlargeBounds with SYSmin / SYSmax (FWNFS.h:255-256, 4023-4028):
      // (a > b) ? b : a keeps a NaN of the first vertex and drops one of a
      // later vertex, so only a non-finite first vertex excludes the box
      for (int c = 1; c < 3; ++c) {
        const float* p = vtx(F[t * 3 + c]);
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = b.lo[a] > p[a] ? p[a] : b.lo[a];
          b.hi[a] = b.hi[a] < p[a] ? p[a] : b.hi[a];
        }
      }
    }
    std::vector<uint> idx;
    idx.reserve((size_t)nF);
    for (uint t = 0; t < (uint)nF; ++t)
      if (!box_bad(tri_boxes[t])) idx.push_back(t);
    nodes.clear();
    data.clear();
    if (idx.empty()) return;
    Box all;
    all.init();
    for (uint t : idx) all.combine(tri_boxes[t]);
    Builder B{tri_boxes.data(), {}};
    B.nodes.reserve(idx.size() / 2 + 4);
    B.nodes.push_back(Node{});
    B.init_node(0, all, idx.data(), (uint)idx.size());
    nodes = std::move(B.nodes);
    data.resize(nodes.size());
    Local root;
    build_node(0, root);
  }

  static float tri_angle(const float* a, const float* b, const float* c, const float* q) {
    float qa[3], qb[3], qc[3];
    for (int d = 0; d < 3; ++d) {
      qa[d] = a[d] - q[d];
      qb[d] = b[d] - q[d];
      qc[d] = c[d] - q[d];
    }
    const float la = std::sqrt(qa[0] * qa[0] + qa[1] * qa[1] + qa[2] * qa[2]);
    const float lb = std::sqrt(qb[0] * qb[0] + qb[1] * qb[1] + qb[2] * qb[2]);
    const float lc = std::sqrt(qc[0] * qc[0] + qc[1] * qc[1] + qc[2] * qc[2]);
    if (la == 0 || lb == 0 || lc == 0) return 0;
    const float ia = 1 / la, ib = 1 / lb, ic = 1 / lc;
    for (int d = 0; d < 3; ++d) {
      qa[d] *= ia;
      qb[d] *= ib;
      qc[d] *= ic;
    }
    const float u[3] = {qb[0] - qa[0], qb[1] - qa[1], qb[2] - qa[2]};
    const float v[3] = {qc[0] - qa[0], qc[1] - qa[1], qc[2] - qa[2]};
    const float cr[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
    const float num = qa[0] * cr[0] + qa[1] * cr[1] + qa[2] * cr[2];
    if (num == 0) return 0;
    const float den = 1 + (qa[0] * qb[0] + qa[1] * qb[1] + qa[2] * qb[2]) +
                      (qa[0] * qc[0] + qa[1] * qc[1] + qa[2] * qc[2]) +
                      (qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2]);
    return 2 * std::atan2(num, den);
  }

  float node_angle(uint ni, const float* q, float beta2) const {
    const Lanes& D = data[ni];
    float qv[3][4], q2l[4], om[4];
    uint desc = 0;
    for (int l = 0; l < 4; ++l) {
      for (int d = 0; d < 3; ++d) qv[d][l] = q[d] - D.P[d][l];
      q2l[l] = qv[0][l] * qv[0][l] + qv[1][l] * qv[1][l] + qv[2][l] * qv[2][l];
      if (q2l[l] <= D.maxP2[l] * beta2) desc |= 1u << l;
    }
    float sum = 0;
    if (desc != 15u) {
      for (int l = 0; l < 4; ++l) {
        const float m2 = 1.0f / q2l[l];
        const float m1 = std::sqrt(m2);
        const float x = qv[0][l] * m1, y = qv[1][l] * m1, z = qv[2][l] * m1;
        float o = -m2 * (x * D.N[0][l] + y * D.N[1][l] + z * D.N[2][l]);
        if (order >= 1) {
          const float x2 = x * x, y2 = y * y, z2 = z * z, m3 = m2 * m1;
          o += m3 * (D.Nii[0][l] + D.Nii[1][l] + D.Nii[2][l] -
                     3.0f * ((x2 * D.Nii[0][l] + y2 * D.Nii[1][l] + z2 * D.Nii[2][l]) +
                             x * y * D.Nxy_yx[l] + x * z * D.Nzx_xz[l] + y * z * D.Nyz_zy[l]));
          if (order >= 2) {
            const float x3 = x2 * x, y3 = y2 * y, z3 = z2 * z, m4 = m2 * m2;
            const float t0[3] = {D.c2[3][l] + D.c2[4][l], D.c2[5][l] + D.c2[0][l],
                                 D.c2[1][l] + D.c2[2][l]};
            const float t1[3] = {y * D.c2[0][l] + z * D.c2[1][l], z * D.c2[2][l] + x * D.c2[3][l],
                                 x * D.c2[4][l] + y * D.c2[5][l]};
            const float a0 = 3.0f * D.Niii[0][l] + t0[0], a1 = 3.0f * D.Niii[1][l] + t0[1],
                        a2 = 3.0f * D.Niii[2][l] + t0[2];
            o += m4 * (1.5f * (x * a0 + y * a1 + z * a2) -
                       7.5f * ((x3 * D.Niii[0][l] + y3 * D.Niii[1][l] + z3 * D.Niii[2][l]) +
                               x * y * z * D.perm[l] + (x2 * t1[0] + y2 * t1[1] + z2 * t1[2])));
          }
        }
        om[l] = o;
        if (!(desc >> l & 1u) && std::isfinite(o)) continue;
        om[l] = 0;
        desc |= 1u << l;
      }
      sum = om[0];
      for (int l = 1; l < 4; ++l) sum += om[l];
    }
    // descend
    float dsum = 0;
    int nch = 0;
    float cres[4] = {0, 0, 0, 0};
    for (int s = 0; s < 4; ++s) {
      const uint c = nodes[ni].child[s];
      if (!((desc >> s) & 1u)) {
        if (c == kEmpty) break;
        ++nch;
        continue;
      }
      if (c == kEmpty) {
        desc &= (1u << s) - 1u;
        break;
      }
      ++nch;
      if (c & kInternal) cres[s] = node_angle(c & ~kInternal, q, beta2);
      else cres[s] = tri_angle(vtx(F[c * 3]), vtx(F[c * 3 + 1]), vtx(F[c * 3 + 2]), q);
    }
    dsum = (desc & 1u) ? cres[0] : 0;
    for (int i = 1; i < nch; ++i) dsum += ((desc >> i) & 1u) ? cres[i] : 0;
    return sum + dsum;
  }

  float solid_angle(const float* q, float beta) const {
    if (nodes.empty()) return 0;
    return node_angle(0, q, beta * beta);
  }
};

}  // namespace

extern "C" {

void* oracle_soup_build(const double* V, int64_t nV, const int32_t* F, int64_t nF, int order) {
  Soup* s = new Soup();
  s->build(V, nV, F, nF, order);
  return s;
}

void oracle_soup_eval(void* h, float accuracy_scale, const double* Q, int64_t nQ, double* W,
                      int nthreads) {
  const Soup* s = (const Soup*)h;
  auto one = [&](int64_t p) {
    float q[3] = {(float)Q[p * 3], (float)Q[p * 3 + 1], (float)Q[p * 3 + 2]};
    W[p] = s->solid_angle(q, accuracy_scale) / (4.0 * 3.1415926535897932384626433832795);
  };
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::thread::hardware_concurrency();
  if (nt == 0) nt = 8;
  if (nQ < 1000 || nt <= 1) {
    for (int64_t p = 0; p < nQ; ++p) one(p);
    return;
  }
  const int64_t slice = std::max<int64_t>((int64_t)std::llround((nQ + 1) / (double)nt), 1);
  std::vector<std::thread> pool;
  int64_t i1 = 0, i2 = std::min<int64_t>(slice, nQ);
  unsigned t = 0;
  for (; t + 1 < nt && i1 < nQ; ++t) {
    pool.emplace_back([=, &one] { for (int64_t k = i1; k < i2; ++k) one(k); });
    i1 = i2;
    i2 = std::min<int64_t>(i2 + slice, nQ);
  }
  if (i1 < nQ) pool.emplace_back([=, &one] { for (int64_t k = i1; k < nQ; ++k) one(k); });
  for (auto& th : pool) th.join();
}

int64_t oracle_soup_nodes(void* h) { return (int64_t)((Soup*)h)->nodes.size(); }

// The 4-wide tree: 4 entries per node in the reference's encoding (item
// index, node | 2^31, ~0 for an empty lane); returns the node count.
int64_t oracle_soup_tree(void* h, uint32_t* child) {
  const Soup* s = (const Soup*)h;
  if (child)
    for (size_t i = 0; i < s->nodes.size(); ++i)
      for (int c = 0; c < 4; ++c) child[i * 4 + c] = s->nodes[i].child[c];
  return (int64_t)s->nodes.size();
}

void oracle_soup_free(void* h) { delete (Soup*)h; }

}  // extern "C"
