// CPU oracle for the triangle-soup fast winding number (TEST INFRASTRUCTURE
// ONLY; used by tests/ and the bench CPU baseline, never by libgwn.so).
//
// Restates, in FP64 over plain arrays, the HDK solid-angle algorithm that
// libigl vendors in include/igl/FastWindingNumberForSoups.h:
//   * per-triangle data (item(), FWNFS.h:6668-6890): area-weighted normal,
//     centroid, and the second-moment integrals behind Nijk;
//   * node data about the node's area-weighted average point, with the
//     parallel-axis shifts of post() (FWNFS.h:6892-7118), here applied to all
//     of a node's triangles at once (a flat sum, independent of any merge
//     order) -- used to check a tree's stored moments;
//   * the far field of pre() (FWNFS.h:7176-7259) and the exact triangle term
//     UTsignedSolidAngleTri (FWNFS.h:6070-6110), walked over a given
//     pre-order tree (root always opened, open iff |q-P|^2 <= maxP2 beta^2,
//     non-finite far field forces opening) -- the semantics of
//     computeSolidAngle (FWNFS.h:7148-7284) on that tree.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct Leaf {
  double P[3], area, N[3], lo[3], hi[3];
  double Niii[3], perm, c2[6];
};

void integrals(const double* a, const double* b, const double* c, const double* P, double* ii,
               double* ij, double* ik, int i) {
  double oab[3], oac[3], ocb[3];
  for (int d = 0; d < 3; ++d) {
    oab[d] = b[d] - a[d];
    oac[d] = c[d] - a[d];
    ocb[d] = b[d] - c[d];
  }
  const double t = oab[i] / oac[i];
  const int j = (i == 2) ? 0 : i + 1, k = (j == 2) ? 0 : j + 1;
  const double jd = t * oac[j] - oab[j], kd = t * oac[k] - oab[k];
  const double xa[3] = {jd * oab[k] - kd * oab[j], kd * oab[i], jd * oab[i]};
  const double xc[3] = {jd * ocb[k] - kd * ocb[j], kd * ocb[i], jd * ocb[i]};
  const double sa = std::sqrt(xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
  const double sc = std::sqrt(xc[0] * xc[0] + xc[1] * xc[1] + xc[2] * xc[2]);
  const double Pai = a[i] - P[i], Pci = c[i] - P[i];
  *ii = sa * (0.5 * Pai * Pai + (2.0 / 3.0) * Pai * oab[i] + 0.25 * oab[i] * oab[i]) +
        sc * (0.5 * Pci * Pci + (2.0 / 3.0) * Pci * ocb[i] + 0.25 * ocb[i] * ocb[i]);
  const int jks[2] = {j, k};
  const double diffs[2] = {jd, kd};
  double* outs[2] = {ij, ik};
  for (int s = 0; s < 2; ++s) {
    if (!outs[s]) continue;
    const int jk = jks[s];
    const double mid = b[jk] + 0.5 * diffs[s];
    const double am = mid - a[jk], cm = mid - c[jk];
    const double Paj = a[jk] - P[jk], Pcj = c[jk] - P[jk];
    *outs[s] = sa * (0.5 * Pai * Paj + (1.0 / 3.0) * Pai * am + (1.0 / 3.0) * Paj * oab[i] +
                     0.25 * oab[i] * am) +
               sc * (0.5 * Pci * Pcj + (1.0 / 3.0) * Pci * cm + (1.0 / 3.0) * Pcj * ocb[i] +
                     0.25 * ocb[i] * cm);
  }
}

void order3(const double* v[3], int ax, int o[3]) {
  o[0] = 0, o[1] = 1, o[2] = 2;
  if (v[0][ax] > v[1][ax]) std::swap(o[0], o[1]);
  if (v[o[0]][ax] > v[2][ax]) std::swap(o[0], o[2]);
  if (v[o[1]][ax] > v[o[2]][ax]) std::swap(o[1], o[2]);
}

Leaf leaf_data(const double* a, const double* b, const double* c) {
  Leaf L;
  double ab[3], ac[3];
  for (int d = 0; d < 3; ++d) {
    ab[d] = b[d] - a[d];
    ac[d] = c[d] - a[d];
    L.lo[d] = std::fmin(a[d], std::fmin(b[d], c[d]));
    L.hi[d] = std::fmax(a[d], std::fmax(b[d], c[d]));
    L.P[d] = (a[d] + b[d] + c[d]) / 3;
    L.Niii[d] = 0;
  }
  L.N[0] = 0.5 * (ab[1] * ac[2] - ab[2] * ac[1]);
  L.N[1] = 0.5 * (ab[2] * ac[0] - ab[0] * ac[2]);
  L.N[2] = 0.5 * (ab[0] * ac[1] - ab[1] * ac[0]);
  L.area = std::sqrt(L.N[0] * L.N[0] + L.N[1] * L.N[1] + L.N[2] * L.N[2]);
  L.perm = 0;
  for (double& x : L.c2) x = 0;
  if (L.area == 0) return L;
  const double n[3] = {L.N[0] / L.area, L.N[1] / L.area, L.N[2] / L.area};
  const double* v[3] = {a, b, c};
  int ox[3], oy[3], oz[3];
  order3(v, 0, ox);
  order3(v, 1, oy);
  order3(v, 2, oz);
  const double dx = v[ox[2]][0] - v[ox[0]][0], dy = v[oy[2]][1] - v[oy[0]][1],
               dz = v[oz[2]][2] - v[oz[0]][2];
  double xx = 0, xy = 0, yy = 0, yz = 0, zz = 0, zx = 0;
  if (dx > 0)
    integrals(v[ox[0]], v[ox[1]], v[ox[2]], L.P, &xx, (dx >= dy && dy > 0) ? &xy : nullptr,
              (dx >= dz && dz > 0) ? &zx : nullptr, 0);
  if (dy > 0)
    integrals(v[oy[0]], v[oy[1]], v[oy[2]], L.P, &yy, (dy >= dz && dz > 0) ? &yz : nullptr,
              (dx < dy && dx > 0) ? &xy : nullptr, 1);
  if (dz > 0)
    integrals(v[oz[0]], v[oz[1]], v[oz[2]], L.P, &zz, (dx < dz && dx > 0) ? &zx : nullptr,
              (dy < dz && dy > 0) ? &yz : nullptr, 2);
  L.Niii[0] = xx * n[0];
  L.Niii[1] = yy * n[1];
  L.Niii[2] = zz * n[2];
  L.perm = 2 * (n[0] * yz + n[1] * zx + n[2] * xy);
  L.c2[0] = 2 * (n[0] * xy) + n[1] * xx;
  L.c2[1] = 2 * (n[0] * zx) + n[2] * xx;
  L.c2[2] = 2 * (n[1] * yz) + n[2] * yy;
  L.c2[3] = 2 * (n[1] * xy) + n[0] * yy;
  L.c2[4] = 2 * (n[2] * zx) + n[0] * zz;
  L.c2[5] = 2 * (n[2] * yz) + n[1] * zz;
  return L;
}

// Node record in the exported 24-double layout.
void node_from_leaves(const std::vector<Leaf>& ls, double* out) {
  double area = 0, areaP[3] = {0, 0, 0}, N[3] = {0, 0, 0}, lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = INFINITY;
    hi[d] = -INFINITY;
  }
  for (const Leaf& L : ls) {
    area += L.area;
    for (int d = 0; d < 3; ++d) {
      areaP[d] += L.P[d] * L.area;
      N[d] += L.N[d];
      lo[d] = std::fmin(lo[d], L.lo[d]);
      hi[d] = std::fmax(hi[d], L.hi[d]);
    }
  }
  double P[3];
  for (int d = 0; d < 3; ++d) P[d] = area > 0 ? areaP[d] / area : 0.5 * (lo[d] + hi[d]);
  if (ls.size() == 1)  // a triangle's own average point is its centroid (FWNFS.h:6685)
    for (int d = 0; d < 3; ++d) P[d] = ls[0].P[d];
  double Nii[3] = {0, 0, 0}, Nxy = 0, Nyx = 0, Nyz = 0, Nzy = 0, Nzx = 0, Nxz = 0;
  double Niii[3] = {0, 0, 0}, perm = 0, c2[6] = {0, 0, 0, 0, 0, 0};
  for (const Leaf& L : ls) {
    // leaf first moments about its centroid are zero; shift to P
    const double dx = L.P[0] - P[0], dy = L.P[1] - P[1], dz = L.P[2] - P[2];
    const double* n = L.N;
    Nii[0] += n[0] * dx;
    Nii[1] += n[1] * dy;
    Nii[2] += n[2] * dz;
    const double lxy = n[0] * dy, lyx = n[1] * dx, lyz = n[1] * dz, lzy = n[2] * dy,
                 lzx = n[2] * dx, lxz = n[0] * dz;
    Nxy += lxy, Nyx += lyx, Nyz += lyz, Nzy += lzy, Nzx += lzx, Nxz += lxz;
    Niii[0] += L.Niii[0] + dx * dx * n[0];
    Niii[1] += L.Niii[1] + dy * dy * n[1];
    Niii[2] += L.Niii[2] + dz * dz * n[2];
    perm += L.perm + (dx * (lyz + lzy) + dy * (lzx + lxz) + dz * (lxy + lyx));
    c2[0] += L.c2[0] + 2 * (n[0] * dx * dy) + n[1] * dx * dx;
    c2[1] += L.c2[1] + 2 * (n[0] * dx * dz) + n[2] * dx * dx;
    c2[2] += L.c2[2] + 2 * (n[1] * dy * dz) + n[2] * dy * dy;
    c2[3] += L.c2[3] + 2 * (n[1] * dy * dx) + n[0] * dy * dy;
    c2[4] += L.c2[4] + 2 * (n[2] * dz * dx) + n[0] * dz * dz;
    c2[5] += L.c2[5] + 2 * (n[2] * dz * dy) + n[1] * dz * dz;
  }
  double mp2 = 0;
  for (int d = 0; d < 3; ++d) {
    const double m = std::fmax(P[d] - lo[d], hi[d] - P[d]);
    mp2 += m * m;
  }
  double r[24] = {P[0], P[1], P[2], mp2, N[0], N[1], N[2], Nii[0], Nii[1], Nii[2],
                  Nxy + Nyx, Nyz + Nzy, Nzx + Nxz, Niii[0], Niii[1], Niii[2], perm,
                  c2[0], c2[1], c2[2], c2[3], c2[4], c2[5], 0};
  std::memcpy(out, r, 23 * sizeof(double));
}

double far_field(const double* m, double dx, double dy, double dz, double r2, int order) {
  const double m2 = 1.0 / r2, m1 = std::sqrt(m2);
  const double qx = dx * m1, qy = dy * m1, qz = dz * m1;
  double om = -m2 * (qx * m[4] + qy * m[5] + qz * m[6]);
  if (order >= 1) {
    const double q2x = qx * qx, q2y = qy * qy, q2z = qz * qz, m3 = m2 * m1;
    om += m3 * (m[7] + m[8] + m[9] -
                3.0 * (q2x * m[7] + q2y * m[8] + q2z * m[9] + qx * qy * m[10] + qx * qz * m[12] +
                       qy * qz * m[11]));
    if (order >= 2) {
      const double m4 = m2 * m2;
      const double* c2 = m + 17;
      const double t0x = c2[3] + c2[4], t0y = c2[5] + c2[0], t0z = c2[1] + c2[2];
      const double t1x = qy * c2[0] + qz * c2[1], t1y = qz * c2[2] + qx * c2[3],
                   t1z = qx * c2[4] + qy * c2[5];
      om += m4 * (1.5 * (qx * (3 * m[13] + t0x) + qy * (3 * m[14] + t0y) + qz * (3 * m[15] + t0z)) -
                  7.5 * (q2x * qx * m[13] + q2y * qy * m[14] + q2z * qz * m[15] +
                         qx * qy * qz * m[16] + q2x * t1x + q2y * t1y + q2z * t1z));
    }
  }
  return om;
}

double tri_solid_angle(const double* a, const double* b, const double* c, const double* q) {
  double qa[3], qb[3], qc[3];
  for (int d = 0; d < 3; ++d) {
    qa[d] = a[d] - q[d];
    qb[d] = b[d] - q[d];
    qc[d] = c[d] - q[d];
  }
  const double la = std::sqrt(qa[0] * qa[0] + qa[1] * qa[1] + qa[2] * qa[2]);
  const double lb = std::sqrt(qb[0] * qb[0] + qb[1] * qb[1] + qb[2] * qb[2]);
  const double lc = std::sqrt(qc[0] * qc[0] + qc[1] * qc[1] + qc[2] * qc[2]);
  if (la == 0 || lb == 0 || lc == 0) return 0;
  for (int d = 0; d < 3; ++d) {
    qa[d] /= la;
    qb[d] /= lb;
    qc[d] /= lc;
  }
  const double u[3] = {qb[0] - qa[0], qb[1] - qa[1], qb[2] - qa[2]};
  const double v[3] = {qc[0] - qa[0], qc[1] - qa[1], qc[2] - qa[2]};
  const double num = qa[0] * (u[1] * v[2] - u[2] * v[1]) + qa[1] * (u[2] * v[0] - u[0] * v[2]) +
                     qa[2] * (u[0] * v[1] - u[1] * v[0]);
  if (num == 0) return 0;
  const double den = 1 + (qa[0] * qb[0] + qa[1] * qb[1] + qa[2] * qb[2]) +
                     (qa[0] * qc[0] + qa[1] * qc[1] + qa[2] * qc[2]) +
                     (qb[0] * qc[0] + qb[1] * qc[1] + qb[2] * qc[2]);
  return 2 * std::atan2(num, den);
}

inline int64_t link_of(const double* rec) {
  int64_t l;
  std::memcpy(&l, rec + 23, sizeof(l));
  return l;
}

}  // namespace

extern "C" {

// Recompute every node's moments of a binary pre-order tree from its
// triangles: leaves by item() (FWNFS.h:6668-6890), internal nodes by the
// two-child post() merge (FWNFS.h:6892-7118, parallel-axis shifts exactly as
// written there), children = x+1 and the node after x+1's subtree.
// out is nnodes x 24 (slot 23 left 0).
void oracle_soup_tree_moments(const double* V, const int32_t* F, const double* nodes,
                              int64_t nnodes, const int32_t* tri_index, double* out) {
  struct Loc {
    double P[3], area, areaP[3], N[3], lo[3], hi[3];
    double Nii[3], Nxy, Nyx, Nyz, Nzy, Nzx, Nxz, Niii[3], perm, c2[6];
  };
  std::vector<Loc> M((size_t)nnodes);
  auto end_of = [&](int64_t x) {
    const int64_t l = link_of(nodes + x * 24);
    return l < 0 ? x + 1 : l;
  };
  for (int64_t x = nnodes - 1; x >= 0; --x) {
    const int64_t l = link_of(nodes + x * 24);
    Loc& m = M[(size_t)x];
    if (l < 0) {
      const int32_t f = tri_index[~l];
      const Leaf L = leaf_data(V + (int64_t)F[f * 3] * 3, V + (int64_t)F[f * 3 + 1] * 3,
                               V + (int64_t)F[f * 3 + 2] * 3);
      for (int d = 0; d < 3; ++d) {
        m.P[d] = L.P[d];
        m.areaP[d] = L.P[d] * L.area;
        m.N[d] = L.N[d];
        m.lo[d] = L.lo[d];
        m.hi[d] = L.hi[d];
        m.Nii[d] = 0;
        m.Niii[d] = L.Niii[d];
      }
      m.area = L.area;
      m.Nxy = m.Nyx = m.Nyz = m.Nzy = m.Nzx = m.Nxz = 0;
      m.perm = L.perm;
      for (int k = 0; k < 6; ++k) m.c2[k] = L.c2[k];
      continue;
    }
    const Loc* ch[2] = {&M[(size_t)(x + 1)], &M[(size_t)end_of(x + 1)]};
    m.area = ch[0]->area + ch[1]->area;
    for (int d = 0; d < 3; ++d) {
      m.N[d] = ch[0]->N[d] + ch[1]->N[d];
      m.areaP[d] = ch[0]->areaP[d] + ch[1]->areaP[d];
      m.lo[d] = std::fmin(ch[0]->lo[d], ch[1]->lo[d]);
      m.hi[d] = std::fmax(ch[0]->hi[d], ch[1]->hi[d]);
    }
    for (int d = 0; d < 3; ++d) m.P[d] = m.area > 0 ? m.areaP[d] / m.area : 0.5 * (m.lo[d] + m.hi[d]);
    for (int d = 0; d < 3; ++d) m.Nii[d] = m.Niii[d] = 0;
    m.Nxy = m.Nyx = m.Nyz = m.Nzy = m.Nzx = m.Nxz = 0;
    m.perm = 0;
    for (int k = 0; k < 6; ++k) m.c2[k] = 0;
    for (int c = 0; c < 2; ++c) {
      const Loc& C = *ch[c];
      const double dx = C.P[0] - m.P[0], dy = C.P[1] - m.P[1], dz = C.P[2] - m.P[2];
      const double* N = C.N;
      m.Nii[0] += C.Nii[0] + N[0] * dx;
      m.Nii[1] += C.Nii[1] + N[1] * dy;
      m.Nii[2] += C.Nii[2] + N[2] * dz;
      const double Nxy = C.Nxy + N[0] * dy, Nyx = C.Nyx + N[1] * dx, Nyz = C.Nyz + N[1] * dz,
                   Nzy = C.Nzy + N[2] * dy, Nzx = C.Nzx + N[2] * dx, Nxz = C.Nxz + N[0] * dz;
      m.Nxy += Nxy, m.Nyx += Nyx, m.Nyz += Nyz, m.Nzy += Nzy, m.Nzx += Nzx, m.Nxz += Nxz;
      m.Niii[0] += C.Niii[0] + 2 * dx * C.Nii[0] + dx * dx * N[0];
      m.Niii[1] += C.Niii[1] + 2 * dy * C.Nii[1] + dy * dy * N[1];
      m.Niii[2] += C.Niii[2] + 2 * dz * C.Nii[2] + dz * dz * N[2];
      m.perm += C.perm + (dx * (Nyz + Nzy) + dy * (Nzx + Nxz) + dz * (Nxy + Nyx));
      m.c2[0] += C.c2[0] + 2 * (dy * C.Nii[0] + dx * C.Nxy + N[0] * dx * dy) + 2 * C.Nyx * dx + N[1] * dx * dx;
      m.c2[1] += C.c2[1] + 2 * (dz * C.Nii[0] + dx * C.Nxz + N[0] * dx * dz) + 2 * C.Nzx * dx + N[2] * dx * dx;
      m.c2[2] += C.c2[2] + 2 * (dz * C.Nii[1] + dy * C.Nyz + N[1] * dy * dz) + 2 * C.Nzy * dy + N[2] * dy * dy;
      m.c2[3] += C.c2[3] + 2 * (dx * C.Nii[1] + dy * C.Nyx + N[1] * dy * dx) + 2 * C.Nxy * dy + N[0] * dy * dy;
      m.c2[4] += C.c2[4] + 2 * (dx * C.Nii[2] + dz * C.Nzx + N[2] * dz * dx) + 2 * C.Nxz * dz + N[0] * dz * dz;
      m.c2[5] += C.c2[5] + 2 * (dy * C.Nii[2] + dz * C.Nzy + N[2] * dz * dy) + 2 * C.Nyz * dz + N[1] * dz * dz;
    }
  }
  for (int64_t x = 0; x < nnodes; ++x) {
    const Loc& m = M[(size_t)x];
    double mp2 = 0;
    for (int d = 0; d < 3; ++d) {
      const double e = std::fmax(m.P[d] - m.lo[d], m.hi[d] - m.P[d]);
      mp2 += e * e;
    }
    const double r[24] = {m.P[0], m.P[1], m.P[2], mp2, m.N[0], m.N[1], m.N[2], m.Nii[0], m.Nii[1],
                          m.Nii[2], m.Nxy + m.Nyx, m.Nyz + m.Nzy, m.Nzx + m.Nxz, m.Niii[0],
                          m.Niii[1], m.Niii[2], m.perm, m.c2[0], m.c2[1], m.c2[2], m.c2[3],
                          m.c2[4], m.c2[5], 0};
    std::memcpy(out + x * 24, r, sizeof(r));
  }
}

// Grouping-independent node moments: every node's triangles shifted to its
// average point at once with the exact parallel-axis identities (used to
// measure how far the reference's merge formula drifts from them).
void oracle_soup_tree_moments_flat(const double* V, const int32_t* F, const double* nodes,
                                   int64_t nnodes, const int32_t* tri_index, double* out) {
  std::vector<int64_t> leaf_prefix(nnodes + 1, 0);
  for (int64_t x = 0; x < nnodes; ++x) leaf_prefix[x + 1] = leaf_prefix[x] + (link_of(nodes + x * 24) < 0);
  for (int64_t x = 0; x < nnodes; ++x) {
    const int64_t l = link_of(nodes + x * 24);
    const int64_t end = l < 0 ? x + 1 : l;
    std::vector<Leaf> ls;
    for (int64_t s = leaf_prefix[x]; s < leaf_prefix[end]; ++s) {
      const int32_t f = tri_index[s];
      ls.push_back(leaf_data(V + (int64_t)F[f * 3] * 3, V + (int64_t)F[f * 3 + 1] * 3,
                             V + (int64_t)F[f * 3 + 2] * 3));
    }
    node_from_leaves(ls, out + x * 24);
    out[x * 24 + 23] = 0;
  }
}

// FP64 evaluation of W on a pre-order tree (computeSolidAngle semantics).
void oracle_soup_tree_eval(const double* V, const int32_t* F, const double* nodes,
                           int64_t nnodes, const int32_t* tri_index, int order,
                           float accuracy_scale, const double* Q, int64_t nQ, double* W,
                           int nthreads) {
  const double beta2 = (double)accuracy_scale * (double)accuracy_scale;
  auto one = [&](int64_t qi) {
    const double* q = Q + qi * 3;
    double acc = 0;
    int64_t x = 0;
    while (x < nnodes) {
      const double* r = nodes + x * 24;
      const int64_t link = link_of(r);
      const bool leaf = link < 0;
      if (x == 0 && !leaf) {
        ++x;
        continue;
      }
      const double dx = q[0] - r[0], dy = q[1] - r[1], dz = q[2] - r[2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      const double r2p = std::fma(dz, dz, std::fma(dy, dy, dx * dx));
      bool open = r2p <= r[3] * beta2;
      if (!open) {
        const double om = far_field(r, dx, dy, dz, r2, order);
        if (std::isfinite(om)) {
          acc += om;
          x = leaf ? x + 1 : link;
          continue;
        }
        open = true;
      }
      if (leaf) {
        const int32_t f = tri_index[~link];
        acc += tri_solid_angle(V + (int64_t)F[f * 3] * 3, V + (int64_t)F[f * 3 + 1] * 3,
                               V + (int64_t)F[f * 3 + 2] * 3, q);
      }
      ++x;
    }
    W[qi] = acc / (4.0 * 3.1415926535897932384626433832795);
  };
  unsigned nt = nthreads > 0 ? (unsigned)nthreads : std::thread::hardware_concurrency();
  if (nt == 0) nt = 8;
  std::vector<std::thread> pool;
  const int64_t chunk = (nQ + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    const int64_t b = t * chunk, e = std::min<int64_t>(nQ, b + chunk);
    if (b >= e) break;
    pool.emplace_back([=, &one] {
      for (int64_t i = b; i < e; ++i) one(i);
    });
  }
  for (auto& th : pool) th.join();
}

// HDK per-triangle data of one triangle, 24-double layout (for tests).
void oracle_soup_leaf(const double* a, const double* b, const double* c, double* out) {
  std::vector<Leaf> ls{leaf_data(a, b, c)};
  node_from_leaves(ls, out);
}

}  // extern "C"
