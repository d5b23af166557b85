"""Seeded synthetic meshes, point clouds and query sets for the benchmark
workloads (no public dataset is involved; these generators are the whole
input specification):

* icosphere(k): icosahedron with k midpoint subdivisions (10*4^k+2 vertices,
  20*4^k triangles), outward-oriented.
* geodesic_sphere(nu): nu-frequency geodesic icosphere (20*nu^2 triangles).
* sh_deform: radial displacement by a random real spherical-harmonic field of
  degree 1..lmax with coefficients N(0, sigma/l).
* delete_random_faces / delete_patch: open holes.
* torus_cloud: area-uniform torus samples with jittered normals and areas.
* exact_workload / soup_workload / cloud_workload / precision_workload /
  served_meshes: the five benchmark configurations.
* loops2d / loops2d_queries: closed wavy 2-D polygons (outer loops, holes
  and doubled loops) for the 2-D segment winding number.
* swept_workload: a deformed ellipsoid under a screw motion and the grid
  around its sweep, for swept-volume signed distances.
"""
from __future__ import annotations

import math

import numpy as np

_PHI = (1.0 + math.sqrt(5.0)) / 2.0


def _icosahedron():
    V = np.array([[-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
                  [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
                  [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]], float)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    return V, _orient_outward(V, F)


def _orient_outward(V, F):
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, (a + b + c) / 3.0) < 0
    F = F.copy()
    F[flip] = F[flip][:, [0, 2, 1]]
    return F


def icosphere(k: int):
    """Unit icosphere by k midpoint subdivisions (vertices projected to r=1)."""
    V, F = _icosahedron()
    for _ in range(k):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (V.shape[0] + 1) + e[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        u0, u1 = uk // (V.shape[0] + 1), uk % (V.shape[0] + 1)
        mid = V[u0] + V[u1]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + V.shape[0]  # midpoints of edges 01, 12, 20
        V = np.concatenate([V, mid])
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        F = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return V, F.astype(np.int32)


def geodesic_sphere(nu: int):
    """nu-frequency geodesic icosphere: 20*nu^2 triangles, 10*nu^2+2 vertices."""
    V0, F0 = _icosahedron()
    ii, jj = np.meshgrid(np.arange(nu + 1), np.arange(nu + 1), indexing="ij")
    mask = ii + jj <= nu
    ii, jj = ii[mask], jj[mask]
    lut = -np.ones((nu + 1, nu + 1), np.int64)
    lut[ii, jj] = np.arange(ii.size)
    # local triangles on the (i, j) lattice
    tris = []
    for i in range(nu):
        for j in range(nu - i):
            tris.append((lut[i, j], lut[i + 1, j], lut[i, j + 1]))
            if i + j < nu - 1:
                tris.append((lut[i + 1, j], lut[i + 1, j + 1], lut[i, j + 1]))
    tris = np.array(tris, np.int64)
    wa = (nu - ii - jj) / nu
    wb = ii / nu
    wc = jj / nu
    P = (wa[None, :, None] * V0[F0[:, 0]][:, None, :] + wb[None, :, None] * V0[F0[:, 1]][:, None, :]
         + wc[None, :, None] * V0[F0[:, 2]][:, None, :])  # 20 x npts x 3
    npts = ii.size
    allP = P.reshape(-1, 3)
    allF = (tris[None, :, :] + (np.arange(20) * npts)[:, None, None]).reshape(-1, 3)
    key = np.round(allP * 1e9).astype(np.int64)
    # unique rows in lexicographic order (first occurrence kept), as
    # np.unique(key, axis=0) orders them, via a stable numeric lexsort
    order = np.lexsort((key[:, 2], key[:, 1], key[:, 0]))
    ks = key[order]
    new_grp = np.ones(ks.shape[0], bool)
    new_grp[1:] = np.any(ks[1:] != ks[:-1], axis=1)
    gid = np.cumsum(new_grp) - 1
    first = order[new_grp]
    inv = np.empty(key.shape[0], np.int64)
    inv[order] = gid
    V = allP[first]
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = inv[allF]
    return V, _orient_outward(V, F).astype(np.int32)


def _real_sh(lmax: int, theta: np.ndarray, phi: np.ndarray):
    """Orthonormal real spherical harmonics Y_lm, l=1..lmax, as (nY, npts)."""
    x = np.cos(theta)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    out = []
    # associated Legendre P_l^m via the standard three-term recurrences
    Pmm = np.ones_like(x)
    P = {}
    for m in range(lmax + 1):
        if m > 0:
            Pmm = -(2 * m - 1) * s * Pmm
        P[(m, m)] = Pmm
        if m + 1 <= lmax:
            P[(m + 1, m)] = x * (2 * m + 1) * Pmm
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * x * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    for l in range(1, lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            nrm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            if m == 0:
                out.append(nrm * P[(l, 0)])
            elif m > 0:
                out.append(math.sqrt(2) * nrm * P[(l, am)] * np.cos(am * phi))
            else:
                out.append(math.sqrt(2) * nrm * P[(l, am)] * np.sin(am * phi))
    return np.array(out)


def sh_deform(V, rng, lmax: int = 8, sigma: float = 0.05):
    """Radial displacement r = 1 + sum_{l=1..lmax} sum_m c_lm Y_lm, c_lm ~ N(0, sigma/l).
    (l = 0 is excluded: sigma/0 is undefined.)"""
    r0 = np.linalg.norm(V, axis=1)
    u = V / r0[:, None]
    theta = np.arccos(np.clip(u[:, 2], -1, 1))
    phi = np.arctan2(u[:, 1], u[:, 0])
    Y = _real_sh(lmax, theta, phi)
    coef = np.concatenate([rng.normal(0.0, sigma / l, size=2 * l + 1) for l in range(1, lmax + 1)])
    r = 1.0 + coef @ Y
    return u * r[:, None]


def delete_random_faces(F, rng, frac: float):
    keep = rng.random(F.shape[0]) >= frac
    return F[keep]


def face_adjacency(F):
    """Edge-adjacent faces in CSR form (offsets, neighbours); each face's
    neighbours in the order the edge pairs are found, as lists of the same
    order would hold them."""
    e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]).astype(np.int64)
    fid = np.tile(np.arange(F.shape[0]), 3)
    e.sort(axis=1)
    key = e[:, 0] * (int(F.max()) + 1) + e[:, 1]
    order = np.argsort(key, kind="stable")
    ks, fs = key[order], fid[order]
    same = ks[1:] == ks[:-1]
    a, b = fs[:-1][same], fs[1:][same]
    # pair k appends b to a's list and a to b's list: sort the (owner, k)
    # entries stably by owner to get each list in pair order
    owner = np.stack([a, b], 1).reshape(-1)
    other = np.stack([b, a], 1).reshape(-1)
    srt = np.argsort(owner, kind="stable")
    off = np.zeros(F.shape[0] + 1, np.int64)
    np.add.at(off, owner + 1, 1)
    return np.cumsum(off), other[srt]


def delete_patch(F, rng, nfaces: int):
    """Remove one connected patch of `nfaces` faces grown by BFS from a seeded face."""
    off, nb = face_adjacency(F)
    start = int(rng.integers(F.shape[0]))
    seen = {start}
    order = [start]
    head = 0
    while len(order) < nfaces and head < len(order):
        f = order[head]
        head += 1
        for g in nb[off[f]:off[f + 1]].tolist():
            if g not in seen and len(order) < nfaces:
                seen.add(g)
                order.append(g)
    keep = np.ones(F.shape[0], bool)
    keep[order] = False
    return F[keep]


def face_normals(V, F):
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    return n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-300)


def vertex_normals(V, F):
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    vn = np.zeros_like(V)
    for c in range(3):
        np.add.at(vn, F[:, c], n)
    return vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-300)


def sample_on_faces(V, F, rng, n):
    f = rng.integers(F.shape[0], size=n)
    u, v = rng.random(n), rng.random(n)
    flip = u + v > 1
    u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
    a, b, c = V[F[f, 0]], V[F[f, 1]], V[F[f, 2]]
    return a + u[:, None] * (b - a) + v[:, None] * (c - a), f


# -------------------------------------------------------------- workloads --
def exact_workload(seed: int = 0, subdiv: int = 4, nq: int = 100_000):
    """Closed icosphere (subdiv 4: 2562 V / 5120 F), radial noise N(0,0.02),
    queries uniform in [-1.5,1.5]^3 (f64)."""
    rng = np.random.default_rng(seed)
    V, F = icosphere(subdiv)
    V = V * (1.0 + rng.normal(0.0, 0.02, size=V.shape[0]))[:, None]
    Q = rng.uniform(-1.5, 1.5, size=(nq, 3))
    return V, F, Q


def soup_mesh(seed: int = 1, subdiv: int = 8, delete_frac: float = 0.01):
    """SH-deformed icosphere (subdiv 8: 1,310,720 F) with 1% of faces deleted."""
    rng = np.random.default_rng(seed)
    V, F = icosphere(subdiv)
    V = sh_deform(V, rng)
    F = delete_random_faces(F, rng, delete_frac)
    return V, F


def soup_queries(V, F, seed: int = 2, nq: int = 10_000_000, near_frac: float = 0.1):
    """90% uniform in the bbox scaled 1.2x about its centre; 10% on a random
    face, offset +-10^U(-4,-1) along the face normal."""
    rng = np.random.default_rng(seed)
    lo, hi = V.min(0), V.max(0)
    c, h = (lo + hi) / 2, (hi - lo) / 2 * 1.2
    n_near = int(round(nq * near_frac))
    n_far = nq - n_near
    Qf = c + rng.uniform(-1, 1, size=(n_far, 3)) * h
    P, f = sample_on_faces(V, F, rng, n_near)
    nrm = face_normals(V, F[f])
    d = 10.0 ** rng.uniform(-4, -1, size=n_near) * rng.choice([-1.0, 1.0], size=n_near)
    Qn = P + nrm * d[:, None]
    Q = np.concatenate([Qf, Qn])
    return Q[rng.permutation(nq)]


def torus_cloud(seed: int = 3, n: int = 2_000_000, R: float = 1.0, r: float = 0.35):
    """Area-uniform torus samples (rejection on (R + r cos v)/(R + r)), radial
    tube offset N(0,0.005), analytic normals with N(0,0.05) tangent jitter,
    areas (4 pi^2 R r / n) * U(0.8,1.2)."""
    rng = np.random.default_rng(seed)
    us, vs = [], []
    need = n
    while need > 0:
        m = int(need * 1.6) + 16
        u = rng.uniform(0, 2 * np.pi, m)
        v = rng.uniform(0, 2 * np.pi, m)
        acc = rng.random(m) < (R + r * np.cos(v)) / (R + r)
        us.append(u[acc][:need])
        vs.append(v[acc][:need])
        need -= int(min(acc.sum(), need))
    u, v = np.concatenate(us), np.concatenate(vs)
    rr = r + rng.normal(0, 0.005, n)
    P = np.stack([(R + rr * np.cos(v)) * np.cos(u), (R + rr * np.cos(v)) * np.sin(u),
                  rr * np.sin(v)], 1)
    Nn = np.stack([np.cos(v) * np.cos(u), np.cos(v) * np.sin(u), np.sin(v)], 1)
    tu = np.stack([-np.sin(u), np.cos(u), np.zeros_like(u)], 1)
    tv = np.stack([-np.sin(v) * np.cos(u), -np.sin(v) * np.sin(u), np.cos(v)], 1)
    Nn = Nn + rng.normal(0, 0.05, (n, 1)) * tu + rng.normal(0, 0.05, (n, 1)) * tv
    Nn /= np.linalg.norm(Nn, axis=1, keepdims=True)
    A = (4 * np.pi ** 2 * R * r / n) * rng.uniform(0.8, 1.2, n)
    return P, Nn, A


def cloud_queries(seed: int = 4, nq: int = 8_000_000):
    rng = np.random.default_rng(seed)
    return rng.uniform([-1.6, -1.6, -0.6], [1.6, 1.6, 0.6], size=(nq, 3))


def precision_workload(seed: int = 5, nu: int = 158, hole: int = 2000, nq: int = 1_000_000):
    """SH-deformed nu=158 geodesic icosphere (499,280 F) minus a 2000-face
    patch; queries at distances 10^-k (k=1..7) along seeded vertex normals,
    half inside, half outside.  Returns V, F, Q, decade index, side."""
    rng = np.random.default_rng(seed)
    V, F = geodesic_sphere(nu)
    V = sh_deform(V, rng)
    F = delete_patch(F, rng, hole)
    VN = vertex_normals(V, F)
    used = np.unique(F)
    per = nq // 14
    Qs, ks, sides = [], [], []
    for k in range(1, 8):
        for side in (-1.0, 1.0):
            vid = used[rng.integers(used.size, size=per)]
            Qs.append(V[vid] + side * (10.0 ** -k) * VN[vid])
            ks.append(np.full(per, k))
            sides.append(np.full(per, side))
    return V, F, np.concatenate(Qs), np.concatenate(ks), np.concatenate(sides)


def served_meshes(seed: int = 6, count: int = 256, fmin: float = 1e3, fmax: float = 2e6,
                  hole_frac: float = 0.2):
    """Specs of the served workload's meshes: nu = round(sqrt(F/20)) >= 7,
    F_target log-uniform in [fmin, fmax]; 20% get a deleted patch."""
    rng = np.random.default_rng(seed)
    ft = np.exp(rng.uniform(np.log(fmin), np.log(fmax), count))
    nus = np.maximum(7, np.round(np.sqrt(ft / 20.0))).astype(int)
    holes = rng.random(count) < hole_frac
    seeds = rng.integers(0, 2**31 - 1, size=count)
    return [dict(nu=int(n), hole=bool(h), seed=int(s)) for n, h, s in zip(nus, holes, seeds)]


def served_mesh(spec):
    rng = np.random.default_rng(spec["seed"])
    V, F = geodesic_sphere(spec["nu"])
    V = sh_deform(V, rng)
    if spec["hole"]:
        F = delete_patch(F, rng, max(1, F.shape[0] // 100))
    return V, F


def loops2d(seed: int = 7, n_segments: int = 1_000_000, n_cells: int = 16):
    """Closed 2-D polylines on an n_cells x n_cells grid of unit cells.  Cell k
    holds an outer counter-clockwise loop (radius 0.4) and, for k % 3 == 1, a
    clockwise hole (radius 0.18), for k % 3 == 2 a second counter-clockwise
    loop (radius 0.18, winding number 2 inside).  Radii carry a wave
    r(t) = r0 (1 + 0.15 sin(5t + phase) + 0.04 sin(23t)).  Segments are split
    between loops in proportion to their radius.  Returns V (#V x 2 float64)
    and E (#E x 2 int32), each loop's vertices consecutive."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n_cells * n_cells):
        cx, cy = k % n_cells + 0.5, k // n_cells + 0.5
        specs.append((cx, cy, 0.4, 1.0))
        if k % 3 == 1:
            specs.append((cx, cy, 0.18, -1.0))
        elif k % 3 == 2:
            specs.append((cx, cy, 0.18, 1.0))
    radii = np.array([sp[2] for sp in specs])
    counts = np.maximum(8, np.floor(n_segments * radii / radii.sum())).astype(np.int64)
    counts[0] += max(0, n_segments - int(counts.sum()))
    Vs, Es, base = [], [], 0
    for (cx, cy, r0, orient), n in zip(specs, counts):
        t = np.arange(n) * (2 * np.pi / n)
        ph = rng.uniform(0, 2 * np.pi)
        r = r0 * (1 + 0.15 * np.sin(5 * t + ph) + 0.04 * np.sin(23 * t))
        V = np.stack([cx + r * np.cos(t), cy + orient * r * np.sin(t)], axis=1)
        idx = np.arange(n)
        Es.append(np.stack([base + idx, base + (idx + 1) % n], axis=1))
        Vs.append(V)
        base += n
    return np.concatenate(Vs), np.concatenate(Es).astype(np.int32)


def loops2d_queries(n_cells: int = 16, seed: int = 8, nq: int = 10_000_000):
    """Uniform query points over the cells' square, grown by 5% per side."""
    rng = np.random.default_rng(seed)
    lo, hi = -0.05 * n_cells, 1.05 * n_cells
    return rng.uniform(lo, hi, (nq, 2))


def _rotation(axis, ang):
    axis = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


def swept_workload(seed: int = 9, subdiv: int = 5, n_transforms: int = 64, res_max: int = 128):
    """Icosphere (subdiv: 20*4^subdiv triangles) with a random spherical-harmonic
    bump field, scaled to an ellipsoid (1, 0.6, 0.4); n_transforms rigid
    motions x -> L x + t of a screw motion (a turn of 1.5 rad about a tilted
    axis while moving 3 units along x and 0.5 up and down); a grid over the
    sweep's box grown by 0.15, res_max points on the longest side, spacing h
    equal on all sides.  Returns V, F, transforms (nT x 3 x 4), GV, res, h."""
    rng = np.random.default_rng(seed)
    V, F = icosphere(subdiv)
    V = sh_deform(V, rng, lmax=6, sigma=0.06) * np.array([1.0, 0.6, 0.4])
    T = np.zeros((n_transforms, 3, 4))
    for k in range(n_transforms):
        u = k / max(n_transforms - 1, 1)
        T[k, :, :3] = _rotation([0.3, 1.0, 0.2], 1.5 * u)
        T[k, :, 3] = [3.0 * u, 0.5 * np.sin(2 * np.pi * u), 0.3 * u]
    P = np.concatenate([V @ T[k, :, :3].T + T[k, :, 3] for k in range(n_transforms)])
    lo, hi = P.min(0) - 0.15, P.max(0) + 0.15
    h = float((hi - lo).max() / (res_max - 1))
    res = np.floor((hi - lo) / h).astype(np.int32) + 1
    xs = [lo[d] + h * np.arange(res[d]) for d in range(3)]
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    GV = np.ascontiguousarray(np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1))
    return (np.ascontiguousarray(V), np.ascontiguousarray(F, dtype=np.int32), T, GV,
            res.astype(np.int32), h)
