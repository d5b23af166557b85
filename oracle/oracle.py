"""ctypes front end of the CPU oracle (test infrastructure only).

``liboracle.so`` is compiled from ``oracle/gwn_oracle.cpp`` (a restatement of
libigl's FP64 winding-number algorithms); ``oracle/_ref/libref_soup.so`` is the
reference's own soup code compiled from the reference tree, present only where
that tree exists.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline / reference arm use this module, always as the checker or the timed
CPU baseline, never as the thing measured on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_SOUP_PATH = os.path.join(HERE, "_ref", "libref_soup.so")

_SOURCES = ["gwn_oracle.cpp", "soup_port.cpp", "soup_hdk.cpp", "wn_hier.cpp", "distance.cpp", "aabb.cpp", "knn.cpp", "eytzinger.cpp", "swept.cpp",
            "point_areas.cpp"]


def build(force: bool = False) -> str:
    """Compile liboracle.so (g++, no FMA contraction, so results match on x86 and Arm)."""
    srcs = [os.path.join(HERE, s) for s in _SOURCES if os.path.exists(os.path.join(HERE, s))]
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= lib_m for s in srcs):
            return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", *srcs,
           "-o", LIB_PATH, "-lpthread"]
    subprocess.run(cmd, check=True)
    return LIB_PATH


def build_ref() -> str | None:
    """Compile the reference soup wrapper where the reference tree exists."""
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True)
    return REF_SOUP_PATH if os.path.exists(REF_SOUP_PATH) else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        p = C.c_void_p
        i64 = C.c_int64
        L.oracle_winding_number.argtypes = [p, i64, p, i64, C.c_int, p, i64, p, C.c_int]
        L.oracle_winding_number.restype = C.c_int
        L.oracle_solid_angle.argtypes = [p, p, p, p]
        L.oracle_solid_angle.restype = C.c_double
        L.oracle_octree_build.argtypes = [p, i64]
        L.oracle_octree_build.restype = p
        L.oracle_octree_sizes.argtypes = [p, p, p]
        L.oracle_octree_export.argtypes = [p, p, p, p, p, p]
        L.oracle_octree_free.argtypes = [p]
        L.oracle_cloud_precompute.argtypes = [p, p, p, p, p, p, i64, C.c_int, p, p, p, C.c_int]
        L.oracle_cloud_precompute.restype = C.c_int
        L.oracle_cloud_eval.argtypes = [p, p, p, i64, p, p, p, i64, p, p, p, C.c_int, p, i64,
                                        C.c_double, p, C.c_int]
        L.oracle_cloud_eval.restype = C.c_int
        L.oracle_num_threads.argtypes = [C.c_int]
        L.oracle_num_threads.restype = C.c_int
        if hasattr(L, "oracle_soup_build"):
            L.oracle_soup_build.argtypes = [p, i64, p, i64, C.c_int]
            L.oracle_soup_build.restype = p
            L.oracle_soup_eval.argtypes = [p, C.c_float, p, i64, p, C.c_int]
            L.oracle_soup_free.argtypes = [p]
            L.oracle_soup_nodes.argtypes = [p]
            L.oracle_soup_nodes.restype = i64
            L.oracle_soup_tree.argtypes = [p, p]
            L.oracle_soup_tree.restype = i64
        if hasattr(L, "oracle_soup_tree_eval"):
            L.oracle_soup_tree_moments.argtypes = [p, p, p, i64, p, p]
            L.oracle_soup_tree_moments_flat.argtypes = [p, p, p, i64, p, p]
            L.oracle_soup_tree_eval.argtypes = [p, p, p, i64, p, C.c_int, C.c_float, p, i64, p,
                                                C.c_int]
            L.oracle_soup_leaf.argtypes = [p, p, p, p]
        if hasattr(L, "oracle_squared_distance"):
            L.oracle_squared_distance.argtypes = [p, p, i64, p, i64, C.c_double, p, p, p,
                                                  C.c_int]
            L.oracle_squared_distance.restype = C.c_int
            L.oracle_point_triangle.argtypes = [p, p, p, p, p]
            L.oracle_point_triangle.restype = C.c_double
            L.oracle_pseudonormal.argtypes = [p, i64, p, i64, p, i64, p, p, p, p]
            L.oracle_pseudonormal.restype = C.c_int
        if hasattr(L, "oracle_knn"):
            L.oracle_knn.argtypes = [p, i64, p, i64, i64, p, p, p, p, p, p, C.c_int]
            L.oracle_knn.restype = C.c_int
        if hasattr(L, "oracle_aabb_build"):
            L.oracle_aabb_build.argtypes = [p, p, i64]
            L.oracle_aabb_build.restype = p
            L.oracle_aabb_free.argtypes = [p]
            L.oracle_aabb_squared_distance.argtypes = [p, p, i64, C.c_double, p, p, p, C.c_int]
        if hasattr(L, "oracle_eytzinger_aabb"):
            L.oracle_eytzinger_slots.argtypes = [i64]
            L.oracle_eytzinger_slots.restype = i64
            L.oracle_eytzinger_aabb.argtypes = [p, p, i64, C.c_int, C.c_int, p, p, p]
            L.oracle_eytzinger_wn_tree.argtypes = [p, p, i64, C.c_int, p, p]
            L.oracle_eytzinger_wn.argtypes = [p, i64, p, p, p, p, p, i64, p, p, p, C.c_int]
            L.oracle_segments_wn.argtypes = [p, i64, p, p, i64, p]
        if hasattr(L, "oracle_flood_fill"):
            L.oracle_flood_fill.argtypes = [p, p]
        if hasattr(L, "oracle_point_areas"):
            L.oracle_point_areas.argtypes = [p, i64, i64, p, C.c_int, p, p, p, C.c_int]
        if hasattr(L, "oracle_winding_number_hier"):
            L.oracle_winding_number_hier.argtypes = [p, i64, p, i64, p, i64, p, C.c_int]
            L.oracle_winding_number_hier.restype = C.c_int
        _lib = L
    return _lib


def _d(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def num_threads(requested: int = 0) -> int:
    return lib().oracle_num_threads(requested)


def winding_number(V, F, O, nthreads: int = 0) -> np.ndarray:
    """Brute-force exact GWN (FP64), dim taken from F.shape[1] (2 or 3)."""
    V, O = _d(V), _d(O)
    F = _d(F, np.int32)
    dim = F.shape[1]
    W = np.empty(O.shape[0], np.float64)
    rc = lib().oracle_winding_number(_ptr(V), V.shape[0], _ptr(F), F.shape[0], dim, _ptr(O),
                                     O.shape[0], _ptr(W), nthreads)
    if rc:
        raise ValueError("oracle_winding_number failed")
    return W


def winding_number_hier(V, F, O, nthreads: int = 0) -> np.ndarray:
    """Hierarchical exact GWN (restated WindingNumberAABB), 3D only."""
    V, O = _d(V), _d(O)
    F = _d(F, np.int32)
    W = np.empty(O.shape[0], np.float64)
    rc = lib().oracle_winding_number_hier(_ptr(V), V.shape[0], _ptr(F), F.shape[0], _ptr(O),
                                          O.shape[0], _ptr(W), nthreads)
    if rc:
        raise ValueError("oracle_winding_number_hier failed")
    return W


def solid_angle(a, b, c, p) -> float:
    a, b, c, p = (_d(x) for x in (a, b, c, p))
    return lib().oracle_solid_angle(_ptr(a), _ptr(b), _ptr(c), _ptr(p))


class Octree:
    """igl::octree outputs in CSR form: pi_off (ncells+1), pi_idx, CH, CN, W."""

    def __init__(self, pi_off, pi_idx, CH, CN, W):
        self.pi_off, self.pi_idx, self.CH, self.CN, self.W = pi_off, pi_idx, CH, CN, W

    @property
    def ncells(self):
        return self.CH.shape[0]

    def point_indices(self):
        return [self.pi_idx[self.pi_off[c]:self.pi_off[c + 1]].tolist() for c in range(self.ncells)]


def octree(P) -> Octree:
    P = _d(P).reshape(-1, 3)
    L = lib()
    h = L.oracle_octree_build(_ptr(P), P.shape[0])
    try:
        nc, ni = C.c_int64(), C.c_int64()
        L.oracle_octree_sizes(h, C.byref(nc), C.byref(ni))
        nc, ni = nc.value, ni.value
        pi_off = np.empty(nc + 1, np.int64)
        pi_idx = np.empty(max(ni, 1), np.int32)[:ni]
        CH = np.empty((nc, 8), np.int32)
        CN = np.empty((nc, 3), np.float64)
        W = np.empty(nc, np.float64)
        L.oracle_octree_export(h, _ptr(pi_off), _ptr(pi_idx), _ptr(CH), _ptr(CN), _ptr(W))
    finally:
        L.oracle_octree_free(h)
    return Octree(pi_off, pi_idx, CH, CN, W)


def num_terms(order: int) -> int:
    return {0: 3, 1: 12, 2: 39}[order]


def cloud_precompute(P, N, A, tree: Octree, order: int = 2, nthreads: int = 0):
    P, N, A = _d(P), _d(N), _d(A).reshape(-1)
    nc = tree.ncells
    CM = np.empty((nc, 3), np.float64)
    R = np.empty(nc, np.float64)
    EC = np.empty((nc, num_terms(order)), np.float64)
    rc = lib().oracle_cloud_precompute(_ptr(P), _ptr(N), _ptr(A), _ptr(tree.pi_off),
                                       _ptr(tree.pi_idx), _ptr(tree.CH), nc, order, _ptr(CM),
                                       _ptr(R), _ptr(EC), nthreads)
    if rc:
        raise ValueError("oracle_cloud_precompute failed")
    return CM, R, EC


def cloud_eval(P, N, A, tree: Octree, CM, R, EC, Q, beta: float = 2.0, nthreads: int = 0):
    P, N, A, Q = _d(P), _d(N), _d(A).reshape(-1), _d(Q)
    CM, R, EC = _d(CM), _d(R), _d(EC)
    order = {3: 0, 12: 1, 39: 2}[EC.shape[1]]
    W = np.empty(Q.shape[0], np.float64)
    rc = lib().oracle_cloud_eval(_ptr(P), _ptr(N), _ptr(A), P.shape[0], _ptr(tree.pi_off),
                                 _ptr(tree.pi_idx), _ptr(tree.CH), tree.ncells, _ptr(CM), _ptr(R),
                                 _ptr(EC), order, _ptr(Q), Q.shape[0], float(beta), _ptr(W),
                                 nthreads)
    if rc:
        raise ValueError("oracle_cloud_eval failed")
    return W


def cloud_fwn(P, N, A, Q, order: int = 2, beta: float = 2.0, nthreads: int = 0):
    """One-shot point-cloud FWN: octree -> precompute -> eval (fast_winding_number.cpp:320-344)."""
    t = octree(P)
    CM, R, EC = cloud_precompute(P, N, A, t, order, nthreads)
    return cloud_eval(P, N, A, t, CM, R, EC, Q, beta, nthreads)


class SoupPort:
    """CPU restatement of the reference's FP32 soup FWN (oracle/soup_hdk.cpp:
    the UT_BVH<4> build, the HDK moments and computeSolidAngle; equal to the
    compiled reference bit for bit on the committed fixtures)."""

    def __init__(self, V, F, order: int = 2):
        self._V = _d(V)
        self._F = _d(F, np.int32)
        self._h = lib().oracle_soup_build(_ptr(self._V), self._V.shape[0], _ptr(self._F),
                                          self._F.shape[0], order)

    def eval(self, Q, accuracy_scale: float = 2.0, nthreads: int = 0) -> np.ndarray:
        Q = _d(Q)
        W = np.empty(Q.shape[0], np.float64)
        lib().oracle_soup_eval(self._h, float(accuracy_scale), _ptr(Q), Q.shape[0], _ptr(W),
                               nthreads)
        return W

    @property
    def nodes(self) -> int:
        return lib().oracle_soup_nodes(self._h)

    def tree(self) -> np.ndarray:
        """The 4-wide tree, #nodes x 4 uint32 in the reference's encoding."""
        n = lib().oracle_soup_tree(self._h, None)
        out = np.empty((n, 4), np.uint32)
        lib().oracle_soup_tree(self._h, _ptr(out))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_soup_free(self._h)
            self._h = None


_ref = None


def ref_soup_available() -> bool:
    return os.path.exists(REF_SOUP_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SOUP_PATH)
        p = C.c_void_p
        L.ref_soup_build.argtypes = [p, C.c_int64, p, C.c_int64, C.c_int]
        L.ref_soup_build.restype = p
        L.ref_soup_eval.argtypes = [p, C.c_float, p, C.c_int64, p]
        L.ref_soup_free.argtypes = [p]
        L.ref_soup_tree.argtypes = [p, p]
        L.ref_soup_tree.restype = C.c_int64
        _ref = L
    return _ref


class RefSoup:
    """The reference's own UT_SolidAngle soup FWN (only where the reference tree exists)."""

    def __init__(self, V, F, order: int = 2):
        self._V = _d(V)
        self._F = _d(F, np.int32)
        self._h = ref_lib().ref_soup_build(_ptr(self._V), self._V.shape[0], _ptr(self._F),
                                           self._F.shape[0], order)

    def eval(self, Q, accuracy_scale: float = 2.0) -> np.ndarray:
        Q = _d(Q)
        W = np.empty(Q.shape[0], np.float64)
        ref_lib().ref_soup_eval(self._h, float(accuracy_scale), _ptr(Q), Q.shape[0], _ptr(W))
        return W

    def tree(self) -> np.ndarray:
        """The reference's own UT_BVH<4> nodes, #nodes x 4 uint32."""
        n = ref_lib().ref_soup_tree(self._h, None)
        out = np.empty((n, 4), np.uint32)
        ref_lib().ref_soup_tree(self._h, _ptr(out))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            ref_lib().ref_soup_free(self._h)
            self._h = None


def soup_tree_moments(V, F, nodes, tri_index, flat: bool = False) -> np.ndarray:
    """Every node's HDK moments recomputed on the CPU from its triangles:
    two-child post() merges over the given tree, or (flat=True) the
    grouping-independent exact shifts."""
    V, F = _d(V), _d(F, np.int32)
    nodes = _d(nodes)
    tri_index = _d(tri_index, np.int32)
    out = np.zeros_like(nodes)
    fn = lib().oracle_soup_tree_moments_flat if flat else lib().oracle_soup_tree_moments
    fn(_ptr(V), _ptr(F), _ptr(nodes), nodes.shape[0], _ptr(tri_index), _ptr(out))
    return out


def soup_tree_eval(V, F, nodes, tri_index, Q, accuracy_scale: float = 2.0, order: int = 2,
                   nthreads: int = 0) -> np.ndarray:
    """FP64 computeSolidAngle/(4 pi) walked over a given pre-order tree."""
    V, F, Q = _d(V), _d(F, np.int32), _d(Q)
    nodes = _d(nodes)
    tri_index = _d(tri_index, np.int32)
    W = np.empty(Q.shape[0], np.float64)
    lib().oracle_soup_tree_eval(_ptr(V), _ptr(F), _ptr(nodes), nodes.shape[0], _ptr(tri_index),
                                order, float(accuracy_scale), _ptr(Q), Q.shape[0], _ptr(W),
                                nthreads)
    return W


# ----------------------------------------------------------- signed distance --
SIGNED_DISTANCE_TYPE_PSEUDONORMAL = 0
SIGNED_DISTANCE_TYPE_WINDING_NUMBER = 1
SIGNED_DISTANCE_TYPE_DEFAULT = 2
SIGNED_DISTANCE_TYPE_UNSIGNED = 3
SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER = 4


def squared_distance(V, F, P, up_sqr_d: float = np.inf, nthreads: int = 0):
    """Brute-force closest triangle (distance.cpp): (sqrD, I, C)."""
    V, P = _d(V), _d(P)
    F = _d(F, np.int32)
    sqrD = np.empty(P.shape[0])
    I = np.empty(P.shape[0], np.int32)
    Cp = np.empty((P.shape[0], 3))
    lib().oracle_squared_distance(_ptr(V), _ptr(F), F.shape[0], _ptr(P), P.shape[0],
                                  float(up_sqr_d), _ptr(sqrD), _ptr(I), _ptr(Cp), nthreads)
    return sqrD, I, Cp


def signed_distance(P, V, F, sign_type, lower_bound=None, upper_bound=None,
                    return_normals: bool = False):
    """igl::signed_distance(P,V,F,sign_type,lower,upper,S,I,C,N) for 3-D
    triangles, restating include/igl/signed_distance.cpp:372-424 (dispatch,
    empty F) and :83-137 (bounds, per-query sign): (S, I, C) or, with
    return_normals, (S, I, C, N) (N set for the pseudonormal type).  The default
    bounds are the reference's (numeric_limits min / max, :426-440)."""
    P, V = _d(P), _d(V)
    F = _d(F, np.int32)
    nP = P.shape[0]
    if F.shape[0] == 0:
        out = np.full(nP, np.nan), np.full(nP, -1, np.int32), np.full((nP, 3), np.nan)
        return out + (np.full((nP, 3), np.nan),) if return_normals else out
    Nrm = np.zeros((nP, 3))
    lo = np.finfo(np.float64).tiny if lower_bound is None else float(lower_bound)
    hi = np.finfo(np.float64).max if upper_bound is None else float(upper_bound)
    max_abs = max(abs(lo), abs(hi))
    with np.errstate(over="ignore"):
        up2 = float(np.float64(max_abs) ** 2)
    low2 = max(max_abs - (hi - lo), 0.0) ** 2
    sqrD, I, Cp = squared_distance(V, F, P, up2)
    if sign_type in (SIGNED_DISTANCE_TYPE_WINDING_NUMBER, SIGNED_DISTANCE_TYPE_DEFAULT):
        s = 1.0 - 2.0 * winding_number(V, F, P)
    elif sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER:
        # fast_winding_number(fwn_bvh, 2, q) on the float copy of V (:64-65, 113-116)
        w = SoupPort(V.astype(np.float32).astype(np.float64), F, order=2).eval(P, 2.0)
        s = 1.0 - 2.0 * np.abs(w)
    elif sign_type == SIGNED_DISTANCE_TYPE_PSEUDONORMAL:
        s = np.empty(nP)
        lib().oracle_pseudonormal(_ptr(V), V.shape[0], _ptr(F), F.shape[0], _ptr(P), nP, _ptr(I),
                                  _ptr(Cp), _ptr(s), _ptr(Nrm))
    else:
        s = np.ones(nP)
    S = s * np.sqrt(sqrD)
    out = (sqrD >= up2) | (sqrD < low2)
    S[out] = np.nan
    I = I.copy()
    I[out] = F.shape[0] + 1
    Cp[out] = 0.0
    return (S, I, Cp, Nrm) if return_normals else (S, I, Cp)


class AABB:
    """igl::AABB<V,3> over triangles, restated (aabb.cpp): build, then
    squared_distance(P) -> (sqrD, I, C)."""

    def __init__(self, V, F):
        self.V, self.F = _d(V), _d(F, np.int32)
        self._h = lib().oracle_aabb_build(_ptr(self.V), _ptr(self.F), self.F.shape[0])

    def squared_distance(self, P, up_sqr_d: float = np.inf, nthreads: int = 0):
        P = _d(P)
        sqrD = np.empty(P.shape[0])
        I = np.empty(P.shape[0], np.int32)
        Cp = np.empty((P.shape[0], 3))
        lib().oracle_aabb_squared_distance(self._h, _ptr(P), P.shape[0], float(up_sqr_d),
                                           _ptr(sqrD), _ptr(I), _ptr(Cp), nthreads)
        return sqrD, I, Cp

    def __del__(self):
        try:
            lib().oracle_aabb_free(self._h)
        except Exception:
            pass


def knn(P, V, k: int, tree: Octree | None = None, nthreads: int = 0):
    """igl::knn(P,V,k,point_indices,CH,CN,W,I) restated (knn.cpp): the
    reference's best-first search over the octree of V."""
    P, V = _d(P), _d(V)
    if tree is None:
        tree = octree(V)
    cols = min(V.shape[0], int(k))
    I = np.empty((P.shape[0], cols), np.int32)
    lib().oracle_knn(_ptr(P), P.shape[0], _ptr(V), V.shape[0], int(k), _ptr(tree.pi_off),
                     _ptr(tree.pi_idx), _ptr(tree.CH), _ptr(tree.CN), _ptr(tree.W), _ptr(I),
                     nthreads)
    return I


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def eytzinger_aabb(PB1, PB2, median_mode: int = 0):
    """igl::eytzinger_aabb(PB1,PB2,B1,B2,leaf) restated (eytzinger_aabb.cpp);
    median_mode 0 = the reference's igl::median, 1 = exact order statistics.
    Empty slots hold NaN boxes."""
    PB1, PB2 = _d(PB1), _d(PB2)
    m, dim = PB1.shape
    nb = int(lib().oracle_eytzinger_slots(m))
    B1 = np.empty((nb, dim)); B2 = np.empty((nb, dim)); leaf = np.empty(nb, np.int32)
    lib().oracle_eytzinger_aabb(_ptr(PB1), _ptr(PB2), m, dim, median_mode, _ptr(B1), _ptr(B2),
                                _ptr(leaf))
    return B1, B2, leaf


def eytzinger_wn_tree(E, leaf, canonical: bool = True):
    """igl::eytzinger_aabb_winding_number_tree(E,leaf,I,C) restated; canonical
    sorts each node's positive and negative vertex lists (the reference's
    order is that of an unordered_map)."""
    E, leaf = _i(E), _i(leaf)
    nb = leaf.shape[0]
    Cc = np.empty(nb + 1, np.int32)
    lib().oracle_eytzinger_wn_tree(_ptr(E), _ptr(leaf), nb, int(canonical), _ptr(Cc), None)
    I = np.empty(int(Cc[-1]), np.int32)
    lib().oracle_eytzinger_wn_tree(_ptr(E), _ptr(leaf), nb, int(canonical), _ptr(Cc), _ptr(I))
    return I, Cc


def eytzinger_winding_number(P, V, E, B1, B2, leaf, I, Cc, nthreads: int = 0):
    """igl::eytzinger_aabb_winding_number(p,V,E,B1,B2,leaf,I,C,wn) restated,
    for every row of P."""
    P, V, B1, B2 = _d(P), _d(V), _d(B1), _d(B2)
    E, leaf, I, Cc = _i(E), _i(leaf), _i(I), _i(Cc)
    W = np.empty(P.shape[0])
    lib().oracle_eytzinger_wn(_ptr(P), P.shape[0], _ptr(V), _ptr(E), _ptr(B1), _ptr(B2),
                              _ptr(leaf), leaf.shape[0], _ptr(I), _ptr(Cc), _ptr(W), nthreads)
    return W


def segments_winding_number(P, V, E):
    """Direct sum of atan2(cross, dot)/(2 pi) over every segment."""
    P, V, E = _d(P), _d(V), _i(E)
    W = np.empty(P.shape[0])
    lib().oracle_segments_wn(_ptr(P), P.shape[0], _ptr(V), _ptr(E), E.shape[0], _ptr(W))
    return W


def segment_boxes(V, E):
    """Per-segment min / max corners (the PB1, PB2 a caller passes to
    eytzinger_aabb)."""
    V, E = _d(V), _i(E)
    A, B = V[E[:, 0]], V[E[:, 1]]
    return np.minimum(A, B), np.maximum(A, B)


def flood_fill(res, S):
    """igl::flood_fill(res,S) restated (swept.cpp): a filled copy of S."""
    S = np.array(S, dtype=np.float64, copy=True)
    r = np.ascontiguousarray(res, dtype=np.int32)
    assert S.size == int(r[0]) * int(r[1]) * int(r[2])
    lib().oracle_flood_fill(_ptr(r), _ptr(S))
    return S


def swept_volume_signed_distance(V, F, transforms, sign_type, GV, res, h, isolevel, S0=None):
    """igl::swept_volume_signed_distance(V,F,transforms,sign_type,GV,res,h,
    isolevel,S0,S) restated (include/igl/swept_volume_signed_distance.cpp:
    21-160): the transforms in order, each over every grid point (vectorised
    over the points, which are independent), with the reference's skip rules,
    AABB closest triangle below (isolevel + sqrt(3) h)^2 (oracle AABB), sign
    by type (exact winding number, the soup code on the float copy of V, the
    pseudonormal test) and the running minimum; then flood_fill for a finite
    isolevel.  transforms: nT x 3 x 4 [linear | translation]."""
    V, GV = _d(V), _d(GV)
    F = _d(F, np.int32)
    T = np.asarray(transforms, dtype=np.float64).reshape(-1, 3, 4)
    n = GV.shape[0]
    S = np.full(n, np.nan) if S0 is None else np.array(S0, dtype=np.float64, copy=True)
    finite = bool(np.isfinite(isolevel))
    iso = float(isolevel) if finite else np.inf
    ext = (iso if finite else 0.0) + np.sqrt(3.0) * h
    min_sqrd = (np.sqrt(3.0) * h + iso) ** 2 if finite else np.inf
    skip = iso - np.sqrt(3.0) * h
    if F.shape[0]:
        lo, hi = V.min(0) - ext, V.max(0) + ext
        tree = AABB(V, F)
        soup = None
        if sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER:
            soup = SoupPort(V.astype(np.float32).astype(np.float64), F, order=2)
        for A in T:
            L, t = A[:, :3], A[:, 3]
            act = np.ones(n, bool)
            if finite:
                act &= ~((S == S) & (S < skip))
            d = GV - t
            gv = np.empty_like(GV)
            for j in range(3):
                gv[:, j] = (d[:, 0] * L[0, j] + d[:, 1] * L[1, j]) + d[:, 2] * L[2, j]
            if finite:
                act &= np.all((lo <= gv) & (gv <= hi), axis=1)
            idx = np.flatnonzero(act)
            if idx.size == 0:
                continue
            q = np.ascontiguousarray(gv[idx])
            sqrd, I, Cp = tree.squared_distance(q, min_sqrd)
            if sign_type in (SIGNED_DISTANCE_TYPE_WINDING_NUMBER, SIGNED_DISTANCE_TYPE_DEFAULT):
                s = 1.0 - 2.0 * winding_number(V, F, q)
            elif sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER:
                s = 1.0 - 2.0 * np.abs(soup.eval(q, 2.0))
            elif sign_type == SIGNED_DISTANCE_TYPE_PSEUDONORMAL:
                s = np.empty(idx.size)
                Nrm = np.empty((idx.size, 3))
                lib().oracle_pseudonormal(_ptr(V), V.shape[0], _ptr(F), F.shape[0], _ptr(q),
                                          idx.size, _ptr(I), _ptr(Cp), _ptr(s), _ptr(Nrm))
            else:
                s = np.ones(idx.size)
            ok = sqrd < min_sqrd
            sd = s * np.sqrt(sqrd)
            cur = S[idx]
            new = np.where(cur == cur, np.where(sd < cur, sd, cur), sd)
            S[idx[ok]] = new[ok]
    if finite:
        S = flood_fill(res, S)
    return S


def point_areas(P, I, N, nthreads: int = 0):
    """igl::copyleft::cgal::point_areas restated (oracle/point_areas.cpp):
    returns (A, T) for the points of I's rows (the first I.shape[0] points
    of P; I may hold a leading block of the rows)."""
    P, N = _d(P), _d(N)
    I = np.ascontiguousarray(I, np.int32)
    n, k = I.shape
    A = np.empty(n, np.float64)
    T = np.empty((n, 3), np.float64)
    lib().oracle_point_areas(_ptr(P), P.shape[0], n, _ptr(I), k, _ptr(N), _ptr(A), _ptr(T),
                             nthreads)
    return A, T
