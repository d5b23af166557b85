"""CPU tests of the oracle itself: pinned against the reference's own golden
vectors and known answers (tests/include/igl/fast_winding_number.cpp:17-53,
tests/include/igl/signed_distance.cpp:4-42) and against analytic cases."""
import os

import numpy as np
import pytest

from oracle import oracle as O


def test_one_point_cloud_golden():
    # tests/include/igl/fast_winding_number.cpp:17-53, tolerance 1e-15 (:52)
    P = np.array([[0.1, 0.2, 0.3]])
    N = np.array([[4.0, 5.0, 6.0]])
    N /= np.linalg.norm(N[0])
    A = np.array([0.7])
    Q = np.array([[0, 0, 0], [4, -3, 2], [-1, 1, 3], [0, 5, -2]], float)
    W = O.cloud_fwn(P, N, A, Q, order=2, beta=2.0)
    expected = np.array([0.38779369004261133, -0.00041235296362485, -0.00362978253577090,
                         -0.00041235296362485])
    assert np.abs(W - expected).max() <= 1e-15


TET_V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
TET_F = np.array([[0, 1, 3], [0, 2, 1], [0, 3, 2], [1, 2, 3]], np.int32)


def test_single_tet_exact():
    # tests/include/igl/signed_distance.cpp:4-42: (.5,.5,.5) is outside the unit tet.
    W = O.winding_number(TET_V, TET_F, [[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]])
    assert abs(W[0]) < 1e-15 and abs(W[1] - 1) < 1e-15


def test_single_triangle_analytic():
    # A unit right triangle seen from far along its normal: Omega ~ area / d^2.
    a, b, c = [0, 0, 0], [1, 0, 0], [0, 1, 0]
    for d in (10.0, 100.0, 1000.0):
        w = O.solid_angle(a, b, c, [1 / 3, 1 / 3, d])
        # solid angle of a small planar patch: A cos / d^2, sign: normal +z, point above
        approx = -(0.5 / d ** 2) / (4 * np.pi)
        assert abs(w - approx) / abs(approx) < 3.0 / d


def test_exact_closed_forms():
    """Closed-form solid angles (the exact path has no numeric golden vector
    in the reference's tests): a unit square seen along its axis from
    distance d subtends 4 asin(1 / (1 + 4 d^2)); each face of a regular
    tetrahedron subtends pi from its centroid; a unit segment seen from
    height h on its bisector subtends 2 atan(1 / (2 h)) (2-D).  Signs as the
    reference's: a point on the side the face normal points to gets W < 0."""
    Vs = np.array([[-0.5, -0.5, 0], [0.5, -0.5, 0], [0.5, 0.5, 0], [-0.5, 0.5, 0]], float)
    Fs = np.array([[0, 1, 2], [0, 2, 3]], np.int32)   # normal +z
    d = np.array([1e-3, 0.1, 0.5, 1.0, 10.0, 1e3])
    W = O.winding_number(Vs, Fs, np.c_[np.zeros((d.size, 2)), d])
    expect = -np.arcsin(1.0 / (1.0 + 4.0 * d ** 2)) / np.pi
    np.testing.assert_allclose(W, expect, rtol=1e-13, atol=1e-17)
    np.testing.assert_allclose(O.winding_number(Vs, Fs, np.c_[np.zeros((d.size, 2)), -d]),
                               -expect, rtol=1e-13, atol=1e-17)
    # regular tetrahedron, outward faces
    T = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float)
    c = T.mean(axis=0)
    for f in ([0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3]):
        a, b, e = T[f]
        n = np.cross(b - a, e - a)
        if n @ (a - c) < 0:
            b, e = e, b
        assert abs(O.solid_angle(a, b, e, c) - 0.25) < 1e-15   # pi / (4 pi), point inside
    # 2-D: unit segment from (-1/2, 0) to (1/2, 0)
    V2 = np.array([[-0.5, 0.0], [0.5, 0.0]])
    E2 = np.array([[0, 1]], np.int32)
    h = np.array([1e-3, 0.25, 1.0, 100.0])
    W2 = O.winding_number(V2, E2, np.c_[np.zeros(h.size), h])
    np.testing.assert_allclose(np.abs(W2), 2.0 * np.arctan(1.0 / (2.0 * h)) / (2.0 * np.pi),
                               rtol=1e-13)
    W2m = O.winding_number(V2, E2, np.c_[np.zeros(h.size), -h])
    np.testing.assert_allclose(W2m, -W2, rtol=1e-13)


@pytest.mark.skipif(not O.ref_soup_available(), reason="reference tree not present")
def test_reference_soup_single_tet_sign():
    r = O.RefSoup(TET_V, TET_F)
    W = r.eval(np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]]))
    assert abs(W[0]) < 1e-6 and abs(W[1] - 1) < 1e-6


def _brute_octree(P):
    """Independent pure-Python statement of octree.cpp:5-170 (recursive)."""
    P = np.asarray(P, float)
    n = P.shape[0]
    pi, ch, cn, w = [list(range(n))], [[-1] * 8], [], []
    mn, mx = P.min(0), P.max(0)
    cn.append(((mn + mx) / 2.0).tolist())
    w.append(float((mx - mn).max()))
    m = [1]

    def helper(index, depth):
        if len(pi[index]) > 1 and depth < 30000:
            ch[index] = [m[0] + i for i in range(8)]
            h = w[index] / 2
            c = cn[index]
            for i in range(8):
                ch.append([-1] * 8)
                pi.append([])
                hh = h / 2
                cn.append([c[0] + (hh if i % 2 else -hh), c[1] + (hh if i in (2, 3, 6, 7) else -hh),
                           c[2] + (hh if i > 3 else -hh)])
                w.append(h)
            for p in pi[index]:
                o = int(P[p, 0] >= c[0]) + 2 * int(P[p, 1] >= c[1]) + 4 * int(P[p, 2] >= c[2])
                pi[m[0] + o].append(p)
            first = m[0]
            m[0] += 8
            for i in range(8):
                helper(first + i, depth + 1)

    helper(0, 0)
    return pi, np.array(ch), np.array(cn), np.array(w)


@pytest.mark.parametrize("seed,n", [(0, 1), (1, 2), (2, 9), (3, 40), (4, 150)])
def test_octree_matches_recursive_statement(seed, n):
    rng = np.random.default_rng(seed)
    P = rng.random((n, 3))
    t = O.octree(P)
    pi, ch, cn, w = _brute_octree(P)
    assert t.point_indices() == pi
    assert np.array_equal(t.CH, ch)
    assert np.array_equal(t.CN, cn)
    assert np.array_equal(t.W, w)


def test_octree_duplicate_points_reach_max_depth():
    # Two identical points never separate: the split recurses to MAX_DEPTH =
    # 30000 (octree.cpp:16, :98), emitting 8 cells per level.
    P = np.array([[0.25, 0.5, 0.75], [0.25, 0.5, 0.75], [0.9, 0.1, 0.3]])
    t = O.octree(P)
    internal = (t.CH[:, 0] != -1).sum()
    assert t.ncells == 1 + 8 * internal
    assert internal == 30000  # the root (3 points) and the pair at depths 1..29999
    sizes = np.diff(t.pi_off)
    assert sizes.max() == 3 and (sizes == 2).sum() == 30000  # depths 1..30000


def test_cloud_direct_matches_bh_far():
    rng = np.random.default_rng(7)
    P = rng.random((300, 3))
    Nn = rng.normal(size=(300, 3))
    Nn /= np.linalg.norm(Nn, axis=1, keepdims=True)
    A = rng.random(300) * 0.01
    Q = rng.random((50, 3)) * 8 + 5  # far from the cloud
    t = O.octree(P)
    CM, R, EC = O.cloud_precompute(P, Nn, A, t, 2)
    Wbh = O.cloud_eval(P, Nn, A, t, CM, R, EC, Q, 2.0)
    Wd = O.cloud_eval(P, Nn, A, t, CM, R, EC, Q, 0.0)
    assert np.abs(Wbh - Wd).max() < 1e-3 * np.abs(Wd).max()  # order-3 truncation


def test_soup_port_reproduces_reference_fixtures_bit_for_bit():
    # The CPU restatement of the HDK soup algorithm (oracle/soup_hdk.cpp) is
    # pinned against the reference's own UT_SolidAngle outputs committed by
    # tests/golden/make_golden.py.
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "soup_reference.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    for name in names:
        V, F, Q, Wref = z[name + "/V"], z[name + "/F"], z[name + "/Q"], z[name + "/W_ref"]
        W = O.SoupPort(V, F, order=2).eval(Q, 2.0)
        assert np.array_equal(W, Wref), name


def test_pair_atan2_polynomial_in_fp32():
    """The FP32 atan2 of the FP32 angle terms (atan2f.cuh, atan2_pairs, used
    by the exact 3-D sum and the 2-D tree walk): its coefficients, evaluated in float32 with the kernel's
    octant reduction, stay within a few ulp of atan2 everywhere."""
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "libigl_gb300", "csrc",
                            "atan2f.cuh")).read()
    body = src[src.index("float atan2_pairs("):]
    body = body[:body.index("\n}\n")]
    coef = [np.float32(float(x)) for x in
            re.findall(r"(?:float p = |p = fmaf\(p, s, )(-?[0-9.]+(?:e[-+][0-9]+)?)f", body)]
    assert len(coef) == 9  # degree 8, highest first
    f32 = np.float32
    rng = np.random.default_rng(0)
    ang = rng.uniform(-np.pi, np.pi, 400_000)
    rad = 10.0 ** rng.uniform(-6, 6, ang.size)
    y = (rad * np.sin(ang)).astype(f32)
    x = (rad * np.cos(ang)).astype(f32)
    ax, ay = np.abs(x), np.abs(y)
    mx, mn = np.maximum(ax, ay), np.minimum(ax, ay)
    t = (mn / mx).astype(f32)
    s = (t * t).astype(f32)
    p = coef[0]
    for c in coef[1:]:
        p = (p * s + c).astype(f32)
    r = (t * p).astype(f32)
    r = np.where(ay > ax, (f32(np.pi / 2) - r).astype(f32), r)
    r = np.where(x < 0, (f32(np.pi) - r).astype(f32), r)
    r = np.copysign(r, y)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    err = np.abs(r - ref)
    assert np.all(err <= 4 * np.spacing(np.abs(ref).astype(f32)) + 1e-12), err.max()


def test_signed_distance_oracle_single_tet_golden():
    """tests/include/igl/signed_distance.cpp:4-42: the point (.5,.5,.5) is
    sqrt(1/12) from the unit tet for every sign type (1e-15; the fast winding
    number sign 1e-7)."""
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    F = np.array([[0, 1, 3], [0, 2, 1], [0, 3, 2], [1, 2, 3]], np.int32)
    P = np.array([[0.5, 0.5, 0.5]])
    for t, tol in ((O.SIGNED_DISTANCE_TYPE_PSEUDONORMAL, 1e-15),
                   (O.SIGNED_DISTANCE_TYPE_WINDING_NUMBER, 1e-15),
                   (O.SIGNED_DISTANCE_TYPE_DEFAULT, 1e-15),
                   (O.SIGNED_DISTANCE_TYPE_UNSIGNED, 1e-15),
                   (O.SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER, 1e-7)):
        S, I, Cp = O.signed_distance(P, V, F, t)
        assert abs(S[0] - np.sqrt(1 / 12)) <= tol, (t, S)
        assert I[0] == 3 and np.allclose(Cp[0], 1 / 3, atol=1e-15)


def test_closest_point_oracle_regions():
    """Ericson's regions on one triangle: vertex, edge and face closest points
    against analytic answers."""
    a, b, c = np.array([0., 0, 0]), np.array([1., 0, 0]), np.array([0., 1, 0])
    L = O.lib()
    cases = [([-1, -1, 0.5], [0, 0, 0]), ([2, -0.5, 0], [1, 0, 0]), ([0.5, -1, 1], [0.5, 0, 0]),
             ([0.2, 0.3, -2], [0.2, 0.3, 0]), ([1, 1, 0], [0.5, 0.5, 0]), ([-1, 0.5, 0], [0, 0.5, 0])]
    for p, cp in cases:
        p = np.array(p, float)
        out = np.empty(3)
        d2 = L.oracle_point_triangle(O._ptr(p), O._ptr(a), O._ptr(b), O._ptr(c), O._ptr(out))
        assert np.allclose(out, cp, atol=1e-15), (p, out)
        assert abs(d2 - np.sum((p - np.array(cp)) ** 2)) < 1e-14


def test_aabb_restatement_matches_brute_force():
    """The AABB restatement (the timed CPU baseline of the signed distance)
    finds the brute-force minimum distance."""
    from libigl_gb300 import synth
    V, F = synth.soup_mesh(seed=31, subdiv=3, delete_frac=0.02)
    rng = np.random.default_rng(32)
    P = rng.uniform(V.min(0) - 0.3, V.max(0) + 0.3, size=(3000, 3))
    P = np.concatenate([P, V[:40]])
    D, I, Cp = O.AABB(V, F).squared_distance(P)
    Db, Ib, Cb = O.squared_distance(V, F, P)
    assert np.array_equal(D, Db)
    # a closest edge or vertex is shared by several triangles (ties), so the
    # indices may differ; the closest points agree
    assert np.abs(Cp - Cb).max() <= 1e-12


def test_knn_oracle_golden():
    """tests/include/igl/knn.cpp:8-73: unit-cube corners (with a distance tie
    in the first query) and the #V <= k branch."""
    V = np.array([[0, 0, 1], [0, 1, 0], [0, 1, 1], [0, 0, 0], [1, 0, 0], [1, 1, 0], [1, 1, 1],
                  [1, 0, 1]], float)
    P = np.array([[0, 0, 0.6], [0.3, 0.1, 0.2], [.7, .6, 0]])
    assert np.array_equal(O.knn(P, V, 3), [[0, 3, 2], [3, 4, 0], [5, 4, 1]])
    V2 = np.array([[0, 0, 0], [1, 1, 1]], float)
    P2 = np.array([[0, 0, 0], [-1, -1, -1], [2, 2, 2]], float)
    assert np.array_equal(O.knn(P2, V2, 10), [[0, 1], [0, 1], [1, 0]])


# ------------------------------------------------- 2-D Eytzinger AABB tree --
def _eytz_cases():
    from libigl_gb300 import synth
    rng = np.random.default_rng(11)
    cases = {}
    cases["loops"] = synth.loops2d(n_segments=3000, n_cells=3)
    n = 1500  # random grid polygon: repeated coordinates, self-intersections
    g = rng.integers(0, 40, (n, 2)).astype(float)
    cases["grid"] = (g, np.c_[np.arange(n), (np.arange(n) + 1) % n].astype(np.int32))
    t = np.linspace(0, 3 * np.pi, 400)  # open spiral
    cases["open"] = (np.c_[t * np.cos(t), t * np.sin(t)] / 10,
                     np.c_[np.arange(399), np.arange(1, 400)].astype(np.int32))
    # a vertex shared by six segments (two triangles and a bow-tie through 0),
    # a zero-length segment and a duplicated segment
    V = np.array([[0, 0], [1, 0], [1, 1], [-1, 0], [-1, -1], [0, 1], [0, -1], [.5, .5]], float)
    E = np.array([[0, 1], [1, 2], [2, 0], [0, 3], [3, 4], [4, 0], [0, 5], [5, 6], [6, 0],
                  [7, 7], [1, 2]], np.int32)
    cases["nonmanifold"] = (V, E)
    return cases


def test_eytzinger_oracle_equals_direct_sum():
    """The hierarchy (eytzinger_aabb_winding_number.cpp:66-110) returns the
    direct sum over every segment (the same per-term formula) for closed,
    open, self-intersecting and non-manifold inputs, with the reference's
    pairing order and with the canonical one."""
    rng = np.random.default_rng(12)
    for name, (V, E) in _eytz_cases().items():
        lo, hi = V.min(0), V.max(0)
        P = rng.uniform(lo - 0.1 * (hi - lo), hi + 0.1 * (hi - lo), (800, 2))
        Wd = O.segments_winding_number(P, V, E)
        B1, B2, leaf = O.eytzinger_aabb(*O.segment_boxes(V, E), median_mode=0)
        for canonical in (False, True):
            I, Cc = O.eytzinger_wn_tree(E, leaf, canonical=canonical)
            assert Cc[0] == 0 and np.all(np.diff(Cc) % 2 == 0)
            W = O.eytzinger_winding_number(P, V, E, B1, B2, leaf, I, Cc)
            np.testing.assert_allclose(W, Wd, rtol=0, atol=1e-12, err_msg=name)


def test_eytzinger_oracle_known_answers():
    """Unit square: 1 inside counter-clockwise, -1 clockwise, 0 outside; a
    point on a vertex adds atan2(0, 0) = 0 for its two segments."""
    V = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    E = np.array([[0, 1], [1, 2], [2, 3], [3, 0]], np.int32)
    P = np.array([[.5, .5], [2, .5], [-.1, -.1], [.25, .75]])
    for orient, want in ((E, [1, 0, 0, 1]), (E[:, ::-1].copy(), [-1, 0, 0, -1])):
        B1, B2, leaf = O.eytzinger_aabb(*O.segment_boxes(V, orient))
        assert leaf.shape == (8,) and list(leaf[:3]) == [-1, -1, -1]
        I, Cc = O.eytzinger_wn_tree(orient, leaf)
        W = O.eytzinger_winding_number(P, V, orient, B1, B2, leaf, I, Cc)
        np.testing.assert_allclose(W, want, atol=1e-15)


def test_eytzinger_median_forms_agree():
    """igl::median's two nth_element calls (median.cpp:14-35) against the
    order statistics: the same tree on distinct centre coordinates; with
    repeated coordinates any difference leaves the winding numbers equal."""
    for name, (V, E) in _eytz_cases().items():
        PB1, PB2 = O.segment_boxes(V, E)
        a = O.eytzinger_aabb(PB1, PB2, median_mode=0)
        b = O.eytzinger_aabb(PB1, PB2, median_mode=1)
        if name in ("loops", "open"):
            assert np.array_equal(a[2], b[2]), name
        P = np.random.default_rng(13).uniform(V.min(0) - .1, V.max(0) + .1, (300, 2))
        Wa = O.eytzinger_winding_number(P, V, E, a[0], a[1], a[2], *O.eytzinger_wn_tree(E, a[2]))
        Wb = O.eytzinger_winding_number(P, V, E, b[0], b[1], b[2], *O.eytzinger_wn_tree(E, b[2]))
        np.testing.assert_allclose(Wa, Wb, atol=1e-12, err_msg=name)
