"""2-D winding numbers over the Eytzinger AABB tree on the GPU against the
CPU restatement of the reference (oracle/eytzinger.cpp):

* igl::eytzinger_aabb: B1, B2 and leaf bit-exact against the restatement
  taking the median as the order statistics (the reference's igl::median
  gives the same tree on distinct centre coordinates; both are checked);
* igl::eytzinger_aabb_winding_number_tree: I and C exactly equal to the
  restatement with each node's vertex lists sorted (the reference's pairing
  order is an unordered_map's);
* igl::eytzinger_aabb_winding_number: plain FP64 within 1e-13 of the
  restatement on the same arrays (CUDA's and the C library's atan2 may differ
  in the last bit), mixed within 1e-4 of FP64 (the precision target) with
  identical rounded winding numbers away from the curve.
"""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(21)
    out = {"loops": synth.loops2d(seed=22, n_segments=20000, n_cells=4)}
    n = 3000
    g = rng.integers(0, 60, (n, 2)).astype(float)
    out["grid"] = (g, np.c_[np.arange(n), (np.arange(n) + 1) % n].astype(np.int32))
    t = np.linspace(0, 3 * np.pi, 700)
    out["open"] = (np.c_[t * np.cos(t), t * np.sin(t)] / 10,
                   np.c_[np.arange(699), np.arange(1, 700)].astype(np.int32))
    V = np.array([[0, 0], [1, 0], [1, 1], [-1, 0], [-1, -1], [0, 1], [0, -1], [.5, .5]], float)
    E = np.array([[0, 1], [1, 2], [2, 0], [0, 3], [3, 4], [4, 0], [0, 5], [5, 6], [6, 0],
                  [7, 7], [1, 2]], np.int32)
    out["nonmanifold"] = (V, E)
    return out


def _queries(V, n, seed):
    lo, hi = V.min(0), V.max(0)
    ext = np.maximum(hi - lo, 1e-9)
    return np.random.default_rng(seed).uniform(lo - 0.1 * ext, hi + 0.1 * ext, (n, 2))


def _same_tree(a, b):
    B1, B2, leaf = a
    R1, R2, rleaf = b
    assert np.array_equal(leaf, rleaf)
    used = leaf != -2
    assert np.array_equal(B1[used], R1[used]) and np.array_equal(B2[used], R2[used])
    assert np.all(np.isnan(B1[~used])) and np.all(np.isnan(B2[~used]))


def test_tree_bit_exact(cuda):
    rng = np.random.default_rng(23)
    for name, (V, E) in _cases().items():
        PB1, PB2 = O.segment_boxes(V, E)
        got = G.eytzinger_aabb(PB1, PB2)
        _same_tree(got, O.eytzinger_aabb(PB1, PB2, median_mode=1))
        if name in ("loops", "open"):
            _same_tree(got, O.eytzinger_aabb(PB1, PB2, median_mode=0))
    # small counts, 1-D and 3-D boxes, many equal centres
    for m in (1, 2, 3, 4, 5, 7, 8, 9, 17, 33, 1000):
        for dim in (1, 2, 3):
            PB1 = rng.integers(0, 5, (m, dim)).astype(float)
            PB2 = PB1 + rng.integers(0, 3, (m, dim))
            _same_tree(G.eytzinger_aabb(PB1, PB2), O.eytzinger_aabb(PB1, PB2, median_mode=1))


def test_tree_device_arrays(cuda):
    torch = cuda
    V, E = synth.loops2d(seed=24, n_segments=200_000, n_cells=8)
    PB1, PB2 = O.segment_boxes(V, E)
    d = G.eytzinger_aabb(torch.from_numpy(PB1).cuda(), torch.from_numpy(PB2).cuda())
    _same_tree(tuple(x.cpu().numpy() for x in d), O.eytzinger_aabb(PB1, PB2, median_mode=1))


def test_pairs_exact(cuda):
    for name, (V, E) in _cases().items():
        _, _, leaf = O.eytzinger_aabb(*O.segment_boxes(V, E), median_mode=0)
        I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
        Ir, Cr = O.eytzinger_wn_tree(E, leaf, canonical=True)
        assert np.array_equal(Cc, Cr), name
        assert np.array_equal(I, Ir), name


def test_eval_fp64_matches_oracle(cuda):
    for name, (V, E) in _cases().items():
        B1, B2, leaf = O.eytzinger_aabb(*O.segment_boxes(V, E), median_mode=0)
        for canonical in (False, True):
            I, Cc = O.eytzinger_wn_tree(E, leaf, canonical=canonical)
            P = _queries(V, 20000, 25)
            W = G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc, precision="fp64")
            Wr = O.eytzinger_winding_number(P, V, E, B1, B2, leaf, I, Cc)
            np.testing.assert_allclose(W, Wr, rtol=0, atol=1e-13, err_msg=name)


def test_eval_mixed_within_target(cuda):
    for name, (V, E) in _cases().items():
        B1, B2, leaf = G.eytzinger_aabb(*O.segment_boxes(V, E))
        I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
        P = _queries(V, 50000, 26)
        # plus points on and next to the curve
        k = np.random.default_rng(27).integers(0, E.shape[0], 2000)
        s = np.random.default_rng(28).uniform(0, 1, (2000, 1))
        on = V[E[k, 0]] * (1 - s) + V[E[k, 1]] * s
        P = np.concatenate([P, on, on + 1e-7, V[E[k, 0]]])
        W64 = G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc, precision="fp64")
        Wm = G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc, precision="mixed")
        assert np.abs(Wm - W64).max() <= 1e-4, name
        far = np.abs(W64 - np.round(W64)) < 0.25
        assert np.array_equal(np.round(Wm[far]), np.round(W64[far])), name


def test_loops_winding_values(cuda):
    """The synthetic loops have winding numbers 0, 1 and 2 only (mixed
    precision: within the 1e-4 target of them)."""
    V, E = synth.loops2d(seed=29, n_segments=100_000, n_cells=6)
    B1, B2, leaf = G.eytzinger_aabb(*O.segment_boxes(V, E))
    I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
    P = synth.loops2d_queries(6, seed=30, nq=200_000)
    W = G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc)
    r = np.round(W)
    assert np.abs(W - r).max() < 1e-4
    assert set(np.unique(r).astype(int)) <= {0, 1, 2}
    Wr = O.segments_winding_number(P[:300], V, E)
    np.testing.assert_allclose(W[:300], Wr, atol=1e-4)


def test_device_and_host_paths_agree(cuda):
    torch = cuda
    V, E = synth.loops2d(seed=31, n_segments=50_000, n_cells=5)
    B1, B2, leaf = G.eytzinger_aabb(*O.segment_boxes(V, E))
    I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
    P = synth.loops2d_queries(5, seed=32, nq=100_000)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (P, V, E, B1, B2, leaf, I, Cc)]
    Id, Cd = G.eytzinger_aabb_winding_number_tree(dev[2], dev[5])
    assert np.array_equal(Id.cpu().numpy(), I) and np.array_equal(Cd.cpu().numpy(), Cc)
    for prec in ("fp64", "mixed"):
        Wh = G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc, precision=prec)
        Wd = G.eytzinger_aabb_winding_number(*dev, precision=prec)
        assert np.array_equal(Wd.cpu().numpy(), Wh), prec


def test_empty_and_tiny(cuda):
    P = np.array([[0.3, 0.2], [5, 5]])
    V = np.zeros((0, 2))
    E = np.zeros((0, 2), np.int32)
    B1, B2, leaf = G.eytzinger_aabb(np.zeros((0, 2)), np.zeros((0, 2)))
    assert leaf.shape == (0,)
    I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
    assert I.shape == (0,) and list(Cc) == [0]
    assert np.array_equal(G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc), [0, 0])
    V = np.array([[0, 0], [1, 0]], float)
    E = np.array([[0, 1]], np.int32)
    B1, B2, leaf = G.eytzinger_aabb(*O.segment_boxes(V, E))
    assert list(leaf) == [0, -2]
    I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
    assert list(Cc) == [0, 0, 0]
    for prec in ("fp64", "mixed"):
        W = G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc, precision=prec)
        np.testing.assert_allclose(W, O.segments_winding_number(P, V, E), atol=1e-7)


def test_bad_indices_raise(cuda):
    V, E = synth.loops2d(seed=33, n_segments=2000, n_cells=2)
    B1, B2, leaf = G.eytzinger_aabb(*O.segment_boxes(V, E))
    I, Cc = G.eytzinger_aabb_winding_number_tree(E, leaf)
    bad = I.copy()
    bad[0] = V.shape[0]
    P = synth.loops2d_queries(2, seed=34, nq=1000)
    for prec in ("fp64", "mixed"):
        with pytest.raises(G.GwnError):
            G.eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, bad, Cc, precision=prec)
    bad_leaf = leaf.copy()
    bad_leaf[np.flatnonzero(leaf >= 0)[0]] = E.shape[0] + 5
    with pytest.raises(G.GwnError):
        G.eytzinger_aabb_winding_number_tree(E, bad_leaf)
