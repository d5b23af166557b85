"""GPU parity of the triangle-soup fast winding number over the binned binary
tree (tree="binned"; the reference's own 4-wide tree is covered by
tests/test_soup_ref_gpu.py).

Checks, through the C ABI:
  * the tree's stored FP64 moments equal the HDK moments recomputed on the CPU
    from each node's triangles (FWNFS.h:6668-7118);
  * the plain FP64 walk equals the CPU oracle's FP64 walk over the same tree
    (computeSolidAngle semantics, FWNFS.h:7148-7284) to rounding;
  * the mixed walk is within the metric bound |dW| <= 1e-4 of the plain FP64
    walk, with identical inside/outside labels outside 0.5 +- 1e-3;
  * against the reference's own FP32 UT_SolidAngle (committed fixtures from
    tests/golden/make_golden.py): tight where the trees coincide (one
    triangle), within the reference's own approximation error elsewhere;
  * against the exact winding number: within the 1e-2 the reference's own
    test allows (tests/include/igl/fast_winding_number.cpp:76).
"""
import os

import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL_MIXED = 1e-4


def golden():
    z = np.load(os.path.join(HERE, "golden", "soup_reference.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    return {n: {k.split("/")[1]: z[k] for k in z.files if k.startswith(n + "/")} for n in names}


@pytest.fixture(scope="module")
def mesh(cuda):
    rng = np.random.default_rng(5)
    V, F = synth.icosphere(5)
    V = synth.sh_deform(V, rng)
    F = synth.delete_random_faces(F, rng, 0.01)
    Q = synth.soup_queries(V, F, seed=6, nq=20000)
    return V, F, Q


def test_tree_moments_match_flat_recomputation(mesh):
    V, F, _ = mesh
    Vs, Fs = V, F[:3000]
    bvh = G.FastWindingNumberBVH(Vs, Fs, order=2, tree="binned")
    nodes, links, tri = bvh.export()
    assert sorted(tri.tolist()) == list(range(Fs.shape[0]))
    ref = O.soup_tree_moments(Vs, Fs, nodes, tri)
    scale = np.abs(ref[:, :23]).max(axis=0) + 1e-300
    rel = np.abs(nodes[:, :23] - ref[:, :23]) / scale
    assert rel.max() < 1e-10, rel.max(axis=0)
    # The reference's SumPermute shift (FWNFS.h:7075) counts the children's
    # first-moment term once; the exact parallel-axis shift counts it twice.
    # Every other moment equals its grouping-independent value.
    flat = O.soup_tree_moments(Vs, Fs, nodes, tri, flat=True)
    relf = np.abs(nodes[:, :23] - flat[:, :23]) / scale
    others = [k for k in range(23) if k != 16]
    assert relf[:, others].max() < 1e-10
    # pre-order skip links: every internal node's subtree is contiguous
    n = nodes.shape[0]
    assert n == 2 * Fs.shape[0] - 1
    internal = links >= 0
    assert np.all(links[internal] > np.nonzero(internal)[0])
    assert np.all(links[internal] <= n)
    assert links[0] == n


def test_fp64_walk_matches_cpu_walk(mesh):
    V, F, Q = mesh
    bvh = G.FastWindingNumberBVH(V, F, order=2, tree="binned")
    nodes, links, tri = bvh.export()
    W64 = bvh.eval(Q, 2.0, precision="fp64")
    Wcpu = O.soup_tree_eval(V, F, nodes, tri, Q, 2.0, order=2)
    assert np.abs(W64 - Wcpu).max() < 1e-11


@pytest.mark.parametrize("tree", ["binned", "reference"])
def test_mixed_within_metric_of_fp64(mesh, tree):
    V, F, Q = mesh
    bvh = G.FastWindingNumberBVH(V, F, order=2, tree=tree)
    for qdt in (np.float64, np.float32):
        Qd = Q.astype(qdt)
        W64 = bvh.eval(Qd, 2.0, precision="fp64", out_dtype=np.float64)
        Wm = bvh.eval(Qd, 2.0, precision="mixed", out_dtype=np.float64)
        err = np.abs(Wm - W64)
        assert err.max() <= TOL_MIXED, err.max()
        out = np.abs(W64 - 0.5) > 1e-3
        assert np.array_equal((Wm > 0.5)[out], (W64 > 0.5)[out])


def test_against_exact_and_orders(mesh):
    V, F, Q = mesh
    Qs = Q[:3000]
    Wex = O.winding_number(V, F, Qs)
    for order, tol in ((2, 1e-2), (1, 2e-1), (0, 5e-1)):
        bvh = G.FastWindingNumberBVH(V, F, order=order, tree="binned")
        W = bvh.eval(Qs, 2.0, precision="fp64")
        assert np.abs(W - Wex).max() < tol, (order, np.abs(W - Wex).max())
        nodes, links, tri = bvh.export()
        Wcpu = O.soup_tree_eval(V, F, nodes, tri, Qs, 2.0, order=order)
        assert np.abs(W - Wcpu).max() < 1e-11


def test_against_reference_fixtures(cuda):
    for name, c in golden().items():
        if "W_exact" not in c:
            continue
        V, F, Q, Wref, Wex = c["V"], c["F"], c["Q"], c["W_ref"], c["W_exact"]
        bvh = G.FastWindingNumberBVH(V, F, order=2, tree="binned")
        W = bvh.eval(Q, 2.0, precision="mixed")
        ref_err = np.abs(Wref - Wex).max()
        if name == "one_tri":
            # same tree (one triangle): only FP32-vs-FP64 arithmetic differs
            assert np.abs(W - Wref).max() < 5e-6, name
        # the reference's own error bound vs exact, with our approximation's
        assert np.abs(W - Wex).max() < max(1e-2, 3 * ref_err), name
        assert np.abs(W - Wref).max() < max(1e-2, 3 * ref_err), name
        far_band = (np.abs(Wex - 0.5) > 0.05)
        assert np.array_equal((W > 0.5)[far_band], (Wex > 0.5)[far_band]), name


def test_single_tet_sign(cuda):
    # tests/include/igl/signed_distance.cpp:4-42: (.5,.5,.5) is outside the unit tet
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    F = np.array([[0, 1, 3], [0, 2, 1], [0, 3, 2], [1, 2, 3]], np.int32)
    W = G.fast_winding_number_soup(V, F, np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1]]))
    assert abs(W[0]) < 1e-6 and abs(W[1] - 1) < 1e-6


def test_edge_cases(cuda):
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [np.nan, 0, 0]], float)
    F = np.array([[0, 1, 3], [0, 2, 1], [0, 3, 2], [1, 2, 3], [4, 1, 2]], np.int32)
    Q = np.array([[0.1, 0.1, 0.1], [2, 2, 2], [0, 0, 0]])
    # a triangle with a NaN vertex is excluded from the tree (FWNFS.h:4606-4615)
    for tree in ("binned", "reference"):
        b = G.FastWindingNumberBVH(V, F, tree=tree)
        assert b.stats["num_triangles"] == 4
        Wt = b.eval(Q, 2.0, precision="mixed")
        # within the order-2 expansion's error at accuracy 2 of the exact 1 / 0
        assert abs(Wt[0] - 1) < 1e-4 and abs(Wt[1]) < 1e-4 and np.isfinite(Wt[2])
        if tree == "reference":  # and the reference's own values (its tree)
            assert np.abs(Wt[:2] - O.SoupPort(V, F).eval(Q[:2], 2.0)).max() < 1e-6
        with pytest.raises(G.GwnError):
            G.FastWindingNumberBVH(V, np.array([[0, 1, 9]], np.int32), tree=tree)
    bvh = G.FastWindingNumberBVH(V, F)
    assert bvh.stats["num_triangles"] == 4
    W = bvh.eval(Q, 2.0, precision="mixed")
    assert abs(W[0] - 1) < 1e-4 and abs(W[1]) < 1e-4 and np.isfinite(W[2])
    # empty mesh and empty queries
    e = G.FastWindingNumberBVH(V, np.zeros((0, 3), np.int32))
    assert np.all(e.eval(Q) == 0)
    assert bvh.eval(np.zeros((0, 3))).shape == (0,)
    # out-of-range index fails loudly
    with pytest.raises(G.GwnError):
        G.FastWindingNumberBVH(V, np.array([[0, 1, 9]], np.int32))


def test_device_tensors_and_repeatability(mesh, cuda):
    torch = cuda
    V, F, Q = mesh
    bvh = G.FastWindingNumberBVH(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    dQ = torch.from_numpy(Q.astype(np.float32)).cuda()
    W1 = bvh.eval(dQ, 2.0, precision="mixed")
    W2 = bvh.eval(dQ, 2.0, precision="mixed")
    assert W1.is_cuda and torch.equal(W1, W2)  # deterministic
    Wh = bvh.eval(Q.astype(np.float32), 2.0, precision="mixed")
    assert np.array_equal(W1.cpu().numpy(), Wh)
    # a query's value does not depend on the batch it is evaluated in
    sub = Q[::7].astype(np.float32)
    Ws = bvh.eval(sub, 2.0, precision="mixed")
    assert np.abs(Ws - Wh[::7]).max() <= 1e-6
    assert G.device_status() == 0


def _check_tree(V, F, Q):
    bvh = G.FastWindingNumberBVH(V, F, order=2, tree="binned")
    nodes, links, tri = bvh.export()
    n = F.shape[0]
    assert sorted(tri.tolist()) == list(range(n))
    assert nodes.shape[0] == 2 * n - 1
    # pre-order with skip links: an internal node's subtree is [p + 1, link)
    internal = links >= 0
    idx = np.nonzero(internal)[0]
    assert np.all(links[idx] > idx + 1) and np.all(links[idx] <= 2 * n - 1)
    if n > 1:
        assert links[0] == 2 * n - 1
    assert sorted((~links[~internal]).tolist()) == list(range(n))
    W64 = bvh.eval(Q, 2.0, precision="fp64")
    Wcpu = O.soup_tree_eval(V, F, nodes, tri, Q, 2.0, order=2)
    assert np.abs(W64 - Wcpu).max() < 1e-11
    Wm = bvh.eval(Q, 2.0, precision="mixed")
    assert np.abs(Wm - W64).max() <= TOL_MIXED


def test_tree_builder_corner_cases(cuda):
    """The binned top-down builder (soup_tree.cu): sizes around the 32
    triangles one warp finishes, triangles whose centroids all coincide (no
    bin separates them: middle splits), and a flat mesh (zero extent on one
    axis)."""
    rng = np.random.default_rng(71)
    V, F = synth.icosphere(3)
    F = np.ascontiguousarray(F, dtype=np.int32)
    Q = np.ascontiguousarray(rng.uniform(-1.3, 1.3, (500, 3)))
    for m in (2, 3, 31, 32, 33, 34, 64, 65, 200):
        _check_tree(V, np.ascontiguousarray(F[:m]), Q)
    # 300 copies of one triangle, flipped every other time: equal centroids
    Fd = np.ascontiguousarray(np.tile(np.array([[0, 1, 2], [0, 2, 1]], np.int32), (150, 1)))
    _check_tree(V, Fd, Q)
    # a flat grid of triangles in z = 0
    g = np.stack(np.meshgrid(np.linspace(0, 1, 30), np.linspace(0, 1, 30), indexing="ij"), -1)
    Vf = np.concatenate([g.reshape(-1, 2), np.zeros((900, 1))], 1)
    a = (np.arange(29)[:, None] * 30 + np.arange(29)[None, :]).ravel()
    Ff = np.concatenate([np.stack([a, a + 30, a + 1], 1), np.stack([a + 1, a + 30, a + 31], 1)])
    _check_tree(np.ascontiguousarray(Vf), np.ascontiguousarray(Ff, dtype=np.int32), Q * 0.8 + 0.3)

