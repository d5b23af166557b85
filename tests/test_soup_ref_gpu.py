"""The reference's own triangle-soup tree, built on the GPU (tree="reference",
the default of FastWindingNumberBVH and gwn_soup_build).

igl::fast_winding_number(V,F,order,bvh) builds UT_BVH<4> with the BOX_AREA
heuristic over float copies of V (include/igl/FastWindingNumberForSoups.h:
4581-5944) and UT_SolidAngle's FP32 per-lane moments (FWNFS.h:6543-7133);
soup_ref.cu rebuilds both on the GPU and the walks take the reference's own
FP32 open test (FWNFS.h:7176-7193).  Checked through the C ABI:
  * the node array equals the reference's own, node for node (fixtures
    exported from the compiled reference by tests/golden/make_golden.py,
    including a grid with exact ties, nodes of more than 1024 boxes and
    degenerate / repeated triangles), and the oracle's restatement of the
    build (oracle/soup_hdk.cpp, itself equal to the reference's) up to
    1.3M triangles;
  * values: the plain FP64 walk equals the reference's own W up to the
    reference's FP32 rounding, the mixed walk within the metric bound
    1e-4 of it, and both with the same inside/outside labels outside
    0.5 +- 1e-3;
  * corner cases: one triangle, <= 4 triangles (the root holds items),
    empty and all-excluded meshes; the closest-triangle search on such a
    handle equals the binned handle's.
"""
import os

import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference computes in FP32 on float copies of V and Q; over the same
# tree cut the FP64 walk differs from it by that rounding only.  On surfaces
# (spheres, the grid) that is below 1e-5.  Soups of random triangles have a
# boundary edge near many queries, where W turns by dW ~ dx / (2 pi d): the
# float rounding of V and Q (~1e-7) at d = 1e-4 moves the reference's own
# value by up to ~2e-4, so there the bound is the reference's error.
SOUPS = {"four_tris", "random_soup", "degenerate_soup"}
TOL_FP64_VS_REF = 1e-5
TOL_FP64_VS_REF_SOUP = 3e-4
P99_FP64_VS_REF = 1e-6
P99_FP64_VS_REF_SOUP = 1e-5
TOL_MIXED = 1e-4


def golden():
    z = np.load(os.path.join(HERE, "golden", "soup_reference.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    return {n: {k.split("/")[1]: z[k] for k in z.files if k.startswith(n + "/")} for n in names}


def test_tree_equals_the_reference_tree(cuda):
    for name, c in golden().items():
        bvh = G.FastWindingNumberBVH(c["V"], c["F"], order=2, tree="reference")
        T = bvh.tree_nodes()
        assert T.shape == c["tree"].shape, name
        assert np.array_equal(T, c["tree"]), name


@pytest.mark.parametrize("subdiv", [6, 8])
def test_tree_equals_the_oracle_tree_at_scale(cuda, subdiv):
    rng = np.random.default_rng(100 + subdiv)
    V, F = synth.icosphere(subdiv)
    V = synth.sh_deform(V, rng)
    F = synth.delete_random_faces(F, rng, 0.01).astype(np.int32)
    T = G.FastWindingNumberBVH(V, F, order=2, tree="reference").tree_nodes()
    To = O.SoupPort(V, F, order=2).tree()
    assert np.array_equal(T, To)


def test_values_match_the_reference(cuda):
    for name, c in golden().items():
        V, F, Q, Wref = c["V"], c["F"], c["Q"], c["W_ref"]
        bvh = G.FastWindingNumberBVH(V, F, order=2, tree="reference")
        W64 = bvh.eval(Q, 2.0, precision="fp64")
        Wm = bvh.eval(Q, 2.0, precision="mixed")
        e64 = np.abs(W64 - Wref)
        em = np.abs(Wm - Wref)
        soup = name in SOUPS
        tol = TOL_FP64_VS_REF_SOUP if soup else TOL_FP64_VS_REF
        p99 = P99_FP64_VS_REF_SOUP if soup else P99_FP64_VS_REF
        assert e64.max() <= tol, (name, e64.max())
        assert np.quantile(e64, 0.99) <= p99, (name, np.quantile(e64, 0.99))
        assert em.max() <= max(TOL_MIXED, tol), (name, em.max())
        # mixed and plain FP64 take the same tree cut: arithmetic only
        assert np.abs(Wm - W64).max() <= TOL_MIXED, name
        out = np.abs(Wref - 0.5) > 1e-3
        assert np.array_equal((W64 > 0.5)[out], (Wref > 0.5)[out]), name
        assert np.array_equal((Wm > 0.5)[out], (Wref > 0.5)[out]), name


def test_float32_queries_and_outputs(cuda):
    c = golden()["sphere5_holes"]
    bvh = G.FastWindingNumberBVH(c["V"], c["F"], order=2)
    Q32 = c["Q"].astype(np.float32)
    W = bvh.eval(Q32, 2.0, precision="mixed")
    assert W.dtype == np.float32
    assert np.abs(W.astype(np.float64) - c["W_ref"]).max() <= TOL_MIXED


@pytest.mark.parametrize("order", [0, 1])
def test_lower_orders_follow_the_reference_algorithm(cuda, order):
    c = golden()["sphere_holes"]
    V, F, Q = c["V"], c["F"], c["Q"]
    ref = O.SoupPort(V, F, order=order).eval(Q, 2.0)
    W = G.FastWindingNumberBVH(V, F, order=order).eval(Q, 2.0, precision="fp64")
    assert np.abs(W - ref).max() <= TOL_FP64_VS_REF_SOUP


def test_small_and_degenerate_meshes(cuda):
    rng = np.random.default_rng(9)
    Q = rng.uniform(-2, 2, (300, 3))
    V = rng.normal(size=(40, 3))
    for m in (1, 2, 3, 4, 5, 6, 7, 33):
        F = rng.integers(0, 40, (m, 3)).astype(np.int32)
        bvh = G.FastWindingNumberBVH(V, F, order=2)
        assert np.array_equal(bvh.tree_nodes(), O.SoupPort(V, F).tree()), m
        W = bvh.eval(Q, 2.0, precision="fp64")
        assert np.abs(W - O.SoupPort(V, F).eval(Q, 2.0)).max() <= TOL_FP64_VS_REF_SOUP, m
    # every triangle excluded (non-finite) and an empty mesh: W = 0
    Vn = V.copy()
    Vn[:, 0] = np.nan
    for Vx, Fx in ((Vn, np.array([[0, 1, 2]], np.int32)), (V, np.zeros((0, 3), np.int32))):
        b = G.FastWindingNumberBVH(Vx, Fx)
        assert b.stats["num_triangles"] == 0
        assert np.all(b.eval(Q) == 0)


def test_closest_triangle_on_a_reference_handle(cuda):
    c = golden()["sphere5_holes"]
    V, F, Q = c["V"], c["F"], c["Q"]
    r = G.FastWindingNumberBVH(V, F, tree="reference")
    b = G.FastWindingNumberBVH(V, F, tree="binned")
    Dr, Ir, Cr = r.squared_distance(Q)
    Db, Ib, Cb = b.squared_distance(Q)
    assert np.abs(Dr - Db).max() <= 1e-12 * max(1.0, float(Db.max()))
    assert np.all((Ir >= 0) & (Ir < F.shape[0]))
    # the reported triangle is at the reported distance
    for i in range(0, Q.shape[0], 97):
        Dd, _, _ = O.squared_distance(V, F[[Ir[i]]], Q[[i]])
        assert abs(Dd[0] - Dr[i]) <= 1e-12 * max(1.0, float(Dr[i]))


def test_host_buffers_equal_the_device_call(cuda):
    """A 4.5M-query host-buffer call (staged copies in and out) equals the
    device-buffer call exactly, in both precisions and for FP32 queries."""
    torch = cuda
    V, F = synth.soup_mesh(seed=1, subdiv=5)
    rng = np.random.default_rng(4)
    Q = rng.uniform(-1.5, 1.5, (4_500_001, 3))
    bvh = G.FastWindingNumberBVH(V, F, order=2)
    for prec in ("mixed", "fp64"):
        Wh = bvh.eval(Q, 2.0, precision=prec)
        Wd = bvh.eval(torch.from_numpy(Q).cuda(), 2.0, precision=prec).cpu().numpy()
        assert np.array_equal(Wh, Wd), prec
    Wh32 = bvh.eval(Q.astype(np.float32), 2.0, precision="mixed")
    Wd32 = bvh.eval(torch.from_numpy(Q.astype(np.float32)).cuda(), 2.0,
                    precision="mixed").cpu().numpy()
    assert np.array_equal(Wh32, Wd32)
