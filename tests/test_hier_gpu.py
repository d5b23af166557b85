"""Hierarchical exact winding number (igl::WindingNumberAABB on the GPU,
hier.cu) against the all-pairs FP64 sum (gwn_winding_number, plain FP64) and
the CPU restatement of the reference hierarchy (oracle/wn_hier.cpp): the
same value up to rounding, so within the mixed-precision target 1e-4 (and
far below it in practice), with identical labels away from 0.5.
"""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _queries(V, n, seed, near=True):
    rng = np.random.default_rng(seed)
    lo, hi = V.min(0), V.max(0)
    ext = hi - lo
    Q = [rng.uniform(lo - 0.3 * ext, hi + 0.3 * ext, (n, 3))]
    if near:
        k = rng.integers(0, V.shape[0], n)
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        for dec in (1e-2, 1e-4, 1e-6):
            Q.append(V[k] + dec * np.linalg.norm(ext) * d)
    return np.ascontiguousarray(np.concatenate(Q))


def _meshes():
    rng = np.random.default_rng(61)
    out = {}
    V, F = synth.icosphere(3)
    out["closed"] = (synth.sh_deform(V, rng, lmax=6, sigma=0.1), F)
    V, F = synth.geodesic_sphere(20)
    V = synth.sh_deform(V, rng, lmax=8, sigma=0.08)
    out["holes"] = (V, synth.delete_patch(synth.delete_random_faces(F, rng, 0.02), rng, 200))
    # duplicated, flipped, degenerate and non-manifold triangles
    V, F = synth.icosphere(2)
    F = np.concatenate([F, F[:10], F[10:20, ::-1], [[0, 0, 1], [2, 2, 2]],
                        [[F[0, 0], F[0, 1], 5], [F[0, 1], F[0, 0], 7]]]).astype(np.int32)
    out["messy"] = (V, F)
    return {k: (np.ascontiguousarray(v), np.ascontiguousarray(f, dtype=np.int32))
            for k, (v, f) in out.items()}


def test_hier_matches_all_pairs(cuda):
    for name, (V, F) in _meshes().items():
        Q = _queries(V, 3000, 62)
        W = G.WindingNumberAABB(V, F).winding_number(Q)
        W64 = G.winding_number(V, F, Q, precision="fp64")
        err = np.abs(W - W64)
        assert err.max() <= 1e-4, (name, err.max())
        assert np.quantile(err, 0.99) <= 1e-6, (name, np.quantile(err, 0.99))
        away = np.abs(W64 - 0.5) > 1e-3
        assert np.array_equal((W > 0.5)[away], (W64 > 0.5)[away]), name


def test_hier_matches_cpu_hierarchy(cuda):
    V, F = _meshes()["holes"]
    Q = _queries(V, 500, 63)
    W = G.WindingNumberAABB(V, F).winding_number(Q)
    Wr = O.winding_number_hier(V, F, Q)
    assert np.abs(W - Wr).max() <= 1e-4


def test_hier_large_mesh_and_device(cuda):
    torch = cuda
    V, F = synth.geodesic_sphere(60)  # 72,000 triangles
    rng = np.random.default_rng(64)
    V = synth.sh_deform(V, rng, lmax=8, sigma=0.05)
    F = synth.delete_patch(F, rng, 500)
    Q = _queries(V, 20000, 65)
    h = G.WindingNumberAABB(torch.from_numpy(V).cuda(), torch.from_numpy(F).cuda())
    Wd = h.winding_number(torch.from_numpy(Q).cuda()).cpu().numpy()
    Wh = G.WindingNumberAABB(V, F).winding_number(Q)
    assert np.array_equal(Wd, Wh)
    sub = np.random.default_rng(66).choice(Q.shape[0], 4000, replace=False)
    W64 = G.winding_number(V, F, Q[sub], precision="fp64")
    assert np.abs(Wh[sub] - W64).max() <= 1e-4


def test_hier_tiny_and_empty(cuda):
    Q = np.array([[0.2, 0.2, 0.3], [5.0, 5.0, 5.0], [0.1, 0.1, -0.2]])
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    for F in (np.zeros((0, 3), np.int32), np.array([[0, 1, 2]], np.int32),
              np.array([[0, 1, 2], [0, 3, 1]], np.int32),
              np.array([[0, 2, 1], [0, 3, 2], [0, 1, 3], [1, 2, 3]], np.int32)):
        W = G.WindingNumberAABB(V, F).winding_number(Q)
        W64 = G.winding_number(V, F, Q, precision="fp64") if F.shape[0] else np.zeros(3)
        np.testing.assert_allclose(W, W64, atol=1e-6)


def test_hier_bad_index_raises(cuda):
    V, F = synth.icosphere(2)
    F = np.ascontiguousarray(F, dtype=np.int32)
    F[3, 1] = V.shape[0] + 4
    with pytest.raises(G.GwnError):
        G.WindingNumberAABB(V, F)


def test_fp64_hierarchy_matches_cpu_hierarchy_and_all_pairs(cuda):
    """The plain-FP64 walk (the reference's: a node's cap for a point
    strictly outside its box, every term in FP64) against the CPU
    restatement of the reference hierarchy (oracle/wn_hier.cpp) and the FP64
    all-pairs sum: rounding only.  Uniform queries 1e-11; queries down to
    1e-6 x the diagonal from the surface, where a triangle term itself loses
    digits (the GPU fuses multiply-adds, the CPU does not), 1e-9."""
    for name, (V, F) in _meshes().items():
        h = G.WindingNumberAABB(V, F)
        for near, tol in ((False, 1e-11), (True, 1e-9)):
            Q = _queries(V, 1000, 67, near=near)
            W64 = h.winding_number(Q, precision="fp64")
            Wr = O.winding_number_hier(V, F, Q)
            Wa = O.winding_number(V, F, Q)
            assert np.abs(W64 - Wr).max() <= tol, (name, near, np.abs(W64 - Wr).max())
            assert np.abs(W64 - Wa).max() <= tol, (name, near, np.abs(W64 - Wa).max())
    # gwn_winding_number in plain FP64 takes the hierarchy from 4096 triangles
    # and 1024 queries, with float64 or float32 queries and results
    V, F = _meshes()["holes"]
    Q = _queries(V, 2000, 68, near=False)
    W = G.winding_number(V, F, Q, precision="fp64")
    assert np.abs(W - O.winding_number(V, F, Q)).max() <= 1e-11
    Q32 = Q.astype(np.float32)
    W32 = G.winding_number(V, F, Q32, precision="fp64")
    assert W32.dtype == np.float32
    ref = O.winding_number(V, F, Q32.astype(np.float64))
    assert np.abs(W32.astype(np.float64) - ref).max() <= 1e-6
    Wm32 = G.winding_number(V, F, Q32, precision="mixed")
    assert np.abs(Wm32.astype(np.float64) - ref).max() <= 1e-4
