"""Closest triangle and signed distance on the GPU (distance.cu) against the
CPU oracle (oracle/distance.cpp: brute force over all triangles with
Ericson's closest point, and the reference's sign rules,
include/igl/signed_distance.cpp:83-137).

Tolerances: squared distances 1e-12 relative plus 1e-14 |d| (both FP64;
the closest point carries an absolute rounding of a few 1e-16, which
dominates d^2 = |p - c|^2 for points very close to the surface), closest
points 1e-9; the triangle index is checked through its
own distance (a tie may pick another triangle at the same distance); signs
from the exact winding number agree to 1e-9; the fast-winding-number sign is
the reference's soup algorithm on its own tree, so S may differ by
2 |dW| |S| with |dW| <= 2e-2 (the reference's own test tolerance against the
exact winding number is 1e-2)."""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tet():
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    F = np.array([[0, 1, 3], [0, 2, 1], [0, 3, 2], [1, 2, 3]], np.int32)
    return V, F


def test_single_tet_golden(cuda):
    """tests/include/igl/signed_distance.cpp:4-42."""
    V, F = _tet()
    P = np.array([[0.5, 0.5, 0.5]])
    for t, tol in ((G.SIGNED_DISTANCE_TYPE_PSEUDONORMAL, 1e-15),
                   (G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER, 1e-15),
                   (G.SIGNED_DISTANCE_TYPE_DEFAULT, 1e-15),
                   (G.SIGNED_DISTANCE_TYPE_UNSIGNED, 1e-15),
                   (G.SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER, 1e-7)):
        S, I, Cp = G.signed_distance(P, V, F, t)
        assert abs(S[0] - np.sqrt(1 / 12)) <= tol, (t, S)
        assert I[0] == 3 and np.allclose(Cp[0], 1 / 3, atol=1e-15)
    # pseudonormal inside / outside / at a vertex region, with its normals
    Q = np.array([[0.5, 0.5, 0.5], [0.1, 0.1, 0.1], [2, 2, 2], [-1, -1, -1], [0.3, -1, 0.3]])
    S, I, Cp, Nn = G.signed_distance(Q, V, F, G.SIGNED_DISTANCE_TYPE_PSEUDONORMAL,
                                     return_normals=True)
    Sr, Ir, Cr, Nr = O.signed_distance(Q, V, F, G.SIGNED_DISTANCE_TYPE_PSEUDONORMAL,
                                       return_normals=True)
    assert np.abs(S - Sr).max() <= 1e-15
    # (0.1, 0.1, 0.1) is equally close to three faces and (-1, -1, -1) to the
    # vertex they share: the closest face (and for the first the normal)
    # follows whichever face each side reached first
    same = I == Ir
    assert same.sum() >= 3 and np.abs(Nn[same] - Nr[same]).max() <= 1e-15


@pytest.fixture(scope="module")
def mesh():
    V, F = synth.soup_mesh(seed=21, subdiv=3, delete_frac=0.02)
    rng = np.random.default_rng(22)
    lo, hi = V.min(0), V.max(0)
    far = rng.uniform(lo - 0.5, hi + 0.5, size=(15000, 3))
    Pn, f = synth.sample_on_faces(V, F, rng, 5000)
    Nn = synth.face_normals(V, F)[f]
    near = Pn + Nn * (rng.choice([-1, 1], (5000, 1)) * 10.0 ** rng.uniform(-7, -1, (5000, 1)))
    return V, F, np.concatenate([far, near, V[:50]])  # and points on vertices (ties)


def _close2(D, Dr):
    return np.abs(D - Dr) <= 1e-12 * Dr + 1e-14 * np.sqrt(Dr) + 1e-300


def _tri_dist2(V, F, P, I):
    out = np.empty(3)
    L = O.lib()
    d = np.empty(len(P))
    for k in range(len(P)):
        t = V[F[I[k]]]
        a, b, c = (np.ascontiguousarray(t[j]) for j in range(3))
        p = np.ascontiguousarray(P[k])
        d[k] = L.oracle_point_triangle(O._ptr(p), O._ptr(a), O._ptr(b), O._ptr(c), O._ptr(out))
    return d


def test_squared_distance_matches_brute_force(mesh, cuda):
    V, F, P = mesh
    bvh = G.FastWindingNumberBVH(V, F)
    D, I, Cp = bvh.squared_distance(P)
    bvh.close()
    Dr, Ir, Cr = O.squared_distance(V, F, P)
    assert np.all(I >= 0)
    assert np.all(_close2(D, Dr))
    # the reported triangle is at the reported distance (tie-safe)
    assert np.all(_close2(_tri_dist2(V, F, P, I), D))
    # a closest edge or vertex is shared by several triangles (ties), so the
    # indices may differ; the closest points agree
    assert np.abs(Cp - Cr).max() <= 1e-9
    # f32 queries: the same up to the query's rounding
    D32, I32, _ = G.FastWindingNumberBVH(V, F).squared_distance(P.astype(np.float32))
    Dr32, _, _ = O.squared_distance(V, F, P.astype(np.float32).astype(np.float64))
    assert np.all(_close2(D32, Dr32))


def test_signed_distance_against_oracle(mesh, cuda):
    V, F, P = mesh
    for t in (G.SIGNED_DISTANCE_TYPE_UNSIGNED, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER,
              G.SIGNED_DISTANCE_TYPE_DEFAULT):
        S, I, Cp = G.signed_distance(P, V, F, t)
        Sr, Ir, Cr = O.signed_distance(P, V, F, t)
        assert np.abs(S - Sr).max() <= 1e-9 * (1 + np.abs(Sr).max()), t
    # pseudonormal: the sign follows the closest feature, so a tie in the
    # closest triangle may pick another feature's normal; compare where the
    # closest triangles agree, and the magnitude everywhere
    S, I, Cp, Nn = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_PSEUDONORMAL,
                                     return_normals=True)
    Sr, Ir, Cr, Nr = O.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_PSEUDONORMAL,
                                       return_normals=True)
    assert np.all(np.abs(np.abs(S) - np.abs(Sr)) <= 1e-12 * (1 + np.abs(Sr)))
    same = I == Ir
    assert same.mean() > 0.5
    assert np.array_equal(np.sign(S[same]), np.sign(Sr[same]))
    assert np.abs(Nn[same] - Nr[same]).max() <= 1e-9
    # and the pseudonormal sign agrees with the exact winding number's
    # away from the surface and the holes' rims
    Sw, _, _ = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER)
    clear = np.abs(Sw) > 1e-3
    assert (np.sign(S[clear]) == np.sign(Sw[clear])).mean() > 0.95
    # fast-winding-number sign
    S, I, Cp = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER)
    Sr, _, _ = O.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER)
    assert np.all(np.abs(S - Sr) <= 2 * 2e-2 * np.abs(Sr) + 1e-12)
    # mixed and plain FP64 exact sign agree to the mixed tolerance
    Sm, _, _ = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER,
                                 precision="mixed")
    S64, _, _ = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER)
    assert np.all(np.abs(Sm - S64) <= 2e-4 * np.abs(S64) + 1e-12)


def test_bounds_empty_and_device(mesh, cuda):
    torch = cuda
    V, F, P = mesh
    lo, hi = -0.05, 0.2
    S, I, Cp = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER, lo, hi)
    Sr, Ir, Cr = O.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER, lo, hi)
    nan = np.isnan(Sr)
    assert nan.any() and (~nan).any()
    assert np.array_equal(np.isnan(S), nan)
    assert np.all(I[nan] == F.shape[0] + 1) and np.all(Cp[nan] == 0)
    assert np.abs(S[~nan] - Sr[~nan]).max() <= 1e-9
    # empty F (signed_distance.cpp:395-402)
    S0, I0, C0 = G.signed_distance(P[:5], V, np.zeros((0, 3), np.int32))
    assert np.all(np.isnan(S0)) and np.all(I0 == -1) and np.all(np.isnan(C0))
    # device tensors give the host result
    Sd, Id, Cd = G.signed_distance(torch.from_numpy(P).cuda(), torch.from_numpy(V).cuda(),
                                   torch.from_numpy(F).cuda(),
                                   G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER)
    Sh, Ih, Ch = G.signed_distance(P, V, F, G.SIGNED_DISTANCE_TYPE_WINDING_NUMBER)
    assert np.array_equal(Sd.cpu().numpy(), Sh) and np.array_equal(Id.cpu().numpy(), Ih)


def test_squared_distance_random_soup_with_skinny_triangles(cuda):
    """Random triangles (many of them long and thin, some degenerate) and
    queries near and far: the FP32 leaf screen never drops the closest
    triangle (exact brute-force distance)."""
    rng = np.random.default_rng(41)
    nF = 3000
    A = rng.uniform(-1, 1, (nF, 3))
    B = A + rng.normal(0, 0.3, (nF, 3))
    # a third of the triangles nearly collinear, a few exactly degenerate
    t = rng.uniform(0, 1, (nF, 1))
    Cc = A + rng.normal(0, 0.3, (nF, 3))
    thin = rng.random(nF) < 0.33
    Cc[thin] = (A + t * (B - A) + rng.normal(0, 1e-6, (nF, 3)))[thin]
    Cc[:10] = A[:10]
    V = np.concatenate([A, B, Cc])
    F = np.stack([np.arange(nF), nF + np.arange(nF), 2 * nF + np.arange(nF)], 1).astype(np.int32)
    P = np.concatenate([rng.uniform(-1.5, 1.5, (6000, 3)),
                        V[rng.integers(0, len(V), 2000)] + rng.normal(0, 1e-4, (2000, 3))])
    D, I, Cp = G.FastWindingNumberBVH(V, F).squared_distance(P)
    Dr, Ir, Cr = O.squared_distance(V, F, P)
    assert np.all(_close2(D, Dr))
    assert np.all(_close2(_tri_dist2(V, F, P, I), D))
