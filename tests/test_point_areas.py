"""Per-point areas of a point cloud (igl::copyleft::cgal::point_areas,
include/igl/copyleft/cgal/point_areas.cpp:60-160) and the CGAL module's
point-cloud winding number that uses them
(copyleft/cgal/fast_winding_number.cpp:9-44).

The reference has no test of its own for this function and CGAL is not in
the image, so the CPU oracle (oracle/point_areas.cpp) restates it with
methods of its own (one-sided Jacobi SVD, a brute-force empty-circle
Delaunay triangulation), independent of the GPU's (scatter-matrix
eigenvectors, the Delaunay star found by inversion), and both are pinned on
analytic cases: a point inside a hexagonal lattice owns its hexagonal
Voronoi cell, (sqrt(3)/2) h^2, and a sampled sphere's areas sum to 4 pi
within the method's own bias."""
import numpy as np
import pytest

from libigl_gb300 import synth
from oracle import oracle as O


def _hex_lattice(h=0.1, n=8, jitter=1e-6, seed=0):
    rng = np.random.default_rng(seed)
    pts = [[h * (i + 0.5 * (j % 2)), h * j * np.sqrt(3) / 2, 0.0]
           for i in range(-n, n + 1) for j in range(-n, n + 1)]
    P = np.array(pts) + rng.normal(0, jitter, (len(pts), 3)) * [1, 1, 0]
    N = np.tile([0.0, 0.0, 1.0], (len(P), 1))
    return P, N


def _knn_brute(P, k):
    d = ((P[:, None, :] - P[None, :, :]) ** 2).sum(-1)
    return np.argsort(d, axis=1, kind="stable")[:, :k].astype(np.int32)


def _sphere(n, seed=1):
    rng = np.random.default_rng(seed)
    P = rng.normal(size=(n, 3))
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    return P, P.copy()


def test_oracle_analytic_cases():
    h = 0.1
    P, N = _hex_lattice(h)
    I = _knn_brute(P, 19)
    A, T = O.point_areas(P, I, N)
    inner = np.linalg.norm(P[:, :2], axis=1) < 0.4
    assert np.abs(A[inner] / (np.sqrt(3) / 2 * h * h) - 1).max() < 1e-4
    assert np.allclose(T[inner], [0, 0, 1], atol=1e-6)
    # flipped normals: T turns towards N, and neighbours whose normal
    # disagrees with the first neighbour's are dropped
    A2, T2 = O.point_areas(P, I, -N)
    assert np.allclose(A2, A) and np.allclose(T2[inner], [0, 0, -1], atol=1e-6)
    Nmix = N.copy()
    Nmix[::2] *= -1
    A3, _ = O.point_areas(P, I, Nmix)
    assert not np.allclose(A3, A)
    # fewer than three kept neighbours: 0
    A1, T1 = O.point_areas(P, I[:, :2], N)
    assert np.all(A1 == 0) and np.all(T1 == 0)
    # a randomly sampled sphere's areas sum to its area within the method's
    # own bias (each point triangulates only its k neighbours: 5% here)
    Ps, Ns = _sphere(3000)
    As, _ = O.point_areas(Ps, _knn_brute(Ps, 16), Ns)
    assert abs(As.sum() / (4 * np.pi) - 1) < 0.1


@pytest.mark.gpu
def test_gpu_matches_oracle(cuda):
    import libigl_gb300 as G
    # lattice, sphere and a noisy torus sample with jittered normals
    cases = []
    P, N = _hex_lattice()
    cases.append((P, N, _knn_brute(P, 19)))
    Ps, Ns = _sphere(4000)
    cases.append((Ps, Ns, G.knn(Ps, Ps, 16)))
    Pt, Nt, _ = synth.torus_cloud(seed=5, n=20_000)
    for k in (8, 21, 40):
        cases.append((Pt, Nt, G.knn(Pt, Pt, k)))
    for P, N, I in cases:
        A, T = G.point_areas(P, I, N, return_T=True)
        Ao, To = O.point_areas(P, I, N)
        rel = np.abs(A - Ao) / np.maximum(np.abs(Ao), 1e-300)
        close = rel <= 1e-9
        # near-cocircular neighbourhoods may triangulate differently in the
        # two methods' rounding: at most one point in a thousand
        assert close.mean() >= 0.999, (I.shape, close.mean(), rel.max())
        assert np.median(rel) <= 1e-12
        dots = np.einsum("ij,ij->i", T, To)
        assert np.all(dots[Ao > 0] > 1 - 1e-9)
    # area sums
    As = G.point_areas(Ps, G.knn(Ps, Ps, 16), Ns)
    assert abs(As.sum() / (4 * np.pi) - 1) < 0.1


@pytest.mark.gpu
def test_gpu_edge_cases(cuda):
    import libigl_gb300 as G
    P, N = _hex_lattice()
    I = _knn_brute(P, 19)
    for k in (1, 2):
        A, T = G.point_areas(P, I[:, :k], N, return_T=True)
        assert np.all(A == 0) and np.all(T == 0)
    # duplicated points in the neighbourhood count once
    P2 = np.concatenate([P, P[:40]])
    N2 = np.concatenate([N, N[:40]])
    I2 = _knn_brute(P2, 24)
    A2 = G.point_areas(P2, I2, N2)
    Ao2, _ = O.point_areas(P2, I2, N2)
    assert np.allclose(A2, Ao2, rtol=1e-9, atol=0)
    # device tensors, and an index outside P raises
    torch = cuda
    Ad = G.point_areas(torch.from_numpy(P).cuda(), torch.from_numpy(I).cuda(),
                       torch.from_numpy(N).cuda())
    assert np.array_equal(Ad.cpu().numpy(), G.point_areas(P, I, N))
    Ib = I.copy()
    Ib[3, 5] = P.shape[0] + 2
    with pytest.raises(G.GwnError):
        G.point_areas(P, Ib, N)
    with pytest.raises(G.GwnError):
        G.point_areas(P, np.zeros((P.shape[0], 200), np.int32), N)


@pytest.mark.gpu
def test_cloud_winding_number_from_points_alone(cuda):
    """copyleft/cgal/fast_winding_number: octree, 21 nearest points, areas,
    expansions, evaluation -- equal to composing the steps by hand, and the
    right inside / outside values on a torus."""
    import libigl_gb300 as G
    P, Nn, _ = synth.torus_cloud(seed=9, n=30_000)
    rng = np.random.default_rng(3)
    Q = rng.uniform([-1.6, -1.6, -0.6], [1.6, 1.6, 0.6], (20_000, 3))
    W = G.fast_winding_number_cloud_points(P, Nn, Q, 2, 2.0, precision="fp64")
    A = G.point_areas(P, G.knn(P, P, 21), Nn)
    Wc = G.fast_winding_number_cloud_oneshot(P, Nn, A, Q, 2, 2.0, precision="fp64")
    assert np.abs(W - Wc).max() <= 1e-12
    # analytic torus (R = 1, r = 0.35): away from the surface W ~ 1 inside
    rho = np.hypot(np.hypot(Q[:, 0], Q[:, 1]) - 1.0, Q[:, 2])
    inside, outside = rho < 0.25, rho > 0.45
    assert np.abs(W[inside] - 1).max() < 0.05 and np.abs(W[outside]).max() < 0.05
    Wm = G.fast_winding_number_cloud_points(P, Nn, Q, 2, 2.0, precision="mixed")
    assert np.abs(Wm - W).max() <= 1e-4
