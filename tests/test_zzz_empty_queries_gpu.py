"""Empty query sets through the GPU entry points whose other tests use
non-empty ones: the point-cloud evaluation (both precisions), the
points-only cloud winding number, knn (with and without a built octree),
point areas of no points, and the signed distance of no points.  The
reference loops over no rows and returns empty outputs
(fast_winding_number.cpp:126-311, knn.cpp:24-136, signed_distance.cpp:83-137);
each call here returns an empty result and launches nothing on a zero-sized
grid."""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth

pytestmark = pytest.mark.gpu


def test_empty_queries(cuda):
    G.device_status(clear=True)  # start from a clear sticky word
    P, Nn, A = synth.torus_cloud(seed=3, n=2000)
    Q0 = np.zeros((0, 3))
    ce = G.CloudExpansion(P, Nn, A, order=2)
    for prec in ("mixed", "fp64"):
        assert ce.eval(Q0, 2.0, precision=prec).shape == (0,)
    assert ce.eval(Q0.astype(np.float32), 2.0).shape == (0,)
    assert G.fast_winding_number_cloud_points(P, Nn, Q0).shape == (0,)
    assert G.knn(Q0, P, 8).shape == (0, 8)
    t = G.Octree(P)
    assert t.knn(Q0, 8).shape == (0, 8)
    A0 = G.point_areas(np.zeros((0, 3)), np.zeros((0, 8), np.int32), np.zeros((0, 3)))
    assert A0.shape == (0,)
    V, F = synth.geodesic_sphere(8)
    for sign_type in (0, 1, 2, 3, 4):
        S, I, C = G.signed_distance(Q0, V, F, sign_type)
        assert S.shape == (0,) and I.shape == (0,) and C.shape == (0, 3)
    # the library is still in a good state afterwards
    W = ce.eval(P[:64] + 0.5, 2.0, precision="fp64")
    assert W.shape == (64,) and np.all(np.isfinite(W))
    assert G.device_status() == 0
