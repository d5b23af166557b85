"""CPU tests of the Python host mirror's argument checks: arrays whose shapes
do not match what the C ABI reads from their pointers are refused with
ValueError before any call into libgwn, so these run without a GPU."""
import numpy as np
import pytest

import libigl_gb300 as gb


@pytest.fixture(scope="module", autouse=True)
def _lib(gwn_lib):
    return gwn_lib


def _cloud(n=4):
    rng = np.random.default_rng(0)
    P = rng.random((n, 3))
    Nrm = rng.standard_normal((n, 3))
    A = np.ones(n)
    off = np.array([0, n], np.int64)            # the root cell holds every point
    idx = np.arange(n, dtype=np.int32)
    CH = np.full((1, 8), -1, np.int32)
    return P, Nrm, A, off, idx, CH


def test_knn_shapes():
    with pytest.raises(ValueError, match="P must be"):
        gb.knn(np.zeros(6), np.zeros((2, 3)), 1)
    with pytest.raises(ValueError, match="V must be"):
        gb.knn(np.zeros((2, 3)), np.zeros((2, 2)), 1)
    with pytest.raises(ValueError, match="k must be non-negative"):
        gb.knn(np.zeros((2, 3)), np.zeros((2, 3)), -1)


def test_point_areas_shapes():
    P = np.zeros((3, 3))
    I = np.zeros((3, 2), np.int32)
    with pytest.raises(ValueError, match="N must be 3 x 3"):
        gb.point_areas(P, I, np.zeros((2, 3)))
    with pytest.raises(ValueError, match="P must be"):
        gb.point_areas(np.zeros((3, 2)), I, np.zeros((3, 3)))
    with pytest.raises(ValueError, match="I must be"):
        gb.point_areas(P, np.zeros((2, 2), np.int32), np.zeros((3, 3)))


def test_cloud_points_shapes():
    with pytest.raises(ValueError, match="N must be 3 x 3"):
        gb.fast_winding_number_cloud_points(np.zeros((3, 3)), np.zeros((4, 3)), np.zeros((1, 3)))
    with pytest.raises(ValueError, match="Q must be"):
        gb.fast_winding_number_cloud_points(np.zeros((3, 3)), np.zeros((3, 3)), np.zeros(3))


def test_cloud_array_overloads_shapes():
    P, Nrm, A, off, idx, CH = _cloud()
    pre = gb.fast_winding_number_cloud_precompute
    with pytest.raises(ValueError, match="pi_offsets must hold"):
        pre(P, Nrm, A, off[:1], idx, CH)
    with pytest.raises(ValueError, match="pi_indices must hold"):
        pre(P, Nrm, A, off, idx[:2], CH)
    with pytest.raises(ValueError, match="CH must be"):
        pre(P, Nrm, A, off, idx, CH[:, :4])
    with pytest.raises(ValueError, match="N must be"):
        pre(P, Nrm[:2], A, off, idx, CH)
    with pytest.raises(ValueError, match="A must hold"):
        pre(P, Nrm, A[:3], off, idx, CH)
    with pytest.raises(ValueError, match="order must be"):
        pre(P, Nrm, A, off, idx, CH, order=3)
    ev = gb.fast_winding_number_cloud
    CM, R, EC = np.zeros((1, 3)), np.zeros(1), np.zeros((1, 39))
    Q = np.zeros((2, 3))
    with pytest.raises(ValueError, match="EC must be"):
        ev(P, Nrm, A, off, idx, CH, CM, R, np.zeros((1, 7)), Q)
    with pytest.raises(ValueError, match="CM must be"):
        ev(P, Nrm, A, off, idx, CH, np.zeros((0, 3)), R, EC, Q)
    with pytest.raises(ValueError, match="Q must be"):
        ev(P, Nrm, A, off, idx, CH, CM, R, EC, np.zeros(3))
    # the reference's 8 * #cells rows are accepted (only the first #cells are read)
    with pytest.raises(ValueError, match="pi_offsets must hold"):
        ev(P, Nrm, A, off[:1], idx, CH, np.zeros((8, 3)), np.zeros(8), np.zeros((8, 39)), Q)


def test_eytzinger_winding_number_shapes():
    P = np.zeros((1, 2))
    V = np.zeros((2, 2))
    E = np.array([[0, 1]], np.int32)
    leaf = np.array([-1, 0], np.int32)
    B1 = np.zeros((2, 2))
    I = np.zeros(0, np.int32)
    Cc = np.zeros(3, np.int32)
    with pytest.raises(ValueError, match="B1 must be 2 x 2"):
        gb.eytzinger_aabb_winding_number(P, V, E, B1[:1], B1, leaf, I, Cc)
    with pytest.raises(ValueError, match="C must hold 3"):
        gb.eytzinger_aabb_winding_number(P, V, E, B1, B1, leaf, I, Cc[:2])
    with pytest.raises(ValueError, match="E must be"):
        gb.eytzinger_aabb_winding_number(P, V, np.zeros((1, 3), np.int32), B1, B1, leaf, I, Cc)


def test_swept_volume_seed_length():
    V = np.zeros((3, 3))
    F = np.array([[0, 1, 2]], np.int32)
    GV = np.zeros((8, 3))
    T = np.tile(np.eye(4)[:3], (1, 1, 1))
    with pytest.raises(ValueError, match="S0 must hold 8"):
        gb.swept_volume_signed_distance(V, F, T, 1, GV, (2, 2, 2), 1.0, 0.0, S0=np.zeros(7))
