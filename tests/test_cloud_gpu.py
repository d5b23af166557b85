"""GPU parity of the point-cloud path: octree bit-exact with igl::octree,
expansion precompute and Barnes-Hut evaluation against the FP64 oracle
(restated include/igl/octree.cpp and fast_winding_number.cpp), through the
C ABI; the reference's own golden vector
(tests/include/igl/fast_winding_number.cpp:17-53, 1e-15)."""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-4


def assert_octree_equal(P):
    off, idx, CH, CN, W = G.octree(P)
    t = O.octree(P)
    assert np.array_equal(CH, t.CH)
    assert np.array_equal(off, t.pi_off)
    assert np.array_equal(idx, t.pi_idx)
    assert np.array_equal(CN.view(np.int64), t.CN.view(np.int64))  # bit-exact centres
    assert np.array_equal(W.view(np.int64), t.W.view(np.int64))


@pytest.mark.parametrize("n", [1, 2, 3, 17, 1000, 50000])
def test_octree_bit_exact_random(cuda, n):
    rng = np.random.default_rng(n)
    assert_octree_equal(rng.random((n, 3)))


def test_octree_bit_exact_structured(cuda):
    rng = np.random.default_rng(3)
    # clustered, on a plane, collinear, integer lattice (ties at centres)
    A = rng.normal(size=(2000, 3)) * 1e-3
    B = np.c_[rng.random(500), rng.random(500), np.zeros(500)]
    C = np.c_[np.linspace(0, 1, 300), np.zeros(300), np.zeros(300)]
    D = np.stack(np.meshgrid(np.arange(6.0), np.arange(6.0), np.arange(6.0)), -1).reshape(-1, 3)
    for P in (A, B, C, D, np.concatenate([A, B + 5])):
        assert_octree_equal(P)


def test_octree_duplicates_reach_max_depth(cuda):
    # identical points recurse to depth 30000 (octree.cpp:16, :98)
    P = np.array([[0.25, 0.5, 0.75], [0.25, 0.5, 0.75], [0.9, 0.1, 0.3], [0.9, 0.1, 0.3],
                  [0.9, 0.1, 0.3], [0.1, 0.1, 0.1]])
    assert_octree_equal(P)
    t = G.Octree(P)
    assert t.sizes()[2] == 30000


def test_octree_torus_config_scale(cuda):
    P, _, _ = synth.torus_cloud(seed=3, n=200_000)
    assert_octree_equal(P)


def test_one_point_cloud_golden(cuda):
    # tests/include/igl/fast_winding_number.cpp:17-53, tolerance 1e-15 (:52)
    P = np.array([[0.1, 0.2, 0.3]])
    N = np.array([[4.0, 5.0, 6.0]])
    N /= np.linalg.norm(N[0])
    A = np.array([0.7])
    Q = np.array([[0, 0, 0], [4, -3, 2], [-1, 1, 3], [0, 5, -2]], float)
    expected = np.array([0.38779369004261133, -0.00041235296362485, -0.00362978253577090,
                         -0.00041235296362485])
    W = G.fast_winding_number_cloud_oneshot(P, N, A, Q, 2, 2.0, precision="fp64")
    assert np.abs(W - expected).max() <= 1e-15
    Wm = G.fast_winding_number_cloud_oneshot(P, N, A, Q, 2, 2.0, precision="mixed")
    assert np.abs(Wm - expected).max() <= TOL_MIXED


@pytest.fixture(scope="module")
def torus(cuda):
    P, Nn, A = synth.torus_cloud(seed=3, n=60_000)
    Q = synth.cloud_queries(seed=4, nq=20_000)
    t = O.octree(P)
    CM, R, EC = O.cloud_precompute(P, Nn, A, t, 2)
    return P, Nn, A, Q, t, CM, R, EC


def test_precompute_matches_oracle(torus):
    P, Nn, A, Q, t, CM, R, EC = torus
    ce = G.CloudExpansion(P, Nn, A, order=2)
    gCM, gR, gEC = ce.export()
    ne = np.diff(t.pi_off) > 0
    assert np.all(np.isnan(gCM[~ne])) and np.all(gR[~ne] == 0) and np.all(gEC[~ne] == 0)
    scale = np.abs(CM[ne]).max()
    assert np.abs(gCM[ne] - CM[ne]).max() <= 1e-13 * scale
    assert np.abs(gR[ne] - R[ne]).max() <= 1e-12 * np.abs(R[ne]).max()
    sc = np.abs(EC[ne]).max(axis=0) + 1e-300
    assert (np.abs(gEC[ne] - EC[ne]) / sc).max() <= 1e-11
    # single-point cells reproduce the oracle bit for bit
    one = np.diff(t.pi_off) == 1
    assert np.array_equal(gCM[one], CM[one]) and np.array_equal(gR[one], R[one])


def test_eval_fp64_matches_oracle(torus):
    P, Nn, A, Q, t, CM, R, EC = torus
    Wref = O.cloud_eval(P, Nn, A, t, CM, R, EC, Q, 2.0)
    ce = G.CloudExpansion(P, Nn, A, order=2)
    W64 = ce.eval(Q, 2.0, precision="fp64")
    assert np.abs(W64 - Wref).max() <= 1e-11
    Wm = ce.eval(Q, 2.0, precision="mixed")
    err = np.abs(Wm - Wref)
    assert err.max() <= TOL_MIXED, err.max()
    out = np.abs(Wref - 0.5) > 1e-3
    assert np.array_equal((Wm > 0.5)[out], (Wref > 0.5)[out])
    Wf = ce.eval(Q.astype(np.float32), 2.0, precision="mixed")
    assert Wf.dtype == np.float32


def test_drop_in_arrays_forms(torus):
    P, Nn, A, Q, t, CM, R, EC = torus
    gCM, gR, gEC = G.fast_winding_number_cloud_precompute(P, Nn, A, t.pi_off, t.pi_idx, t.CH, 2)
    ne = np.diff(t.pi_off) > 0
    assert np.abs(gCM[ne] - CM[ne]).max() <= 1e-13 * np.abs(CM[ne]).max()
    # evaluation over caller arrays, including the reference's 8*#cells-row outputs
    nc = t.ncells
    CM8 = np.vstack([CM, np.zeros((7 * nc, 3))])
    EC8 = np.vstack([EC, np.zeros((7 * nc, EC.shape[1]))])
    R8 = np.concatenate([R, np.zeros(7 * nc)])
    Qs = Q[:4000]
    Wref = O.cloud_eval(P, Nn, A, t, CM, R, EC, Qs, 2.0)
    W = G.fast_winding_number_cloud(P, Nn, A, t.pi_off, t.pi_idx, t.CH, CM8, R8, EC8, Qs, 2.0,
                                    precision="fp64")
    assert np.abs(W - Wref).max() <= 1e-11


@pytest.mark.parametrize("order", [0, 1])
def test_lower_orders(cuda, order):
    P, Nn, A = synth.torus_cloud(seed=8, n=20_000)
    Q = synth.cloud_queries(seed=9, nq=4000)
    t = O.octree(P)
    CM, R, EC = O.cloud_precompute(P, Nn, A, t, order)
    Wref = O.cloud_eval(P, Nn, A, t, CM, R, EC, Q, 2.0)
    ce = G.CloudExpansion(P, Nn, A, order=order)
    assert np.abs(ce.eval(Q, 2.0, precision="fp64") - Wref).max() <= 1e-11
    assert np.abs(ce.eval(Q, 2.0, precision="mixed") - Wref).max() <= TOL_MIXED


def test_direct_sum_beta_nonpositive(cuda):
    P, Nn, A = synth.torus_cloud(seed=10, n=3000)
    Q = synth.cloud_queries(seed=11, nq=500)
    t = O.octree(P)
    CM, R, EC = O.cloud_precompute(P, Nn, A, t, 2)
    Wref = O.cloud_eval(P, Nn, A, t, CM, R, EC, Q, 0.0)
    ce = G.CloudExpansion(P, Nn, A, order=2)
    # the direct sum adds thousands of dipoles of magnitude up to ~10: rounding
    # of the summation order is ~1e-16 * sum |term|
    W64 = ce.eval(Q, 0.0, precision="fp64")
    assert np.abs(W64 - Wref).max() <= 1e-10, np.abs(W64 - Wref).max()
    Wm = ce.eval(Q, -1.0, precision="mixed")
    assert np.abs(Wm - Wref).max() <= TOL_MIXED, np.abs(Wm - Wref).max()


def test_query_on_a_point_gives_half_dipole(cuda):
    # direct_eval returns 0.5 when the point coincides with the query (:164-166)
    P = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    Nn = np.array([[0, 0, 1.0]] * 3)
    A = np.array([0.1, 0.1, 0.1])
    Q = P.copy()
    t = O.octree(P)
    CM, R, EC = O.cloud_precompute(P, Nn, A, t, 2)
    Wref = O.cloud_eval(P, Nn, A, t, CM, R, EC, Q, 2.0)
    for prec in ("fp64", "mixed"):
        W = G.fast_winding_number_cloud_oneshot(P, Nn, A, Q, 2, 2.0, precision=prec)
        assert np.abs(W - Wref).max() <= 1e-12
