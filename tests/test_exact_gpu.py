"""GPU parity of the exact winding number (igl::winding_number) against the
FP64 oracle (restated solid_angle.cpp / winding_number.cpp), through the C ABI."""
import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# FP64 GPU vs FP64 oracle: same formula, different atan2/sqrt implementations
# and summation order -> rounding level.
TOL_FP64 = 1e-11
# Mixed vs FP64 oracle: the metric bound |dW| <= 1e-4.
TOL_MIXED = 1e-4


@pytest.fixture(scope="module")
def c1(cuda):
    V, F, Q = synth.exact_workload(seed=0, subdiv=4, nq=100_000)
    W = O.winding_number(V, F, Q)
    return V, F, Q, W


def test_exact_fp64_matches_oracle_full_config(c1):
    V, F, Q, Wref = c1
    W = G.winding_number(V, F, Q, precision="fp64")
    assert W.dtype == np.float64
    assert np.abs(W - Wref).max() <= TOL_FP64
    assert np.array_equal(W > 0.5, Wref > 0.5)


def test_exact_mixed_matches_oracle_full_config(c1):
    V, F, Q, Wref = c1
    W = G.winding_number(V, F, Q, precision="mixed")
    err = np.abs(W - Wref)
    assert err.max() <= TOL_MIXED, err.max()
    # labels identical outside the 0.5 +- 1e-3 band (and, for this closed mesh, everywhere)
    out = np.abs(Wref - 0.5) > 1e-3
    assert np.array_equal((W > 0.5)[out], (Wref > 0.5)[out])
    assert np.array_equal(W > 0.5, Wref > 0.5)


def test_exact_near_surface_and_float_io(cuda):
    rng = np.random.default_rng(11)
    V, F = synth.icosphere(3)
    V = synth.sh_deform(V, rng)
    F = synth.delete_random_faces(F, rng, 0.02)  # holes -> fractional W
    P, f = synth.sample_on_faces(V, F, rng, 3000)
    n = synth.face_normals(V, F[f])
    d = 10.0 ** rng.uniform(-7, -1, size=3000) * rng.choice([-1.0, 1.0], 3000)
    Q = P + n * d[:, None]
    Wref = O.winding_number(V, F, Q)
    Wm = G.winding_number(V, F, Q, precision="mixed")
    W64 = G.winding_number(V, F, Q, precision="fp64")
    assert np.abs(W64 - Wref).max() <= 1e-9
    assert np.abs(Wm - Wref).max() <= TOL_MIXED
    out = np.abs(Wref - 0.5) > 1e-3
    assert np.array_equal((Wm > 0.5)[out], (Wref > 0.5)[out])
    # float32 queries in, float32 out
    Qf = Q.astype(np.float32)
    Wf = G.winding_number(V, F, Qf, precision="mixed")
    assert Wf.dtype == np.float32
    Wref_f = O.winding_number(V, F, Qf.astype(np.float64))
    far = np.abs(d) > 1e-4
    assert np.abs(Wf[far] - Wref_f[far]).max() <= TOL_MIXED


def test_exact_edge_cases(cuda):
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    F = np.array([[0, 1, 3], [0, 2, 1], [0, 3, 2], [1, 2, 3]], np.int32)
    # empty query set
    assert G.winding_number(V, F, np.zeros((0, 3))).shape == (0,)
    # empty mesh -> W = 0
    W = G.winding_number(V, np.zeros((0, 3), np.int32), np.array([[0.1, 0.1, 0.1]]))
    assert np.all(W == 0)
    # queries on a vertex and on a face, against the oracle.  On a vertex
    # the incident triangles' terms are atan2(+-0, +0) = 0 in the reference's
    # formula (no zero guards, solid_angle.cpp:21-54) and here alike, so the
    # values agree to rounding.  On a face the triangle's determinant is
    # zero up to rounding and its term is +-pi by the sign of that rounding:
    # the reference's own value depends on its compiler's contraction of
    # multiply-adds, so only W modulo 1/2 is defined there.
    Q = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1], [0.25, 0.25, 0], [0.2, 0, 0.3],
                  [0.1, 0.1, 0.1], [0.5, 0.5, 0.5]])
    Wref = O.winding_number(V, F, Q)
    on_vertex, on_face = slice(0, 3), slice(3, 5)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-6)):  # mixed: far faces in FP32
        W = G.winding_number(V, F, Q, precision=prec)
        assert np.all(np.isfinite(W))
        assert np.abs(W[on_vertex] - Wref[on_vertex]).max() < tol
        d = (W[on_face] - Wref[on_face]) * 2.0
        assert np.abs(d - np.round(d)).max() < 2 * tol
        assert np.abs(W[5:] - Wref[5:]).max() < 1e-6
    # out-of-range index -> GWN_ERR_INVALID_ARGUMENT, loudly
    with pytest.raises(G.GwnError):
        G.winding_number(V, np.array([[0, 1, 7]], np.int32), Q)


def test_exact_2d_edges(cuda):
    # unit square polygon, counter-clockwise
    V = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    E = np.array([[0, 1], [1, 2], [2, 3], [3, 0]], np.int32)
    Q = np.array([[0.5, 0.5], [2.0, 0.5], [0.1, 0.9]])
    W = G.winding_number(V, E, Q, precision="fp64")
    Wref = O.winding_number(V, E, Q)
    assert np.abs(W - Wref).max() < 1e-12
    # signed_angle (signed_angle.cpp:14-45) over a star polygon with 400
    # edges, a self-overlapping loop and an open polyline, 4000 queries
    rng = np.random.default_rng(12)
    t = np.sort(rng.uniform(0, 2 * np.pi, 400))
    r = 1 + 0.4 * np.sin(7 * t) + 0.05 * rng.normal(size=400)
    star = np.stack([r * np.cos(t), r * np.sin(t)], 1)
    loop = 0.5 * np.stack([np.cos(2 * t[::4]), np.sin(2 * t[::4])], 1) + 0.2
    Vs = np.concatenate([star, loop])
    Es = np.concatenate([np.stack([np.arange(400), (np.arange(400) + 1) % 400], 1),
                         400 + np.stack([np.arange(99), np.arange(1, 100)], 1)]).astype(np.int32)
    Qs = rng.uniform(-1.6, 1.6, (4000, 2))
    Wref = O.winding_number(Vs, Es, Qs)
    W64 = G.winding_number(Vs, Es, Qs, precision="fp64")
    assert np.abs(W64 - Wref).max() < 1e-12
    Wm = G.winding_number(Vs, Es, Qs, precision="mixed")
    assert np.abs(Wm - Wref).max() < TOL_MIXED


def test_exact_device_tensors(cuda):
    torch = cuda
    V, F, Q = synth.exact_workload(seed=3, subdiv=3, nq=5000)
    Wref = O.winding_number(V, F, Q)
    dV = torch.from_numpy(V).cuda()
    dF = torch.from_numpy(F).cuda()
    dQ = torch.from_numpy(Q).cuda()
    W = G.winding_number(dV, dF, dQ, precision="mixed")
    assert W.is_cuda
    assert np.abs(W.cpu().numpy() - Wref).max() <= TOL_MIXED
    assert G.device_status() == 0
