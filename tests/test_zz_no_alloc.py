"""gwn_winding_number_noalloc: the exact winding number for callers that must
not allocate device memory during a call (hosts that own all device memory
through their own pool, latency-critical loops where cudaMalloc/cudaFree would
synchronize).  Its scratch is a static device array of fixed capacity inside
libgwn.  The test calls it twice in a row through the C ABI (different meshes,
so the shared scratch is reused with a different tile count) and compares
each result with gwn_winding_number's mixed path within the tests' metric
tolerance, plus the oracle.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import _native as N
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-4  # the metric bound the other exact-path tests use


def _noalloc(torch, V, F, Q):
    L = N.load()
    dV = torch.from_numpy(np.ascontiguousarray(V, np.float64)).cuda()
    dF = torch.from_numpy(np.ascontiguousarray(F, np.int32)).cuda()
    dQ = torch.from_numpy(np.ascontiguousarray(Q, np.float64)).cuda()
    dW = torch.full((Q.shape[0],), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    N.check(L.gwn_winding_number_noalloc(
        C.c_void_p(dV.data_ptr()), V.shape[0], C.c_void_p(dF.data_ptr()), F.shape[0],
        C.c_void_p(dQ.data_ptr()), Q.shape[0], C.c_void_p(dW.data_ptr()),
        C.c_void_p(st.data_ptr()), C.c_void_p(stream)))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    return dW.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(cuda):
    torch = cuda
    rng = np.random.default_rng(21)
    cases = []
    V1, F1, Q1 = synth.exact_workload(seed=4, subdiv=4, nq=30_000)   # 5120 triangles
    cases.append((V1, F1, Q1))
    V2, F2 = synth.icosphere(3)                                       # 1280 triangles, holes
    V2 = synth.sh_deform(V2, rng)
    F2 = synth.delete_random_faces(F2, rng, 0.05)
    P, f = synth.sample_on_faces(V2, F2, rng, 5000)
    n = synth.face_normals(V2, F2[f])
    d = 10.0 ** rng.uniform(-6, -1, 5000) * rng.choice([-1.0, 1.0], 5000)
    Q2 = np.concatenate([P + n * d[:, None], rng.uniform(-1.5, 1.5, (5000, 3))])
    cases.append((V2, F2, Q2))
    for V, F, Q in cases:  # two calls in a row on the shared static scratch
        W_na = _noalloc(torch, V, F, Q)
        W_ref = G.winding_number(V, F, Q, precision="mixed")
        assert np.all(np.isfinite(W_na))
        assert np.abs(W_na - W_ref).max() <= TOL
        W64 = O.winding_number(V, F, Q)
        assert np.abs(W_na - W64).max() <= TOL
        out = np.abs(W64 - 0.5) > 1e-3
        assert np.array_equal((W_na > 0.5)[out], (W64 > 0.5)[out])


def test_noalloc_rejects_more_than_the_static_capacity(cuda):
    torch = cuda
    L = N.load()
    # valid device buffers; the call must refuse on the size alone, before
    # launching anything
    V = torch.zeros((3, 3), dtype=torch.float64, device="cuda")
    F = torch.zeros((65537, 3), dtype=torch.int32, device="cuda")
    Q = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    W = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.gwn_winding_number_noalloc(V.data_ptr(), 3, F.data_ptr(), 65537, Q.data_ptr(), 1,
                                      W.data_ptr(), None, None)
    assert rc == 1  # GWN_ERR_INVALID_ARGUMENT
    assert b"65536" in L.gwn_last_error()


def _noalloc_raw(torch, V, F, Q, status):
    """One call with device buffers; `status` is a device int32 tensor or None."""
    L = N.load()
    dV = torch.from_numpy(np.ascontiguousarray(V, np.float64)).cuda()
    dF = torch.from_numpy(np.ascontiguousarray(F, np.int32)).cuda()
    dQ = torch.from_numpy(np.ascontiguousarray(Q, np.float64)).cuda()
    dW = torch.zeros((Q.shape[0],), dtype=torch.float64, device="cuda")
    N.check(L.gwn_winding_number_noalloc(
        C.c_void_p(dV.data_ptr()), V.shape[0], C.c_void_p(dF.data_ptr()), F.shape[0],
        C.c_void_p(dQ.data_ptr()), Q.shape[0], C.c_void_p(dW.data_ptr()),
        C.c_void_p(status.data_ptr()) if status is not None else None,
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return dW.cpu().numpy()


def test_noalloc_reports_device_failures_with_and_without_a_status_word(cuda):
    """A triangle index outside V is reported in the caller's status word, or,
    when the caller passes none, in the library's static word that
    gwn_device_status reads; so is a bulk-copy wait that runs out (made to run
    out on purpose through gwn_debug_fail_next_waits).  Afterwards the entry
    point still matches the allocating path."""
    torch = cuda
    L = N.load()
    G.device_status(clear=True)
    V, F, Q = synth.exact_workload(seed=8, subdiv=2, nq=1000)
    Fbad = F.copy()
    Fbad[7, 1] = V.shape[0] + 5  # built on the host: one index past the end of V
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    _noalloc_raw(torch, V, Fbad, Q, st)
    assert int(st.item()) & 2  # GWN_STATUS_BAD_INPUT
    assert G.device_status(clear=True) == 0  # nothing leaked into the sticky words
    _noalloc_raw(torch, V, Fbad, Q, None)
    assert G.device_status(clear=True) & 2
    try:
        L.gwn_debug_fail_next_waits(1)
        _noalloc_raw(torch, V, F, Q, None)
    finally:
        L.gwn_debug_fail_next_waits(0)
    assert G.device_status(clear=True) & 1  # GWN_STATUS_WAIT_TIMEOUT
    assert G.device_status(clear=True) == 0
    W = _noalloc_raw(torch, V, F, Q, None)
    assert G.device_status(clear=True) == 0
    assert np.abs(W - G.winding_number(V, F, Q, precision="mixed")).max() <= TOL
