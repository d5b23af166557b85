"""Device-side failure reporting, exercised without faulting the GPU.

The reference reports nothing (asserts only: winding_number.cpp:56,
fast_winding_number.cpp:37).  Here a bounded mbarrier wait that runs out sets
GWN_STATUS_WAIT_TIMEOUT and the kernel returns after draining its copies, and
an out-of-range index sets GWN_STATUS_BAD_INPUT.  gwn_debug_fail_next_waits
makes the next ring kernel withhold one mbarrier arrival (a flag that nothing
sets), so its first wait runs out of its budget; the tests check the status
the host sees and that the device keeps working afterwards."""
import ctypes as C

import numpy as np
import pytest

import libigl_gb300 as G
from libigl_gb300 import _native as N
from libigl_gb300 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # GWN_ERR_TIMEOUT


@pytest.fixture
def lib(cuda):
    L = N.load()
    L.gwn_debug_fail_next_waits(0)
    yield L
    L.gwn_debug_fail_next_waits(0)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_injected_wait_timeout_is_reported_and_device_recovers(lib, precision):
    # 320 triangles: below the hierarchy's threshold, so the all-pairs ring
    # kernels run
    V, F, Q = synth.exact_workload(seed=3, subdiv=2, nq=3000)
    Wref = O.winding_number(V, F, Q)
    assert lib.gwn_debug_fail_next_waits(1) == 0
    with pytest.raises(N.GwnError) as e:
        G.winding_number(V, F, Q, precision=precision)
    assert e.value.code == TIMEOUT
    assert b"bounded device wait" in lib.gwn_last_error()
    # the injection is spent and the context is usable: the next call is exact
    W = G.winding_number(V, F, Q, precision=precision)
    assert np.abs(W - Wref).max() <= (1e-11 if precision == "fp64" else 1e-4)


def test_injected_timeout_on_device_memory_goes_to_the_sticky_word(lib, cuda):
    torch = cuda
    V, F, Q = synth.exact_workload(seed=5, subdiv=2, nq=2000)
    dV = torch.from_numpy(V).cuda()
    dF = torch.from_numpy(F.astype(np.int32)).cuda()
    dQ = torch.from_numpy(Q).cuda()
    dW = torch.zeros(Q.shape[0], dtype=torch.float64, device="cuda")
    assert G.device_status(clear=True) == 0
    lib.gwn_debug_fail_next_waits(1)
    N.check(lib.gwn_winding_number(dV.data_ptr(), V.shape[0], 3, dF.data_ptr(), F.shape[0],
                                   dQ.data_ptr(), N.GWN_F64, Q.shape[0], dW.data_ptr(),
                                   N.GWN_F64, N.GWN_MIXED, N.GWN_DEVICE, None))
    assert G.device_status(clear=True) & 1  # GWN_STATUS_WAIT_TIMEOUT
    assert G.device_status(clear=True) == 0  # cleared
