"""CPU tests of the C-ABI boundary: libgwn.so builds for sm_103a, loads, and
exports exactly the functions include/gwn.h declares (no compute calls)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(inc, fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(gwn_\w+)\s*\(", src, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("gwn_winding_number", "gwn_soup_build", "gwn_soup_eval", "gwn_octree_build",
              "gwn_cloud_build", "gwn_cloud_eval", "gwn_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(gwn_lib):
    from libigl_gb300 import _native
    out = subprocess.run(["nm", "-D", "--defined-only", _native.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = declared_functions() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    # the Python binding knows every declared entry point
    assert declared_functions() <= set(_native.SIGNATURES)


def test_version_and_error_without_gpu(gwn_lib):
    from libigl_gb300 import _native
    assert gwn_lib.gwn_version() == 100
    # argument validation happens before any device work
    rc = gwn_lib.gwn_winding_number(None, 0, 4, None, 0, None, 0, 0, None, 0, 1, 0, None)
    assert rc == 1
    assert b"dim" in gwn_lib.gwn_last_error()


def test_mesh_arguments_refused_before_any_device_work(gwn_lib):
    """F rows that index an empty V, or a null V for vertices, are refused on
    the host (GWN_ERR_INVALID_ARGUMENT) before anything is launched, so this
    runs without a GPU."""
    import ctypes as C
    L = gwn_lib
    F = (C.c_int32 * 3)(0, 0, 0)
    O = (C.c_double * 3)(0.0, 0.0, 0.0)
    W = (C.c_double * 1)()
    Vbuf = (C.c_double * 3)(0.0, 0.0, 0.0)
    # triangles over an empty V
    for call in (
        lambda: L.gwn_winding_number(Vbuf, 0, 3, F, 1, O, 1, 1, W, 1, 1, 0, None),
        lambda: L.gwn_winding_number_noalloc(Vbuf, 0, F, 1, O, 1, W, None, None),
        lambda: L.gwn_soup_build(Vbuf, 0, F, 1, 2, 0, None, C.byref(C.c_void_p())),
    ):
        assert call() == 1
        assert b"no vertices" in L.gwn_last_error()
    # vertices behind a null pointer, with or without triangles
    for call in (
        lambda: L.gwn_winding_number(None, 3, 3, None, 0, O, 1, 1, W, 1, 1, 0, None),
        lambda: L.gwn_winding_number_noalloc(None, 3, None, 0, O, 1, W, None, None),
        lambda: L.gwn_winding_number_noalloc(None, 3, F, 1, O, 1, W, None, None),
    ):
        assert call() == 1
        assert b"V must be non-null" in L.gwn_last_error()
    # the wait-injection hook validates its argument without a device
    assert L.gwn_debug_fail_next_waits(-1) == 1
    assert L.gwn_debug_fail_next_waits(0) == 0


def test_octree_arrays_refused_before_any_device_work(gwn_lib):
    """The array forms of the cloud precompute and evaluation check the
    caller's octree (CSR point lists, CH) and its point arrays on the host,
    so a null or out-of-range argument is an error before any launch."""
    import ctypes as C
    import numpy as np
    L = gwn_lib
    P = np.zeros((2, 3))
    N = np.zeros((2, 3))
    A = np.ones(2)
    off = np.array([0, 2], dtype=np.int64)      # one cell holding both points
    idx = np.array([0, 1], dtype=np.int32)
    CH = np.full(8, -1, dtype=np.int32)
    CM, R, EC = np.zeros(3), np.zeros(1), np.zeros(39)
    Q, W = np.zeros(3), np.zeros(1)

    def ptr(a):
        return None if a is None else a.ctypes.data_as(C.c_void_p)

    def pre(P_, N_, A_, off_, idx_, CH_):
        return L.gwn_cloud_precompute_arrays(ptr(P_), ptr(N_), ptr(A_), 2, ptr(off_), ptr(idx_),
                                             ptr(CH_), 1, 2, ptr(CM), ptr(R), ptr(EC))

    def ev(P_, N_, A_, off_, idx_, CH_):
        return L.gwn_cloud_eval_arrays(ptr(P_), ptr(N_), ptr(A_), 2, ptr(off_), ptr(idx_),
                                       ptr(CH_), 1, ptr(CM), ptr(R), ptr(EC), 2, ptr(Q), 1, 2.0,
                                       ptr(W), 0)

    for call in (pre, ev):
        assert call(P, N, A, off, None, CH) == 1
        assert b"pi_indices must be non-null" in L.gwn_last_error()
        assert call(None, N, A, off, idx, CH) == 1
        assert b"P, N and A must be non-null" in L.gwn_last_error()
        assert call(P, N, A, off, np.array([0, 2], dtype=np.int32), CH) == 1
        assert b"point index out of range" in L.gwn_last_error()
        CH_bad = np.array([5, 1, 1, 1, 1, 1, 1, 1], dtype=np.int32)
        assert call(P, N, A, off, idx, CH_bad) == 1
        assert b"CH child id out of range" in L.gwn_last_error()


def test_soup_walk_stats_refuses_null_queries(gwn_lib):
    """A non-null handle is not dereferenced before the argument checks."""
    import ctypes as C
    L = gwn_lib
    counters = (C.c_ulonglong * 7)()
    fake = C.c_void_p(1)
    assert L.gwn_soup_walk_stats(fake, 2.0, None, 4, 0, counters) == 1
    assert b"Q must be non-null" in L.gwn_last_error()
    q = (C.c_double * 3)()
    assert L.gwn_soup_walk_stats(fake, float("inf"), q, 1, 0, counters) == 1
    assert b"accuracy_scale must be finite" in L.gwn_last_error()


def test_size_limits_refused_before_any_device_work(gwn_lib):
    """Every entry point's largest accepted size is checked on the host:
    one past it is GWN_ERR_INVALID_ARGUMENT before anything is read from the
    arrays or launched (the small buffers below are never read)."""
    import ctypes as C
    L = gwn_lib
    big31, big30 = 2 ** 31, 2 ** 30
    buf = (C.c_double * 64)()
    ibuf = (C.c_int32 * 64)()
    fake = C.c_void_p(1)          # a handle that is refused before it is read
    res = (C.c_int32 * 3)(2 ** 14, 2 ** 14, 2 ** 14)
    cases = [
        ("queries", lambda: L.gwn_winding_number(buf, 3, 3, ibuf, 1, buf, 1, big31, buf, 1, 1,
                                                 0, None)),
        ("queries", lambda: L.gwn_soup_eval(fake, 2.0, buf, 1, big31, buf, 1, 1, 0, None)),
        ("nQ < 2^31", lambda: L.gwn_cloud_eval(fake, 2.0, buf, 1, big31, buf, 1, 1, 0, None)),
        ("queries", lambda: L.gwn_wn_aabb_eval_precision(fake, buf, big31, buf, 1, 0, None)),
        ("queries", lambda: L.gwn_knn(buf, big31, buf, 1, 1, ibuf, 0, None)),
        ("queries", lambda: L.gwn_signed_distance(buf, big31, buf, 3, ibuf, 1, 2, 0.0, 1.0, buf,
                                                  ibuf, buf, None, 0, 0, None)),
        ("primitives", lambda: L.gwn_eytzinger_aabb(buf, buf, big30, 2, buf, buf, ibuf, 0, None)),
        ("segments", lambda: L.gwn_eytzinger_winding_number_tree(ibuf, big30, ibuf, 2, ibuf,
                                                                  None, 0, None)),
        ("queries", lambda: L.gwn_eytzinger_winding_number(buf, big31, buf, 2, ibuf, 1, buf, buf,
                                                           ibuf, 2, ibuf, 0, ibuf, buf, 0, 0,
                                                           None)),
        ("grid points", lambda: L.gwn_swept_volume_signed_distance(
            buf, 3, ibuf, 1, buf, 1, 1, buf, big31, ibuf, 1.0, float("nan"), None, buf, 0, 0,
            None)),
        ("grid too large", lambda: L.gwn_flood_fill(res, buf, 0, None)),
        ("no-allocation limit", lambda: L.gwn_winding_number_noalloc(buf, 3, ibuf, 65537, buf, 1,
                                                                     buf, None, None)),
    ]
    for what, call in cases:
        assert call() == 1, what
        assert what.encode() in L.gwn_last_error(), (what, L.gwn_last_error())


def test_server_wait_refuses_nan_timeout(gwn_lib):
    """A NaN timeout is refused before the server is touched (a fake handle
    is never read)."""
    import ctypes as C
    L = gwn_lib
    assert L.gwn_server_wait(C.c_void_p(1), 1, float("nan"), None) == 1
    assert b"NaN" in L.gwn_last_error()
    assert L.gwn_server_wait(None, 1, 1.0, None) == 1
    assert b"server is null" in L.gwn_last_error()


def test_server_submit_refuses_non_finite_accuracy(gwn_lib):
    """As gwn_soup_eval: a non-finite accuracy_scale is refused, before the
    server is touched (a fake handle is never read)."""
    import ctypes as C
    L = gwn_lib
    rid = C.c_int64(0)
    rc = L.gwn_server_submit(C.c_void_p(1), 1, None, 1, 0, None, 1, float("inf"), 1,
                             C.byref(rid))
    assert rc == 1
    assert b"accuracy_scale must be finite" in L.gwn_last_error()
