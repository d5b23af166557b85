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
