"""ctypes binding of libgwn.so (include/gwn.h).

The library is built in-tree by ``libigl_gb300.build`` and loaded from
``libigl_gb300/_lib/libgwn.so``.  There is no fallback: if the library is
missing or no CUDA device is present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgwn.so")

GWN_OK = 0
GWN_F32, GWN_F64 = 0, 1
GWN_PLAIN_FP64, GWN_MIXED = 0, 1
GWN_HOST, GWN_DEVICE = 0, 1
GWN_TREE_REFERENCE, GWN_TREE_BINNED = 0, 1

STATUS_NAMES = {
    1: "GWN_ERR_INVALID_ARGUMENT",
    2: "GWN_ERR_CUDA",
    3: "GWN_ERR_OUT_OF_MEMORY",
    4: "GWN_ERR_NO_DEVICE",
    5: "GWN_ERR_TIMEOUT",
    6: "GWN_ERR_BUSY",
    7: "GWN_ERR_INTERNAL",
}

# Every exported entry point with its ctypes signature; tests check that the
# library exports exactly these names (the declarations of include/gwn.h).
_p, _i, _i64, _f, _d = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_double
SIGNATURES = {
    "gwn_last_error": ([], C.c_char_p),
    "gwn_version": ([], _i),
    "gwn_device_status": ([_p, _i], _i),
    "gwn_debug_fail_next_waits": ([_i], _i),
    "gwn_winding_number": ([_p, _i64, _i, _p, _i64, _p, _i, _i64, _p, _i, _i, _i, _p], _i),
    "gwn_winding_number_noalloc": ([_p, _i64, _p, _i64, _p, _i64, _p, _p, _p], _i),
    "gwn_soup_build": ([_p, _i64, _p, _i64, _i, _i, _p, _p], _i),
    "gwn_soup_build_tree": ([_p, _i64, _p, _i64, _i, _i, _i, _p, _p], _i),
    "gwn_soup_tree_nodes": ([_p, _p, _p], _i),
    "gwn_soup_eval": ([_p, _f, _p, _i, _i64, _p, _i, _i, _i, _p], _i),
    "gwn_soup_stats_get": ([_p, _p], _i),
    "gwn_soup_free": ([_p], None),
    "gwn_soup_export": ([_p, _p, _p], _i),
    "gwn_soup_walk_stats": ([_p, _f, _p, _i64, _i, _p], _i),
    "gwn_octree_build": ([_p, _i64, _i, _p, _p], _i),
    "gwn_octree_sizes": ([_p, _p, _p, _p], _i),
    "gwn_octree_export": ([_p, _p, _p, _p, _p, _p, _i, _p], _i),
    "gwn_octree_free": ([_p], None),
    "gwn_cloud_build": ([_p, _p, _p, _p, _i, _i, _p, _p], _i),
    "gwn_cloud_export": ([_p, _p, _p, _p, _i, _p], _i),
    "gwn_cloud_eval": ([_p, _d, _p, _i, _i64, _p, _i, _i, _i, _p], _i),
    "gwn_cloud_free": ([_p], None),
    "gwn_cloud_precompute_arrays": ([_p, _p, _p, _i64, _p, _p, _p, _i64, _i, _p, _p, _p], _i),
    "gwn_profile_enable": ([_i], _i),
    "gwn_launch_count": ([], C.c_ulonglong),
    "gwn_soup_squared_distance": ([_p, _p, _i, _i64, _d, _p, _p, _p, _i, _p], _i),
    "gwn_octree_knn": ([_p, _p, _i, _i64, _i64, _p, _i, _p], _i),
    "gwn_knn": ([_p, _i64, _p, _i64, _i64, _p, _i, _p], _i),
    "gwn_point_areas": ([_p, _i64, _p, _i64, _p, _p, _p, _i, _p], _i),
    "gwn_cloud_winding_number_points": ([_p, _p, _i64, _p, _i, _i64, _i, _d, _p, _i, _i, _i,
                                         _p], _i),
    "gwn_eytzinger_slots": ([_i64], _i64),
    "gwn_wn_aabb_build": ([_p, _i64, _p, _i64, _i, _p, _p], _i),
    "gwn_wn_aabb_eval": ([_p, _p, _i64, _p, _i, _p], _i),
    "gwn_wn_aabb_eval_precision": ([_p, _p, _i64, _p, _i, _i, _p], _i),
    "gwn_wn_aabb_free": ([_p], None),
    "gwn_swept_volume_signed_distance": ([_p, _i64, _p, _i64, _p, _i64, _i, _p, _i64, _p, _d,
                                          _d, _p, _p, _i, _i, _p], _i),
    "gwn_flood_fill": ([_p, _p, _i, _p], _i),
    "gwn_eytzinger_aabb": ([_p, _p, _i64, _i, _p, _p, _p, _i, _p], _i),
    "gwn_eytzinger_winding_number_tree": ([_p, _i64, _p, _i64, _p, _p, _i, _p], _i),
    "gwn_eytzinger_winding_number": ([_p, _i64, _p, _i64, _p, _i64, _p, _p, _p, _i64, _p, _i64,
                                      _p, _p, _i, _i, _p], _i),
    "gwn_signed_distance": ([_p, _i64, _p, _i64, _p, _i64, _i, _d, _d, _p, _p, _p, _p, _i, _i,
                             _p], _i),
    "gwn_server_create": ([_i64, _i64, C.c_int32, _p], _i),
    "gwn_server_add_mesh": ([_p, _p, _i64, _p, _i64, _i, _p], _i),
    "gwn_server_remove_mesh": ([_p, _i64], _i),
    "gwn_server_submit": ([_p, _i64, _p, _i, _i64, _p, _i, _f, _i, _p], _i),
    "gwn_server_wait": ([_p, _i64, _d, _p], _i),
    "gwn_server_stats_get": ([_p, _p], _i),
    "gwn_server_destroy": ([_p], _i),
    "gwn_profile_read": ([_p, _i, _p, _i, _p], _i),
    "gwn_cloud_eval_arrays": ([_p, _p, _p, _i64, _p, _p, _p, _i64, _p, _p, _p, _i, _p, _i64, _d,
                               _p, _i], _i),
}


class GwnError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load libgwn.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m libigl_gb300.build` "
            "(nvcc, sm_103a); there is no CPU fallback")
    L = C.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def exported_symbols(path: str = LIB_PATH):
    L = C.CDLL(path)
    return {n for n in SIGNATURES if hasattr(L, n)}


def check(rc: int):
    if rc != GWN_OK:
        msg = load().gwn_last_error()
        raise GwnError(rc, msg.decode() if msg else "")
