"""Served winding-number queries over the gwn_server C ABI (include/gwn.h).

A ``Server`` keeps triangle meshes resident on the GPU (built soup trees,
bounded by an HBM budget with least-recently-used eviction) and evaluates
requests against them with continuous batching: a native worker thread
groups the requests pending whenever a batch slot frees up, and runs each
batch, whatever mix of meshes it holds, as one captured CUDA graph.

Each request computes ``igl::fast_winding_number(bvh, accuracy_scale, Q, W)``
for its mesh (libigl's fast_winding_number.h:189-194); the results equal
``FastWindingNumberBVH(V, F).eval(Q, accuracy_scale, precision)``.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _native as N

_PREC = {"fp64": N.GWN_PLAIN_FP64, "plain": N.GWN_PLAIN_FP64, "mixed": N.GWN_MIXED}


class ServerStats(C.Structure):
    _fields_ = [(name, C.c_int64) for name in (
        "requests_done", "queries_done", "batches", "builds", "evictions", "resident_meshes",
        "resident_bytes", "peak_resident_bytes", "budget_bytes", "refined", "pending",
        "kernels_per_batch")] + [("batch_gpu_ms", C.c_double), ("walk_gpu_ms", C.c_double)]


class Request:
    """A submitted request: ``wait()`` returns (W, latency seconds)."""

    __slots__ = ("server", "id", "Q", "W")

    def __init__(self, server, rid, Q, W):
        self.server, self.id, self.Q, self.W = server, rid, Q, W

    def wait(self, timeout: float | None = None):
        return self.server.wait(self, timeout)


class Server:
    def __init__(self, hbm_budget_bytes: int = 120 << 30, max_batch_queries: int = 1 << 22,
                 slots: int = 3):
        self._L = N.load()
        h = C.c_void_p()
        N.check(self._L.gwn_server_create(int(hbm_budget_bytes), int(max_batch_queries),
                                          int(slots), C.byref(h)))
        self._h = h
        self._lock = threading.Lock()
        self._live = {}

    def add_mesh(self, V, F, order: int = 2) -> int:
        V = np.ascontiguousarray(V, np.float64)
        F = np.ascontiguousarray(F, np.int32)
        if V.ndim != 2 or V.shape[1] != 3 or F.ndim != 2 or F.shape[1] != 3:
            raise ValueError("V must be #V x 3 and F #F x 3")
        mid = C.c_int64()
        N.check(self._L.gwn_server_add_mesh(self._h, V.ctypes.data, V.shape[0], F.ctypes.data,
                                            F.shape[0], int(order), C.byref(mid)))
        return mid.value

    def remove_mesh(self, mesh_id: int) -> None:
        N.check(self._L.gwn_server_remove_mesh(self._h, int(mesh_id)))

    def submit(self, mesh_id: int, Q, accuracy_scale: float = 2.0, precision="mixed",
               out_dtype=None) -> Request:
        Q = np.asarray(Q)
        if Q.dtype not in (np.float32, np.float64):
            Q = Q.astype(np.float64)
        Q = np.ascontiguousarray(Q)
        if Q.ndim != 2 or Q.shape[1] != 3:
            raise ValueError("Q must be #Q x 3")
        wdt = np.dtype(out_dtype) if out_dtype is not None else Q.dtype
        W = np.empty(Q.shape[0], wdt)
        rid = C.c_int64()
        N.check(self._L.gwn_server_submit(
            self._h, int(mesh_id), Q.ctypes.data,
            N.GWN_F64 if Q.dtype == np.float64 else N.GWN_F32, Q.shape[0], W.ctypes.data,
            N.GWN_F64 if wdt == np.float64 else N.GWN_F32, C.c_float(accuracy_scale),
            _PREC[precision] if isinstance(precision, str) else int(precision), C.byref(rid)))
        req = Request(self, rid.value, Q, W)
        with self._lock:
            self._live[rid.value] = req  # keeps Q and W alive until waited for
        return req

    def wait(self, req: Request, timeout: float | None = None):
        lat = C.c_double()
        rc = self._L.gwn_server_wait(self._h, req.id, -1.0 if timeout is None else float(timeout),
                                     C.byref(lat))
        if rc == 5:  # GWN_ERR_TIMEOUT: still queued
            raise TimeoutError(N.load().gwn_last_error().decode())
        with self._lock:
            self._live.pop(req.id, None)
        N.check(rc)
        return req.W, lat.value

    def stats(self) -> dict:
        st = ServerStats()
        N.check(self._L.gwn_server_stats_get(self._h, C.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.check(self._L.gwn_server_destroy(self._h))
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
