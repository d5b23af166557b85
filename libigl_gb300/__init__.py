"""libigl_gb300: GB300-native generalized winding numbers.

Python host mirror of libigl's winding-number interface over the C ABI of
``libgwn.so`` (include/gwn.h).  Functions keep libigl's names and argument
meaning:

* ``winding_number(V, F, O)``            -- igl::winding_number(V,F,O,W)
* ``fast_winding_number_soup_precompute`` / ``FastWindingNumberBVH`` /
  ``fast_winding_number_soup``           -- igl::fast_winding_number soup overloads
* ``octree(P)``                          -- igl::octree
* ``fast_winding_number_cloud_precompute`` / ``fast_winding_number_cloud`` /
  ``fast_winding_number_cloud_oneshot``  -- point-cloud overloads
* ``Server``                             -- resident meshes, continuously batched
  soup requests (no libigl counterpart)

Arrays may be NumPy arrays (host memory: the call copies in, computes on the
GPU, copies out) or CUDA torch tensors (device memory: the work is enqueued on
torch's current stream and the result stays on the device).  Every call runs
on the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import _native as NV  # for functions whose arguments are named N
from ._native import GwnError
from .serve import Server

__all__ = [
    "GwnError", "winding_number", "FastWindingNumberBVH",
    "fast_winding_number_soup_precompute", "fast_winding_number_soup",
    "Octree", "octree", "CloudExpansion", "fast_winding_number_cloud_precompute",
    "fast_winding_number_cloud", "fast_winding_number_cloud_oneshot", "device_status",
    "Server", "signed_distance", "knn", "eytzinger_aabb", "eytzinger_aabb_winding_number_tree",
    "eytzinger_aabb_winding_number", "swept_volume_signed_distance", "flood_fill",
    "WindingNumberAABB", "point_areas", "fast_winding_number_cloud_points",
]

_PREC = {"fp64": N.GWN_PLAIN_FP64, "plain": N.GWN_PLAIN_FP64, "mixed": N.GWN_MIXED}


def _prec(p) -> int:
    if isinstance(p, int):
        return p
    return _PREC[p]


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def _torch():
    import torch
    return torch


def _stream_ptr():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Arg:
    """A contiguous argument array with its pointer, memory kind and dtype code."""

    def __init__(self, x, dtype=None, allowed=(np.float32, np.float64)):
        if _is_torch_cuda(x):
            torch = _torch()
            if dtype is not None:
                x = x.to(dtype=getattr(torch, np.dtype(dtype).name))
            elif x.dtype not in (torch.float32, torch.float64):
                x = x.to(torch.float64)
            self.obj = x.contiguous()
            self.ptr = C.c_void_p(self.obj.data_ptr())
            self.mem = N.GWN_DEVICE
            self.np_dtype = np.dtype(str(self.obj.dtype).replace("torch.", ""))
        else:
            a = np.asarray(x)
            if dtype is not None:
                a = np.ascontiguousarray(a, dtype=dtype)
            elif a.dtype.type not in allowed:
                a = np.ascontiguousarray(a, dtype=np.float64)
            else:
                a = np.ascontiguousarray(a)
            self.obj = a
            self.ptr = a.ctypes.data_as(C.c_void_p)
            self.mem = N.GWN_HOST
            self.np_dtype = a.dtype
        self.code = N.GWN_F64 if self.np_dtype == np.float64 else N.GWN_F32

    @property
    def shape(self):
        return tuple(self.obj.shape)


def _need_rows(a, cols: int, name: str, rows: int | None = None):
    """Raise ValueError unless ``a`` (an _Arg) is a rows x cols matrix (any
    number of rows when ``rows`` is None): the C ABI reads rows * cols
    elements from the pointer it is given."""
    shape = a.shape
    if len(shape) != 2 or shape[1] != cols or (rows is not None and shape[0] != rows):
        want = f"{rows if rows is not None else '#'} x {cols}"
        raise ValueError(f"{name} must be {want}, got shape {shape}")


def _need_len(a, n: int, name: str):
    """Raise ValueError unless ``a`` holds exactly n elements."""
    size = int(np.prod(a.shape)) if len(a.shape) else 1
    if size != n:
        raise ValueError(f"{name} must hold {n} elements, got shape {tuple(a.shape)}")


def _same_mem(*args):
    mems = {a.mem for a in args}
    if len(mems) != 1:
        raise ValueError("mix of host (NumPy) and device (torch CUDA) arrays in one call")
    return mems.pop()


def _empty_like_mem(mem, shape, np_dtype, like=None):
    if mem == N.GWN_DEVICE:
        torch = _torch()
        return torch.empty(shape, dtype=getattr(torch, np.dtype(np_dtype).name),
                           device=like.obj.device)
    return np.empty(shape, dtype=np_dtype)


def _ptr_of(x):
    if _is_torch_cuda(x):
        return C.c_void_p(x.data_ptr())
    return x.ctypes.data_as(C.c_void_p)


def device_status(clear: bool = True) -> int:
    """Status bits recorded by device-memory calls (see gwn_device_status)."""
    flags = C.c_uint(0)
    N.check(N.load().gwn_device_status(C.byref(flags), int(clear)))
    return flags.value


# --------------------------------------------------------------- exact GWN --
def winding_number(V, F, O, precision="mixed", out_dtype=None):
    """igl::winding_number(V,F,O,W) (include/igl/winding_number.h:35-44).

    V: #V x dim vertex positions, F: #F x dim simplices (dim 3 triangles,
    dim 2 edges), O: #O x dim queries.  Returns W (#O,) in O's dtype unless
    ``out_dtype`` is given.  ``precision`` is "mixed" (FP32 bulk + FP64
    near-field / threshold re-evaluation) or "fp64" (plain FP64).
    """
    L = N.load()
    Va = _Arg(V, np.float64)
    Fa = _Arg(F, np.int32, allowed=(np.int32,))
    Oa = _Arg(O)
    mem = _same_mem(Va, Fa, Oa)
    dim = Fa.shape[1] if len(Fa.shape) == 2 else 3
    if len(Va.shape) != 2 or Va.shape[1] != dim:
        raise ValueError(f"V must be #V x {dim}")
    if len(Oa.shape) != 2 or Oa.shape[1] != dim:
        raise ValueError(f"O must be #O x {dim}")
    wdt = np.dtype(out_dtype) if out_dtype is not None else Oa.np_dtype
    W = _empty_like_mem(mem, (Oa.shape[0],), wdt, like=Oa)
    stream = _stream_ptr() if mem == N.GWN_DEVICE else None
    N.check(L.gwn_winding_number(Va.ptr, Va.shape[0], dim, Fa.ptr, Fa.shape[0], Oa.ptr, Oa.code,
                                 Oa.shape[0], _ptr_of(W),
                                 N.GWN_F64 if wdt == np.float64 else N.GWN_F32,
                                 _prec(precision), mem, stream))
    return W


# ---------------------------------------------------------- triangle soup --
class _SoupStats(C.Structure):
    _fields_ = [("num_triangles", C.c_int64), ("num_nodes", C.c_int64),
                ("device_bytes", C.c_int64), ("order", C.c_int32), ("max_depth", C.c_int32),
                ("tree", C.c_int32), ("reserved", C.c_int32), ("tree_nodes", C.c_int64)]


TREE_REFERENCE, TREE_BINNED = N.GWN_TREE_REFERENCE, N.GWN_TREE_BINNED


class FastWindingNumberBVH:
    """Device-resident soup tree + moments (igl::FastWindingNumberBVH,
    include/igl/fast_winding_number.h:140-147).  Built by
    ``fast_winding_number_soup_precompute``; owns device copies of V and F."""

    def __init__(self, V, F, order: int = 2, tree: str = "reference"):
        """``tree``: "reference" -- libigl's own 4-wide SAH tree, built on the
        GPU node for node (results equal the reference's up to its FP32
        rounding); "binned" -- a binary tree of binned splits (a different
        tree cut)."""
        L = N.load()
        Va = _Arg(V, np.float64)
        Fa = _Arg(F, np.int32, allowed=(np.int32,))
        mem = _same_mem(Va, Fa)
        if len(Va.shape) != 2 or Va.shape[1] != 3 or len(Fa.shape) != 2 or Fa.shape[1] != 3:
            raise ValueError("V must be #V x 3 and F #F x 3")
        kinds = {"reference": N.GWN_TREE_REFERENCE, "binned": N.GWN_TREE_BINNED}
        if tree not in kinds:
            raise ValueError(f"tree must be one of {sorted(kinds)}")
        h = C.c_void_p()
        stream = _stream_ptr() if mem == N.GWN_DEVICE else None
        N.check(L.gwn_soup_build_tree(Va.ptr, Va.shape[0], Fa.ptr, Fa.shape[0], int(order),
                                      kinds[tree], mem, stream, C.byref(h)))
        self._h = h
        self.order = order
        self.tree = tree

    def tree_nodes(self) -> np.ndarray:
        """The 4-wide tree as the reference stores it (tree="reference"):
        #nodes x 4 uint32, a triangle index, node | 2^31, or 2^32-1 (empty)."""
        n = C.c_int64(0)
        N.check(N.load().gwn_soup_tree_nodes(self._h, C.byref(n), None))
        out = np.empty((n.value, 4), np.uint32)
        N.check(N.load().gwn_soup_tree_nodes(self._h, C.byref(n), out.ctypes.data_as(C.c_void_p)))
        return out

    def eval(self, Q, accuracy_scale: float = 2.0, precision="mixed", out_dtype=None):
        """W(p) = computeSolidAngle(p, accuracy_scale) / 4pi for every row of Q."""
        L = N.load()
        Qa = _Arg(Q)
        if len(Qa.shape) != 2 or Qa.shape[1] != 3:
            raise ValueError("Q must be #Q x 3")
        wdt = np.dtype(out_dtype) if out_dtype is not None else Qa.np_dtype
        W = _empty_like_mem(Qa.mem, (Qa.shape[0],), wdt, like=Qa)
        stream = _stream_ptr() if Qa.mem == N.GWN_DEVICE else None
        N.check(L.gwn_soup_eval(self._h, C.c_float(accuracy_scale), Qa.ptr, Qa.code, Qa.shape[0],
                                _ptr_of(W), N.GWN_F64 if wdt == np.float64 else N.GWN_F32,
                                _prec(precision), Qa.mem, stream))
        return W

    def eval_ptr(self, q_ptr, q_dtype: int, nq: int, w_ptr, w_dtype: int, accuracy_scale=2.0,
                 precision="mixed", stream=None):
        """Raw device-pointer evaluation (no allocation on the Python side)."""
        N.check(N.load().gwn_soup_eval(self._h, C.c_float(accuracy_scale), C.c_void_p(q_ptr),
                                       q_dtype, nq, C.c_void_p(w_ptr), w_dtype, _prec(precision),
                                       N.GWN_DEVICE, C.c_void_p(stream)))

    def export(self):
        """(nodes (num_nodes x 24 float64, pre-order), links (int64), tri_index (int32))."""
        st = self.stats
        nodes = np.empty((st["num_nodes"], 24), np.float64)
        tri = np.empty(st["num_triangles"], np.int32)
        N.check(N.load().gwn_soup_export(self._h, nodes.ctypes.data_as(C.c_void_p),
                                         tri.ctypes.data_as(C.c_void_p)))
        links = nodes[:, 23].copy().view(np.int64)
        return nodes, links, tri

    def squared_distance(self, Q, up_sqr_d: float = float("inf")):
        """igl::AABB::squared_distance(V,F,Q,sqrD,I,C) over this mesh's
        triangles: (sqrD, I, C) -- smallest squared distance (below
        up_sqr_d), input triangle index (-1 if none) and closest point."""
        L = N.load()
        Qa = _Arg(Q)
        if len(Qa.shape) != 2 or Qa.shape[1] != 3:
            raise ValueError("Q must be #Q x 3")
        n = Qa.shape[0]
        D = _empty_like_mem(Qa.mem, (n,), np.float64, like=Qa)
        I = _empty_like_mem(Qa.mem, (n,), np.int32, like=Qa)
        Cp = _empty_like_mem(Qa.mem, (n, 3), np.float64, like=Qa)
        stream = _stream_ptr() if Qa.mem == N.GWN_DEVICE else None
        N.check(L.gwn_soup_squared_distance(self._h, Qa.ptr, Qa.code, n, C.c_double(up_sqr_d),
                                            _ptr_of(D), _ptr_of(I), _ptr_of(Cp), Qa.mem,
                                            stream))
        return D, I, Cp

    def walk_stats(self, Q, accuracy_scale: float = 2.0) -> dict:
        """Work counters of one instrumented mixed evaluation of Q (float64)."""
        Qa = _Arg(Q, np.float64)
        out = (C.c_ulonglong * 7)()
        N.check(N.load().gwn_soup_walk_stats(self._h, C.c_float(accuracy_scale), Qa.ptr,
                                             Qa.shape[0], Qa.mem, out))
        keys = ["warp_steps", "node_visits", "far_field", "exact_fp32", "exact_fp64_near",
                "fp64_rechecks", "threshold_refines"]
        return dict(zip(keys, [int(x) for x in out]))

    @property
    def stats(self) -> dict:
        st = _SoupStats()
        N.check(N.load().gwn_soup_stats_get(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _SoupStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            N.load().gwn_soup_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fast_winding_number_soup_precompute(V, F, order: int = 2) -> FastWindingNumberBVH:
    """igl::fast_winding_number(V,F,order,fwn_bvh) (fast_winding_number.h:176-181)."""
    return FastWindingNumberBVH(V, F, order)


def fast_winding_number_soup(V, F, Q, order: int = 2, accuracy_scale: float = 2.0,
                             precision="mixed"):
    """One-shot soup FWN, igl::fast_winding_number(V,F,Q,W) (fast_winding_number.h:157-163):
    order 2, accuracy_scale 2."""
    bvh = FastWindingNumberBVH(V, F, order)
    try:
        return bvh.eval(Q, accuracy_scale, precision)
    finally:
        bvh.close()


# ---------------------------------------------------------------- octree --
class Octree:
    """igl::octree output (include/igl/octree.h:44-50), device-resident.

    ``export()`` returns (pi_offsets, pi_indices, CH, CN, W): point_indices in
    CSR form plus the child table, centres and widths, bit-exact with the
    reference."""

    def __init__(self, P):
        L = N.load()
        Pa = _Arg(P, np.float64)
        if len(Pa.shape) != 2 or Pa.shape[1] != 3:
            raise ValueError("P must be #P x 3")
        h = C.c_void_p()
        stream = _stream_ptr() if Pa.mem == N.GWN_DEVICE else None
        N.check(L.gwn_octree_build(Pa.ptr, Pa.shape[0], Pa.mem, stream, C.byref(h)))
        self._h = h
        self.num_points = Pa.shape[0]

    def sizes(self):
        nc, ni, md = C.c_int64(), C.c_int64(), C.c_int32()
        N.check(N.load().gwn_octree_sizes(self._h, C.byref(nc), C.byref(ni), C.byref(md)))
        return nc.value, ni.value, md.value

    def export(self):
        nc, ni, _ = self.sizes()
        off = np.empty(nc + 1, np.int64)
        idx = np.empty(max(ni, 1), np.int32)
        CH = np.empty((nc, 8), np.int32)
        CN = np.empty((nc, 3), np.float64)
        W = np.empty(nc, np.float64)
        P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        N.check(N.load().gwn_octree_export(self._h, P(off), P(idx), P(CH), P(CN), P(W),
                                           N.GWN_HOST, None))
        return off, idx[:ni], CH, CN, W

    def point_indices(self):
        off, idx, *_ = self.export()
        return [idx[off[c]:off[c + 1]].tolist() for c in range(off.shape[0] - 1)]

    def knn(self, Q, k: int):
        """igl::knn over this octree's points: I (#Q x min(k, #points)),
        nearest first, equal distances by index."""
        Qa = _Arg(Q)
        if len(Qa.shape) != 2 or Qa.shape[1] != 3:
            raise ValueError("Q must be #Q x 3")
        cols = min(int(k), self.num_points)
        I = _empty_like_mem(Qa.mem, (Qa.shape[0], cols), np.int32, like=Qa)
        stream = _stream_ptr() if Qa.mem == N.GWN_DEVICE else None
        N.check(N.load().gwn_octree_knn(self._h, Qa.ptr, Qa.code, Qa.shape[0], int(k), _ptr_of(I),
                                        Qa.mem, stream))
        return I

    def close(self):
        if getattr(self, "_h", None):
            N.load().gwn_octree_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def octree(P):
    """igl::octree(P, point_indices, CH, CN, W) -> (pi_offsets, pi_indices, CH, CN, W)."""
    t = Octree(P)
    try:
        return t.export()
    finally:
        t.close()


# ------------------------------------------------------------ point cloud --
class CloudExpansion:
    """Device-resident octree + order-k expansion of a point cloud
    (igl::fast_winding_number precompute, fast_winding_number.h:35-53)."""

    def __init__(self, P, Nrm, A, order: int = 2, tree: Octree | None = None):
        L = N.load()
        own = tree is None
        if own:
            tree = Octree(P)
        Na = _Arg(Nrm, np.float64)
        Aa = _Arg(np.asarray(A).reshape(-1) if not _is_torch_cuda(A) else A.reshape(-1),
                  np.float64)
        _need_rows(Na, 3, "N", tree.num_points)
        _need_len(Aa, tree.num_points, "A")
        h = C.c_void_p()
        stream = _stream_ptr() if Na.mem == N.GWN_DEVICE else None
        N.check(L.gwn_cloud_build(tree._h, None, Na.ptr, Aa.ptr, int(order), Na.mem, stream,
                                  C.byref(h)))
        self._h = h
        self.order = order
        self.num_terms = {0: 3, 1: 12, 2: 39}[order]
        self.tree = tree
        self.ncells = tree.sizes()[0]

    def export(self):
        """(CM, R, EC) with one row per octree cell (rows >= #cells of the
        reference's 8*#cells-row outputs are not produced)."""
        nc = self.ncells
        CM = np.empty((nc, 3))
        R = np.empty(nc)
        EC = np.empty((nc, self.num_terms))
        P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        N.check(N.load().gwn_cloud_export(self._h, P(CM), P(R), P(EC), N.GWN_HOST, None))
        return CM, R, EC

    def eval(self, Q, beta: float = 2.0, precision="mixed", out_dtype=None):
        L = N.load()
        Qa = _Arg(Q)
        if len(Qa.shape) != 2 or Qa.shape[1] != 3:
            raise ValueError("Q must be #Q x 3")
        wdt = np.dtype(out_dtype) if out_dtype is not None else Qa.np_dtype
        W = _empty_like_mem(Qa.mem, (Qa.shape[0],), wdt, like=Qa)
        stream = _stream_ptr() if Qa.mem == N.GWN_DEVICE else None
        N.check(L.gwn_cloud_eval(self._h, C.c_double(beta), Qa.ptr, Qa.code, Qa.shape[0],
                                 _ptr_of(W), N.GWN_F64 if wdt == np.float64 else N.GWN_F32,
                                 _prec(precision), Qa.mem, stream))
        return W

    def close(self):
        if getattr(self, "_h", None):
            N.load().gwn_cloud_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _octree_arrays(P, Nrm, A, pi_offsets, pi_indices, CH):
    """The caller's cloud and octree arrays as contiguous host arrays, with
    the shapes the C ABI reads checked first."""
    P, Nrm, A = _f64(P), _f64(Nrm), _f64(np.asarray(A).reshape(-1))
    off = np.ascontiguousarray(pi_offsets, np.int64).reshape(-1)
    idx = np.ascontiguousarray(pi_indices, np.int32).reshape(-1)
    CH = np.ascontiguousarray(CH, np.int32)
    if P.ndim != 2 or P.shape[1] != 3:
        raise ValueError(f"P must be #P x 3, got shape {P.shape}")
    if Nrm.shape != P.shape:
        raise ValueError(f"N must be {P.shape[0]} x 3, got shape {Nrm.shape}")
    if A.shape[0] != P.shape[0]:
        raise ValueError(f"A must hold {P.shape[0]} elements, got {A.shape[0]}")
    if CH.ndim != 2 or CH.shape[1] != 8 or CH.shape[0] < 1:
        raise ValueError(f"CH must be #cells x 8 with at least the root, got shape {CH.shape}")
    if off.shape[0] != CH.shape[0] + 1:
        raise ValueError(f"pi_offsets must hold #cells + 1 = {CH.shape[0] + 1} entries, "
                         f"got {off.shape[0]}")
    if idx.shape[0] < off[-1]:
        raise ValueError(f"pi_indices must hold pi_offsets[-1] = {off[-1]} entries, "
                         f"got {idx.shape[0]}")
    return P, Nrm, A, off, idx, CH


def fast_winding_number_cloud_precompute(P, Nrm, A, pi_offsets, pi_indices, CH, order: int = 2):
    """igl::fast_winding_number(P,N,A,point_indices,CH,expansion_order,CM,R,EC)
    over caller-held octree arrays (host memory).  Returns (CM, R, EC) with
    #cells rows."""
    P, Nrm, A, off, idx, CH = _octree_arrays(P, Nrm, A, pi_offsets, pi_indices, CH)
    nc = CH.shape[0]
    if order not in (0, 1, 2):
        raise ValueError("order must be 0, 1 or 2")
    nt = {0: 3, 1: 12, 2: 39}[order]
    CM, R, EC = np.empty((nc, 3)), np.empty(nc), np.empty((nc, nt))
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    N.check(N.load().gwn_cloud_precompute_arrays(p(P), p(Nrm), p(A), P.shape[0], p(off), p(idx),
                                                 p(CH), nc, int(order), p(CM), p(R), p(EC)))
    return CM, R, EC


def fast_winding_number_cloud(P, Nrm, A, pi_offsets, pi_indices, CH, CM, R, EC, Q,
                              beta: float = 2.0, precision="mixed"):
    """igl::fast_winding_number(P,N,A,point_indices,CH,CM,R,EC,Q,beta,WN) over
    caller-held arrays (host memory); CM/R/EC may carry the reference's
    8*#cells rows, only the first #cells are read."""
    P, Nrm, A, off, idx, CH = _octree_arrays(P, Nrm, A, pi_offsets, pi_indices, CH)
    Q = _f64(Q)
    if Q.ndim != 2 or Q.shape[1] != 3:
        raise ValueError(f"Q must be #Q x 3, got shape {Q.shape}")
    nc = CH.shape[0]
    CM, R, EC = _f64(CM), _f64(np.asarray(R).reshape(-1)), _f64(EC)
    if CM.ndim != 2 or CM.shape[1] != 3 or CM.shape[0] < nc or R.shape[0] < nc:
        raise ValueError(f"CM must be at least {nc} x 3 and R hold at least {nc} entries")
    if EC.ndim != 2 or EC.shape[1] not in (3, 12, 39) or EC.shape[0] < nc:
        raise ValueError(f"EC must be at least {nc} x (3, 12 or 39), got shape {EC.shape}")
    CM, R, EC = np.ascontiguousarray(CM[:nc]), R[:nc], np.ascontiguousarray(EC[:nc])
    order = {3: 0, 12: 1, 39: 2}[EC.shape[1]]
    W = np.empty(Q.shape[0])
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    N.check(N.load().gwn_cloud_eval_arrays(p(P), p(Nrm), p(A), P.shape[0], p(off), p(idx), p(CH),
                                           nc, p(CM), p(R), p(EC), order, p(Q), Q.shape[0],
                                           float(beta), p(W), _prec(precision)))
    return W


def fast_winding_number_cloud_oneshot(P, Nrm, A, Q, order: int = 2, beta: float = 2.0,
                                      precision="mixed"):
    """igl::fast_winding_number(P,N,A,Q,order,beta,WN) (fast_winding_number.h:104-131):
    octree -> precompute -> evaluate, all on the device."""
    ce = CloudExpansion(P, Nrm, A, order)
    try:
        return ce.eval(Q, beta, precision)
    finally:
        ce.close()
        ce.tree.close()


def point_areas(P, I, N, return_T: bool = False):
    """igl::copyleft::cgal::point_areas(P,I,N,A[,T])
    (include/igl/copyleft/cgal/point_areas.h:40-53): per-point Voronoi
    areas from the neighbour lists I (#P x k, e.g. ``knn(P, P, k)``).
    Returns A (#P,), and T (#P x 3) too when return_T."""
    L = NV.load()
    Pa = _Arg(P, np.float64)
    Ia = _Arg(I, np.int32, allowed=(np.int32,))
    Na = _Arg(N, np.float64)
    mem = _same_mem(Pa, Ia, Na)
    _need_rows(Pa, 3, "P")
    _need_rows(Na, 3, "N", Pa.shape[0])
    if len(Ia.shape) != 2 or Ia.shape[0] != Pa.shape[0]:
        raise ValueError("I must be #P x k")
    n, k = Ia.shape
    A = _empty_like_mem(mem, (n,), np.float64, like=Pa)
    T = _empty_like_mem(mem, (n, 3), np.float64, like=Pa) if return_T else None
    stream = _stream_ptr() if mem == NV.GWN_DEVICE else None
    NV.check(L.gwn_point_areas(Pa.ptr, n, Ia.ptr, k, Na.ptr, _ptr_of(A),
                               _ptr_of(T) if return_T else None, mem, stream))
    return (A, T) if return_T else A


def fast_winding_number_cloud_points(P, Nrm, Q, order: int = 2, beta: float = 2.0,
                                     precision="mixed", out_dtype=None):
    """igl::copyleft::cgal::fast_winding_number(P,N,Q,expansion_order,beta,WN)
    (include/igl/copyleft/cgal/fast_winding_number.h:20-36): the areas come
    from the 21 nearest points of each point (point_areas)."""
    L = NV.load()
    Pa = _Arg(P, np.float64)
    Na = _Arg(Nrm, np.float64)
    Qa = _Arg(Q)
    mem = _same_mem(Pa, Na, Qa)
    _need_rows(Pa, 3, "P")
    _need_rows(Na, 3, "N", Pa.shape[0])
    _need_rows(Qa, 3, "Q")
    wdt = np.dtype(out_dtype) if out_dtype is not None else Qa.np_dtype
    W = _empty_like_mem(mem, (Qa.shape[0],), wdt, like=Qa)
    stream = _stream_ptr() if mem == NV.GWN_DEVICE else None
    NV.check(L.gwn_cloud_winding_number_points(
        Pa.ptr, Na.ptr, Pa.shape[0], Qa.ptr, Qa.code, Qa.shape[0], int(order), float(beta),
        _ptr_of(W), NV.GWN_F64 if wdt == np.float64 else NV.GWN_F32, _prec(precision), mem,
        stream))
    return W


def knn(P, V, k: int):
    """igl::knn(P,V,k,point_indices,CH,CN,W,I) (include/igl/knn.h): the k
    points of V nearest to each row of P, nearest first (equal distances by
    index); the octree of V is built inside.  Host arrays or CUDA tensors."""
    Pa, Va = _Arg(P, np.float64), _Arg(V, np.float64)
    _same_mem(Pa, Va)
    _need_rows(Pa, 3, "P")
    _need_rows(Va, 3, "V")
    if int(k) < 0:
        raise ValueError("k must be non-negative")
    cols = min(int(k), Va.shape[0])
    I = _empty_like_mem(Pa.mem, (Pa.shape[0], cols), np.int32, like=Pa)
    stream = _stream_ptr() if Pa.mem == N.GWN_DEVICE else None
    N.check(N.load().gwn_knn(Pa.ptr, Pa.shape[0], Va.ptr, Va.shape[0], int(k), _ptr_of(I),
                             Pa.mem, stream))
    return I


# ------------------------------------------ hierarchical exact winding --
class WindingNumberAABB:
    """igl::WindingNumberAABB (include/igl/WindingNumberAABB.h) on the GPU:
    the exact winding number of a triangle mesh through a tree of boundary
    caps.  ``WindingNumberAABB(V, F).winding_number(Q)``; V, F host arrays or
    CUDA tensors (copied to the device), Q likewise."""

    def __init__(self, V, F):
        Va = _Arg(V, np.float64)
        Fa = _Arg(F, np.int32, allowed=(np.int32,))
        _same_mem(Va, Fa)
        if Va.shape[1:] != (3,) or Fa.shape[1:] != (3,):
            raise ValueError("V must be #V x 3 and F #F x 3")
        self._h = C.c_void_p()
        stream = _stream_ptr() if Va.mem == N.GWN_DEVICE else None
        N.check(N.load().gwn_wn_aabb_build(Va.ptr, Va.shape[0], Fa.ptr, Fa.shape[0], Va.mem,
                                           stream, C.byref(self._h)))

    def winding_number(self, Q, precision="mixed"):
        """W of every row of Q; ``precision`` "fp64" walks as the reference
        does with every term in FP64, "mixed" takes FP32 terms away from the
        surface (see gwn_wn_aabb_eval_precision)."""
        Qa = _Arg(Q, np.float64)
        if len(Qa.shape) != 2 or Qa.shape[1] != 3:
            raise ValueError("Q must be #Q x 3")
        W = _empty_like_mem(Qa.mem, (Qa.shape[0],), np.float64, like=Qa)
        stream = _stream_ptr() if Qa.mem == N.GWN_DEVICE else None
        N.check(N.load().gwn_wn_aabb_eval_precision(self._h, Qa.ptr, Qa.shape[0], _ptr_of(W),
                                                    _prec(precision), Qa.mem, stream))
        return W

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            N.load().gwn_wn_aabb_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------- 2-D Eytzinger AABB winding --
def eytzinger_aabb(PB1, PB2):
    """igl::eytzinger_aabb(PB1,PB2,B1,B2,leaf) (include/igl/eytzinger_aabb.h):
    (B1, B2, leaf) of the tree over the m primitive boxes (m x dim corners);
    empty slots have leaf -2 and NaN boxes.  Host arrays or CUDA tensors."""
    A1, A2 = _Arg(PB1, np.float64), _Arg(PB2, np.float64)
    _same_mem(A1, A2)
    if len(A1.shape) != 2 or A1.shape != A2.shape:
        raise ValueError("PB1 and PB2 must both be m x dim")
    m, dim = A1.shape
    L = N.load()
    nb = int(L.gwn_eytzinger_slots(m))
    B1 = _empty_like_mem(A1.mem, (nb, dim), np.float64, like=A1)
    B2 = _empty_like_mem(A1.mem, (nb, dim), np.float64, like=A1)
    leaf = _empty_like_mem(A1.mem, (nb,), np.int32, like=A1)
    stream = _stream_ptr() if A1.mem == N.GWN_DEVICE else None
    N.check(L.gwn_eytzinger_aabb(A1.ptr, A2.ptr, m, dim, _ptr_of(B1), _ptr_of(B2), _ptr_of(leaf),
                                 A1.mem, stream))
    return B1, B2, leaf


def eytzinger_aabb_winding_number_tree(E, leaf):
    """igl::eytzinger_aabb_winding_number_tree(E,leaf,I,C): (I, C), each
    internal node's boundary-vertex pairs (positive vertices ascending paired
    with negative vertices ascending)."""
    Ea = _Arg(E, np.int32, allowed=(np.int32,))
    La = _Arg(leaf, np.int32, allowed=(np.int32,))
    _same_mem(Ea, La)
    nb = La.shape[0]
    L = N.load()
    Cc = _empty_like_mem(La.mem, (nb + 1,), np.int32, like=La)
    stream = _stream_ptr() if La.mem == N.GWN_DEVICE else None
    nE = Ea.shape[0] if len(Ea.shape) == 2 else 0
    N.check(L.gwn_eytzinger_winding_number_tree(Ea.ptr, nE, La.ptr, nb, _ptr_of(Cc), None,
                                                La.mem, stream))
    total = int(Cc[-1])
    I = _empty_like_mem(La.mem, (total,), np.int32, like=La)
    if total:
        N.check(L.gwn_eytzinger_winding_number_tree(Ea.ptr, nE, La.ptr, nb, _ptr_of(Cc),
                                                    _ptr_of(I), La.mem, stream))
    return I, Cc


def eytzinger_aabb_winding_number(P, V, E, B1, B2, leaf, I, Cc, precision="mixed"):
    """igl::eytzinger_aabb_winding_number(p,V,E,B1,B2,leaf,I,C,wn) for every
    row of P (#P x 2): the winding number of each point with respect to the
    segments E of V (2-D).  ``precision`` "fp64" follows the reference's
    arithmetic; "mixed" is FP32 with FP64 where it matters."""
    Pa, Va, B1a, B2a = (_Arg(x, np.float64) for x in (P, V, B1, B2))
    Ea, La, Ia, Ca = (_Arg(x, np.int32, allowed=(np.int32,)) for x in (E, leaf, I, Cc))
    _same_mem(Pa, Va, B1a, B2a, Ea, La, Ia, Ca)
    if len(Pa.shape) != 2 or Pa.shape[1] != 2 or (Va.shape[0] and Va.shape[1:] != (2,)):
        raise ValueError("P and V must be #P x 2 / #V x 2")
    if Ea.shape[0] and Ea.shape[1:] != (2,):
        raise ValueError(f"E must be #E x 2, got shape {Ea.shape}")
    slots = La.shape[0]
    if slots:
        _need_rows(B1a, 2, "B1", slots)
        _need_rows(B2a, 2, "B2", slots)
        _need_len(Ca, slots + 1, "C")
    n = Pa.shape[0]
    W = _empty_like_mem(Pa.mem, (n,), np.float64, like=Pa)
    stream = _stream_ptr() if Pa.mem == N.GWN_DEVICE else None
    nE = Ea.shape[0] if len(Ea.shape) == 2 else 0
    N.check(N.load().gwn_eytzinger_winding_number(
        Pa.ptr, n, Va.ptr, Va.shape[0], Ea.ptr, nE, B1a.ptr, B2a.ptr, La.ptr, La.shape[0],
        Ia.ptr, Ia.shape[0], Ca.ptr, _ptr_of(W), _prec(precision), Pa.mem, stream))
    return W


# ------------------------------------------------------- signed distance --
SIGNED_DISTANCE_TYPE_PSEUDONORMAL = 0
SIGNED_DISTANCE_TYPE_WINDING_NUMBER = 1
SIGNED_DISTANCE_TYPE_DEFAULT = 2
SIGNED_DISTANCE_TYPE_UNSIGNED = 3
SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER = 4


def signed_distance(P, V, F, sign_type=SIGNED_DISTANCE_TYPE_DEFAULT, lower_bound=None,
                    upper_bound=None, precision=None, return_normals: bool = False):
    """igl::signed_distance(P,V,F,sign_type,lower_bound,upper_bound,S,I,C,N)
    (include/igl/signed_distance.h:61-71) for 3-D triangles: (S, I, C).

    Bounds default to the reference's bound-less overload (DBL_MIN, DBL_MAX).
    ``precision`` selects how the sign's winding number is computed; by
    default plain FP64 for the exact winding number (as the reference) and
    mixed precision for the fast winding number (the reference's is FP32).
    With ``return_normals`` also N (the pseudonormal type's normals, else 0).
    Host arrays or CUDA torch tensors (all of one kind)."""
    L = N.load()
    Pa = _Arg(P, np.float64)
    Va = _Arg(V, np.float64)
    Fa = _Arg(F, np.int32, allowed=(np.int32,))
    _same_mem(Pa, Va, Fa)
    if len(Pa.shape) != 2 or Pa.shape[1] != 3 or Va.shape[1:] != (3,) or Fa.shape[1:] != (3,):
        raise ValueError("P and V must be #P x 3 / #V x 3 and F #F x 3 (3-D triangles)")
    if precision is None:
        precision = "mixed" if sign_type == SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER else "fp64"
    lo = np.finfo(np.float64).tiny if lower_bound is None else float(lower_bound)
    hi = np.finfo(np.float64).max if upper_bound is None else float(upper_bound)
    n = Pa.shape[0]
    S = _empty_like_mem(Pa.mem, (n,), np.float64, like=Pa)
    I = _empty_like_mem(Pa.mem, (n,), np.int32, like=Pa)
    Cp = _empty_like_mem(Pa.mem, (n, 3), np.float64, like=Pa)
    Nm = _empty_like_mem(Pa.mem, (n, 3), np.float64, like=Pa)
    if sign_type != SIGNED_DISTANCE_TYPE_PSEUDONORMAL:
        Nm[:] = 0
    stream = _stream_ptr() if Pa.mem == N.GWN_DEVICE else None
    N.check(L.gwn_signed_distance(Pa.ptr, n, Va.ptr, Va.shape[0], Fa.ptr, Fa.shape[0],
                                  int(sign_type), C.c_double(lo), C.c_double(hi), _ptr_of(S),
                                  _ptr_of(I), _ptr_of(Cp), _ptr_of(Nm), _prec(precision),
                                  Pa.mem, stream))
    return (S, I, Cp, Nm) if return_normals else (S, I, Cp)


# ---------------------------------------------------------- swept volume --
def _affine_rows(transforms):
    T = np.asarray(transforms, dtype=np.float64)
    if T.ndim == 2 and T.shape[1] == 12:
        return np.ascontiguousarray(T)
    if T.ndim == 3 and T.shape[1:] in ((3, 4), (4, 4)):
        return np.ascontiguousarray(T[:, :3, :4].reshape(-1, 12))
    raise ValueError("transforms must be nT x 3 x 4, nT x 4 x 4 or nT x 12")


def swept_volume_signed_distance(V, F, transforms, sign_type, GV, res, h, isolevel, S0=None,
                                 precision=None):
    """igl::swept_volume_signed_distance(V,F,transforms,sign_type,GV,res,h,
    isolevel,S0,S) (include/igl/swept_volume_signed_distance.h): the signed
    distance at grid points GV (#GV x 3, a res[0] x res[1] x res[2] grid, x
    fastest, spacing h) to the volume swept by the mesh under the rigid
    motions ``transforms`` (nT x 3 x 4 or 4 x 4 affine matrices, applied as
    x -> L x + t).  ``S0`` seeds the running minimum (default all NaN).  Host
    arrays or CUDA tensors for V, F, GV, S0 (all of one kind); transforms on
    the host.  ``precision``: how the sign's winding number is computed,
    mixed by default (FP32 with FP64 near the mesh and for results within
    1e-3 of 0.5); "fp64" is the reference's arithmetic."""
    Va, Ga = _Arg(V, np.float64), _Arg(GV, np.float64)
    Fa = _Arg(F, np.int32, allowed=(np.int32,))
    _same_mem(Va, Fa, Ga)
    if Ga.shape[1:] != (3,) or Va.shape[1:] != (3,) or Fa.shape[1:] != (3,):
        raise ValueError("V, GV must be #x3 float and F #F x 3 int32")
    T = _affine_rows(transforms)
    r = np.ascontiguousarray(res, dtype=np.int32).reshape(3)
    if precision is None:
        precision = "mixed"
    n = Ga.shape[0]
    S = _empty_like_mem(Ga.mem, (n,), np.float64, like=Ga)
    S0p = None
    if S0 is not None:
        S0a = _Arg(S0, np.float64)
        _same_mem(Ga, S0a)
        _need_len(S0a, n, "S0")
        S0p = S0a.ptr
    stream = _stream_ptr() if Ga.mem == N.GWN_DEVICE else None
    N.check(N.load().gwn_swept_volume_signed_distance(
        Va.ptr, Va.shape[0], Fa.ptr, Fa.shape[0], T.ctypes.data_as(C.c_void_p), T.shape[0],
        int(sign_type), Ga.ptr, n, r.ctypes.data_as(C.c_void_p), float(h), float(isolevel),
        S0p, _ptr_of(S), _prec(precision), Ga.mem, stream))
    return S


def flood_fill(res, S):
    """igl::flood_fill(res,S) (include/igl/flood_fill.h): fills the NaN entries
    of S (res[0] x res[1] x res[2], x fastest) in place and returns S."""
    Sa = _Arg(S, np.float64)
    if Sa.mem == N.GWN_HOST and Sa.obj is not S:
        raise ValueError("S must be a contiguous float64 array (filled in place)")
    if Sa.mem == N.GWN_DEVICE and Sa.obj.data_ptr() != S.data_ptr():
        raise ValueError("S must be a contiguous float64 tensor (filled in place)")
    r = np.ascontiguousarray(res, dtype=np.int32).reshape(3)
    stream = _stream_ptr() if Sa.mem == N.GWN_DEVICE else None
    N.check(N.load().gwn_flood_fill(r.ctypes.data_as(C.c_void_p), Sa.ptr, Sa.mem, stream))
    return S


# ------------------------------------------------------------- profiling --
def profile_enable(on: bool = True, accumulate: bool = False) -> None:
    """Record CUDA events around each phase of this thread's calls (of the
    last call only, or, with ``accumulate``, of every call until the next
    profile_enable)."""
    N.check(N.load().gwn_profile_enable(0 if not on else (2 if accumulate else 1)))


def profile_read() -> dict:
    """{phase name: milliseconds} of the recorded phases (the last call's, or
    summed over every call in accumulate mode); waits for them."""
    names = C.create_string_buffer(1 << 18)
    ms = (C.c_float * 8192)()
    n = C.c_int(0)
    N.check(N.load().gwn_profile_read(names, 1 << 18, ms, 8192, C.byref(n)))
    keys = names.value.decode().split(";") if names.value else []
    out = {}
    for k, v in zip(keys, list(ms)[: n.value]):
        out[k] = out.get(k, 0.0) + float(v)
    return out


def launch_count() -> int:
    """Kernels launched by libgwn in this process so far."""
    return int(N.load().gwn_launch_count())


def launch_count_of(fn) -> int:
    """Kernels libgwn launches while running fn() (same thread, nothing concurrent)."""
    a = launch_count()
    fn()
    return launch_count() - a
