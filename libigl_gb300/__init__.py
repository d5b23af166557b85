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

Arrays may be NumPy arrays (host memory: the call copies in, computes on the
GPU, copies out) or CUDA torch tensors (device memory: the work is enqueued on
torch's current stream and the result stays on the device).  Every call runs
on the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from ._native import GwnError

__all__ = [
    "GwnError", "winding_number", "FastWindingNumberBVH",
    "fast_winding_number_soup_precompute", "fast_winding_number_soup",
    "Octree", "octree", "CloudExpansion", "fast_winding_number_cloud_precompute",
    "fast_winding_number_cloud", "fast_winding_number_cloud_oneshot", "device_status",
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
