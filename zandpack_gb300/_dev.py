"""Device-array helpers for the reference-name shims: torch CUDA tensors are
passed to libzandgpu by pointer on the current torch stream."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import ZGInvalid


def _torch():
    import torch
    return torch


def as_c128(x, name="array"):
    torch = _torch()
    if not (isinstance(x, torch.Tensor) and x.is_cuda):
        raise ZGInvalid(1, "%s must be a CUDA tensor" % name)
    if x.dtype != torch.complex128:
        raise ZGInvalid(1, "%s must be complex128" % name)
    if not x.is_contiguous():
        raise ZGInvalid(1, "%s must be contiguous" % name)
    return x


def ptr(x):
    return C.c_void_p(x.data_ptr())


def stream_of(x):
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)


def host_f64(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
