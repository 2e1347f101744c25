"""Device versions of the kernels ``zand`` imports from Zandpack/mpi_funcs.py,
under the same names and argument meaning, for complex128 CUDA tensors
(torch).  ``Y`` arrays carry the Runge-Kutta slot axis first, like the
reference's ``SIGS``/``PSIS``/``OMGS``."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _dev
from ._lib import check, lib


def abs2(x):
    """|x|^2 (Zandpack/mpi_funcs.py:18-20)."""
    return x.real ** 2 + x.imag ** 2


def MM(A, B, OUT):
    """``np.matmul(A, B, out=OUT)`` (Zandpack/mpi_funcs.py:24-25); device
    tensors go through ``torch.matmul``."""
    torch = _dev._torch()
    if isinstance(A, torch.Tensor):
        torch.matmul(A, B, out=OUT)
    else:
        np.matmul(A, B, out=OUT)


_multiply = np.multiply


def _terr2(Y, CT):
    Y = _dev.as_c128(Y, "Y")
    ns = Y.shape[0]
    ct = _dev.host_f64(CT)
    if ct.size != ns:
        raise AssertionError("CT has %d entries for %d slots" % (ct.size, ns))
    count = Y[0].numel() if ns else 0
    res = np.zeros(1)
    check(lib().zg_terr2_c128(_dev.ptr(Y), count, ns, ct.ctypes.data_as(C.c_void_p), count,
                              res.ctypes.data_as(C.c_void_p), _dev.stream_of(Y)))
    return float(res[0])


def TERR2_sig(y1, CT):
    """sum |sum_j CT_j y_j|^2 over sigma slots (Zandpack/mpi_funcs.py:247-248)."""
    return _terr2(y1, CT)


def TERR2_psi(y2, CT):
    """Zandpack/mpi_funcs.py:249-250."""
    return _terr2(y2, CT)


def TERR2_omg(y3, CT):
    """Zandpack/mpi_funcs.py:251-252."""
    return _terr2(y3, CT)


def _step_fourth(Y, CH):
    Y = _dev.as_c128(Y, "Y")
    ns = Y.shape[0]
    ch = _dev.host_f64(CH)
    if ch.size != ns:
        raise AssertionError("CH has %d entries for %d slots" % (ch.size, ns))
    count = Y[0].numel()
    check(lib().zg_step_fourth_c128(_dev.ptr(Y), count, ns, ch.ctypes.data_as(C.c_void_p), count,
                                    _dev.stream_of(Y)))


def step_fourth_sig(Y1, CH):
    """Y1[-1] = sum_j CH_j Y1[j] in place (Zandpack/mpi_funcs.py:254-255)."""
    _step_fourth(Y1, CH)


def step_fourth_psi(Y2, CH):
    """Zandpack/mpi_funcs.py:256-257."""
    _step_fourth(Y2, CH)


def step_fourth_omg(Y3, CH):
    """Zandpack/mpi_funcs.py:258-259."""
    _step_fourth(Y3, CH)


def OuterSubtraction_hard_opti(A, B, C_, out):
    """out[k,a,x,c,aa,xx,:] += (A[k,a,x,0] - B[k,aa,xx,0]) * C[k,a,x,c,aa,xx,:]
    (Zandpack/mpi_funcs.py:91-102), broadcast on the device."""
    a = A[..., 0][:, :, :, None, None, None, None]
    b = B[..., 0][:, None, None, None, :, :, None]
    out += (a - b) * C_
