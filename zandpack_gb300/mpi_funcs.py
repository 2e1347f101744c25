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
    """``np.matmul(A, B, out=OUT)`` (Zandpack/mpi_funcs.py:24-25) on CUDA
    tensors.  ``zand`` calls it in two forms.  The stage combination
    ``MM(SIGS[idx].transpose(..., 0), B[i, idx], out)`` (Zandpack/mpi/zand:
    306-313), a product with a vector whose left operand is a set of
    Runge-Kutta slots viewed slot-axis-last, runs on this library's combination
    kernel (``zg_combine_c128``).  Every other form is a plain complex GEMM of
    the worker's stage body, which this package replaces as a whole (``zg_rhs``);
    it goes to ``torch.matmul`` (cuBLAS), as a library GEMM."""
    torch = _dev._torch()
    for name, x in (("A", A), ("OUT", OUT)):
        if not (isinstance(x, torch.Tensor) and x.is_cuda):
            raise _lib_invalid("%s must be a CUDA tensor" % name)
    if np.ndim(B) == 1 and A.dim() >= 2 and A.shape[-1] == len(B):
        slots = A.movedim(-1, 0)
        bh = B.detach().cpu().numpy() if isinstance(B, torch.Tensor) else np.asarray(B)
        if (slots.is_contiguous() and A.dtype == torch.complex128 and OUT.is_contiguous()
                and OUT.dtype == torch.complex128 and tuple(OUT.shape) == tuple(A.shape[:-1])
                and not np.any(np.imag(bh))):
            b = _dev.host_f64(np.real(bh))
            ns = slots.shape[0]
            count = OUT.numel()
            idx = np.arange(ns, dtype=np.int32)
            check(lib().zg_combine_c128(_dev.ptr(slots), count, ns, b.ctypes.data_as(C.c_void_p),
                                        idx.ctypes.data_as(C.c_void_p), ns, _dev.ptr(OUT), count,
                                        _dev.stream_of(OUT)))
            return
    Bd = B if isinstance(B, torch.Tensor) else torch.as_tensor(np.asarray(B), device=A.device).to(A.dtype)
    torch.matmul(A, Bd, out=OUT)


def _lib_invalid(msg):
    from ._lib import ZGInvalid
    return ZGInvalid(1, msg)


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
    (Zandpack/mpi_funcs.py:91-102), in one pass of ``zg_outer_subtraction_c128``."""
    A = _dev.as_c128(A, "A")
    B = _dev.as_c128(B, "B")
    C_ = _dev.as_c128(C_, "C")
    out = _dev.as_c128(out, "out")
    if A.dim() != 4 or B.dim() != 4 or C_.dim() != 7 or tuple(out.shape) != tuple(C_.shape):
        raise AssertionError("OuterSubtraction_hard_opti: A (nk,na,nx,*), B (nk,NA,NX,*), C and out 7-D alike")
    nk, na, nx, noT, NA, NX, NO = C_.shape
    if tuple(A.shape[:3]) != (nk, na, nx) or tuple(B.shape[:3]) != (nk, NA, NX):
        raise AssertionError("OuterSubtraction_hard_opti: A/B do not match C")
    shape = np.array(C_.shape, np.int64)
    check(lib().zg_outer_subtraction_c128(_dev.ptr(A), int(A.shape[3]), _dev.ptr(B), int(B.shape[3]),
                                          _dev.ptr(C_), _dev.ptr(out), shape.ctypes.data_as(C.c_void_p),
                                          _dev.stream_of(out)))
