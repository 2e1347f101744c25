"""Device versions of the stage-combination and error kernels of
Zandpack/func_step_forward.py, under the same names, for complex128 CUDA
tensors (torch).  ``Y`` carries the Runge-Kutta slot axis first."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _dev
from ._lib import check, lib
from .mpi_funcs import _terr2


def _combine(Y, b, out, idx):
    Y = _dev.as_c128(Y, "Y")
    out = _dev.as_c128(out, "out")
    ns = Y.shape[0]
    count = Y[0].numel() if ns else 0
    if out.numel() != count:
        raise AssertionError("out has %d elements, a slot has %d" % (out.numel(), count))
    bb = _dev.host_f64(b)
    ix = np.ascontiguousarray(np.asarray(idx, dtype=np.int32).ravel())
    if bb.size < ns:
        raise AssertionError("b has fewer entries than slots")
    check(lib().zg_combine_c128(_dev.ptr(Y), count, ns, bb.ctypes.data_as(C.c_void_p),
                                ix.ctypes.data_as(C.c_void_p), int(ix.size), _dev.ptr(out), count,
                                _dev.stream_of(Y)))


def step_sig_forward_nb(Sig_v, b, out, idx):
    """out = sum_{i in idx} b[i] Sig_v[i] (Zandpack/func_step_forward.py:16-28)."""
    _combine(Sig_v, b, out, idx)


def step_psi_forward_nb(Psi_v, b, out, idx):
    """Zandpack/func_step_forward.py:54-68."""
    _combine(Psi_v, b, out, idx)


def step_omg_forward_nb(Omg_v, b, out, idx):
    """Zandpack/func_step_forward.py:92-109."""
    _combine(Omg_v, b, out, idx)


def step_omg_forward_nb_fermi_opti(Omg_v, b, out, idx, fp_loc, fp_all):
    """Like ``step_omg_forward_nb`` but leaves ``out`` untouched where both the
    row pole (``fp_loc``) and the column pole (``fp_all``) are Fermi poles
    (Zandpack/func_step_forward.py:112-139), in one pass of
    ``zg_combine_fermi_skip_c128``.  ``Omg_v`` is (RK, k, a, x, c, a, x, c)."""
    torch = _dev._torch()
    Omg_v = _dev.as_c128(Omg_v, "Omg_v")
    out = _dev.as_c128(out, "out")
    if Omg_v.dim() != 8 or tuple(out.shape) != tuple(Omg_v.shape[1:]):
        raise AssertionError("Omg_v must be 8-D and out its slot shape")
    fl = np.ascontiguousarray(np.asarray(fp_loc, bool).astype(np.uint8))
    fa = np.ascontiguousarray(np.asarray(fp_all, bool).astype(np.uint8))
    if fl.size != Omg_v.shape[3] or fa.size != Omg_v.shape[6]:
        raise AssertionError("fp_loc/fp_all must have one entry per pole of the row/column lead axis")
    bb = _dev.host_f64(b)
    ix = np.ascontiguousarray(np.asarray(idx, dtype=np.int32).ravel())
    ns = Omg_v.shape[0]
    if bb.size < ns:
        raise AssertionError("b has fewer entries than slots")
    fld = torch.from_numpy(fl).to(out.device)
    fad = torch.from_numpy(fa).to(out.device)
    shape = np.array(Omg_v.shape[1:], np.int64)
    count = out.numel()
    check(lib().zg_combine_fermi_skip_c128(_dev.ptr(Omg_v), count, ns, bb.ctypes.data_as(C.c_void_p),
                                           ix.ctypes.data_as(C.c_void_p), int(ix.size), _dev.ptr(out),
                                           shape.ctypes.data_as(C.c_void_p), _dev.ptr(fld), _dev.ptr(fad),
                                           _dev.stream_of(out)))


def TERR2_sig_nb(Sig_v, CH):
    """Zandpack/func_step_forward.py:39-53."""
    return _terr2(Sig_v, CH)


def TERR2_psi_nb(Psi_v, b):
    """Zandpack/func_step_forward.py:75-91."""
    return _terr2(Psi_v, b)


def TERR2_omg_nb(Omg_v, b):
    """Zandpack/func_step_forward.py:141-159."""
    return _terr2(Omg_v, b)
