"""Readers of the ``<name>_save/`` output of a propagation, with the names and
argument meaning of the reference's post-processing helpers
(Zandpack/mpi_tools.py:13-144).

The files are those ``zand``/``nozand`` (and ``zandpack_gb300.zand``) write:
``current_<lead>_<step>.npy``, ``times<step>.npy``, ``DM<step>.npy`` (or
``.npz`` with ``compress_mat``), ``DMt<step>.npy``, ``PIa<step>.npy``.  Files
are ordered by their natural order (digit groups compared as integers).
"""
from __future__ import annotations

import io
import lzma
import os
import re

import numpy as np

from .arrays_io import flexload

__all__ = ["natural_keys", "combine_currents", "rectified_charge", "combine_dm", "herm_insert_tril", "combine_pi"]


def atoi(text):
    return int(text) if text.isdigit() else text


def natural_keys(text):
    """Sort key: the digit groups of ``text`` compared as integers
    (Zandpack/mpi_tools.py:13-17)."""
    return [atoi(c) for c in re.split(r"(\d+)", text)]


def _sorted(d, pred):
    return sorted((v for v in os.listdir(d) if pred(v)), key=natural_keys)


def combine_currents(dirs, n=2):
    """(T, [J_0, ..., J_{n-1}]) over the save directories ``dirs``
    (Zandpack/mpi_tools.py:19-49): every ``current_<lead>_<step>`` file of a
    lead stacked in natural order, the ``times*`` files concatenated with the
    last entry of each directory dropped (the time after the last step)."""
    C = [[] for _ in range(n)]
    T = []
    count = 0
    for d in dirs:
        for ff in _sorted(d, lambda v: "current_" in v):
            vals = ff.split("_")
            if len(vals) != 2:
                C[int(vals[1])].append(flexload(os.path.join(d, ff)))
        for ff in _sorted(d, lambda v: "times" in v):
            T.append(np.load(os.path.join(d, ff)))
        count += 1
    CC = [np.vstack(C[i]) for i in range(n)]
    T = np.hstack(T)[:-count]
    return T, CC


def rectified_charge(dirs, n=2, wgts=(0.5, -0.5), idx=0):
    """Per directory, the charge passed by the weighted current
    sum_k wgts[k] J_k (k-point ``idx``): [t[1:], cumulative Simpson integral]
    (Zandpack/mpi_tools.py:51-59)."""
    from scipy.integrate import cumulative_simpson
    res = []
    for d in dirs:
        t, j = combine_currents([d], n=n)
        Jt = np.zeros(len(t))
        for k in range(n):
            Jt += wgts[k] * j[k][:, idx]
        res.append([t[1:].copy(), cumulative_simpson(Jt, x=t)])
    return res


def herm_insert_tril(A):
    """In place: the strict lower triangle from the conjugate of the upper one
    (undoes ``dm_triu_only``; Zandpack/mpi_tools.py:113-118)."""
    n = A.shape[-1]
    il = np.tril_indices(n, -1)
    A[..., il[0], il[1]] = np.conj(A[..., il[1], il[0]])
    return A


def _lossy_archive(d, names):
    if "LossyDensityMatrix.npz.xz" in names:
        with lzma.open(os.path.join(d, "LossyDensityMatrix.npz.xz"), "rb") as f:
            return np.load(io.BytesIO(f.read()))
    if "LossyDensityMatrix.npz" in names:
        return np.load(os.path.join(d, "LossyDensityMatrix.npz"))
    return None


def combine_dm(dirs, times_label="DMt", insert_tril=False, split=None, split_rank=None, prefer_lossy_dm=True,
               lossy_dm_arc=False, prefer_full=True):
    """(T, DM): the saved density matrices of ``dirs`` in natural file order
    (``.npy`` or ``.npz``) and the ``times_label`` time files
    (Zandpack/mpi_tools.py:61-111).  A directory without ``DM`` files (or with
    ``prefer_full=False``) is read from its ``LossyDensityMatrix.npz[.xz]``
    archive instead (``dm`` transposed to time-first, and ``tdm``); with
    ``lossy_dm_arc`` the archive itself is returned.  ``insert_tril`` restores
    the lower triangle of ``dm_triu_only`` files; ``split``/``split_rank``
    read one of ``split`` contiguous shares of the files."""
    DM, T = [], []
    for d in dirs:
        names = os.listdir(d)
        arc = _lossy_archive(d, names)
        files = _sorted(d, lambda v: "DM" in v and "DMt" not in v)
        if not (len(files) > 0 and prefer_full):
            if lossy_dm_arc:
                return arc
            dm = arc["dm"].transpose(3, 0, 1, 2).copy()
            if insert_tril:
                herm_insert_tril(dm)
            return arc["tdm"], dm
        tfiles = _sorted(d, lambda v: times_label in v)
        if split is not None and split_rank is not None:
            assert split < len(files)
            idx = np.array_split(np.arange(len(files)), split)[split_rank]
            files = [files[i] for i in idx]
            tfiles = [tfiles[i] for i in idx]
        for ff in files:
            dm = flexload(os.path.join(d, ff))
            if insert_tril:
                herm_insert_tril(dm)
            DM.append(dm)
        for ff in tfiles:
            T.append(np.load(os.path.join(d, ff)))
    return np.hstack(T), np.vstack(DM)


def combine_pi(dirs, times_label="DMt"):
    """(T, PI): the saved ``PIa`` arrays and time files of ``dirs``
    (Zandpack/mpi_tools.py:120-144); ``.npz`` archives (``compress_mat``) are
    read as well."""
    DM, T = [], []
    for d in dirs:
        for ff in _sorted(d, lambda v: "PIa" in v):
            DM.append(flexload(os.path.join(d, ff)))
        for ff in _sorted(d, lambda v: times_label in v):
            T.append(np.load(os.path.join(d, ff)))
    return np.hstack(T), np.vstack(DM)
