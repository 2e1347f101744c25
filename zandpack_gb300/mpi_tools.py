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


def natural_keys(text):
    """Sort key: the digit groups of ``text`` compared as integers
    (Zandpack/mpi_tools.py:13-17)."""
    return [int(part) if part.isdigit() else part for part in re.split(r"(\d+)", text)]


def _step_files(d, keep):
    """The names in directory ``d`` for which ``keep(name)`` holds, in natural order."""
    return sorted(filter(keep, os.listdir(d)), key=natural_keys)


def _read_all(d, names, load=np.load):
    return [load(os.path.join(d, name)) for name in names]


def combine_currents(dirs, n=2):
    """(T, [J_0, ..., J_{n-1}]) over the save directories ``dirs``
    (Zandpack/mpi_tools.py:19-49): every ``current_<lead>_<step>`` file of a
    lead stacked in natural order, and the ``times*`` files concatenated with
    as many trailing entries dropped as there are directories (the time after
    the last step), as the reference does."""
    leads = [[] for _ in range(n)]
    times = []
    for d in dirs:
        for name in _step_files(d, lambda v: "current_" in v):
            fields = name.split("_")
            if len(fields) != 2:  # current_<lead>_<step>
                leads[int(fields[1])].append(flexload(os.path.join(d, name)))
        times.extend(_read_all(d, _step_files(d, lambda v: "times" in v)))
    T = np.hstack(times)
    return T[:T.shape[0] - len(dirs)], [np.vstack(rows) for rows in leads]


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
    mats, times = [], []
    for d in dirs:
        dm_names = _step_files(d, lambda v: "DM" in v and "DMt" not in v)
        if not dm_names or not prefer_full:
            archive = _lossy_archive(d, os.listdir(d))
            if lossy_dm_arc:
                return archive
            dm = archive["dm"].transpose(3, 0, 1, 2).copy()
            return archive["tdm"], herm_insert_tril(dm) if insert_tril else dm
        t_names = _step_files(d, lambda v: times_label in v)
        if split is not None and split_rank is not None:
            assert split < len(dm_names)
            share = np.array_split(np.arange(len(dm_names)), split)[split_rank]
            dm_names = [dm_names[i] for i in share]
            t_names = [t_names[i] for i in share]
        for dm in _read_all(d, dm_names, flexload):
            mats.append(herm_insert_tril(dm) if insert_tril else dm)
        times.extend(_read_all(d, t_names))
    return np.hstack(times), np.vstack(mats)


def combine_pi(dirs, times_label="DMt"):
    """(T, PI): the saved ``PIa`` arrays and time files of ``dirs``
    (Zandpack/mpi_tools.py:120-144); ``.npz`` archives (``compress_mat``) are
    read as well."""
    pis, times = [], []
    for d in dirs:
        pis.extend(_read_all(d, _step_files(d, lambda v: "PIa" in v), flexload))
        times.extend(_read_all(d, _step_files(d, lambda v: times_label in v)))
    return np.hstack(times), np.vstack(pis)
