"""Readers and writers for the reference's on-disk formats.

* ``Arrays/``: one ``<key>.npy`` per array, ``xi``/``Ixi`` as compressed
  ``.npz`` (``Writer.write_to_file_compressed``, Zandpack/Writer.py:61-151),
  read lazily by key with a ``.npy`` -> ``.npz`` fallback (``flexload`` and
  ``load_dictionary``, Zandpack/Loader.py:12-43).
* ``<name>_save/``: restart files ``last_sig/last_time/last_stepsize`` and
  ``last_psi/last_omg`` (full padded arrays, complex128) as ``zand`` and
  ``psinought`` write them (Zandpack/mpi/zand:221-237,412-420,539-541;
  Zandpack/cmdtools/psinought:490-491).
"""
from __future__ import annotations

import os

import numpy as np


def flexload(filepath: str):
    """Load ``filepath``; a ``.npz`` archive yields its first array; a missing
    ``.npy`` falls back to the ``.npz`` of the same stem (Zandpack/Loader.py:12-31)."""
    try:
        f = np.load(filepath)
        if isinstance(f, np.ndarray):
            return f
        return f[f.files[0]]
    except (OSError, ValueError):
        pass
    alt = filepath.replace(".npy", ".npz")
    try:
        return np.load(alt)["arr_0"]
    except (OSError, ValueError, KeyError):
        raise FileNotFoundError("cannot load %s (nor %s)" % (filepath, alt)) from None


class load_dictionary:
    """Lazy ``Arrays`` dictionary: ``D[key]`` loads ``<dir><key>.npy``
    (Zandpack/Loader.py:33-43)."""

    def __init__(self, dir):
        self.dir = dir

    def __getitem__(self, x):
        return flexload(self.dir + x + ".npy")

    def __contains__(self, x):
        return os.path.exists(self.dir + x + ".npy") or os.path.exists(self.dir + x + ".npz")

    def __str__(self):
        return "load_dictionary class instance, using " + str(self.dir)


def write_arrays(dirname: str, arrays: dict) -> None:
    """Write an ``Arrays`` directory: ``xi`` and ``Ixi`` compressed, the rest
    as ``.npy`` (the layout ``write_to_file_compressed`` produces)."""
    os.makedirs(dirname, exist_ok=True)
    for k, v in arrays.items():
        if k in ("xi", "Ixi"):
            np.savez_compressed(os.path.join(dirname, k), v)
        else:
            np.save(os.path.join(dirname, k), v)


REQUIRED_KEYS = ("H_Ortho", "DM_Ortho", "psi_shape", "Xpp", "Xpm", "GG_P", "GL_P",
                 "diff_GGP_GLP", "diff_GGM_GLM", "xi", "Ixi", "zero_tol")


def read_arrays(D, keys=REQUIRED_KEYS) -> dict:
    """Materialise the keys ``zand`` reads from an ``Arrs`` mapping."""
    return {k: np.asarray(D[k]) for k in keys}
