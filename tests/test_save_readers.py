"""The ``_save`` readers (``zandpack_gb300.mpi_tools``) against the outputs
of the reference's own readers (Zandpack/mpi_tools.py:19-144) on the same
synthetic save directories (``tests/golden/make_save_golden.py``): plain
``.npy`` runs, ``compress_mat``/``dm_triu_only`` archives, lossy archives
(plain and ``.xz``), split reads and the rectified charge."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
from make_save_golden import build_save_dirs, reader_outputs  # noqa: E402


def test_readers_match_reference(tmp_path):
    path = os.path.join(GOLDEN, "save_readers.npz")
    if not os.path.exists(path):
        pytest.skip("fixture save_readers.npz missing")
    ref = np.load(path)
    from zandpack_gb300 import mpi_tools
    got = reader_outputs(mpi_tools, build_save_dirs(str(tmp_path)))
    assert set(got) == set(ref.files)
    for k in ref.files:
        np.testing.assert_array_equal(np.asarray(got[k]), ref[k], err_msg=k)


def test_herm_insert_tril_restores_triu_only_files():
    from zandpack_gb300.mpi_tools import herm_insert_tril
    rng = np.random.default_rng(3)
    A = rng.standard_normal((2, 1, 6, 6)) + 1j * rng.standard_normal((2, 1, 6, 6))
    H = (A + A.conj().transpose(0, 1, 3, 2)) / 2
    np.testing.assert_array_equal(herm_insert_tril(np.triu(H)), H)
