"""Golden outputs of the reference's ``_save`` readers
(Zandpack/mpi_tools.py:19-144) on synthetic save directories.

``build_save_dirs(root)`` writes, from a fixed seed, four directories in the
layouts the drivers produce: a plain run (``DM``/``DMt``/``times``/
``current_*``/``PIa`` every 3 steps), a ``compress_mat``+``dm_triu_only`` run
(``.npz`` archives, upper triangles), and two that hold only a
``LossyDensityMatrix`` archive (plain and ``.xz``).  ``main`` runs the
reference readers on them (numba stubbed, see ``refharness``) and stores what
they return in ``tests/golden/save_readers.npz``; the tests rebuild the same
directories and compare.

    python tests/golden/make_save_golden.py
"""
from __future__ import annotations

import io
import lzma
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

N_ORB = 5
CHUNK = 3
N_CHUNKS = 3


def build_save_dirs(root):
    rng = np.random.default_rng(77)
    n = N_ORB
    dirs = {}
    for name, compress in (("plain", False), ("triu", True)):
        d = os.path.join(root, name + "_save")
        os.makedirs(d)
        t = 0.0
        for c in range(N_CHUNKS):
            step = (c + 1) * CHUNK
            k = CHUNK + (1 if c == 0 else 0)  # the first chunk holds the initial sigma too
            A = rng.standard_normal((k, 1, n, n)) + 1j * rng.standard_normal((k, 1, n, n))
            dm = ((A + A.conj().transpose(0, 1, 3, 2)) / 2).astype(np.complex64)
            tt = t + np.cumsum(rng.uniform(0.01, 0.02, k)) - (0.0 if c else 0.01)
            t = float(tt[-1])
            if compress:
                np.savez_compressed(os.path.join(d, "DM%d" % step), np.triu(dm))
            else:
                np.save(os.path.join(d, "DM%d" % step), dm)
            np.save(os.path.join(d, "DMt%d" % step), tt)
            np.save(os.path.join(d, "times%d" % step), tt)
            # currents and PI are recorded once per accepted step: CHUNK per file
            for lead in range(2):
                np.save(os.path.join(d, "current_%d_%d" % (lead, step)), rng.standard_normal((CHUNK, 1)))
            pi = (rng.standard_normal((CHUNK, 1, 2, n, n))
                  + 1j * rng.standard_normal((CHUNK, 1, 2, n, n))).astype(np.complex64)
            np.save(os.path.join(d, "PIa%d" % step), pi)
        np.save(os.path.join(d, "current_0.npy"), np.zeros(1))  # two-part name: skipped by the reader
        dirs[name] = d
    for name, xz in (("lossy", False), ("lossyxz", True)):
        d = os.path.join(root, name + "_save")
        os.makedirs(d)
        nt = 6
        dm = (rng.standard_normal((1, n, n, nt)) + 1j * rng.standard_normal((1, n, n, nt))).astype(np.complex64)
        tdm = np.linspace(0.0, 1.0, nt)
        buf = io.BytesIO()
        np.savez(buf, dm=dm, tdm=tdm)
        if xz:
            with lzma.open(os.path.join(d, "LossyDensityMatrix.npz.xz"), "wb") as f:
                f.write(buf.getvalue())
        else:
            with open(os.path.join(d, "LossyDensityMatrix.npz"), "wb") as f:
                f.write(buf.getvalue())
        dirs[name] = d
    return dirs


def reader_outputs(mt, dirs):
    """Outputs of the readers in module ``mt`` (reference or ours) on ``dirs``."""
    out = {}
    T, C = mt.combine_currents([dirs["plain"]])
    out["cc_T"], out["cc_J0"], out["cc_J1"] = T, C[0], C[1]
    T, C = mt.combine_currents([dirs["plain"], dirs["triu"]])
    out["cc2_T"], out["cc2_J0"] = T, C[0]
    r = mt.rectified_charge([dirs["plain"]])
    out["rq_t"], out["rq_q"] = r[0][0], r[0][1]
    out["dm_T"], out["dm"] = mt.combine_dm([dirs["plain"]])
    out["dmt_T"], out["dmt"] = mt.combine_dm([dirs["triu"]], insert_tril=True)
    out["dms_T"], out["dms"] = mt.combine_dm([dirs["plain"]], split=2, split_rank=1)
    out["dml_T"], out["dml"] = mt.combine_dm([dirs["lossy"]])
    out["dmx_T"], out["dmx"] = mt.combine_dm([dirs["lossyxz"]], insert_tril=True)
    out["pi_T"], out["pi"] = mt.combine_pi([dirs["plain"]])
    return out


def main():
    sys.path.insert(0, HERE)
    import refharness
    refharness._install_stubs()
    import importlib
    mt = importlib.import_module("Zandpack.mpi_tools")
    with tempfile.TemporaryDirectory() as root:
        out = reader_outputs(mt, build_save_dirs(root))
    path = os.path.join(HERE, "save_readers.npz")
    np.savez_compressed(path, **out)
    print("%d outputs -> %s (%.0f KB)" % (len(out), path, os.path.getsize(path) / 1024))


if __name__ == "__main__":
    main()
