"""Generate the steady-state fixtures by running the UNMODIFIED reference
``cmdtools/psinought`` in-process (see ``refharness.run_psinought``).

Usage (in a container that has the reference checkout):

    python tests/golden/make_psinought_golden.py [mini2 mini3 c1]

For each case this reads the input ``Arrays`` of ``tests/golden/<case>.npz``
(the bytes the reference ``zand`` runs consumed), writes them with the case's
``Initial.py``/``Bias.py``, runs psinought (Krylov tolerance ``steptol=1e-12``)
and stores its ``last_psi``/``last_omg`` (complex128, shapes
``(1, NL, NX, NOT, NO)`` and ``(1, NL, NX, NOT, NL, NX, NOT)``) in
``tests/golden/psi0_<case>.npz``.
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import refharness  # noqa: E402
from make_golden import initial_py  # noqa: E402
from zandpack_gb300.arrays_io import write_arrays  # noqa: E402
from zandpack_gb300.workloads import make_workload  # noqa: E402

ARRAY_KEYS = ("H_Ortho", "DM_Ortho", "psi_shape", "Xpp", "Xpm", "GG_P", "GL_P", "GG_M", "GL_M", "diff_GGP_GLP",
              "diff_GGM_GLM", "xi", "Ixi", "zero_tol", "num_leads", "num_poles_fermi", "num_lorentzians", "noT",
              "kT_i", "mu_i")


def make_case(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    arrays = {k: z[k] for k in ARRAY_KEYS if k in z.files}
    p = json.loads(str(z["params"]))
    w = make_workload(name)
    with tempfile.TemporaryDirectory(prefix="zpsi0_") as d:
        write_arrays(os.path.join(d, "SaveFile", "Arrays"), arrays)
        with open(os.path.join(d, "Initial.py"), "w") as f:
            f.write(initial_py(w, p["t1"], p["stepsize"]))
        with open(os.path.join(d, "Bias.py"), "w") as f:
            f.write(w.bias_source())
        psi, omg, log = refharness.run_psinought(d, "SaveFile", ["steptol=1e-12"])
    if "Converged psi" not in log:
        raise RuntimeError("reference psinought did not converge:\n" + log[-2000:])
    np.savez_compressed(os.path.join(HERE, "psi0_%s.npz" % name), PSI=psi.astype(np.complex128),
                        OMG=omg.astype(np.complex128))
    print(name, psi.shape, omg.shape, [l for l in log.splitlines() if "Converged" in l])


if __name__ == "__main__":
    for c in sys.argv[1:] or ["mini2", "mini3", "c1"]:
        make_case(c)
