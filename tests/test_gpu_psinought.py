"""Steady state on the GPU (``zandpack_gb300.psinought``, the reference's
psinought) against the unmodified reference's output (``psi0_*.npz``): psi and
Omega to 1e-8 relative to their largest entries, and the state is a fixed point
of the device's own time-dependent right-hand side (k_psi and k_Omega vanish
to 1e-9 of the size of k_psi's source term)."""
import os

import numpy as np
import pytest

from conftest import golden_callbacks, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["mini2", "mini3", "c1"])
def test_steady_state_matches_reference(case):
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.psinought import steady_state
    z = load_golden(case)
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "psi0_%s.npz" % case))
    p = z["params"]
    bias, dH = golden_callbacks(p)
    res = steady_state(z, p["hbar"], bias, dH, t0=p["t0"], tol=1e-12)
    assert res.converged, (res.iterations, res.residual)
    P, O = ref["PSI"], ref["OMG"]
    nt = res.psi.shape[3]
    assert np.abs(res.psi - P[..., :nt, :]).max() <= 1e-8 * np.abs(P).max()
    assert np.abs(res.omg - O[:, :, :, :nt, :, :, :nt]).max() <= 1e-8 * np.abs(O).max()
    # fixed point of the time-dependent equations at sigma0 (k_sigma need not vanish)
    tr = Trajectory(z, p["hbar"])
    L = tr.layout
    tr.set_slot(tr.stages, L.pack(z["DM_Ortho"], res.psi, res.omg))
    dm0 = np.asarray(z["DM_Ortho"])
    dh = dH(p["t0"], dm0)
    tr.stage_input(0)
    mode = _lib.ZG_DH_NONE
    if not np.isscalar(dh):
        tr.set_dH(np.asarray(dh)[0])
        mode = _lib.ZG_DH_MATRIX
    tr.rhs(0, p["t0"], 1.0, [bias(p["t0"], a) for a in range(L.NL)], mode)
    _, kp, ko = L.unpack(tr.get_slot(0))
    tr.rhs(0, p["t0"], 1.0, [bias(p["t0"], a) for a in range(L.NL)], mode)  # same input: k of psi = 0 state
    tr.set_slot(tr.stages, L.pack(z["DM_Ortho"], 0 * res.psi, 0 * res.omg))
    tr.stage_input(0)
    tr.rhs(0, p["t0"], 1.0, [bias(p["t0"], a) for a in range(L.NL)], mode)
    _, kp0, _ = L.unpack(tr.get_slot(0))
    tr.close()
    scale = np.abs(kp0).max()
    assert np.abs(kp).max() <= 1e-9 * scale
    assert np.abs(ko).max() <= 1e-9 * scale


def test_psinought_command_line(tmp_path):
    """``python -m zandpack_gb300.psinought Dir=... file=...``: reads a run
    directory like the reference and writes ``<file>_save/last_psi.npy``,
    ``last_omg.npy`` (padded layout) and the MESSAGE files."""
    import json
    import sys
    from zandpack_gb300 import psinought
    from zandpack_gb300.arrays_io import write_arrays
    from zandpack_gb300.workloads import make_workload
    z = load_golden("mini2")
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "psi0_mini2.npz"))
    p = z["params"]
    keys = ("H_Ortho", "DM_Ortho", "psi_shape", "Xpp", "Xpm", "GG_P", "GL_P", "GG_M", "GL_M", "diff_GGP_GLP",
            "diff_GGM_GLM", "xi", "Ixi", "zero_tol")
    write_arrays(str(tmp_path / "SaveFile" / "Arrays"), {k: z[k] for k in keys})
    (tmp_path / "Initial.py").write_text("hbar=%r\nt0=%r\n" % (p["hbar"], p["t0"]))
    (tmp_path / "Bias.py").write_text(make_workload("mini2").bias_source())
    cwd = os.getcwd()
    try:
        for m in ("Initial", "Bias"):
            sys.modules.pop(m, None)
        res = psinought.main(["Dir=" + str(tmp_path), "file=SaveFile", "steptol=1e-12"])
    finally:
        os.chdir(cwd)
        sys.path[:] = [q for q in sys.path if os.path.realpath(q) != os.path.realpath(str(tmp_path))]
        for m in ("Initial", "Bias"):
            sys.modules.pop(m, None)
    assert res.converged
    P = np.load(tmp_path / "SaveFile_save" / "last_psi.npy")
    O = np.load(tmp_path / "SaveFile_save" / "last_omg.npy")
    nt = P.shape[3]
    assert np.abs(P - ref["PSI"][..., :nt, :]).max() <= 1e-8 * np.abs(ref["PSI"]).max()
    assert O.shape[3] == nt and np.abs(O).max() > 0
    assert (tmp_path / "psinought_dpsi_MESSAGE.txt").read_text() == "Success"
