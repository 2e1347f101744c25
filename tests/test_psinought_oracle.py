"""The steady-state oracle (psinought restated in NumPy) against the
unmodified reference psinought's output (``tests/golden/psi0_*.npz``): psi and
Omega to 1e-9 relative (the reference's Krylov tolerance is 1e-12 relative to
the right-hand side), and the psi derivative the reference checks vanishes."""
import os

import numpy as np
import pytest

from conftest import golden_callbacks, load_golden


@pytest.mark.parametrize("case", ["mini2", "mini3", "c1"])
def test_steady_state_oracle_matches_reference(case):
    from oracle.psinought_np import SteadyState
    z = load_golden(case)
    ref = np.load(os.path.join(os.path.dirname(__file__), "golden", "psi0_%s.npz" % case))
    p = z["params"]
    bias, dH = golden_callbacks(p)
    H = z["H_Ortho"] + dH(p["t0"], z["DM_Ortho"])
    na = int(z["psi_shape"][1])
    ss = SteadyState(z, p["hbar"], H, [bias(p["t0"], a) for a in range(na)])
    psi, omg = ss.solve()
    P, O = ref["PSI"][0], ref["OMG"][0]
    nt = psi.shape[2]
    assert np.abs(psi - P[:, :, :nt]).max() <= 1e-9 * np.abs(P).max()
    assert np.abs(omg - O[:, :, :nt, :, :, :nt]).max() <= 1e-9 * np.abs(O).max()
    assert np.abs(ss.dpsi(psi, omg)).max() <= 1e-12 * np.abs(ss.rhs()).max()
