"""The oracle's restatement of the in-process stepper ``AdaptiveDOP``
(``oracle.zand_np.adaptive_dop``) against fixtures of the unmodified
reference stepper (``tests/golden/make_inprocess_golden.py``): same accepted
steps and times, density matrices and lead currents to 1e-12."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_callbacks, load_golden


@pytest.mark.parametrize("case", ["mini2", "mini3"])
def test_adaptive_dop_oracle_matches_reference(case):
    from oracle import zand_np as zo
    path = os.path.join(GOLDEN, "inproc_%s.npz" % case)
    g = np.load(path)
    c = json.loads(str(g["params"]))
    z = load_golden(case)
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    sig0, psi0, omg0 = prob.zero_state()
    sig0 = sig0 + np.asarray(z["DM_Ortho"])
    out = zo.adaptive_dop(prob, sig0, psi0, omg0, c["eps"], c["t0"], c["t1"], dH, bias, h_guess=c["h_guess"])
    assert len(out["times"]) == len(g["times"])
    np.testing.assert_allclose(out["times"], g["times"], rtol=0, atol=1e-14)
    assert np.abs(out["dm"] - g["dm"]).max() < 1e-12
    for a in range(prob.NL):
        np.testing.assert_allclose(out["currents"][a], g["current_%d" % a], rtol=1e-12, atol=1e-15)
