"""Several k-points: the oracle against the unmodified reference ``zand`` run
on ``mini2`` with two k-points (fixture ``k2_mini2``): per-stage derivatives
of every k-point at 1e-12 relative, and the adaptive run (the error norm sums
over the k-points, so they share one step sequence) with the time grid, the
final sigma of each k-point and the per-k-point lead currents."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_callbacks, load_golden
from oracle import zand_np as zo
from test_oracle_golden import _stage_ks


@pytest.fixture(scope="module")
def k2():
    if not os.path.exists(os.path.join(GOLDEN, "k2_mini2.npz")):
        pytest.skip("fixture k2_mini2 missing")
    return load_golden("k2_mini2")


def test_kpoint_stage_derivatives_match_reference(k2):
    z = k2
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    assert prob.NK == 2
    for a in p["keep"]:
        got = _stage_ks(prob, z, a, bias, dH)
        for g, name in zip(got, ("ksig", "kpsi", "komg")):
            ref = z["%s_%d" % (name, a)]
            assert np.abs(g - ref).max() / np.abs(ref).max() < 1e-12, (a, name)


def test_kpoint_trajectory_matches_reference(k2):
    z = k2
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    out = zo.propagate(prob, p["t0"], p["t1"], p["stepsize"], p["eps"], bias, dH,
                       state=(z["DM_Ortho"], None, None))
    TE = np.array(out["TE_hist"])
    assert len(TE) == len(z["TE_hist"])
    np.testing.assert_allclose(TE, z["TE_hist"], rtol=1e-7)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-10)
    assert np.abs(out["sig"][-1] - z["sig_final"]).max() < 1e-11
    J = np.array(out["currents"])          # (steps, NK, NL)
    assert np.abs(J.transpose(2, 0, 1) - z["currents"]).max() < 1e-10
