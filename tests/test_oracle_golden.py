"""Pin the oracle against fixtures made by running the unmodified reference.

Per-stage derivatives of the recorded attempts must agree to 1e-12 relative
(max-norm over each array), and a full adaptive run must reproduce the
reference's attempt count, accept/reject sequence, time grid, final sigma and
lead currents.
"""
import numpy as np

from conftest import golden_callbacks
from oracle import zand_np as zo


def _stage_ks(prob, z, a, bias, dH):
    ys, yp, yo = z["y_sig_%d" % a], z["y_psi_%d" % a], z["y_omg_%d" % a]
    h = float(z["h_%d" % a])
    t = float(z["t_attempt"][a])
    SIGS = np.zeros((8,) + ys.shape, complex)
    PSIS = np.zeros((8,) + yp.shape, complex)
    OMGS = np.zeros((8,) + yo.shape, complex)
    SIGS[-1], PSIS[-1], OMGS[-1] = ys, yp, yo
    for i in range(7):
        if i == 0:
            s, ps, om = ys, yp, yo
        else:
            ix = zo.idxholder[i]
            s, ps, om = (zo.stage_combine(Y, zo.B[i], ix) for Y in (SIGS, PSIS, OMGS))
        ts = t + zo.A[i] * h
        ks, kp, ko, _, _ = prob.rhs(h, s, ps, om, prob.H0 + dH(ts, s), [bias(ts, l) for l in range(prob.NL)])
        SIGS[i], PSIS[i], OMGS[i] = ks, kp, ko
    return SIGS[:7], PSIS[:7], OMGS[:7]


def test_stage_derivatives_match_reference(golden):
    case, z = golden
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    for a in p["keep"]:
        got = _stage_ks(prob, z, a, bias, dH)
        for g, name in zip(got, ("ksig", "kpsi", "komg")):
            ref = z["%s_%d" % (name, a)]
            scale = max(np.abs(ref).max(), 1e-300)
            assert np.abs(g - ref).max() / scale < 1e-12, (case, a, name)


def test_trajectory_matches_reference(golden):
    case, z = golden
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    out = zo.propagate(prob, p["t0"], p["t1"], p["stepsize"], p["eps"], bias, dH,
                       state=(z["DM_Ortho"], None, None))
    TE = np.array(out["TE_hist"])
    assert len(TE) == len(z["TE_hist"])
    assert ((TE < p["eps"]) == (z["TE_hist"] < p["eps"])).all()
    np.testing.assert_allclose(TE, z["TE_hist"], rtol=1e-7)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-10)
    assert np.abs(out["sig"][-1] - z["sig_final"]).max() < 1e-11
    J = np.array(out["currents"])[:, 0, :].T
    assert np.abs(J - z["currents"]).max() < 1e-10


def test_tableau_identities():
    """Row sums of B equal A (the check at Zandpack/mpi_RK4pars_dev.py:203-205),
    CH carries the stored y with weight 1, and CT = b5 - b4 sums to zero."""
    for i in range(1, zo.RK_N):
        ix = zo.idxholder[i]
        assert abs(zo.B[i, ix[:-1]].sum() - zo.A[i]) < 1e-14
        assert zo.B[i, 7] == 1.0
    assert abs(zo.CT.sum()) < 1e-15
    assert zo.CH[-1] == 1.0 and abs(zo.CH[:-1].sum() - 1) < 1e-15
    # DOP54's last stage row equals b5 (first-same-as-last)
    assert np.allclose(zo.B[6, :6], zo.CH[:6]) and zo.CH[6] == 0.0


def test_c1_full_span_prefix():
    """The n=20 chain over 0-50 fs (``c1_50fs``: 5414 attempts of the
    unmodified ``zand``): the oracle reproduces the first 300 attempts' error
    norms and accept decisions and the stage derivatives of attempt 0 (the
    whole span runs on the GPU in ``tests/test_gpu_parity.py``)."""
    import os
    import pytest
    from conftest import GOLDEN, load_golden
    if not os.path.exists(os.path.join(GOLDEN, "c1_50fs.npz")):
        pytest.skip("fixture c1_50fs missing")
    z = load_golden("c1_50fs")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    got = _stage_ks(prob, z, 0, bias, dH)
    for g, name in zip(got, ("ksig", "kpsi", "komg")):
        ref = z["%s_0" % name]
        assert np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300) < 1e-12
    out = zo.propagate(prob, p["t0"], p["t1"], p["stepsize"], p["eps"], bias, dH,
                       state=(z["DM_Ortho"], None, None), max_attempts=300)
    TE = np.array(out["TE_hist"])
    assert len(TE) == 300
    assert ((TE < p["eps"]) == (z["TE_hist"][:300] < p["eps"])).all()
    np.testing.assert_allclose(TE, z["TE_hist"][:300], rtol=1e-7)
    k = len(out["times"])
    np.testing.assert_allclose(out["times"], z["times"][:k], rtol=0, atol=1e-9)
