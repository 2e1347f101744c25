"""Pin the ``nozand`` oracle (non-orthogonal basis) against fixtures made by
running the unmodified reference ``nozand``: per-stage derivatives to 1e-12
relative, and a full adaptive run with the reference's attempt sequence, time
grid, final sigma' and lead currents."""
import numpy as np

from conftest import golden_callbacks
from oracle import nozand_np as nz
from oracle import zand_np as zo
from test_oracle_golden import _stage_ks


def test_nozand_stage_derivatives_match_reference(golden_nz):
    case, z = golden_nz
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = nz.NonorthProblem(z, p["hbar"])
    assert not prob.orthogonal
    for a in p["keep"]:
        got = _stage_ks(prob, z, a, bias, dH)
        for g, name in zip(got, ("ksig", "kpsi", "komg")):
            ref = z["%s_%d" % (name, a)]
            scale = max(np.abs(ref).max(), 1e-300)
            assert np.abs(g - ref).max() / scale < 1e-12, (case, a, name, np.abs(g - ref).max() / scale)


def test_nozand_trajectory_matches_reference(golden_nz):
    case, z = golden_nz
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = nz.NonorthProblem(z, p["hbar"])
    out = zo.propagate(prob, p["t0"], p["t1"], p["stepsize"], p["eps"], bias, dH,
                       state=(prob.sig0, None, None))
    TE = np.array(out["TE_hist"])
    assert len(TE) == len(z["TE_hist"])
    assert ((TE < p["eps"]) == (z["TE_hist"] < p["eps"])).all()
    np.testing.assert_allclose(TE, z["TE_hist"], rtol=1e-7)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-10)
    assert np.abs(out["sig"][-1] - z["sig_final"]).max() < 1e-11
    J = np.array(out["currents"])[:, 0, :].T
    assert np.abs(J - z["currents"]).max() < 1e-10


def test_nozand_is_a_similarity_transform_of_zand(golden_nz):
    """With S = 1 the non-orthogonal equations are zand's; in general the
    sigma' derivative is S^-1/2 (zand's sigma derivative in the orthogonal
    basis) S^-1/2 at the corresponding state."""
    case, z = golden_nz
    p = z["params"]
    prob = nz.NonorthProblem(z, p["hbar"])
    po = zo.Problem(z, p["hbar"])
    rng = np.random.default_rng(5)
    sig_o = z["DM_Ortho"]
    psi_o = np.zeros(po.zero_state()[1].shape, complex)
    for a in range(po.NL):
        nt = po.noT_lead[a]
        psi_o[:, a, :, :nt] = 1e-2 * (rng.standard_normal(psi_o[:, a, :, :nt].shape)
                                      + 1j * rng.standard_normal(psi_o[:, a, :, :nt].shape))
    omg = np.zeros(po.zero_state()[2].shape, complex)
    delta = [0.1 * (a + 1) for a in range(po.NL)]
    ks_o, kp_o, ko_o, _, _ = po.rhs(0.01, sig_o, psi_o, omg, po.H0, delta)
    Sm05 = prob.Sm05
    sig_n = Sm05 @ sig_o @ Sm05
    psi_n = psi_o @ Sm05[0].T
    ks_n, kp_n, ko_n, _, _ = prob.rhs(0.01, sig_n, psi_n, omg, prob.H0, delta)
    scale = np.abs(ks_n).max()
    assert np.abs(ks_n - Sm05 @ ks_o @ Sm05).max() / scale < 1e-10
    assert np.abs(kp_n - kp_o @ Sm05[0].T).max() / np.abs(kp_n).max() < 1e-10
    assert np.abs(ko_n - ko_o).max() / max(np.abs(ko_n).max(), 1e-300) < 1e-10
