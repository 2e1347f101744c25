"""Host side of the non-orthogonal basis (``nozand``): the transformed
constants handed to the device agree with the oracle's, and the compact
layout built on them keeps the coupling-orbital supports of the orthogonal
case (the round-off residues of S^1/2 xi are cleaned to the tolerance
supports)."""
import numpy as np

from oracle import nozand_np as nz
from zandpack_gb300.layout import CompactLayout
from zandpack_gb300.nonorth import NonorthBasis


def test_transformed_constants_match_oracle(golden_nz):
    case, z = golden_nz
    p = z["params"]
    b = NonorthBasis(z)
    prob = nz.NonorthProblem(z, p["hbar"])
    assert not b.orthogonal
    np.testing.assert_array_equal(b.H0, prob.H0)
    np.testing.assert_allclose(b.Sm1, prob.Sm1, rtol=0, atol=0)
    np.testing.assert_allclose(b.sigma(z["DM_Ortho"]), prob.sig0, rtol=0, atol=0)
    L = CompactLayout(b.arrays, p["hbar"])
    C0 = b.constant_term(L)
    a, x, c = L.modes[:, 0], L.modes[:, 1], L.modes[:, 2]
    ref = (prob.GLP[0][a, x, c][:, None] * prob.xi[0][a, x, c]) @ prob.Sm1[0].T
    np.testing.assert_allclose(C0, ref, rtol=0, atol=1e-14 * np.abs(ref).max())


def test_layout_supports_survive_the_transform(golden_nz):
    from conftest import load_golden
    case, z = golden_nz
    p = z["params"]
    zo = load_golden(case[3:])  # the same case in the orthogonal basis
    Lo = CompactLayout(zo, zo["params"]["hbar"])
    Ln = CompactLayout(NonorthBasis(z).arrays, p["hbar"])
    assert (Ln.N, Ln.Ns, Ln.nc) == (Lo.N, Lo.Ns, Lo.nc)
    np.testing.assert_array_equal(Ln.lead_cols, Lo.lead_cols)
