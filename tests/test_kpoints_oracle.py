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


def test_kpoint_arrays_slices_dict_and_lazy_mapping(tmp_path):
    """kpoint_arrays gives the NK = 1 Arrays of one k-point, from a dict or a
    lazy ``load_dictionary`` mapping; k-point 0 of the two-k-point workload is
    the one-k-point workload."""
    from zandpack_gb300.arrays_io import load_dictionary, write_arrays
    from zandpack_gb300.engine import kpoint_arrays
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.workloads import make_kpoint_workload, make_workload
    w2, w1 = make_kpoint_workload("mini2"), make_workload("mini2")
    write_arrays(str(tmp_path / "A"), w2.arrays)
    lazy = load_dictionary(str(tmp_path / "A") + "/")
    for src in (w2.arrays, lazy):
        a0 = kpoint_arrays(src, 0)
        for key in ("H_Ortho", "DM_Ortho", "xi", "GL_P"):
            np.testing.assert_array_equal(np.asarray(a0[key]), np.asarray(w1.arrays[key]))
        assert int(a0["psi_shape"][0]) == 1
        L1 = CompactLayout(kpoint_arrays(src, 1), w2.hbar)
        assert L1.N == CompactLayout(w1.arrays, w1.hbar).N
