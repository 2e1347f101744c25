"""Synthetic-input generation: Pade poles against the reference's ``Hu_poles``
(fixture from ``tests/golden/make_golden.py pade``) and the structure of the
generated ``Arrays``."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from zandpack_gb300.pade import psd_poles, fermi_expanded
from zandpack_gb300.workloads import make_workload


@pytest.mark.parametrize("N", [2, 3, 20, 30, 40])
def test_psd_poles_match_reference(N):
    z = np.load(os.path.join(GOLDEN, "hu_poles.npz"))
    zz, cc = psd_poles(N)
    np.testing.assert_allclose(zz, z["z_%d" % N], rtol=1e-12)
    np.testing.assert_allclose(cc, z["c_%d" % N], rtol=1e-9)


def test_fermi_expansion_accuracy():
    z, c = psd_poles(30)
    E = np.linspace(-0.5, 0.5, 101)
    beta = 1 / 0.025
    assert np.abs(fermi_expanded(E, z, c, beta) - 1 / (1 + np.exp(E * beta))).max() < 1e-10


@pytest.mark.parametrize("name,N,Npad", [("c1", 112, 112), ("c2", 2816, 3584), ("c3", 4480, 6400)])
def test_mode_counts(name, N, Npad):
    A = make_workload(name).arrays
    L, NX, NOT, n = (int(v) for v in A["psi_shape"][1:])
    assert L * NX * NOT == Npad
    live = (np.abs(A["GG_P"]) > 0) | (np.abs(A["GL_P"]) > 0)
    assert live.sum() == N
    # Fermi-pole modes carry no source: GG == GL exactly
    N_L = int(A["num_lorentzians"])
    assert (A["diff_GGP_GLP"][:, :, N_L:] == 0).all() and (A["diff_GGM_GLM"][:, :, N_L:] == 0).all()
    np.testing.assert_array_equal(A["Ixi"], A["xi"].conj())
