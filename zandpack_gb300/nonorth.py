"""The non-orthogonal-basis propagation of the reference's ``nozand``
(Zandpack/mpi/nozand).

``nozand`` propagates sigma' = S^-1/2 sigma S^-1/2 and psi' (rows
S^-1/2 psi) with the overlap S entering through S^-1; Omega is the same.  The
``Arrays`` hold the Loewdin-orthogonal quantities plus ``S^(-0.5)``; nozand
maps them to the non-orthogonal basis once (:259-320, :376, :698-812):

* S^1/2 = inv(S^-1/2), S^-1 = (S^-1/2)^2;
* H0' = S^1/2 H_Ortho S^1/2, entries below 1e-13 set to zero, replaced by its
  Hermitian part when the non-Hermitian part is below 1e-6;
* xi' rows = S^1/2 xi (``transform_vec_Tv``), Ixi' rows = Ixi S^1/2
  (``transform_vec_vT``);
* the initial sigma' = S^-1/2 DM_Ortho S^-1/2 (:306), and a psi loaded from a
  full save, rows S^-1/2 psi (:722).

``NonorthBasis`` does the same on the host and gives the device what
``zg_set_overlap`` takes: S^-1 and the constant psi term S^-1 (GL_P xi') of
every compact mode (nozand's ``dPsi_const``, :1002-1003, from the full xi').

The compact layout needs exact supports.  After the transformation, xi' and
Ixi' carry round-off residues (|v| ~ 1e-17) outside the coupling orbitals;
the reference drops everything at most ``dot_prod_zero_tol`` from the
supports it uses (``orbidx_*``, :917-931, :378-386), so the transformed rows of
lead a are cleaned to the lead's tolerance supports (xi' to ``S_xi[a]``, Ixi'
to ``S_alpha[a]``).  The one term where the reference keeps such entries is
the Omega xi term (xi' on the Ixi support of all leads); there they contribute
at the level of the residues themselves.
"""
from __future__ import annotations

import numpy as np

from .layout import CompactLayout
from .layout import _noT_lead as _layout_noT

__all__ = ["NonorthBasis"]


class NonorthBasis:
    def __init__(self, arrays, dot_prod_zero_tol=1e-10):
        Sm05 = np.asarray(arrays["S^(-0.5)"], np.complex128)
        if Sm05.ndim != 3 or Sm05.shape[0] != 1:
            raise ValueError("S^(-0.5) must have shape (1, NO, NO)")
        self.Sm05 = Sm05
        self.S05 = np.linalg.inv(Sm05)
        self.Sm1 = Sm05 @ Sm05
        n = Sm05.shape[-1]
        self.orthogonal = bool(np.abs(self.S05 @ self.S05 - np.eye(n)).max() < 1e-10)
        H0 = self.S05 @ np.asarray(arrays["H_Ortho"], np.complex128) @ self.S05
        H0[np.abs(H0) < 1e-13] = 0.0
        if np.abs(H0 - H0.transpose(0, 2, 1).conj()).max() < 1e-6:
            H0 = 0.5 * (H0 + H0.conj().transpose(0, 2, 1))
        self.H0 = H0
        S05 = self.S05[0]
        xi_full = np.asarray(arrays["xi"], np.complex128) @ S05.T
        ixi_full = np.asarray(arrays["Ixi"], np.complex128) @ S05
        self.xi_full = xi_full
        tol = float(dot_prod_zero_tol)
        NL = int(arrays["psi_shape"][1])
        xi_c = np.zeros_like(xi_full)
        ixi_c = np.zeros_like(ixi_full)
        # tolerance supports per lead, on the rows the reference computes (c < noT_a)
        noT_lead = _noT_lead(arrays)
        NOT = int(noT_lead.max())
        for a in range(NL):
            nt = noT_lead[a]
            s_xi = (np.abs(xi_full[0, a, :, :nt]) > tol).any(axis=(0, 1))
            s_al = (np.abs(ixi_full[0, a, :, :NOT]) > tol).any(axis=(0, 1))
            xi_c[0, a][..., s_xi] = xi_full[0, a][..., s_xi]
            ixi_c[0, a][..., s_al] = ixi_full[0, a][..., s_al]
        A = dict(arrays)
        A["H_Ortho"] = H0
        A["xi"] = xi_c
        A["Ixi"] = ixi_c
        self.arrays = A

    def sigma(self, dm_ortho):
        """sigma' of an orthogonal-basis density matrix (nozand:306)."""
        return self.Sm05 @ np.asarray(dm_ortho, np.complex128).reshape(self.Sm05.shape) @ self.Sm05

    def psi(self, psi_ortho):
        """psi' rows S^-1/2 psi of an orthogonal-basis psi (nozand:722)."""
        return np.asarray(psi_ortho, np.complex128) @ self.Sm05[0].T

    def constant_term(self, layout: CompactLayout):
        """C0[m] = S^-1 (GL_P[m] xi'[m]) for the compact modes m (N x n)."""
        a, x, c = layout.modes[:, 0], layout.modes[:, 1], layout.modes[:, 2]
        rows = layout.GLP[:, None] * self.xi_full[0, a, x, c]
        return np.ascontiguousarray(rows @ self.Sm1[0].T)


def _noT_lead(arrays):
    return _layout_noT(np.asarray(arrays["GG_P"]), np.asarray(arrays["GL_P"]), np.asarray(arrays["zero_tol"]))
