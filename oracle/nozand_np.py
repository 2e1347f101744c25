"""ORACLE -- test infrastructure only.

A CPU restatement, in NumPy, of the reference's non-orthogonal-basis driver
``nozand`` (Zandpack/mpi/nozand): the same DOP54 propagation as ``zand`` but
of sigma' = S^-1/2 sigma S^-1/2 and psi' (rows S^-1/2 psi), with the overlap
S entering the right-hand side through S^-1.  Padded reference layout, one
k-point.

Only ``tests/`` use this module, as the checker.  It is pinned against
fixtures produced by running the unmodified reference ``nozand``
(``tests/golden/make_golden.py``, cases ``nz_*``).

Per stage, with H~ = S^-1 (H0' + dH(ts, sigma')) and P = sum_a psi'_a^T Ixi'_a:

* sigma: ``k = (h/hbar) [ -i (S^-1 H_t sigma' - h.c.) - hbar dis
  + (P S^-1 + h.c.)/hbar ]`` (nozand:456-500; ``PI_np`` there no longer adds
  the conjugate, :120-140);
* psi: ``k = -i h [ psi' H~^T/hbar - (X+ + Delta) psi'/hbar
  + S^-1 (GL_P xi') + dGP xi'_S sigma'_S^T + S^-1_(:,S) (Omega xi'_S/hbar^2) ]``
  (:1003, :1075-1214);
* Omega: as ``zand`` with the transformed xi', Ixi' (:1216-1290).

The transformed constants (:259-278, :376, :776-812): S^1/2 = inv(S^-1/2),
S^-1 = (S^-1/2)^2, ``H0' = S^1/2 H_Ortho S^1/2`` with entries below 1e-13 set
to zero and, when its non-Hermitian part is below 1e-6, replaced by its
Hermitian part; ``xi'`` rows ``S^1/2 xi`` (``transform_vec_Tv``), ``Ixi'`` rows
``Ixi S^1/2`` (``transform_vec_vT``).
"""
from __future__ import annotations

import numpy as np

from .zand_np import Problem


def lowdin_factors(Sm05):
    """(S^-1/2, S^1/2, S^-1, orthogonal) as nozand:259-267 derives them."""
    Sm05 = np.asarray(Sm05, np.complex128)
    S05 = np.linalg.inv(Sm05)
    Sm1 = Sm05 @ Sm05
    orthogonal = bool(np.abs(S05 @ S05 - np.eye(Sm1.shape[-1])).max() < 1e-10)
    return Sm05, S05, Sm1, orthogonal


def nonorth_h0(H_Ortho, S05):
    """H0' (nozand:269-278)."""
    H0 = S05 @ np.asarray(H_Ortho, np.complex128) @ S05
    H0[np.abs(H0) < 1e-13] = 0.0
    if np.abs(H0 - H0.transpose(0, 2, 1).conj()).max() < 1e-6:
        H0 = 0.5 * (H0 + H0.conj().transpose(0, 2, 1))
    return H0


class NonorthProblem(Problem):
    """Constants of one ``nozand`` propagation.  ``self.H0`` is H0' (what the
    caller adds dH(ts, sigma') to); ``self.sig0`` the initial sigma'."""

    def __init__(self, arrays, hbar, dot_prod_zero_tol=1e-10):
        Sm05, S05, Sm1, orth = lowdin_factors(arrays["S^(-0.5)"])
        D = dict(arrays)
        D["H_Ortho"] = nonorth_h0(arrays["H_Ortho"], S05)
        D["xi"] = np.asarray(arrays["xi"], np.complex128) @ S05[0].T
        D["Ixi"] = np.asarray(arrays["Ixi"], np.complex128) @ S05[0]
        super().__init__(D, hbar, dot_prod_zero_tol)
        self.Sm05, self.S05, self.Sm1, self.orthogonal = Sm05, S05, Sm1, orth
        self.sig0 = Sm05 @ np.asarray(arrays["DM_Ortho"], np.complex128) @ Sm05   # :306

    def rhs(self, h, sig, psi, omg, Ht, delta, diss=0.0):
        hbar = self.hbar
        NK, NL, NX, NOT, NO = self.NK, self.NL, self.NX, self.NOT, self.NO
        Sm1 = self.Sm1
        delta = np.asarray(delta, dtype=np.float64)
        # ---- sigma (:456-500)
        X = Ht @ sig
        if not self.orthogonal:
            X = Sm1 @ X
        Dm = (X - X.transpose(0, 2, 1).conj()) * (-1j) - hbar * np.asarray(diss)
        Q = np.zeros((NK, NO, NO), complex)
        J = np.zeros((NK, NL))
        for a in range(NL):
            S = self.S_alpha[a]
            pa = psi[:, a].reshape(NK, NX * NOT, NO)
            ia = self.Ixi[:, a][..., S].reshape(NK, NX * NOT, len(S))
            res = np.zeros((NK, NO, NO), complex)
            res[:, :, S] = np.matmul(pa.transpose(0, 2, 1), ia)
            res /= hbar
            Q += res
            J[:, a] = (np.trace(res, axis1=1, axis2=2) + np.trace(res.conj().transpose(0, 2, 1), axis1=1,
                                                                  axis2=2)).real / hbar   # :478-486
        Q = Q @ Sm1
        Q = Q + Q.transpose(0, 2, 1).conj()
        ksig = (Dm + Q) * (h / hbar)
        # ---- psi and Omega, one lead of rows at a time (:1075-1290)
        Ht_til = Sm1 @ Ht if not self.orthogonal else Ht
        kpsi = np.zeros_like(psi)
        komg = np.zeros_like(omg)
        psi_tilde = psi.conj()
        Xpm_d = self.Xpm + delta[None, :, None, None]
        SI = self.S_all
        xi_S = (self.xi[..., SI] / hbar ** 2).reshape(NK, NL * NX * NOT, len(SI))
        Sm1_sub = Sm1[:, :, SI]                                                  # :1031
        for a in range(NL):
            nt = self.noT_lead[a]
            tp = psi[:, a, :, :nt]
            to = omg[:, a, :, :nt]
            Xpp_d = self.Xpp[:, a, :, :nt] + delta[a]
            xa = self.xi[:, a, :, :nt]
            kp = np.matmul(tp.reshape(NK, NX * nt, NO), (Ht_til / hbar).transpose(0, 2, 1)).reshape(tp.shape)
            kp -= (Xpp_d / hbar)[..., None] * tp
            const = self.GLP[:, a, :, :nt, None] * xa                             # dPsi_const (:1002-1003)
            kp += np.matmul(const.reshape(NK, NX * nt, NO), Sm1.transpose(0, 2, 1)).reshape(tp.shape)
            Sx = self.S_xi[a]
            kp += self.dGP[:, a, :, :nt, None] * np.matmul(
                xa[..., Sx].reshape(NK, NX * nt, len(Sx)), sig[:, :, Sx].transpose(0, 2, 1)).reshape(tp.shape)
            r = np.matmul(to.reshape(NK, NX * nt, NL * NX * NOT), xi_S)          # :1199-1210
            kp += np.matmul(r, Sm1_sub.transpose(0, 2, 1)).reshape(tp.shape)
            kp *= -1j * h
            kpsi[:, a, :, :nt] = kp
            ko = np.zeros_like(to)
            rows = tp.reshape(NK, NX * nt, NO)
            for b in range(NL):
                Sb = self.S_alpha[b]
                rhs_b = (self.dGM[:, b, :, :, None] * self.Ixi[:, b])[..., Sb].reshape(NK, NX * NOT, len(Sb))
                ko[:, :, :, b] = np.matmul(h * rows[..., Sb], rhs_b.transpose(0, 2, 1)).reshape(NK, NX, nt, NX, NOT)
            lhs = (self.dGP[:, a, :, :nt, None] * xa)[..., Sx].reshape(NK, NX * nt, len(Sx))
            rt = (h * psi_tilde.reshape(NK, NL * NX * NOT, NO)[..., Sx]).transpose(0, 2, 1)
            ko += np.matmul(lhs, rt).reshape(ko.shape)
            s = 1j * h / hbar
            Ad = Xpp_d[..., 0] * s
            Bd = Xpm_d[..., 0] * s
            ko += (Ad[:, :, None, None, None, None] - Bd[:, None, None, :, :, None]) * to
            komg[:, a, :, :nt] = ko
        return ksig, kpsi, komg, None, J
