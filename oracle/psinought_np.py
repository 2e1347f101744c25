"""ORACLE -- test infrastructure only.

A CPU restatement, in NumPy, of the reference's steady-state tool
``Zandpack/cmdtools/psinought``: the stationary psi of the AME equations at a
fixed density matrix, with Omega eliminated, and the Omega that goes with it.
Padded reference layout, one k-point.

Only ``tests/`` use this module, as the checker.  It is pinned against the
unmodified reference run in-process (``tests/golden/make_psinought_golden.py``).

The reference solves ``A psi = b`` with a preconditioned Krylov method
(scipy ``cgs``, ``:133-150,421-425``); the solution is the same whatever method
converges, so this restatement builds the (small) real matrix of ``A`` and
solves it directly.
"""
from __future__ import annotations

import numpy as np

from .zand_np import find_max_orbital_idx_per_lead


class SteadyState:
    """Operator, right-hand side and Omega reconstruction of psinought.

    ``H`` is ``H_Ortho + dH(t0, DM0)`` (psinought:115), ``bias_a`` the lead
    biases at t0, added to Xpp and Xpm of each lead (:137-141)."""

    def __init__(self, arrays, hbar, H, bias_a):
        D = arrays
        self.hbar = float(hbar)
        self.dm0 = np.asarray(D["DM_Ortho"], np.complex128)[0]
        self.h0 = np.asarray(H, np.complex128).reshape(self.dm0.shape)
        noT = int(max(find_max_orbital_idx_per_lead(D["GG_P"], D["GL_P"], D["zero_tol"])))  # :119-124
        sl = (0, slice(None), slice(None), slice(0, noT))
        self.xi = np.asarray(D["xi"])[sl]          # (na, nx, noT, no)
        self.ixi = np.asarray(D["Ixi"])[sl]
        self.glp = np.asarray(D["GL_P"])[sl]
        self.dP = np.asarray(D["GG_P"])[sl] - self.glp                 # deltaP (:193)
        self.dM = np.asarray(D["GG_M"])[sl] - np.asarray(D["GL_M"])[sl]  # deltaM (:191)
        self.xpp = np.array(np.asarray(D["Xpp"])[sl], np.complex128)
        self.xpm = np.array(np.asarray(D["Xpm"])[sl], np.complex128)
        for a, v in enumerate(bias_a):
            self.xpp[a] += v
            self.xpm[a] += v
        self.na, self.nx, self.noT, self.no = self.xi.shape
        self.C = self.na * self.nx * self.noT

    def _flat(self, arr):
        return arr.reshape(self.C, *arr.shape[3:])

    def apply(self, psi):
        """``Av3`` (psinought:198-226), vectorised over the modes: for every
        mode (a,x,c),
            (xpp_ax0 - h0) psi_axc
            + sum_{a'x'c'} xi_{a'x'c'} FRAC (dM_{a'x'c'} (ixi_{a'x'c'} . psi_axc)
                                             + dP_axc (conj psi_{a'x'c'} . xi_axc))
        with FRAC = i / (xpm_{a'x'c'} - xpp_ax0)."""
        P = self._flat(np.asarray(psi).reshape(self.na, self.nx, self.noT, self.no))
        xi, ixi = self._flat(self.xi), self._flat(self.ixi)
        xpp0 = np.broadcast_to(self.xpp[:, :, :1], self.xpp.shape).reshape(self.C)  # X_ax0 (:208)
        xpm = self._flat(self.xpm)
        frac = 1j / (xpm[None, :] - xpp0[:, None])                                # (:209)
        src = (P @ ixi.T) * self._flat(self.dM)[None, :] + self._flat(self.dP)[:, None] * (xi @ P.conj().T)
        out = P * xpp0[:, None] - P @ self.h0.T + (frac * src) @ xi
        return out.reshape(self.na, self.nx, self.noT, self.no)

    def rhs(self):
        """``B3`` (psinought:228-237): hbar glp xi + hbar dP dm0 xi."""
        xi = self.xi
        return self.hbar * (self.glp[..., None] * xi + self.dP[..., None] * np.einsum("ij,axcj->axci", self.dm0, xi))

    def omega(self, psi):
        """Omega of the stationary psi (psinought:443-451)."""
        P = self._flat(np.asarray(psi).reshape(self.na, self.nx, self.noT, self.no))
        xi, ixi = self._flat(self.xi), self._flat(self.ixi)
        xpp = self._flat(self.xpp)
        xpm = self._flat(self.xpm)
        src = (P @ ixi.T) * self._flat(self.dM)[None, :] + self._flat(self.dP)[:, None] * (xi @ P.conj().T)
        om = -src * (1j * self.hbar) / (xpm[None, :] - xpp[:, None])
        return om.reshape(self.na, self.nx, self.noT, self.na, self.nx, self.noT)

    def dpsi(self, psi, omg):
        """The psi derivative psinought checks (:456-462): zero at the steady state."""
        P = np.asarray(psi).reshape(self.na, self.nx, self.noT, self.no)
        xi = self._flat(self.xi)
        out = (np.einsum("ij,axcj->axci", self.h0, P) - self.xpp[..., None] * P + self.rhs()
               + (omg.reshape(self.C, self.C) @ xi).reshape(P.shape) / self.hbar)
        return out

    def solve(self):
        """Direct solve of the real-linear system (real and imaginary parts)."""
        n = self.C * self.no
        Amat = np.zeros((2 * n, 2 * n))
        e = np.zeros(n, np.complex128)
        for k in range(2 * n):
            e[:] = 0
            e[k % n] = 1.0 if k < n else 1j
            col = self.apply(e).ravel()
            Amat[:n, k] = col.real
            Amat[n:, k] = col.imag
        b = self.rhs().ravel()
        x = np.linalg.solve(Amat, np.concatenate([b.real, b.imag]))
        psi = (x[:n] + 1j * x[n:]).reshape(self.na, self.nx, self.noT, self.no)
        return psi, self.omega(psi)
