"""Compact mode layout of the AME state on the device.

The reference stores the auxiliary modes padded: psi is (NK, NL, NX, NOT, NO)
and Omega is (NK, NL, NX, NOT, NL, NX, NOT), where NOT is the largest eigen
count of any lead (``find_max_orbital_idx_per_lead``,
Zandpack/mpi_splitter.py:555-580; Zandpack/mpi/zand:122-123).  Workers compute
only rows c < noT_a of their lead (Zandpack/mpi/zand:520-533).

The device keeps only the modes whose rows can ever be nonzero, ordered

    [ sourced modes (dGP != 0 or dGM != 0), by lead | source-free modes, by lead ]

and Omega as two dense blocks,

    OmA = Omega[:, sourced]            (N x N_s)
    OmB = Omega[sourced, source-free]  (N_s x N_f)

because Omega[r, c] with both r and c source-free has no source term
(``dGM[c] = 0`` kills the psi.Ixi source, ``dGP[r] = 0`` the xi.conj(psi)
source; Zandpack/mpi/zand:784-809) and starts at zero, so it stays exactly zero;
``nozand`` skips the same block (Zandpack/mpi/nozand:820-823).  A mode is
dropped entirely ("dead") when it has no source at all (GL_P = dGP = dGM = 0)
and its initial psi row and Omega row and column are zero: its psi row and
Omega row then form a closed homogeneous system that stays zero.  Rank-padding
modes of every lead are dead in this sense.

All classifications use exact zeros; the tolerance-based supports the reference
applies (``orbidx_*`` with ``dot_prod_zero_tol``, Zandpack/mpi/zand:254-281,
589-602) are applied on top, so the compact state evolves by the same equations.

Orbital columns: each lead a couples through the set C_a (the exact support of
its live xi/Ixi rows), padded to a common width ``nc``.  The per-mode
coefficient rows are stored gathered on C_a:

* ``XI``   = xi[m, C_a]                        (GL_P xi and dGP xi sigma^T terms)
* ``IXI``  = Ixi[m, C_a] on S_alpha[a], else 0   (PI and the psi.Ixi source)
* ``XIS``  = xi[m, C_a] / hbar^2 on S_all, else 0 (the Omega xi term)
* ``XIT2`` = xi[m, C_a] on S_xi[a], else 0       (the xi.conj(psi) source)
"""
from __future__ import annotations

import numpy as np

__all__ = ["CompactLayout", "LayoutError"]


class LayoutError(ValueError):
    """Input the compact layout cannot represent exactly."""


def _noT_lead(GG_P, GL_P, zero_tol):
    live = (np.abs(GG_P).max(axis=0) >= zero_tol) | (np.abs(GL_P).max(axis=0) >= zero_tol)
    return np.array([np.where(live[a])[1].max() + 1 for a in range(live.shape[0])])


class CompactLayout:
    def __init__(self, arrays, hbar, dot_prod_zero_tol=1e-10, psi0=None, omg0=None):
        D = arrays
        H0 = np.asarray(D["H_Ortho"], dtype=np.complex128)
        if H0.ndim != 3 or H0.shape[1] != H0.shape[2]:
            raise LayoutError("H_Ortho must have shape (NK, NO, NO)")
        if H0.shape[0] != 1:
            raise LayoutError("a trajectory holds one k-point (NK = 1); engine.Propagator runs one per k-point")
        self.hbar = float(hbar)
        self.H0 = H0[0]
        self.n = n = H0.shape[-1]
        self.NL = NL = int(D["psi_shape"][1])
        self.NX = NX = int(D["psi_shape"][2])
        self.noT_lead = _noT_lead(np.asarray(D["GG_P"]), np.asarray(D["GL_P"]), np.asarray(D["zero_tol"]))
        self.NOT = NOT = int(self.noT_lead.max())
        sl = (0, slice(None), slice(None), slice(0, NOT))
        Xpp = np.asarray(D["Xpp"])[sl]
        Xpm = np.asarray(D["Xpm"])[sl]
        GLP = np.asarray(D["GL_P"])[sl]
        dGP = np.asarray(D["diff_GGP_GLP"])[sl]
        dGM = np.asarray(D["diff_GGM_GLM"])[sl]
        xi = np.asarray(D["xi"])[sl]
        Ixi = np.asarray(D["Ixi"])[sl]
        if xi.shape != (NL, NX, NOT, n) or Ixi.shape != (NL, NX, NOT, n):
            raise LayoutError("xi/Ixi must cover (NL, NX, >=NOT, NO)")
        tol = float(dot_prod_zero_tol)
        # reference asserts: X+ constant along c within noT, X- along all NOT (Zandpack/mpi/zand:578-581)
        for a in range(NL):
            if not np.allclose(Xpp[a, :, :self.noT_lead[a]], Xpp[a, :, :1]):
                raise LayoutError("Xpp must be constant along the eigen axis")
        if not np.allclose(Xpm, Xpm[:, :, :1]):
            raise LayoutError("Xpm must be constant along the eigen axis")
        S_alpha = [np.where((np.abs(Ixi[a]) > tol).any(axis=(0, 1)))[0] for a in range(NL)]
        S_all = np.where((np.abs(Ixi) > tol).any(axis=(0, 1, 2)))[0]
        S_xi = [np.where((np.abs(xi[a, :, :self.noT_lead[a]]) > tol).any(axis=(0, 1)))[0] for a in range(NL)]
        self.S_alpha, self.S_all, self.S_xi = S_alpha, S_all, S_xi

        psi0 = None if psi0 is None else np.asarray(psi0)[0]
        omg0 = None if omg0 is None else np.asarray(omg0)[0]
        # rows the reference never computes (c >= noT_a) must not be sourced as columns
        for a in range(NL):
            nt = self.noT_lead[a]
            if nt < NOT:
                src = np.abs(dGM[a, :, nt:, None] * Ixi[a, :, nt:][..., S_alpha[a]]).max(initial=0.0)
                if src > 0:
                    raise LayoutError("lead %d: diff_GGM_GLM * Ixi nonzero beyond noT; such Omega columns "
                                      "are not representable" % a)
                if omg0 is not None and np.abs(omg0[:, :, :, a, :, nt:]).max(initial=0.0) > 0:
                    raise LayoutError("initial Omega nonzero in columns beyond noT of lead %d" % a)
        sourced = (dGP != 0) | (dGM != 0)
        live = np.zeros((NL, NX, NOT), bool)
        for a in range(NL):
            nt = self.noT_lead[a]
            blk = sourced[a, :, :nt] | (GLP[a, :, :nt] != 0)
            if psi0 is not None:
                blk |= (psi0[a, :, :nt] != 0).any(axis=-1)
            if omg0 is not None:
                blk |= (omg0[a, :, :nt] != 0).any(axis=(-3, -2, -1))
                blk |= (omg0[:, :, :, a, :, :nt] != 0).any(axis=(0, 1, 2))
            live[a, :, :nt] = blk
        order = []
        for cls in (True, False):
            for a in range(NL):
                for x in range(NX):
                    for c in range(self.noT_lead[a]):
                        if live[a, x, c] and bool(sourced[a, x, c]) == cls:
                            order.append((a, x, c))
        self.modes = np.array(order, dtype=np.int64).reshape(-1, 3)
        self.N = N = len(order)
        self.Ns = Ns = int(sum(1 for (a, x, c) in order if sourced[a, x, c]))
        self.Nf = N - Ns
        if N == 0:
            raise LayoutError("no live auxiliary modes")
        ma, mx, mc = self.modes[:, 0], self.modes[:, 1], self.modes[:, 2]
        self.mode_lead = ma.astype(np.int32)
        # per-lead orbital column set: exact support of live xi/Ixi rows
        cols = []
        for a in range(NL):
            sel = ma == a
            sup = (xi[ma[sel], mx[sel], mc[sel]] != 0).any(axis=0) | (Ixi[ma[sel], mx[sel], mc[sel]] != 0).any(axis=0)
            cols.append(np.where(sup)[0])
        self.nc = nc = max(1, max(len(c) for c in cols))
        self.lead_cols = np.zeros((NL, nc), np.int32)
        self.lead_ncols = np.array([len(c) for c in cols], np.int32)
        self.colmap = -np.ones((NL, n), np.int32)  # orbital -> k within lead a, or -1
        for a in range(NL):
            self.lead_cols[a, :len(cols[a])] = cols[a]
            self.colmap[a, cols[a]] = np.arange(len(cols[a]))
        self.Xp = Xpp[ma, mx, 0].copy()
        self.Xm = Xpm[ma, mx, 0].copy()
        self.GLP = GLP[ma, mx, mc].copy()
        self.dGP = dGP[ma, mx, mc].copy()
        self.dGM = dGM[ma, mx, mc].copy()
        XI = np.zeros((N, nc), complex)
        IXI = np.zeros((N, nc), complex)
        XIS = np.zeros((N, nc), complex)
        XIT2 = np.zeros((N, nc), complex)
        hb2 = self.hbar ** 2
        sa_all = np.zeros(n, bool)
        sa_all[S_all] = True
        for a in range(NL):
            sel = np.where(ma == a)[0]
            cc = cols[a]
            k = len(cc)
            in_alpha = np.isin(cc, S_alpha[a])
            in_xi = np.isin(cc, S_xi[a])
            xr = xi[ma[sel], mx[sel], mc[sel]][:, cc]
            ir = Ixi[ma[sel], mx[sel], mc[sel]][:, cc]
            XI[sel, :k] = xr
            IXI[sel, :k] = np.where(in_alpha[None, :], ir, 0)
            XIS[sel, :k] = np.where(sa_all[cc][None, :], xr / hb2, 0)
            XIT2[sel, :k] = np.where(in_xi[None, :], xr, 0)
        self.XI, self.IXI, self.XIS, self.XIT2 = XI, IXI, XIS, XIT2
        # row ranges per (class, lead): sourced rows [s_start[a], s_start[a+1]), free rows likewise
        self.s_start = np.zeros(NL + 1, np.int64)
        self.f_start = np.zeros(NL + 1, np.int64)
        for a in range(NL):
            self.s_start[a + 1] = self.s_start[a] + int(((ma == a) & (np.arange(N) < Ns)).sum())
            self.f_start[a + 1] = self.f_start[a] + int(((ma == a) & (np.arange(N) >= Ns)).sum())
        self.f_start += Ns
        # flat state: [sigma n*n | psi N*n | OmA N*Ns | OmB Ns*Nf]
        self.off_sig = 0
        self.off_psi = n * n
        self.off_omA = self.off_psi + N * n
        self.off_omB = self.off_omA + N * Ns
        self.size = self.off_omB + Ns * self.Nf
        self.padded_modes = NL * NX * NOT
        if omg0 is not None:
            self._check_ff_zero(omg0)

    def _check_ff_zero(self, omg0):
        free = self.modes[self.Ns:]
        if len(free):
            a, x, c = free[:, 0], free[:, 1], free[:, 2]
            blk = omg0[a, x, c][:, a, x, c]
            if np.abs(blk).max() > 0:
                raise LayoutError("initial Omega has a nonzero block between source-free modes")

    # -------------------------------------------------------------- state maps
    def pack(self, sig, psi, omg, dtype=np.complex128):
        """Padded reference arrays (NK=1 leading axis optional) -> flat compact vector."""
        sig = np.asarray(sig).reshape(self.n, self.n)
        psi = np.asarray(psi).reshape(self.NL, self.NX, self.NOT, self.n)
        omg = np.asarray(omg).reshape(self.NL, self.NX, self.NOT, self.NL, self.NX, self.NOT)
        a, x, c = self.modes[:, 0], self.modes[:, 1], self.modes[:, 2]
        Ns = self.Ns
        y = np.empty(self.size, dtype)
        y[:self.off_psi] = sig.ravel()
        y[self.off_psi:self.off_omA] = psi[a, x, c].ravel()
        full = omg[a, x, c][:, a, x, c]
        y[self.off_omA:self.off_omB] = full[:, :Ns].ravel()
        y[self.off_omB:] = full[:Ns, Ns:].ravel()
        return y

    def unpack(self, y):
        """Flat compact vector -> padded (sig (1,n,n), psi (1,NL,NX,NOT,n),
        omg (1,NL,NX,NOT,NL,NX,NOT)); modes outside the layout are zero."""
        n, N, Ns = self.n, self.N, self.Ns
        y = np.asarray(y)
        sig = y[:self.off_psi].reshape(1, n, n).astype(np.complex128)
        psi = np.zeros((1, self.NL, self.NX, self.NOT, n), np.complex128)
        omg = np.zeros((1, self.NL, self.NX, self.NOT, self.NL, self.NX, self.NOT), np.complex128)
        a, x, c = self.modes[:, 0], self.modes[:, 1], self.modes[:, 2]
        psi[0, a, x, c] = y[self.off_psi:self.off_omA].reshape(N, n)
        full = np.zeros((N, N), np.complex128)
        full[:, :Ns] = y[self.off_omA:self.off_omB].reshape(N, Ns)
        full[:Ns, Ns:] = y[self.off_omB:].reshape(Ns, self.Nf)
        omg[0, a[:, None], x[:, None], c[:, None], a[None, :], x[None, :], c[None, :]] = full
        return sig, psi, omg

    def views(self, y):
        """(sig n x n, psi N x n, OmA N x Ns, OmB Ns x Nf) views of a flat vector."""
        n, N, Ns, Nf = self.n, self.N, self.Ns, self.Nf
        return (y[:self.off_psi].reshape(n, n), y[self.off_psi:self.off_omA].reshape(N, n),
                y[self.off_omA:self.off_omB].reshape(N, Ns), y[self.off_omB:].reshape(Ns, Nf))

    def summary(self):
        return dict(n=self.n, NL=self.NL, NX=self.NX, NOT=self.NOT, N=self.N, Ns=self.Ns, Nf=self.Nf,
                    nc=self.nc, padded_modes=self.padded_modes, state_complex=self.size)
