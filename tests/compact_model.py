"""NumPy model of the device RHS in the compact layout (test helper).

It evaluates, term by term, the same contractions the CUDA kernels evaluate,
on the flat compact state of ``zandpack_gb300.layout.CompactLayout``.  Tests
compare it with the padded oracle on the CPU, which checks the layout and the
restated equations before any GPU run.
"""
import numpy as np


def rhs_compact(L, y, Ht, delta, h, diss=0.0):
    hb = L.hbar
    n, N, Ns, Nf, nc = L.n, L.N, L.Ns, L.Nf, L.nc
    sig, psi, omA, omB = L.views(y)
    delta = np.asarray(delta, float)
    lead = L.mode_lead
    # sigma: -i[H, sig] + (P + P^H)/hbar
    T = Ht @ sig
    Pc = np.zeros((L.NL, n, nc), complex)
    Pfull = np.zeros((n, n), complex)
    J = np.zeros(L.NL)
    for a in range(L.NL):
        rows = lead == a
        Pc[a] = psi[rows].T @ L.IXI[rows]
        k = L.lead_ncols[a]
        Pfull[:, L.lead_cols[a, :k]] += Pc[a][:, :k]
        J[a] = 2 * np.real(np.sum(Pc[a][L.lead_cols[a], np.arange(nc)])) / hb ** 2
    ksig = (h / hb) * (-1j * (T - T.conj().T) + (Pfull + Pfull.conj().T) / hb) - h * np.asarray(diss)
    # psi
    R1 = psi @ Ht.T
    sigC = np.stack([sig[:, L.lead_cols[a]] for a in range(L.NL)])           # (NL, n, nc)
    R2 = np.einsum("mk,mik->mi", L.XI, sigC[lead])
    Z = np.zeros((L.NL, N, nc), complex)
    for b in range(L.NL):
        sc = slice(L.s_start[b], L.s_start[b + 1])
        fc = slice(L.f_start[b], L.f_start[b + 1])
        Z[b] = omA[:, sc] @ L.XIS[sc]
        Z[b, :Ns] += omB[:, slice(fc.start - Ns, fc.stop - Ns)] @ L.XIS[fc]
    G = np.stack([psi[:, L.lead_cols[a]] for a in range(L.NL)], axis=1)    # (N, NL, nc)
    kpsi = R1 / hb - ((L.Xp + delta[lead]) / hb)[:, None] * psi + L.dGP[:, None] * R2
    for b in range(L.NL):
        cm = L.colmap[b]
        has = cm >= 0
        kpsi[:, has] += Z[b][:, cm[has]]
        rows = lead == b
        kpsi[np.ix_(rows, has)] += L.GLP[rows, None] * L.XI[rows][:, cm[has]]
    kpsi *= -1j * h
    # Omega
    s = 1j * h / hb
    Xpd = L.Xp + delta[lead]
    Xmd = L.Xm + delta[lead]
    U = L.dGM[:, None] * L.IXI          # per column mode
    V = L.dGP[:, None] * L.XIT2         # per row mode
    kA = h * np.einsum("mlk,lk->ml", G[:, lead[:Ns]], U[:Ns])
    kA += h * np.einsum("mk,lmk->ml", V, G[:Ns][:, lead].conj())
    kA += s * (Xpd[:, None] - Xmd[None, :Ns]) * omA
    kB = h * np.einsum("mk,fmk->mf", V[:Ns], G[Ns:][:, lead[:Ns]].conj())
    kB += s * (Xpd[:Ns, None] - Xmd[None, Ns:]) * omB
    k = np.empty_like(y)
    ks, kp, ka, kb = L.views(k)
    ks[...] = ksig
    kp[...] = kpsi
    ka[...] = kA
    kb[...] = kB
    return k, J
