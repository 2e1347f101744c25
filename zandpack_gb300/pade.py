"""Pade spectrum decomposition (PSD) of the Fermi function.

Restates the published [N-1/N] scheme of J. Hu, R.-X. Xu and Y. J. Yan,
J. Chem. Phys. 133, 101106 (2010) and 134, 244106 (2011), the method the
reference selects with ``pole_mode='JieHu2011'`` (Zandpack/PadeDecomp.py:136-152,
Zandpack/TimedependentTransport.py:72-83).

With x = beta (E - mu) the expansion reads

    f(x) = 1/(1+e^x) ~= 1/2 - sum_j eta_j [ 1/(x - i xi_j) + 1/(x + i xi_j) ]

The poles xi_j are 2/lambda_j for the positive eigenvalues lambda_j of the
2N x 2N symmetric tridiagonal matrix with off-diagonal entries
1/sqrt(b_m b_{m+1}), b_m = 2m - 1.  The zeros zeta_k of the numerator come from
the same matrix with its first row and column removed.  The residues are

    eta_j = (N b_{N+1} / 2) prod_k (zeta_k^2 - xi_j^2) / prod_{k != j} (xi_k^2 - xi_j^2).

This module is input preparation for synthetic workloads (it builds the
``Arrays`` a ``zand`` run reads); it is not on the propagation path.
"""
from __future__ import annotations

import numpy as np


def _b(m):
    return 2.0 * m - 1.0


def _tridiag_positive_eigs(M: int, drop_first: bool) -> np.ndarray:
    idx = np.arange(1, M + 1, dtype=np.float64)
    off = 1.0 / np.sqrt(_b(idx[:-1]) * _b(idx[1:]))
    T = np.diag(off, 1) + np.diag(off, -1)
    if drop_first:
        T = T[1:, 1:]
    e = np.linalg.eigvalsh(T)
    return np.sort(e[e > 1e-15])[::-1]


def psd_poles(N: int):
    """Return (z, eta): z = 1j*xi_j (upper-half-plane poles in units of kT, as
    ``Hu_poles`` returns them, sorted by increasing |xi|) and real residues eta_j."""
    if N < 1:
        raise ValueError("need at least one pole")
    xi = 2.0 / _tridiag_positive_eigs(2 * N, drop_first=False)
    zeta = 2.0 / _tridiag_positive_eigs(2 * N, drop_first=True)
    const = N * _b(N + 1) / 2.0
    eta = np.empty(N)
    # products evaluated as sums of logs with sign tracking (N up to ~60)
    for j in range(N):
        num = zeta ** 2 - xi[j] ** 2
        den = np.delete(xi, j) ** 2 - xi[j] ** 2
        sign = np.prod(np.sign(num)) * np.prod(np.sign(den))
        logmag = np.sum(np.log(np.abs(num))) - np.sum(np.log(np.abs(den)))
        eta[j] = const * sign * np.exp(logmag)
    return 1j * xi, eta


def fermi_expanded(E, z, eta, beta, mu=0.0):
    """Pade-expanded Fermi function at (possibly complex) energies E; same form as
    ``FD_expanded`` (Zandpack/PadeDecomp.py:36-42)."""
    E = np.atleast_1d(np.asarray(E, dtype=np.complex128))
    xp = mu + z / beta
    xm = mu - z / beta
    d = (1.0 / beta) * (1.0 / np.subtract.outer(E, xp) + 1.0 / np.subtract.outer(E, xm)) * eta
    return 0.5 - d.sum(axis=1)
