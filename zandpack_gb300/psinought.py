"""Steady state of the AME equations on the GPU (the reference's ``psinought``,
Zandpack/cmdtools/psinought:180-491).

At a fixed density matrix sigma0 (``DM_Ortho``) and the biases and dH at t0,
the stationary psi solves ``k_psi(sigma0, psi, Omega(psi)) = 0``, where
``Omega(psi)`` is the Omega of ``dOmega/dt = 0``
(``Omega = i hbar S(psi) / (X+ + Delta_a - X- - Delta_b)``, psinought:443-451).
The map is affine in psi and real-linear (the second Omega source is
conjugate-linear), so it is solved as a real linear system with restarted
GMRES (real inner products ``Re <u, v>`` on complex vectors), right-
preconditioned by the inverse of the dominant term of k_psi,
``r_m -> i hbar r_m (H^T - X+_m - Delta)^{-1}``, applied through the
eigenpairs of H.  The reference uses scipy's ``cgs`` with a block-Woodbury
preconditioner; the solution is the same.

Operator and preconditioner run in libzandgpu (``zg_stationary_*``, FP64);
the Krylov bookkeeping (a few vectors of N*n complex) uses torch tensors on the
same device.

    python -m zandpack_gb300.psinought Dir=<run dir> file=SaveFile [steptol=1e-8 maxiter=10000]

reads ``<file>/Arrays`` and ``Initial.py``/``Bias.py`` like the reference and
writes ``<file>_save/last_psi.npy`` and ``last_omg.npy`` (padded layout) plus
the ``psinought_dpsi_MESSAGE.txt``/``psinought_dsig_MESSAGE.txt`` verdicts.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
import sys
import time
from typing import Callable, Optional

import numpy as np

from . import _lib
from ._lib import check, lib
from .engine import Trajectory
from .layout import CompactLayout


@dataclasses.dataclass
class SteadyResult:
    psi: np.ndarray        # (1, NL, NX, NOT, NO) complex128
    omg: np.ndarray        # (1, NL, NX, NOT, NL, NX, NOT) complex128
    iterations: int
    residual: float        # ||k_psi|| / ||k_psi(psi = 0)|| at the solution
    converged: bool
    seconds: float


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def steady_state(arrays, hbar, bias: Callable, dH: Callable, t0: float = 0.0, tol: float = 1e-10,
                 maxiter: int = 2000, restart: int = 40, device: int = 0, layout: Optional[CompactLayout] = None,
                 x0: Optional[np.ndarray] = None) -> SteadyResult:
    """Solve for the stationary psi (and Omega) at sigma0 = ``arrays['DM_Ortho']``.

    ``bias(t, a)`` and ``dH(t, sigma)`` are the reference's callbacks; dH is
    evaluated once at (t0, sigma0) as psinought does (psinought:115).  ``tol``
    is the relative residual of the preconditioned GMRES."""
    import torch
    L = layout if layout is not None else CompactLayout(arrays, hbar)
    tr = Trajectory(arrays, hbar, precision="f64", device=device, layout=L)
    try:
        dm0 = np.asarray(arrays["DM_Ortho"], np.complex128).reshape(1, L.n, L.n)
        tr.set_y(dm0[0])
        dh = dH(t0, dm0)
        H = np.asarray(arrays["H_Ortho"], np.complex128).reshape(L.n, L.n)
        mode = _lib.ZG_DH_NONE
        if not (np.isscalar(dh) and dh == 0):
            dhm = np.asarray(dh, np.complex128).reshape(L.n, L.n)
            tr.set_dH(dhm)
            H = H + dhm
            mode = _lib.ZG_DH_MATRIX
        lam, V = np.linalg.eigh((H + H.conj().T) / 2)
        V = np.ascontiguousarray(V, np.complex128)
        lam = np.ascontiguousarray(lam, np.float64)
        delta = np.zeros(_lib.ZG_MAX_LEADS)
        delta[:L.NL] = [bias(t0, a) for a in range(L.NL)]
        check(lib().zg_stationary_setup(tr._h, float(t0), delta.ctypes.data_as(C.c_void_p), mode, 0.0,
                                        V.ctypes.data_as(C.c_void_p), lam.ctypes.data_as(C.c_void_p)))
        dev = torch.device("cuda", device)
        shape = (L.N, L.n)
        zero = torch.zeros(shape, dtype=torch.complex128, device=dev)
        buf = torch.empty(shape, dtype=torch.complex128, device=dev)

        def F(psi):  # k_psi(psi), affine
            check(lib().zg_stationary_apply(tr._h, _ptr(psi), _ptr(buf)))
            return buf.clone()

        def M(r):
            out = torch.empty(shape, dtype=torch.complex128, device=dev)
            check(lib().zg_stationary_precond(tr._h, _ptr(r.contiguous()), _ptr(out)))
            return out

        f0 = F(zero)
        b = -f0                                   # L(psi) = F(psi) - F(0) = -F(0)

        def Lop(v):
            return F(v) - f0

        def rdot(u, v):
            return float(torch.real(torch.vdot(u.reshape(-1), v.reshape(-1))))

        bnorm = float(torch.linalg.vector_norm(b))
        x = torch.zeros(shape, dtype=torch.complex128, device=dev)
        if x0 is not None:
            x = torch.as_tensor(np.asarray(x0, np.complex128).reshape(shape), device=dev)
        t_start = time.perf_counter()
        its, res = 0, float("inf")
        converged = bnorm == 0.0
        while not converged and its < maxiter:
            r = b - Lop(x) if its > 0 or x0 is not None else b.clone()
            beta = float(torch.linalg.vector_norm(r))
            res = beta / bnorm
            if res <= tol:
                converged = True
                break
            Vs = [r / beta]
            Hm = np.zeros((restart + 1, restart))
            cs, sn = np.zeros(restart), np.zeros(restart)
            g = np.zeros(restart + 1)
            g[0] = beta
            k_used = 0
            for j in range(restart):
                w = Lop(M(Vs[j]))
                for i in range(j + 1):       # modified Gram-Schmidt, twice
                    hij = rdot(Vs[i], w)
                    Hm[i, j] += hij
                    w = w - hij * Vs[i]
                for i in range(j + 1):
                    hij = rdot(Vs[i], w)
                    Hm[i, j] += hij
                    w = w - hij * Vs[i]
                hn = float(torch.linalg.vector_norm(w))
                Hm[j + 1, j] = hn
                for i in range(j):           # earlier Givens rotations
                    a_, b_ = Hm[i, j], Hm[i + 1, j]
                    Hm[i, j], Hm[i + 1, j] = cs[i] * a_ + sn[i] * b_, -sn[i] * a_ + cs[i] * b_
                den = np.hypot(Hm[j, j], Hm[j + 1, j])
                cs[j], sn[j] = (1.0, 0.0) if den == 0 else (Hm[j, j] / den, Hm[j + 1, j] / den)
                Hm[j, j] = cs[j] * Hm[j, j] + sn[j] * Hm[j + 1, j]
                Hm[j + 1, j] = 0.0
                g[j + 1] = -sn[j] * g[j]
                g[j] = cs[j] * g[j]
                its += 1
                k_used = j + 1
                res = abs(g[j + 1]) / bnorm
                if res <= tol or hn == 0.0 or its >= maxiter:
                    break
                Vs.append(w / hn)
            y = np.linalg.solve(np.triu(Hm[:k_used, :k_used]), g[:k_used]) if k_used else np.zeros(0)
            z = torch.zeros(shape, dtype=torch.complex128, device=dev)
            for i in range(k_used):
                z = z + float(y[i]) * Vs[i]
            x = x + M(z)
            if res <= tol:
                # confirm with the true residual
                rt = float(torch.linalg.vector_norm(b - Lop(x))) / bnorm
                res = rt
                converged = rt <= 10 * tol
        secs = time.perf_counter() - t_start
        # final state: y = (sigma0, psi, Omega(psi))
        F(x)
        sig, psi, omg = L.unpack(tr.get_slot(tr.stages))
        return SteadyResult(psi=psi, omg=omg, iterations=its, residual=res, converged=converged, seconds=secs)
    finally:
        tr.close()


def _parse(args):
    opts = {"file": "SaveFile", "maxiter": "10000", "steptol": "1e-8", "restart": "40", "checkderivative": "True"}
    for a in args:
        k, _, v = a.replace(" ", "").partition("=")
        opts[k] = v
    return opts


def main(argv=None):
    """The psinought command line: Dir=<run directory> file=<Arrays parent>."""
    from .arrays_io import load_dictionary
    argv = sys.argv[1:] if argv is None else argv
    opts = _parse(argv)
    if "Dir" not in opts:
        raise SystemExit("usage: python -m zandpack_gb300.psinought Dir=<run dir> [file=SaveFile steptol=1e-8]")
    os.chdir(opts["Dir"])
    sys.path.insert(0, os.getcwd())
    import importlib
    Initial = importlib.import_module("Initial")
    Bias = importlib.import_module("Bias")
    arrays = load_dictionary(opts["file"] + "/Arrays/")
    A = {k: arrays[k] for k in ("H_Ortho", "DM_Ortho", "psi_shape", "Xpp", "Xpm", "GG_P", "GL_P", "GG_M", "GL_M",
                                "diff_GGP_GLP", "diff_GGM_GLM", "xi", "Ixi", "zero_tol")}
    res = steady_state(A, Initial.hbar, Bias.bias, Bias.dH, t0=float(Initial.t0), tol=float(opts["steptol"]),
                       maxiter=int(opts["maxiter"]), restart=int(opts["restart"]))
    print("psinought: %s psi in %d iterations (%.3f s), relative residual %.2e"
          % ("Converged" if res.converged else "Did not converge:", res.iterations, res.seconds, res.residual))
    save = opts["file"] + "_save"
    os.makedirs(save, exist_ok=True)
    np.save(os.path.join(save, "last_psi.npy"), res.psi)
    np.save(os.path.join(save, "last_omg.npy"), res.omg)
    ok_psi = res.converged
    # the sigma derivative at the fixed density matrix (psinought:467-477)
    hbar = float(Initial.hbar)
    dm0 = np.asarray(A["DM_Ortho"], np.complex128)[0]
    dh = Bias.dH(float(Initial.t0), np.asarray(A["DM_Ortho"]))
    h0 = np.asarray(A["H_Ortho"], np.complex128)[0] + (0 if np.isscalar(dh) else np.asarray(dh)[0])
    L = CompactLayout(A, hbar)
    Ixi = np.asarray(A["Ixi"])[0][:, :, :L.NOT]
    P = res.psi[0]
    PI = sum((lambda pa, ia: (pa.reshape(-1, L.n).T @ ia.reshape(-1, L.n))
              + (pa.reshape(-1, L.n).T @ ia.reshape(-1, L.n)).conj().T)(P[a], Ixi[a]) for a in range(L.NL)) / hbar
    dsig = (-1j / hbar) * (h0 @ dm0 - dm0 @ h0) + PI / hbar
    print("psinought: max(|DM derivative|) %.3e" % np.abs(dsig).max())
    with open("psinought_dpsi_MESSAGE.txt", "w") as f:
        f.write("Success" if ok_psi else "Failure")
    with open("psinought_dsig_MESSAGE.txt", "w") as f:
        f.write("Success" if np.abs(dsig).max() < 1e-2 else "Failure")
    return res


if __name__ == "__main__":
    main()
