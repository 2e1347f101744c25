"""ORACLE -- test infrastructure only.

A CPU restatement, in NumPy, of the reference's AME propagation path: the
``zand`` stage body (master sigma part Zandpack/mpi/zand:297-408, worker psi/Omega
part :692-848) and its Dormand-Prince 5(4) controller, in the reference's
padded layout psi (NK, NL, NX, NOT, NO), Omega (NK, NL, NX, NOT, NL, NX, NOT).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this module, as the checker.  The product (``zandpack_gb300``) never imports
it.  It is pinned against fixtures produced by running the unmodified reference
(``tests/golden/make_golden.py``).

Differences from the reference that do not change results:

* each lead's rows are computed in one piece instead of per worker chunk
  (``partition_scheme3``, Zandpack/mpi_splitter.py:582-654);
* the support of xi in the second Omega source is taken per lead, where the
  reference takes it per worker chunk (Zandpack/mpi/zand:600-602); both drop
  only entries whose magnitude is at most ``dot_prod_zero_tol`` and coincide
  whenever entries outside a lead's support are exactly zero.
"""
from __future__ import annotations

import math

import numpy as np

# ----------------------------------------------------------------- tableau
# DOP54 as Zandpack/mpi_RK4pars_dev.py:118-149 writes it
RK_N = 7
_V = np.full((7, 8), np.nan)
_V[0, 0] = 0
_V[1, 0:2] = 1 / 5, 1 / 5
_V[2, 0:3] = 3 / 10, 3 / 40, 9 / 40
_V[3, 0:4] = 4 / 5, 44 / 45, -56 / 15, 32 / 9
_V[4, 0:5] = 8 / 9, 19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729
_V[5, 0:6] = 1, 9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656
_V[6, 0:7] = 1, 35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84
_b5 = np.array([35 / 384, 0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84, 0])
_b4 = np.array([5179 / 57600, 0, 7571 / 16695, 393 / 640, -92097 / 339200, 187 / 2100, 1 / 40])
A = _V[:, 0].copy()
B = np.zeros((7, 8))
B[:, :7] = _V[:, 1:]
B[1:, 7] = 1.0
CT = _b5 - _b4
CH = np.hstack((_b5, [1.0]))
idxholder = {0: None, 1: [0, 7], 2: [0, 1, 7], 3: [0, 1, 2, 7], 4: [0, 1, 2, 3, 7],
             5: [0, 1, 2, 3, 4, 7], 6: [0, 1, 2, 3, 4, 5, 7]}


def hnew_func(h, TE, eps):
    """Zandpack/mpi_RK4pars_dev.py:148-149."""
    with np.errstate(divide="ignore"):
        return 0.9 * h * ((eps / np.float64(TE)) ** 0.2)


# ------------------------------------------------------ reference kernels
def abs2(x):
    """Zandpack/mpi_funcs.py:18-20."""
    return x.real ** 2 + x.imag ** 2


def stage_combine(Y, b, idx):
    """``MM(Y[idx].transpose(..., 0), b[idx], out)`` (Zandpack/mpi/zand:306-313)
    and ``step_*_forward_nb`` (Zandpack/func_step_forward.py:16-109)."""
    idx = list(idx)
    return np.tensordot(np.asarray(b)[idx], Y[idx], axes=(0, 0))


def terr2(Y, ct):
    """``TERR2_*`` (Zandpack/mpi_funcs.py:247-252): sum |sum_j CT_j Y_j|^2."""
    return float(abs2(np.tensordot(ct, Y, axes=(0, 0))).sum())


def step_fourth(Y, ch):
    """``step_fourth_*`` (Zandpack/mpi_funcs.py:254-259): Y[-1] = sum_j CH_j Y_j."""
    Y[-1] = np.tensordot(ch, Y, axes=(0, 0))


def outer_subtraction(A, B, C, out):
    """``OuterSubtraction_hard_opti`` (Zandpack/mpi_funcs.py:91-102):
    out[k,a,x,c,aa,xx,:] += (A[k,a,x,0] - B[k,aa,xx,0]) * C[k,a,x,c,aa,xx,:]."""
    d = A[..., 0][:, :, :, None, None, None, None] - B[..., 0][:, None, None, None, :, :, None]
    out += d * C


def combine_fermi_skip(Y, b, out, idx, fp_loc, fp_all):
    """``step_omg_forward_nb_fermi_opti`` (Zandpack/func_step_forward.py:112-139):
    the stage combination of Omega slots (RK, k, a, x, c, a', x', c') written
    only where the row pole x and the column pole x' are not both Fermi poles."""
    full = stage_combine(Y, b, idx)
    skip = np.asarray(fp_loc, bool)[None, None, :, None, None, None, None] & \
        np.asarray(fp_all, bool)[None, None, None, None, None, :, None]
    skip = np.broadcast_to(skip, out.shape)
    out[~skip] = full[~skip]


def find_max_orbital_idx_per_lead(GG_P, GL_P, zero_tol):
    """Zandpack/mpi_splitter.py:555-580."""
    live = (np.abs(GG_P).max(axis=0) >= zero_tol) | (np.abs(GL_P).max(axis=0) >= zero_tol)
    return np.array([np.where(live[a])[1].max() + 1 for a in range(live.shape[0])])


# ------------------------------------------------------------------ RHS
class Problem:
    """Constants of one propagation, derived as ``zand`` derives them
    (Zandpack/mpi/zand:113-124,254-281,568-664)."""

    def __init__(self, arrays, hbar, dot_prod_zero_tol=1e-10):
        D = arrays
        self.hbar = float(hbar)
        self.H0 = np.asarray(D["H_Ortho"], dtype=np.complex128)
        self.NK, self.NO = self.H0.shape[0], self.H0.shape[-1]
        self.NL, self.NX = int(D["psi_shape"][1]), int(D["psi_shape"][2])
        self.noT_lead = find_max_orbital_idx_per_lead(D["GG_P"], D["GL_P"], D["zero_tol"])
        self.NOT = NOT = int(max(self.noT_lead))
        sl = (slice(None), slice(None), slice(None), slice(0, NOT))
        self.Xpp = np.asarray(D["Xpp"])[sl]
        self.Xpm = np.asarray(D["Xpm"])[sl]
        self.GLP = np.asarray(D["GL_P"])[sl]
        self.dGP = np.asarray(D["diff_GGP_GLP"])[sl]
        self.dGM = np.asarray(D["diff_GGM_GLM"])[sl]
        self.xi = np.asarray(D["xi"])[sl]
        self.Ixi = np.asarray(D["Ixi"])[sl]
        tol = dot_prod_zero_tol
        for a in range(self.NL):
            nt = self.noT_lead[a]
            # *hard_opti assumes X+/X- constant along c (Zandpack/mpi/zand:578-581)
            for c in range(nt):
                assert np.allclose(self.Xpp[:, a, :, c], self.Xpp[:, a, :, 0])
        for c in range(NOT):
            assert np.allclose(self.Xpm[:, :, :, c], self.Xpm[:, :, :, 0])
        self.S_alpha = [np.where((np.abs(self.Ixi[:, a]) > tol).any(axis=(0, 1, 2)))[0]
                        for a in range(self.NL)]
        self.S_all = np.where((np.abs(self.Ixi) > tol).any(axis=(0, 1, 2, 3)))[0]
        self.S_xi = [np.where((np.abs(self.xi[:, a, :, :self.noT_lead[a]]) > tol).any(axis=(0, 1, 2)))[0]
                     for a in range(self.NL)]

    def zero_state(self):
        NK, NL, NX, NOT, NO = self.NK, self.NL, self.NX, self.NOT, self.NO
        return (np.zeros((NK, NO, NO), complex), np.zeros((NK, NL, NX, NOT, NO), complex),
                np.zeros((NK, NL, NX, NOT, NL, NX, NOT), complex))

    def pi_and_currents(self, psi):
        """``Q_np`` per lead (Zandpack/mpi/zand:91-110,363-366) and the lead
        currents ``Re Tr(PI_a)/hbar`` (:368-378)."""
        NK, NO, NOT = self.NK, self.NO, self.NOT
        PI = np.zeros((NK, self.NL, NO, NO), complex)
        for a in range(self.NL):
            S = self.S_alpha[a]
            pa = psi[:, a].reshape(NK, self.NX * NOT, NO)
            ia = self.Ixi[:, a][..., S].reshape(NK, self.NX * NOT, len(S))
            res = np.zeros((NK, NO, NO), complex)
            res[:, :, S] = np.matmul(pa.transpose(0, 2, 1), ia)
            res += res.transpose(0, 2, 1).conj()
            PI[:, a] = res / self.hbar
        J = np.trace(PI, axis1=2, axis2=3).real / self.hbar  # (NK, NL)
        return PI, J

    def rhs(self, h, sig, psi, omg, Ht, delta, diss=0.0):
        """Stage derivatives k = h f(t, y) of sigma, psi, Omega, plus PI and the
        currents, for stage input (sig, psi, omg), H(t) = ``Ht`` and lead biases
        ``delta`` (Appendix-A equations of ``zand``)."""
        hbar = self.hbar
        NK, NL, NX, NOT, NO = self.NK, self.NL, self.NX, self.NOT, self.NO
        delta = np.asarray(delta, dtype=np.float64)
        # ---- sigma (Zandpack/mpi/zand:340-387)
        Dm = Ht @ sig
        Dm = Dm - Dm.transpose(0, 2, 1).conj()
        Dm = Dm * (-1j)
        Dm = Dm - hbar * np.asarray(diss)
        PI, J = self.pi_and_currents(psi)
        ksig = (Dm + PI.sum(axis=1)) * (h / hbar)
        # ---- psi and Omega, one lead of rows at a time (:713-809)
        kpsi = np.zeros_like(psi)
        komg = np.zeros_like(omg)
        psi_tilde = psi.conj()
        Xpm_d = self.Xpm + delta[None, :, None, None]
        xi_S = (self.xi[..., self.S_all] / hbar ** 2).reshape(NK, NL * NX * NOT, len(self.S_all))
        for a in range(NL):
            nt = self.noT_lead[a]
            tp = psi[:, a, :, :nt]                       # (NK, NX, nt, NO)
            to = omg[:, a, :, :nt]                       # (NK, NX, nt, NL, NX, NOT)
            Xpp_d = self.Xpp[:, a, :, :nt] + delta[a]
            xa = self.xi[:, a, :, :nt]
            kp = np.matmul(tp.reshape(NK, NX * nt, NO), (Ht / hbar).transpose(0, 2, 1)).reshape(tp.shape)
            kp -= (Xpp_d / hbar)[..., None] * tp
            kp += self.GLP[:, a, :, :nt, None] * xa
            kp += self.dGP[:, a, :, :nt, None] * np.matmul(
                xa.reshape(NK, NX * nt, NO), sig.transpose(0, 2, 1)).reshape(tp.shape)
            kp[..., self.S_all] += np.matmul(to.reshape(NK, NX * nt, NL * NX * NOT), xi_S).reshape(
                NK, NX, nt, len(self.S_all))
            kp *= -1j * h
            kpsi[:, a, :, :nt] = kp
            ko = np.zeros_like(to)
            rows = tp.reshape(NK, NX * nt, NO)
            for b in range(NL):
                Sb = self.S_alpha[b]
                rhs_b = (self.dGM[:, b, :, :, None] * self.Ixi[:, b])[..., Sb].reshape(NK, NX * NOT, len(Sb))
                ko[:, :, :, b] = np.matmul(h * rows[..., Sb], rhs_b.transpose(0, 2, 1)).reshape(NK, NX, nt, NX, NOT)
            Sx = self.S_xi[a]
            lhs = (self.dGP[:, a, :, :nt, None] * xa)[..., Sx].reshape(NK, NX * nt, len(Sx))
            rt = (h * psi_tilde.reshape(NK, NL * NX * NOT, NO)[..., Sx]).transpose(0, 2, 1)
            ko += np.matmul(lhs, rt).reshape(ko.shape)
            s = 1j * h / hbar
            Ad = Xpp_d[..., 0] * s                          # (NK, NX)
            Bd = Xpm_d[..., 0] * s                          # (NK, NL, NX)
            ko += (Ad[:, :, None, None, None, None] - Bd[:, None, None, :, :, None]) * to
            komg[:, a, :, :nt] = ko
        return ksig, kpsi, komg, PI, J


# ------------------------------------------------------------ DOP54 loop
def propagate(prob, t0, t1, h, eps, bias, dH, state=None, dissipator=None, max_attempts=None,
              replay_h=None, on_attempt=None):
    """The ``zand`` adaptive loop (Zandpack/mpi/zand:297-430).

    Reproduces the reference's controller: 7 stages, accept iff TE < eps,
    h <- 0.9 h (eps/TE)^(1/5) after every attempt, and time advanced by the
    step size proposed for the NEXT step (``t0 += h`` after ``h = hnew(...)``,
    :406-427), until t >= t1.  Returns a dict of histories.
    """
    hbar = prob.hbar
    sig0, psi0, omg0 = state if state is not None else (None, None, None)
    z = prob.zero_state()
    sig0 = z[0] + np.asarray(prob.H0 * 0 if sig0 is None else sig0)
    psi0 = z[1] if psi0 is None else np.array(psi0, dtype=complex)
    omg0 = z[2] if omg0 is None else np.array(omg0, dtype=complex)
    SIGS = np.zeros((RK_N + 1,) + sig0.shape, complex)
    PSIS = np.zeros((RK_N + 1,) + psi0.shape, complex)
    OMGS = np.zeros((RK_N + 1,) + omg0.shape, complex)
    SIGS[-1], PSIS[-1], OMGS[-1] = sig0, psi0, omg0
    t = float(t0)
    out = dict(times=[t], sig=[SIGS[-1].copy()], currents=[], h_hist=[], TE_hist=[], t_attempt=[])
    attempts = 0
    while t < t1:
        accepted = False
        while not accepted:
            if max_attempts is not None and attempts >= max_attempts:
                return out
            if replay_h is not None:
                h = replay_h[attempts]
            J0 = None
            for i in range(RK_N):
                if i == 0:
                    ys, yp, yo = SIGS[-1], PSIS[-1], OMGS[-1]
                else:
                    ix = idxholder[i]
                    ys = stage_combine(SIGS, B[i], ix)
                    yp = stage_combine(PSIS, B[i], ix)
                    yo = stage_combine(OMGS, B[i], ix)
                ts = t + A[i] * h
                Ht = prob.H0 + dH(ts, ys)
                delta = [bias(ts, a) for a in range(prob.NL)]
                diss = dissipator(ts, ys) if dissipator is not None else 0.0
                ks, kp, ko, PI, J = prob.rhs(h, ys, yp, yo, Ht, delta, diss)
                SIGS[i], PSIS[i], OMGS[i] = ks, kp, ko
                if i == 0:
                    J0 = J
            TE = math.sqrt(terr2(SIGS[:RK_N], CT) + terr2(PSIS[:RK_N], CT) + terr2(OMGS[:RK_N], CT))
            out["h_hist"].append(h)
            out["TE_hist"].append(TE)
            out["t_attempt"].append(t)
            if on_attempt is not None:
                on_attempt(attempts, t, h, (SIGS, PSIS, OMGS))
            attempts += 1
            accepted = TE < eps
            h = float(hnew_func(h, TE, eps))
        out["currents"].append(J0)
        step_fourth(SIGS, CH)
        step_fourth(PSIS, CH)
        step_fourth(OMGS, CH)
        t += h
        out["times"].append(t)
        out["sig"].append(SIGS[-1].copy())
    out["state"] = (SIGS[-1].copy(), PSIS[-1].copy(), OMGS[-1].copy())
    return out


# ------------------------------------------------- in-process DOP stepper
def adaptive_dop(prob, sig0, psi0, omg0, eps, t0, t1, dH, delta_func, h_guess=None, dH_given=True,
                 fixed_mode=False, faithful_k7=True, max_steps=None):
    """The reference's in-process ``AdaptiveDOP`` loop
    (Zandpack/TimedependentTransport.py:3392-3560) with ``f`` = the ``zand``
    stage body (``Problem.rhs`` with h = 1):

    * ``h = (t1 - t0)/1000`` unless ``h_guess`` (:3474-3478);
    * ``while t0 <= t1`` (:3491), attempts repeated while ``TE > eps`` (:3493);
    * stage inputs ``y + sum_j B[i, j] k_j`` at ``t0 + A[i] h`` (:3495-3535),
      ``k_i = h f``; ``k7 = h * k6`` (:3537) unless ``faithful_k7`` is False;
    * ``TE = sqrt(sum |sum_j CT_j k_j|^2)`` with CT = b5 - b4 (:3410-3416),
      ``h <- 0.9 h (eps/TE)^(1/5)`` (:3443-3444);
    * density matrix and ``Jk(PI(psi_a, Ixi_a))`` recorded before the update
      (:3547-3549), ``y <- y + sum_j b5_j k_j`` (:3551), ``t0 += h`` (:3553).
    """
    hbar = prob.hbar
    NL = prob.NL
    CT = _b5 - _b4
    sig, psi, omg = (np.array(x, dtype=complex) for x in (sig0, psi0, omg0))
    h = (t1 - t0) / 1000 if h_guess is None else float(h_guess)
    times, dms, cur, TEs = [], [], [[] for _ in range(NL)], []

    def f(t, s, p, o):
        d = dH(t, s) if dH is not None else 0.0
        Ht = prob.H0 + d if dH_given else np.asarray(d) + 0 * prob.H0
        delta = [delta_func(t, a) for a in range(NL)]
        ks, kp, ko, _, _ = prob.rhs(1.0, s, p, o, Ht, delta)
        return ks, kp, ko

    steps = 0
    while t0 <= t1:
        if max_steps is not None and steps >= max_steps:
            break
        TE = 10 * eps
        while TE > eps:
            ks = []
            for i in range(RK_N):
                if i == RK_N - 1 and faithful_k7:
                    ks.append(tuple(h * v for v in ks[5]))
                    break
                y = [sig, psi, omg]
                for j in range(i):
                    for q in range(3):
                        y[q] = y[q] + B[i, j] * ks[j][q]
                ks.append(tuple(h * v for v in f(t0 + A[i] * h, *y)))
            if fixed_mode:
                break
            TE = math.sqrt(sum(terr2(np.array([k[q] for k in ks]), CT) for q in range(3)))
            TEs.append(TE)
            with np.errstate(divide="ignore"):
                h = float(0.9 * h * (np.float64(eps) / np.float64(TE)) ** (1 / 5))
        dms.append(sig.copy())
        _, J = prob.pi_and_currents(psi)
        for a in range(NL):
            cur[a].append(J[:, a])
        upd = [sum(_b5[j] * ks[j][q] for j in range(RK_N)) for q in range(3)]
        sig, psi, omg = sig + upd[0], psi + upd[1], omg + upd[2]
        times.append(t0)
        t0 += h
        steps += 1
    return dict(times=np.array(times), dm=np.array(dms), currents=[np.array(c) for c in cur], TE=TEs,
                state=(sig, psi, omg))
