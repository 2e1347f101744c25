"""The reference's in-process right-hand side and stepper signatures, on the
device.

``make_f(arrays, hbar)`` returns ``f(t, old_sig, old_psi, old_omega, dH,
delta_variant, dH_given=True) -> (D_sig, D_psi, D_omega)``, the signature of
the function ``TD_Transport.make_f`` builds (Zandpack/TimedependentTransport.py:
2754-2776): the time derivatives (not multiplied by a step size) of the
density matrix and of the auxiliary-mode vectors and matrices at time t.
``dH(t, sigma)`` returns an (nk, no, no) array or 0.0; with ``dH_given`` it is
added to H0, otherwise it is H(t) itself.  ``delta_variant(t, a)`` is the bias
of lead a.  The equations are those of the ``zand`` stage body
(Zandpack/mpi/zand:318-387, :713-809); the arrays are in ``zand``'s padded
layout: sigma (nk, no, no), psi (nk, NL, NX, NOT, no), Omega
(nk, NL, NX, NOT, NL, NX, NOT).  Every evaluation runs on the GPU through
libzandgpu's C ABI (one trajectory per k-point, ``zg_rhs`` with h = 1); the
arrays cross the host boundary because the signature takes and returns host
arrays.

``AdaptiveDOP(f, sig0, psi0, omega0, eps, t0, t1, dH, delta_func, Ixi, ...)``
is the reference's in-process Dormand-Prince stepper
(Zandpack/TimedependentTransport.py:3392-3560) for an ``f`` made by
``make_f``: the state stays on the device between steps, stage inputs, error
norm and update run there, and only the callbacks' sigma (when ``dH`` needs
it) and the recorded density matrices cross to the host.
"""
from __future__ import annotations

import math
import time as _time

import numpy as np

from . import _lib
from .engine import Trajectory, kpoint_arrays
from .layout import CompactLayout, LayoutError
from .tableau import DOP54


class DeviceRHS:
    """``f`` of ``make_f``: one device trajectory per k-point."""

    def __init__(self, arrays, hbar, precision="f64", device=0, dot_prod_zero_tol=1e-10):
        self.hbar = float(hbar)
        self.H0 = np.asarray(arrays["H_Ortho"], np.complex128)
        self.NK, self.n = self.H0.shape[0], self.H0.shape[-1]
        self.precision = precision
        self.trajs = []
        for k in range(self.NK):
            A = arrays if self.NK == 1 else kpoint_arrays(arrays, k)
            L = CompactLayout(A, hbar, dot_prod_zero_tol)
            self.trajs.append(Trajectory(A, hbar, precision, device, layout=L))
        L = self.trajs[0].layout
        self.NL, self.NX, self.NOT = L.NL, L.NX, L.NOT
        self.psi_shape = (self.NK, L.NL, L.NX, L.NOT, self.n)
        self.omg_shape = (self.NK, L.NL, L.NX, L.NOT, L.NL, L.NX, L.NOT)
        # padded entries the compact layout holds: live mode rows of psi, and of
        # Omega the columns of sourced modes plus the sourced x free block
        a, x, c = L.modes[:, 0], L.modes[:, 1], L.modes[:, 2]
        self._psi_live = np.zeros((L.NL, L.NX, L.NOT), bool)
        self._psi_live[a, x, c] = True
        npad = L.NL * L.NX * L.NOT
        lin = np.ravel_multi_index((a, x, c), (L.NL, L.NX, L.NOT))
        keep = np.zeros((npad, npad), bool)
        keep[np.ix_(lin, lin[:L.Ns])] = True
        keep[np.ix_(lin[:L.Ns], lin[L.Ns:])] = True
        self._omg_keep = keep

    def close(self):
        for tr in self.trajs:
            tr.close()

    def _check_representable(self, psi, omg):
        """The device keeps only the entries the compact layout holds; a state
        with other nonzero entries is refused rather than silently cut."""
        npad = self._omg_keep.shape[0]
        for k in range(self.NK):
            if np.any(psi[k][~self._psi_live]):
                raise LayoutError("psi is nonzero in auxiliary modes the compact layout drops "
                                  "(rank padding without a source)")
            if np.any(omg[k].reshape(npad, npad)[~self._omg_keep]):
                raise LayoutError("Omega is nonzero outside the blocks the compact layout holds "
                                  "(the source-free x source-free block or dropped modes)")

    def load_state(self, sig, psi, omg, check=True):
        sig = np.asarray(sig, np.complex128).reshape(self.NK, self.n, self.n)
        psi = np.asarray(psi, np.complex128).reshape(self.psi_shape)
        omg = np.asarray(omg, np.complex128).reshape(self.omg_shape)
        if check:
            self._check_representable(psi, omg)
        for k, tr in enumerate(self.trajs):
            tr.set_slot(tr.stages, tr.layout.pack(sig[k], psi[k], omg[k]))

    def _H_terms(self, t, sig, dH, dH_given):
        """(dH mode, per-k dH matrices) for H(t) = H0 + dH(t, sig), or dH(t, sig)."""
        d = dH(t, sig) if dH is not None else 0.0
        if dH_given and np.isscalar(d) and d == 0:
            return _lib.ZG_DH_NONE, None
        d = np.broadcast_to(np.asarray(d, np.complex128), (self.NK, self.n, self.n))
        if not dH_given:
            d = d - self.H0
        return _lib.ZG_DH_MATRIX, d

    def stage(self, slot, t, h, dH, delta_variant, dH_given, want_J=False):
        """k_slot = h f(t, Y_slot) for the stage input already formed on the
        device (``zg_stage_input``); returns the stage-0 currents when asked."""
        sig = np.stack([tr.stage_sigma().copy() for tr in self.trajs]) if dH is not None else None
        mode, d = self._H_terms(t, sig, dH, dH_given)
        delta = [float(delta_variant(t, a)) for a in range(self.NL)]
        Js = []
        for k, tr in enumerate(self.trajs):
            if d is not None:
                tr.set_dH(d[k])
            Js.append(tr.rhs(slot, t, h, delta, mode, 0.0, currents=want_J))
        return np.array(Js) if want_J else None

    def __call__(self, t, old_sig, old_psi, old_omega, dH, delta_variant, dH_given=True):
        self.load_state(old_sig, old_psi, old_omega)
        for tr in self.trajs:
            tr.stage_input(0)
        self.stage(0, float(t), 1.0, dH, delta_variant, dH_given)
        D_sig = np.empty((self.NK, self.n, self.n), np.complex128)
        D_psi = np.empty(self.psi_shape, np.complex128)
        D_omg = np.empty(self.omg_shape, np.complex128)
        for k, tr in enumerate(self.trajs):
            s, p, o = tr.layout.unpack(tr.get_slot(0))
            D_sig[k], D_psi[k], D_omg[k] = s[0], p[0], o[0]
        return D_sig, D_psi, D_omg


def make_f(arrays, hbar, precision="f64", device=0, dot_prod_zero_tol=1e-10):
    """``f(t, old_sig, old_psi, old_omega, dH, delta_variant, dH_given=True)``
    on the device for the propagation described by ``arrays`` (the ``Arrays/``
    of ``TD_Transport.tofile``), as ``TD_Transport.make_f`` returns it
    (Zandpack/TimedependentTransport.py:2754-2776)."""
    return DeviceRHS(arrays, hbar, precision, device, dot_prod_zero_tol)


def _dop54_stepper_tableau(h, faithful_k7):
    """DOP54 as the in-process stepper applies it (Zandpack/DOP54.py; CT = b5 - b4,
    CH = b5).  The reference sets ``k7 = h * k6`` (TimedependentTransport.py:
    3537) instead of the seventh stage, so its error norm takes
    CT[5] k6 + CT[6] h k6: the coefficient of k6 becomes CT[5] + h CT[6] and the
    seventh stage is never used (b5[6] = 0)."""
    CT = np.array(DOP54.CT, np.float64)
    if faithful_k7:
        CT[5] += h * CT[6]
        CT[6] = 0.0
    return CT


def AdaptiveDOP(f, sig0, psi0, omega0, eps, t0, t1, dH, delta_func, Ixi, h_guess=None, dH_given=True,
                print_to_file=True, fixed_mode=False, name="Runge-Kutta", write_func=None, print_step=50,
                plot=False, use_GPU=False, atol=None, rtol=None, elec_names=("left", "right"),
                faithful_k7=True):
    """The reference's in-process adaptive Dormand-Prince loop
    (Zandpack/TimedependentTransport.py:3392-3560) on the device.

    Behaviour kept from the reference: the loop runs while ``t0 <= t1``; an
    attempt is repeated while ``TE > eps`` (TE the unscaled 2-norm of
    sum_j CT_j k_j over sigma, psi and Omega) with ``h <- 0.9 h (eps/TE)^(1/5)``
    after every attempt; the density matrix and the lead currents
    ``2 Re Tr(PI_a)/hbar`` (``Jk(PI(...))``, :3175-3176) are recorded at the
    start of every accepted step together with its time; the state then
    becomes ``y + sum_j b5_j k_j`` and ``t0 += h`` with the step size proposed
    for the next step.  ``faithful_k7`` reproduces the reference's
    ``k7 = h * k6`` (:3537; see ``_dop54_stepper_tableau``); False uses the
    seventh stage as DOP54 defines it.  Returns ``(times, data)`` with
    ``data['current_<name>']`` per lead and ``data['density matrix']``.

    ``name + '.txt'`` receives the progress lines, and every ``print_step``
    steps the state is saved as ``name_last_{sig,psi,omega,time}.npy`` like the
    reference.  ``Ixi`` is accepted for the signature: the currents use the
    Ixi of the arrays ``f`` was made from.  The reference's ``atol``/``rtol``
    branch returns 1 for every input (``1**x``) and ``plot`` needs matplotlib:
    both are refused.
    """
    if not isinstance(f, DeviceRHS):
        raise TypeError("AdaptiveDOP runs an f made by zandpack_gb300.rhs.make_f (the right-hand side on the GPU)")
    if atol is not None or rtol is not None:
        raise ValueError("the atol/rtol error function of the reference is not supported")
    if plot:
        raise ValueError("plot=True is not supported")
    if sig0 is None or psi0 is None or omega0 is None:
        sig0 = np.load(name + "_last_sig.npy")
        psi0 = np.load(name + "_last_psi.npy")
        omega0 = np.load(name + "_last_omega.npy")
        if t0 is None:
            t0 = float(np.load(name + "_last_time.npy").ravel()[0])
    f.load_state(sig0, psi0, omega0)
    h = (t1 - t0) / 1000 if h_guess is None else 0.0 + h_guess
    tab = DOP54
    T0 = t0
    step = 0
    times, dms = [], []
    data = {"current_" + e: [] for e in elec_names}
    with open(name + ".txt", "w") as fh:
        fh.write("\n\n\n\n\nStart (Wait for compilation)\n")
    start = _time.time()
    nstage = tab.RK_N - 1 if faithful_k7 else tab.RK_N
    while t0 <= t1:
        TE = 10 * eps
        while TE > eps:
            J0 = None
            for i in range(nstage):
                for tr in f.trajs:
                    tr.stage_input(i)
                J = f.stage(i, t0 + tab.A[i] * h, h, dH, delta_func, dH_given, want_J=(i == 0))
                if i == 0:
                    J0 = J
            if fixed_mode:
                break
            CT = _dop54_stepper_tableau(h, faithful_k7)
            err = 0.0
            for tr in f.trajs:
                tr.set_error_weights(CT)
                err += float(tr.error_norm2().sum())
            TE = math.sqrt(err)
            with np.errstate(divide="ignore"):
                h = float(0.9 * h * (np.float64(eps) / np.float64(TE)) ** (1 / 5))
        dms.append(np.stack([tr.get_sigma() for tr in f.trajs]))
        for ie, e in enumerate(elec_names):
            data["current_" + e].append(np.asarray(J0)[:, ie] if ie < f.NL else np.zeros(f.NK))
        for tr in f.trajs:
            tr.step_fourth()
        times.append(t0)
        t0 += h
        if step % print_step == 0:
            with open(name + ".txt", "a") as fh:
                fh.write(str((t0 - T0) / (t1 - T0) * 100) + " %\n")
                fh.write("current timestep: " + str(h) + "fs\n")
                fh.write("delta t: " + str(_time.time() - start) + "seconds\n")
                if write_func is not None:
                    s, p, o = _padded_state(f)
                    write_func(fh, t0 - h, s, p, o)
            s, p, o = _padded_state(f)
            np.save(name + "_last_sig", s)
            np.save(name + "_last_psi", p)
            np.save(name + "_last_omega", o)
            np.save(name + "_last_time", np.array(times[-1]))
            np.save("_times", np.array(times))
            np.save("_#electrons_device", np.trace(np.array(dms), axis1=2, axis2=3))
        step += 1
    data["density matrix"] = np.array(dms)
    with open(name + ".txt", "a") as fh:
        fh.write("100%\n")
        fh.write("Runtime: " + str(_time.time() - start) + "seconds")
    return np.array(times), data


def _padded_state(f):
    parts = [tr.get_y() for tr in f.trajs]
    return tuple(np.concatenate([p[i] for p in parts]) for i in range(3))
