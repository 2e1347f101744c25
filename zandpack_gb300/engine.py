"""Device trajectory and the ``zand`` adaptive loop on top of libzandgpu.

``Trajectory`` owns one propagation on the GPU: the compact-layout constants,
the Runge-Kutta state slots and scratch (``zg_traj``).  ``Propagator`` drives it
with the reference's Dormand-Prince 5(4) controller
(Zandpack/mpi/zand:297-430): seven stages per attempt, stage inputs from the
tableau rows, user callbacks ``bias(t, a)``, ``dH(t, sigma)`` and
``dissipator(t, sigma)`` evaluated at every stage time, the unscaled absolute
error test ``TE < eps``, ``h <- 0.9 h (eps/TE)^(1/5)`` after every attempt, and
time advanced by the step size proposed for the next step, as the reference
does (``t0 += h`` after ``h = hnew(h, TE)``).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Callable, Optional

import numpy as np

from . import _lib
from ._lib import check, lib
from .layout import CompactLayout
from .tableau import DOP54, Tableau

PREC = {"f64": _lib.ZG_PREC_F64, "mixed": _lib.ZG_PREC_MIXED}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Trajectory:
    """One AME propagation resident on the GPU."""

    def __init__(self, arrays, hbar, precision="f64", device=0, psi0=None, omg0=None,
                 dot_prod_zero_tol=1e-10, layout: Optional[CompactLayout] = None, nonorth: bool = False):
        """``nonorth``: propagate in the non-orthogonal basis of ``arrays['S^(-0.5)']``
        as the reference's ``nozand`` does; states (``set_y``, ``get_y``) are then
        sigma' and psi' (``NonorthBasis.sigma``/``psi`` map orthogonal ones)."""
        self.basis = None
        if nonorth:
            from .nonorth import NonorthBasis
            self.basis = NonorthBasis(arrays, dot_prod_zero_tol)
            arrays = self.basis.arrays
        L = layout if layout is not None else CompactLayout(arrays, hbar, dot_prod_zero_tol, psi0=psi0, omg0=omg0)
        self.layout = L
        self.precision = precision
        keep = dict(
            mode_lead=np.ascontiguousarray(L.mode_lead, np.int32),
            s_start=np.ascontiguousarray(L.s_start, np.int64),
            f_start=np.ascontiguousarray(L.f_start, np.int64),
            lead_cols=np.ascontiguousarray(L.lead_cols, np.int32),
            colmap=np.ascontiguousarray(L.colmap, np.int32),
            H0=np.ascontiguousarray(L.H0, np.complex128),
            Xp=np.ascontiguousarray(L.Xp, np.complex128), Xm=np.ascontiguousarray(L.Xm, np.complex128),
            GLP=np.ascontiguousarray(L.GLP, np.complex128), dGP=np.ascontiguousarray(L.dGP, np.complex128),
            dGM=np.ascontiguousarray(L.dGM, np.complex128),
            XI=np.ascontiguousarray(L.XI, np.complex128), IXI=np.ascontiguousarray(L.IXI, np.complex128),
            XIS=np.ascontiguousarray(L.XIS, np.complex128), XIT2=np.ascontiguousarray(L.XIT2, np.complex128),
        )
        st = _lib.zg_layout(n=L.n, n_leads=L.NL, n_modes=L.N, n_sourced=L.Ns, nc=L.nc, hbar=L.hbar,
                            **{k: _ptr(v) for k, v in keep.items()})
        h = C.c_void_p()
        check(lib().zg_traj_create(int(device), C.byref(st), PREC[precision], C.byref(h)))
        self._h = h
        info = np.zeros(8, np.int64)
        check(lib().zg_traj_info(self._h, _ptr(info)))
        self.size = int(info[6])
        self.stages = int(info[7])
        assert self.size == L.size
        self._buf = np.empty(self.size, np.complex128)
        self._sig = np.empty((L.n, L.n), np.complex128)
        self._delta = np.zeros(_lib.ZG_MAX_LEADS, np.float64)
        self._J = np.zeros(L.NL, np.float64)
        if self.basis is not None:
            Sm1 = np.ascontiguousarray(self.basis.Sm1[0])
            C0 = self.basis.constant_term(L)
            check(lib().zg_set_overlap(self._h, _ptr(Sm1), _ptr(C0)))

    def close(self):
        if getattr(self, "_h", None):
            lib().zg_traj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ----------------------------------------------------------- tableau
    def set_tableau(self, tab: Tableau):
        B = np.nan_to_num(np.asarray(tab.B, np.float64), nan=0.0)
        Bz = np.zeros_like(B)
        for i in range(1, tab.RK_N):
            ix = tab.idxholder[i]
            Bz[i, ix] = B[i, ix]
        args = [np.ascontiguousarray(x, np.float64) for x in (tab.A, Bz, tab.CT, tab.CH)]
        check(lib().zg_set_tableau(self._h, tab.RK_N, *[_ptr(a) for a in args]))
        self.stages = tab.RK_N
        self._tab_args = args

    def set_error_weights(self, CT):
        """Replace the error weights CT of the current tableau (the stages, the
        stage rows and the update weights stay)."""
        if getattr(self, "_tab_args", None) is None:
            self.set_tableau(DOP54)
        A, Bz, _, CH = self._tab_args
        CT = np.ascontiguousarray(CT, np.float64)
        assert CT.shape == (self.stages,)
        check(lib().zg_set_tableau(self._h, self.stages, _ptr(A), _ptr(Bz), _ptr(CT), _ptr(CH)))
        self._tab_args = [A, Bz, CT, CH]

    # ------------------------------------------------------------- state
    def set_slot(self, slot, y):
        y = np.ascontiguousarray(y, np.complex128)
        assert y.size == self.size
        check(lib().zg_set_state(self._h, int(slot), _ptr(y)))

    def get_slot(self, slot):
        out = np.empty(self.size, np.complex128)
        check(lib().zg_get_state(self._h, int(slot), _ptr(out)))
        return out

    def set_y(self, sig, psi=None, omg=None):
        L = self.layout
        if psi is None and omg is None:  # psi = Omega = 0: only sigma crosses to the device
            s = np.ascontiguousarray(np.asarray(sig, np.complex128).reshape(L.n, L.n))
            check(lib().zg_set_sigma(self._h, _ptr(s)))
            return
        if psi is None or omg is None:
            z = L.unpack(np.zeros(L.size, complex))
            psi = z[1] if psi is None else psi
            omg = z[2] if omg is None else omg
        self.set_slot(self.stages, L.pack(sig, psi, omg))

    def get_y(self):
        return self.layout.unpack(self.get_slot(self.stages))

    # -------------------------------------------------------------- stages
    def stage_input(self, stage):
        check(lib().zg_stage_input(self._h, int(stage)))

    def stage_sigma(self):
        check(lib().zg_get_stage_sigma(self._h, _ptr(self._sig)))
        return self._sig

    def set_dH(self, dH):
        dH = np.ascontiguousarray(np.asarray(dH, np.complex128).reshape(self.layout.n, self.layout.n))
        check(lib().zg_set_dH(self._h, _ptr(dH)))

    def set_dissipator(self, D):
        """dissipator(ts, sigma) for the coming ``rhs`` calls ((1,n,n) or (n,n)); None: off."""
        if D is None:
            check(lib().zg_set_dissipator(self._h, None))
            return
        D = np.ascontiguousarray(np.asarray(D, np.complex128).reshape(self.layout.n, self.layout.n))
        check(lib().zg_set_dissipator(self._h, _ptr(D)))

    def rhs(self, stage, ts, h, delta, dH_mode=_lib.ZG_DH_NONE, hubbard_U=0.0, currents=False):
        d = self._delta
        d[:] = 0.0
        d[:len(delta)] = delta
        Jp = _ptr(self._J) if currents else None
        check(lib().zg_rhs(self._h, int(stage), float(ts), float(h), _ptr(d), int(dH_mode),
                           float(hubbard_U), Jp))
        return self._J.copy() if currents else None

    # ------------------------------------------------ kernel implementation
    def set_impl(self, impl):
        """Kernels of the mixed path's small products and dOmega/dt:
        ``_lib.ZG_IMPL_*`` (``zg_set_impl``)."""
        check(lib().zg_set_impl(self._h, int(impl)))

    def get_impl(self):
        """(current implementation, list of the supported ones)."""
        impl, avail = C.c_int(), C.c_int()
        check(lib().zg_get_impl(self._h, C.byref(impl), C.byref(avail)))
        return impl.value, [i for i in range(_lib.ZG_IMPL_COUNT) if avail.value >> i & 1]

    def set_schedule(self, sched):
        """Where the second stream forks off: ``_lib.ZG_SCHED_*`` (``zg_set_schedule``)."""
        check(lib().zg_set_schedule(self._h, int(sched)))

    def get_schedule(self):
        v = C.c_int()
        check(lib().zg_get_schedule(self._h, C.byref(v)))
        return v.value

    def tune(self, reps=5):
        """Time one right-hand side of every supported implementation under both
        stream schedules and keep the fastest (``zg_tune``); returns
        ((impl, schedule), {(impl, schedule): ms per RHS}) over the supported ones.
        Overwrites k slot 0."""
        best = C.c_int()
        nv = _lib.ZG_IMPL_COUNT * _lib.ZG_SCHED_COUNT
        ms = np.zeros(nv)
        check(lib().zg_tune(self._h, int(reps), C.byref(best), _ptr(ms)))
        n = _lib.ZG_IMPL_COUNT
        times = {(v % n, v // n): float(ms[v]) for v in range(nv) if ms[v] >= 0}
        return (best.value % n, best.value // n), times

    def error_norm2(self):
        e = np.zeros(3)
        check(lib().zg_error_norm2(self._h, _ptr(e)))
        return e

    def attempt_native(self, t, h, eps, bias, hubbard_U=None, currents=True):
        """One controller attempt inside the library (``zg_attempt``): bias is
        a ``zg_bias`` (see ``native_bias``), dH the device Hubbard term or none.
        Returns (TE, accepted, t_new, h_new, stage-0 currents)."""
        tt, hh = C.c_double(t), C.c_double(h)
        TE, acc = C.c_double(), C.c_int()
        mode = _lib.ZG_DH_HUBBARD if hubbard_U is not None else _lib.ZG_DH_NONE
        Jp = _ptr(self._J) if currents else None
        check(lib().zg_attempt(self._h, C.byref(tt), C.byref(hh), float(eps), C.byref(bias), mode,
                               float(hubbard_U or 0.0), C.byref(TE), C.byref(acc), Jp))
        return TE.value, bool(acc.value), tt.value, hh.value, (self._J.copy() if currents else None)

    def get_sigma(self):
        buf = np.empty((self.layout.n, self.layout.n), np.complex128)
        check(lib().zg_get_sigma(self._h, self.stages, _ptr(buf)))
        return buf

    def step_fourth(self):
        check(lib().zg_step_fourth(self._h))

    # -- graph-launched attempts (controller on the device)
    def graph_prepare(self, bias, hubbard_U=None):
        """Capture one controller attempt as a CUDA graph (``zg_graph_prepare``)."""
        mode = _lib.ZG_DH_HUBBARD if hubbard_U is not None else _lib.ZG_DH_NONE
        check(lib().zg_graph_prepare(self._h, C.byref(bias), mode, float(hubbard_U or 0.0)))
        if not hasattr(self, "_recs"):
            self._recs = (_lib.zg_attempt_rec * _lib.ZG_GRAPH_MAX_BATCH)()

    def graph_set(self, t, h, eps, t1):
        check(lib().zg_graph_set(self._h, float(t), float(h), float(eps), float(t1)))

    def graph_run(self, count):
        """Launch ``count`` attempts, one host sync.  Returns (records, t, h,
        done); each record is (t, h, TE, h_next, accepted, status, J[:L])."""
        n, tt, hh, done = C.c_int(), C.c_double(), C.c_double(), C.c_int()
        check(lib().zg_graph_run(self._h, int(count), C.cast(self._recs, C.c_void_p), C.byref(n), C.byref(tt),
                                 C.byref(hh), C.byref(done)))
        L = self.layout.NL
        recs = [(r.t, r.h, r.TE, r.h_next, bool(r.accepted), r.status, np.array(r.J[:L]))
                for r in self._recs[:n.value]]
        return recs, tt.value, hh.value, bool(done.value)


def native_bias(spec, n_leads):
    """``zg_bias`` for the analytic bias specifications of ``workloads``
    (exp_ramp, gauss, sin: +V/2 on lead 0, -V/2 on lead 1; step_lead0: V on
    lead 0; zero)."""
    b = _lib.zg_bias()
    k = spec["kind"]
    w = [0.0] * _lib.ZG_MAX_LEADS
    if k in ("exp_ramp", "gauss", "sin"):
        w[0], w[1] = 0.5, -0.5
    elif k == "step_lead0":
        w[0] = 1.0
    for i in range(_lib.ZG_MAX_LEADS):
        b.w[i] = w[i] if i < n_leads else 0.0
    b.kind = _lib.ZG_BIAS["step" if k == "step_lead0" else k]
    b.V0 = float(spec.get("V0", 0.0))
    b.tau = float(spec.get("tau", 1.0))
    b.tc = float(spec.get("tc", 0.0))
    b.sigma = float(spec.get("sigma", 1.0))
    b.f = float(spec.get("f", 0.0))
    return b


_PER_K = ("H_Ortho", "DM_Ortho", "Xpp", "Xpm", "GG_P", "GL_P", "GG_M", "GL_M", "diff_GGP_GLP", "diff_GGM_GLM",
          "xi", "Ixi", "S^(-0.5)")


def kpoint_arrays(arrays, k):
    """The ``Arrays`` of k-point ``k`` alone (NK = 1): every per-k array sliced
    to ``[k:k+1]`` (the leading NK axis, Zandpack/mpi/zand:113-124)."""
    nk = int(np.asarray(arrays["H_Ortho"]).shape[0])
    out = {}
    if hasattr(arrays, "keys"):
        keys = list(arrays.keys())
    else:  # a lazy Arrays mapping: the keys zand reads, plus the overlap when present
        from .arrays_io import REQUIRED_KEYS
        keys = list(REQUIRED_KEYS) + [k for k in ("S^(-0.5)",) if k in arrays]
    for key in keys:
        v = arrays[key]
        if key in _PER_K:
            v = np.asarray(v)[k:k + 1]
        elif key == "psi_shape":
            v = np.array(v).copy()
            v[0] = 1
        out[key] = v
    assert int(np.asarray(out["H_Ortho"]).shape[0]) == 1 and nk > k
    return out


class Propagator:
    """The ``zand`` time loop on the device (Zandpack/mpi/zand:297-430).

    ``bias(t, a)`` and ``dH(t, sigma)`` are the reference's callbacks; ``dH``
    receives sigma with the k axis, shape (NK, n, n), and may return 0.0.
    ``hubbard_U`` selects the built-in density-dependent term
    U * diag(Re sigma_ii - 0.5) evaluated on the device instead of ``dH``.
    ``nonorth=True`` runs the reference's ``nozand`` instead (non-orthogonal
    basis of ``arrays['S^(-0.5)']``): the state, the callbacks' sigma and the
    returned sigma are then sigma' (start from ``traj.basis.sigma(DM_Ortho)``).

    Several k-points (NK > 1): one device trajectory per k-point
    (``self.trajs``); every stage runs on all of them, the error norm is summed
    over them and the controller is shared, as in ``zand`` where the k axis is
    a batch axis of every array and ``TERR2_*`` sums over it.  States,
    sigma and currents then carry the k axis (currents per step: NK x NL).
    """

    def __init__(self, arrays, hbar, bias: Callable, dH: Optional[Callable] = None,
                 dissipator: Optional[Callable] = None, hubbard_U: Optional[float] = None,
                 precision="f64", device=0, tableau: Tableau = DOP54, psi0=None, omg0=None,
                 dot_prod_zero_tol=1e-10, dH_depends_on_sigma=True, nonorth: bool = False):
        self.NK = int(np.asarray(arrays["H_Ortho"]).shape[0])
        self.trajs = []
        for k in range(self.NK):
            A = arrays if self.NK == 1 else kpoint_arrays(arrays, k)
            p0 = None if psi0 is None else np.asarray(psi0)[k:k + 1]
            o0 = None if omg0 is None else np.asarray(omg0)[k:k + 1]
            self.trajs.append(Trajectory(A, hbar, precision, device, psi0=p0, omg0=o0,
                                         dot_prod_zero_tol=dot_prod_zero_tol, nonorth=nonorth))
        self.traj = self.trajs[0]
        if tableau is not DOP54:
            for tr in self.trajs:
                tr.set_tableau(tableau)
        self.tab = tableau
        self.bias = bias
        self.dH = dH
        self.dissipator = dissipator
        self.hubbard_U = hubbard_U
        self.dH_depends_on_sigma = dH_depends_on_sigma
        self.NL = self.traj.layout.NL
        self.n_rhs = 0

    def close(self):
        for tr in self.trajs:
            tr.close()

    def set_state(self, sig, psi=None, omg=None):
        if self.NK == 1:
            self.traj.set_y(sig, psi, omg)
            return
        sig = np.asarray(sig)
        for k, tr in enumerate(self.trajs):
            tr.set_y(sig[k:k + 1], None if psi is None else np.asarray(psi)[k:k + 1],
                     None if omg is None else np.asarray(omg)[k:k + 1])

    def get_y(self):
        """(sigma, psi, Omega) in the reference layout, with the k axis."""
        parts = [tr.get_y() for tr in self.trajs]
        return tuple(np.concatenate([p[i] for p in parts]) for i in range(3))

    def get_sigma(self):
        return np.concatenate([tr.get_y()[0] for tr in self.trajs]) if self.NK > 1 else self.traj.get_y()[0]

    def step_fourth(self):
        for tr in self.trajs:
            tr.step_fourth()

    def _stage(self, i, t, h, want_J):
        ts = t + self.tab.A[i] * h
        for tr in self.trajs:
            tr.stage_input(i)
        modes = [(_lib.ZG_DH_NONE, 0.0)] * self.NK
        if self.hubbard_U is not None:
            modes = [(_lib.ZG_DH_HUBBARD, float(self.hubbard_U))] * self.NK
        elif self.dH is not None:
            sig = (np.stack([tr.stage_sigma().copy() for tr in self.trajs])
                   if self.dH_depends_on_sigma else None)
            dh = self.dH(ts, sig)
            if not (np.isscalar(dh) and dh == 0):
                dh = np.asarray(dh)
                for k, tr in enumerate(self.trajs):
                    tr.set_dH(dh[k] if dh.ndim == 3 else dh)
                modes = [(_lib.ZG_DH_MATRIX, 0.0)] * self.NK
        if self.dissipator is not None:
            dz = self.dissipator(ts, np.stack([tr.stage_sigma().copy() for tr in self.trajs]))
            for k, tr in enumerate(self.trajs):
                off = np.isscalar(dz) and dz == 0
                tr.set_dissipator(None if off else (np.asarray(dz)[k] if np.ndim(dz) == 3 else dz))
        delta = [self.bias(ts, a) for a in range(self.NL)]
        self.n_rhs += 1
        Js = [tr.rhs(i, ts, h, delta, m, U, currents=want_J) for tr, (m, U) in zip(self.trajs, modes)]
        if not want_J:
            return None
        return Js[0] if self.NK == 1 else np.array(Js)

    def attempt(self, t, h):
        """One attempt of all stages from the stored y; returns (TE, J at stage 0, err2 parts)."""
        J0 = None
        for i in range(self.tab.RK_N):
            J = self._stage(i, t, h, want_J=(i == 0))
            if i == 0:
                J0 = J
        e = sum(tr.error_norm2() for tr in self.trajs)
        TE = math.sqrt(float(e.sum()))
        return TE, J0, e

    def run(self, t0, t1, h, eps, max_attempts=None, replay_h=None, force_accept=None, record_sigma=True,
            on_step=None):
        """Propagate from t0 until t >= t1 exactly as ``zand`` does; returns histories.

        Replay mode (for comparisons on a fixed time grid): ``replay_h[i]`` is
        the step size of attempt i and, after the last attempt, the final
        advance; ``force_accept[i]`` overrides the accept decision of attempt i.
        """
        t = float(t0)
        out = dict(times=[t], sig=[], currents=[], h_hist=[], TE_hist=[], t_attempt=[], accepted=[])
        if record_sigma:
            out["sig"].append(self.get_sigma())
        attempts = 0
        while t < t1:
            accepted = False
            while not accepted:
                if max_attempts is not None and attempts >= max_attempts:
                    return out
                if replay_h is not None:
                    h = float(replay_h[attempts])
                TE, J0, _ = self.attempt(t, h)
                out["h_hist"].append(h)
                out["TE_hist"].append(TE)
                out["t_attempt"].append(t)
                attempts += 1
                accepted = TE < eps if force_accept is None else bool(force_accept[attempts - 1])
                out["accepted"].append(accepted)
                h = self.tab.hnew(h, TE, eps)
                if replay_h is not None and attempts < len(replay_h):
                    h = float(replay_h[attempts])
            out["currents"].append(J0)
            self.step_fourth()
            t += h
            out["times"].append(t)
            if record_sigma:
                out["sig"].append(self.get_sigma())
            if on_step is not None:
                on_step(t, h)
        return out
