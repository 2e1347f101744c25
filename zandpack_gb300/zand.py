"""``zand`` on one GPU: ``python -m zandpack_gb300.zand Dir=/path/to/run``.

Drop-in for ``mpirun -np P zand Dir=...`` (Zandpack/mpi/zand): the same inputs
and outputs, no MPI ranks.

Inputs, read from ``Dir`` exactly as the reference does (Zandpack/mpi/zand:31-77):

* ``Initial.py``: ``Arrs, t0, t1, stepsize, print_timings, usesave, saveevery,
  name, eps, hbar, n_dm_compress, save_PI, checkpoints, save_checkpoints,
  LoadFromFull``;
* ``Bias.py``: ``bias(t, a)``, ``dH(t, sigma)``, ``dissipator(t, sigma)``.
  Optional extension: ``dH_device = {"kind": "hubbard", "U": <eV>}`` evaluates
  U*diag(Re sigma_ii - 0.5) on the device instead of calling ``dH``; the
  environment variable ``ZANDGPU_PRECISION`` (``f64`` or ``mixed``) picks the
  arithmetic (default ``f64``, the reference's).

``Initial.py`` may import ``Zandpack.td_constants``/``Zandpack.Loader`` and
``Bias.py`` may import ``mpi4py``; when those packages are absent, minimal
stand-ins are installed (the constants, the ``Arrays`` loader, and a
one-rank ``MPI.COMM_WORLD``).

Outputs in ``<name>_save/`` (Zandpack/mpi/zand:221-237,412-486): ``DM<step>``
(complex64, every ``n_dm_compress``-th sigma), ``DMt<step>``, ``times<step>``,
``current_<lead>_<step>``, ``PIa<step>`` when ``save_PI``, written every
``saveevery`` accepted steps; at checkpoints ``last_sig``, ``last_time``,
``last_stepsize`` and the full-layout ``last_psi``/``last_omg`` (complex128,
the files ``psinought`` writes and ``LoadFromFull`` reads).  Restarts read
``last_sig/last_time/last_stepsize`` and, with ``LoadFromFull``, ``last_psi``/
``last_omg``; the reference's per-worker restart files depend on its rank
partition and are not read.

The controller is the reference's: seven DOP54 stages per attempt, accept
iff TE < eps, h <- 0.9 h (eps/TE)^(1/5) after every attempt, time advanced by
the step size proposed for the next step, currents from stage 0 of each
accepted attempt.

``ZandRun(nonorth=True)`` (``python -m zandpack_gb300.nozand Dir=...``) is the
reference's ``nozand`` (Zandpack/mpi/nozand): the same run directory plus
``Arrays/S^(-0.5)``; it propagates sigma' = S^-1/2 sigma S^-1/2, starts from
S^-1/2 DM_Ortho S^-1/2 (:306), saves sigma' (``DM*``, ``last_sig``) and
``PIa`` without the conjugate term (:120-140), and honours nozand's
``Initial.py`` flags (:84-95, :547-577): ``compress_mat`` (``.npz`` archives for
``DM``/``PIa``), ``dm_triu_only`` (strict lower triangle zeroed, with
``compress_mat``) and ``dm_occ_only`` (entries where |S| <= 1e-6 zeroed).
``last_psi`` is loaded (``LoadFromFull``) and written in the orthogonal basis,
as ``psinought`` writes it: rows S^-1/2 psi on load (:722), S^1/2 psi' on save.
"""
from __future__ import annotations

import importlib
import inspect
import os
import sys
import time
import types

import numpy as np


def _install_standins():
    """Stand-ins for imports that run files written for the reference use."""
    try:
        import Zandpack.td_constants  # noqa: F401
    except Exception:
        from . import arrays_io, constants
        pkg = types.ModuleType("Zandpack")
        pkg.__path__ = []
        td = types.ModuleType("Zandpack.td_constants")
        td.hbar = constants.HBAR
        td.electron_charge = constants.ELECTRON_CHARGE
        ld = types.ModuleType("Zandpack.Loader")
        ld.load_dictionary = arrays_io.load_dictionary
        ld.flexload = arrays_io.flexload
        pkg.td_constants, pkg.Loader = td, ld
        sys.modules.setdefault("Zandpack", pkg)
        sys.modules.setdefault("Zandpack.td_constants", td)
        sys.modules.setdefault("Zandpack.Loader", ld)
    try:
        import mpi4py  # noqa: F401
    except Exception:
        m = types.ModuleType("mpi4py")
        mpi = types.ModuleType("mpi4py.MPI")

        class _Comm:
            def Get_rank(self):
                return 0

            def Get_size(self):
                return 1

            def Barrier(self):
                pass

            def bcast(self, obj, root=0):
                return obj
        mpi.COMM_WORLD = _Comm()
        m.MPI = mpi
        sys.modules.setdefault("mpi4py", m)
        sys.modules.setdefault("mpi4py.MPI", mpi)


def parse_dir(args):
    """The ``Dir=`` argument as zand parses it (Zandpack/mpi/zand:31-54)."""
    check = ["Dir" in v for v in args]
    if sum(check) > 1:
        raise AssertionError("Dont specify several directories.")
    if True in check:
        a = args[check.index(True)]
        if "=" not in a:
            raise AssertionError("Specify path like this: Dir=/path/to/somewhere/")
        return a.replace(" ", "").split("=")[1]
    return None


class ZandRun:
    """One propagation as ``zand`` runs it, driven through the GPU engine."""

    def __init__(self, run_dir=None, precision=None, device=0, log=print, nonorth=False):
        _install_standins()
        self.nonorth = bool(nonorth)
        if run_dir is not None:
            os.chdir(run_dir)
        cwd = os.getcwd()
        if cwd not in sys.path:
            sys.path.insert(0, cwd)
        for mname in ("Initial", "Bias"):
            sys.modules.pop(mname, None)
        I = importlib.import_module("Initial")
        B = importlib.import_module("Bias")
        self.I, self.B = I, B
        self.log = log
        self.precision = precision or os.environ.get("ZANDGPU_PRECISION", "f64")
        self.device = device
        self.name = I.name
        self.hbar = float(I.hbar)
        self.eps = float(I.eps)
        self.t0, self.t1 = float(I.t0), float(I.t1)
        self.stepsize = float(I.stepsize)
        self.saveevery = int(I.saveevery)
        self.n_dm_compress = int(I.n_dm_compress)
        self.save_PI = bool(I.save_PI)
        self.usesave = bool(I.usesave)
        self.LoadFromFull = bool(getattr(I, "LoadFromFull", False))
        cps = np.array(getattr(I, "checkpoints", []), dtype=float)
        cps = cps[cps > self.t0]
        self.checkpoints = cps[cps < self.t1]
        self.checkpoint_done = np.zeros(len(self.checkpoints), dtype=int)
        self.save_checkpoints = bool(getattr(I, "save_checkpoints", False))
        from .arrays_io import REQUIRED_KEYS, read_arrays
        self.arrays = read_arrays(I.Arrs, REQUIRED_KEYS + (("S^(-0.5)",) if self.nonorth else ()))
        # output flags that only nozand reads (Zandpack/mpi/nozand:84-95)
        self.compress_mat = bool(getattr(I, "compress_mat", False)) and self.nonorth
        self.dm_triu_only = bool(getattr(I, "dm_triu_only", False)) and self.nonorth
        self.dm_occ_only = bool(getattr(I, "dm_occ_only", False)) and self.nonorth

    # ---------------------------------------------------------------- run
    def run(self):
        from .engine import Propagator
        from .tableau import selected
        I, B = self.I, self.B
        save = self.name + "_save/"
        os.makedirs(save, exist_ok=True)
        for f in os.listdir(save):
            if f[0:2] == "DM":
                os.remove(save + f)
        t0, h = self.t0, self.stepsize
        Sm05 = np.asarray(self.arrays["S^(-0.5)"], np.complex128) if self.nonorth else None
        sig0 = self.arrays["DM_Ortho"]
        if self.nonorth:
            sig0 = Sm05 @ np.asarray(sig0, np.complex128) @ Sm05  # Zandpack/mpi/nozand:306
        psi0 = omg0 = None
        if self.usesave:
            try:
                sig0 = np.load(save + "last_sig.npy")
            except OSError:
                self.log("Using /Arrays/DM_Ortho.npy!")
            try:
                t0 = float(np.load(save + "last_time.npy"))
                h = float(np.load(save + "last_stepsize.npy"))
            except OSError:
                pass
            if self.LoadFromFull:
                psi0 = np.load(save + "last_psi.npy")
                omg0 = np.load(save + "last_omg.npy")
                if self.nonorth:  # rows S^-1/2 psi (Zandpack/mpi/nozand:722)
                    psi0 = np.concatenate([np.asarray(psi0[k:k + 1], np.complex128) @ Sm05[k].T
                                           for k in range(Sm05.shape[0])])
        dh_dev = getattr(B, "dH_device", None)
        hub = float(dh_dev["U"]) if isinstance(dh_dev, dict) and dh_dev.get("kind") == "hubbard" else None
        diss = getattr(B, "dissipator", None)
        pr = Propagator(self.arrays, self.hbar, B.bias, dH=None if hub is not None else B.dH,
                        dissipator=diss, hubbard_U=hub, precision=self.precision, device=self.device,
                        tableau=selected(), psi0=psi0, omg0=omg0, nonorth=self.nonorth)
        self.prop = pr
        tr = pr.traj
        L = tr.layout
        pr.set_state(sig0, psi0, omg0)  # psi = Omega = 0 when not loaded
        self.log("zandpack_gb300 %s: %s, precision %s, n=%d, %d live modes of %d padded, eps=%g" % (
            "nozand" if self.nonorth else "zand", self.name, self.precision, L.n, L.N, L.padded_modes, self.eps))
        occ_mask = None
        if self.dm_occ_only:
            S05 = np.concatenate([x.basis.S05 for x in pr.trajs])
            occ_mask = np.abs(S05 @ S05) > 1e-6                    # Zandpack/mpi/nozand:261-262
        self.log("Timedependent Bias:\n" + _source(B.bias))
        NL = L.NL
        currents = [[] for _ in range(NL)]
        DM = [pr.get_sigma()]
        times = [t0]
        PI_holder = []
        step_count = 0
        TIME_START = time.time()
        t = t0
        TE = 0.0
        while t < self.t1:
            accepted = False
            while not accepted:
                TE, J0, _ = pr.attempt(t, h)
                accepted = TE < self.eps
                old_h = h
                h = pr.tab.hnew(h, TE, self.eps)
            for a in range(NL):
                currents[a].append(np.array([J0[a]]) if pr.NK == 1 else np.asarray(J0)[:, a])
            if self.save_PI:
                PI_holder.append(np.concatenate([self._pi_from_state(x.layout, x) for x in pr.trajs]))
            # checkpoints: the state before the update, as the reference saves it
            passed = (t > self.checkpoints) * (self.checkpoint_done == 0)
            if self.save_checkpoints and passed.any():
                sig, psi, omg = pr.get_y()
                np.save(save + "last_sig", sig)
                np.save(save + "last_time", t)
                np.save(save + "last_stepsize", old_h)
                if self.nonorth:  # back to the orthogonal basis: rows S^1/2 psi'
                    psi = np.concatenate([psi[k:k + 1] @ x.basis.S05[0].T for k, x in enumerate(pr.trajs)])
                np.save(save + "last_psi", psi)
                np.save(save + "last_omg", omg)
                self.checkpoint_done[np.where(passed)[0][0]] = 1
            pr.step_fourth()
            t += h
            DM.append(np.concatenate([self._sigma(x) for x in pr.trajs]))
            times.append(t + 0.0)
            step_count += 1
            if np.mod(step_count, self.saveevery) == 0 and step_count >= self.saveevery:
                dm_arr = np.array(DM[::self.n_dm_compress]).astype(np.complex64)
                if occ_mask is not None:
                    dm_arr = dm_arr * occ_mask
                if self.compress_mat:
                    if self.dm_triu_only:
                        dm_arr = np.triu(dm_arr)
                    np.savez_compressed(save + "DM" + str(step_count), dm_arr)
                else:
                    np.save(save + "DM" + str(step_count), dm_arr)
                dm_times = np.array(times[-len(DM):])
                np.save(save + "DMt" + str(step_count), dm_times[::self.n_dm_compress])
                if self.save_PI:
                    pi_arr = np.array(PI_holder[::self.n_dm_compress]).astype(np.complex64)
                    if self.compress_mat:
                        np.savez_compressed(save + "PIa" + str(step_count), pi_arr)
                    else:
                        np.save(save + "PIa" + str(step_count), pi_arr)
                np.save(save + "times" + str(step_count), times[-len(DM):])
                for k, c in enumerate(currents):
                    np.save(save + "current_" + str(k) + "_" + str(step_count), c[-len(DM):])
                DM = []
                PI_holder = []
                self.log("t=" + str(np.round(t, 3)) + " | #steps=" + str(step_count) + " | eps=" + format(TE, ".3e"))
                for k, c in enumerate(currents):
                    self.log("    Bias_%d: %s   | J_%d: %s" % (k, np.round(B.bias(t, k), 6), k, np.round(c[-1], 6)))
        self.log("RUNTIME: %s" % (time.time() - TIME_START))
        self.steps = step_count
        self.t_end = t
        return self

    def _sigma(self, tr):
        n = tr.layout.n
        buf = np.empty((n, n), np.complex128)
        from ._lib import check, lib
        import ctypes
        check(lib().zg_get_sigma(tr._h, tr.stages, buf.ctypes.data_as(ctypes.c_void_p)))
        return buf[None]

    def _pi_from_state(self, L, tr):
        """PI_a = (P_a + P_a^H)/hbar of the stage-0 state (Zandpack/mpi/zand:91-110,363-366);
        nozand keeps P_a/hbar (Zandpack/mpi/nozand:120-140)."""
        sig, psi, _ = tr.get_y()
        n = L.n
        PI = np.zeros((1, L.NL, n, n), complex)
        for a in range(L.NL):
            rows = L.mode_lead == a
            m = L.modes[rows]
            pa = psi[0, m[:, 0], m[:, 1], m[:, 2]]
            P = np.zeros((n, n), complex)
            k = L.lead_ncols[a]
            P[:, L.lead_cols[a, :k]] = pa.T @ L.IXI[rows][:, :k]
            PI[0, a] = (P if self.nonorth else P + P.conj().T) / L.hbar
        return PI


def _source(f):
    try:
        return inspect.getsource(f)
    except (OSError, TypeError):
        return repr(f)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    d = parse_dir(argv)
    ZandRun(d).run()


if __name__ == "__main__":
    main()
