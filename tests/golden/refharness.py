"""Run the UNMODIFIED reference ``zand`` (or ``nozand``) in-process to make
golden fixtures.

Fixture generation only: needs the reference checkout (``ZANDPACK_REF``,
default ``/root/reference``) and is never imported by the GPU tests, ``smoke()``
or ``bench.py``.

The reference needs numba and mpi4py, which this image lacks.  The harness
therefore installs, in ``sys.modules`` only:

* a no-op ``numba`` (``njit`` -> identity, ``prange`` -> ``range``,
  ``vectorize`` -> ``numpy.vectorize``): the decorated loops then run as the same
  arithmetic in plain Python;
* a fake ``mpi4py.MPI`` whose ranks are threads of this process
  (``bcast/Bcast/Send/Recv/Barrier``; ``Abort`` ends the thread);
* a stub ``Zandpack`` package object so ``Zandpack/__init__.py`` (which imports
  sisl) never runs.

``sys.pycache_prefix`` points at a scratch directory so Python compiles the
reference's ``.py`` sources afresh and never uses the ``__pycache__`` shipped
with it.  The ``zand`` source is compiled and executed as it is on disk.

Instrumentation wraps reference functions by name (the wrappers call the
originals): ``TERR2_{sig,psi,omg}`` see every attempt's stage derivatives,
``step_fourth_*`` every accepted state, ``hnew_func`` every (h, TE) pair, and
``numpy.save`` every output file.
"""
from __future__ import annotations

import contextlib
import copy
import io
import os
import queue
import sys
import tempfile
import threading
import types

import numpy as np

REF = os.environ.get("ZANDPACK_REF", "/root/reference")
ZDIR = os.path.join(REF, "Zandpack")

_tl = threading.local()


class _World:
    def __init__(self, size):
        self.size = size
        self.bar = threading.Barrier(size)
        self.slot = None
        self.q = {}
        self.lock = threading.Lock()

    def Q(self, k):
        with self.lock:
            return self.q.setdefault(k, queue.Queue())


_W = None


class _Comm:
    def Get_rank(self):
        return _tl.rank

    def Get_size(self):
        return _W.size

    def bcast(self, obj, root=0):
        if _tl.rank == root:
            _W.slot = obj
        _W.bar.wait(timeout=600)
        v = copy.deepcopy(_W.slot)
        _W.bar.wait(timeout=600)
        return v

    def Bcast(self, buf, root=0):
        if _tl.rank == root:
            _W.slot = np.array(buf, copy=True)
        _W.bar.wait(timeout=600)
        buf[...] = _W.slot
        _W.bar.wait(timeout=600)

    def Send(self, buf, dest, tag=0):
        _W.Q((_tl.rank, dest, tag)).put(np.array(buf, copy=True))

    def Recv(self, buf, source, tag=0):
        buf[...] = _W.Q((source, _tl.rank, tag)).get(timeout=600)

    def Barrier(self):
        _W.bar.wait(timeout=600)

    def Abort(self, *a):
        raise SystemExit(0)


class _Win:
    """``MPI.Win`` shared-memory window: every rank sees rank 0's buffer
    (what ``nozand`` uses for the global psi and the H/sigma broadcast)."""

    def __init__(self, buf, itemsize):
        self.buf, self.itemsize = buf, itemsize

    @staticmethod
    def Allocate_shared(nbytes, itemsize, comm=None):
        if _tl.rank == 0:
            _W.slot = bytearray(max(int(nbytes), 16))
        _W.bar.wait(timeout=600)
        buf = _W.slot
        _W.bar.wait(timeout=600)
        return _Win(buf, itemsize)

    def Shared_query(self, rank):
        return memoryview(self.buf), self.itemsize


class _Dtype:
    def __init__(self, size):
        self.size = size

    def Get_size(self):
        return self.size


def _install_stubs():
    if getattr(_install_stubs, "done", False):
        return
    sys.pycache_prefix = tempfile.mkdtemp(prefix="zref_pyc_")
    nb = types.ModuleType("numba")

    def njit(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f
    nb.njit = nb.jit = njit
    nb.prange = range

    def vectorize(*a, **k):
        return lambda f: np.vectorize(f)
    nb.vectorize = vectorize

    class _T:
        def __call__(self, *a, **k):
            return self
    nb.float64 = nb.float32 = nb.complex128 = nb.complex64 = nb.int64 = _T()
    sys.modules["numba"] = nb
    m = types.ModuleType("mpi4py")
    mpi = types.ModuleType("mpi4py.MPI")
    mpi.COMM_WORLD = _Comm()
    mpi.Win = _Win
    mpi.DOUBLE_COMPLEX = _Dtype(16)
    mpi.Finalize = lambda: None
    m.MPI = mpi
    sys.modules["mpi4py"] = m
    sys.modules["mpi4py.MPI"] = mpi
    pkg = types.ModuleType("Zandpack")
    pkg.__path__ = [ZDIR]
    pkg.__version__ = "1.0"
    sys.modules["Zandpack"] = pkg
    if ZDIR not in sys.path:
        sys.path.insert(0, ZDIR)
    _install_stubs.done = True


def reference_modules():
    """Import the reference's propagation modules (numba stubbed)."""
    _install_stubs()
    import importlib
    mods = {}
    for name in ("mpi_funcs", "mpi_RK4pars_dev", "mpi_splitter", "func_step_forward", "PadeDecomp"):
        mods[name] = importlib.import_module("Zandpack." + name)
    return mods


class Recorder:
    def __init__(self, keep_attempts):
        self.keep = set(keep_attempts)
        self.lock = threading.Lock()
        self.k = {}        # (kind, rank, attempt) -> array
        self.attempt = {}  # (kind, rank) -> counter
        self.hnew = []     # (h, TE, eps)
        self.sig_states = []
        self.saves = []    # (filename, array)
        self.ystate = {}   # (kind, rank, attempt) -> state the attempt started from

    def next_attempt(self, kind):
        key = (kind, _tl.rank)
        with self.lock:
            a = self.attempt.get(key, 0)
            self.attempt[key] = a + 1
        return a


def run_zand(workdir: str, nranks: int, keep_attempts=(0,), keep_states=True, script="zand"):
    """Execute the reference ``zand`` (or ``nozand``, ``script="nozand"``) in
    ``workdir`` (holding Initial.py/Bias.py) with ``nranks`` thread-ranks;
    return the Recorder."""
    global _W
    os.environ.setdefault("OMP_NUM_THREADS", "1")  # start_print reads it
    mods = reference_modules()
    mf = sys.modules["Zandpack.mpi_funcs"]
    fsf = sys.modules["Zandpack.func_step_forward"]
    rk = sys.modules["Zandpack.mpi_RK4pars_dev"]
    rec = Recorder(keep_attempts)
    orig = {k: getattr(mf, k) for k in ("TERR2_sig", "TERR2_psi", "TERR2_omg",
                                        "step_fourth_sig", "step_fourth_psi", "step_fourth_omg")}
    orig_nb = {k: getattr(fsf, "TERR2_%s_nb" % k) for k in ("sig", "psi", "omg")}
    orig_hnew = rk.hnew_func

    def wrap_terr(kind, nb=False):
        f = orig_nb[kind] if nb else orig["TERR2_" + kind]

        def w(Y, CT):
            a = rec.next_attempt(kind)
            if a in rec.keep:
                # Y is the view Y_all[0:RK_N]; its base holds y_n at index RK_N
                base = Y.base
                with rec.lock:
                    rec.k[(kind, _tl.rank, a)] = np.array(Y, copy=True)
                    if base is not None and base.shape[0] == Y.shape[0] + 1:
                        rec.ystate[(kind, _tl.rank, a)] = np.array(base[-1], copy=True)
            return f(Y, CT)
        return w

    def wrap_sf(kind):
        f = orig["step_fourth_" + kind]

        def w(Y, CH):
            f(Y, CH)
            if kind == "sig" and keep_states:
                with rec.lock:
                    rec.sig_states.append(np.array(Y[-1], copy=True))
        return w

    def hnew(h, TE, eps):
        with rec.lock:
            rec.hnew.append((float(h), float(TE), float(eps)))
        return orig_hnew(h, TE, eps)

    np_save = np.save

    def save(fn, arr, *a, **k):
        with rec.lock:
            rec.saves.append((str(fn), np.array(arr, copy=True)))
        return np_save(fn, arr, *a, **k)

    for kind in ("sig", "psi", "omg"):
        setattr(mf, "TERR2_" + kind, wrap_terr(kind))
        setattr(fsf, "TERR2_%s_nb" % kind, wrap_terr(kind, nb=True))
        setattr(mf, "step_fourth_" + kind, wrap_sf(kind))
    rk.hnew_func = hnew
    np.save = save
    spath = os.path.join(ZDIR, "mpi", script)
    code = compile(open(spath).read(), spath, "exec")
    _W = _World(nranks)
    errs = {}
    old = os.getcwd()
    os.chdir(workdir)
    sys.path.insert(0, workdir)
    for m in ("Initial", "Bias"):
        sys.modules.pop(m, None)
    saved_argv = sys.argv
    sys.argv = ["zand"]

    def run(r):
        _tl.rank = r
        try:
            exec(code, {"__name__": "__zand__", "__file__": spath})
        except SystemExit:
            pass
        except Exception as e:  # workers end on bcast(None) unpacking
            errs[r] = repr(e)
    out = io.StringIO()
    try:
        with contextlib.redirect_stdout(out):
            th = [threading.Thread(target=run, args=(r,), daemon=True) for r in range(nranks)]
            for t in th:
                t.start()
            th[0].join()
            for t in th[1:]:
                t.join(timeout=30)
    finally:
        os.chdir(old)
        sys.path.remove(workdir)
        sys.argv = saved_argv
        np.save = np_save
        for k, f in orig.items():
            setattr(mf, k, f)
        for k, f in orig_nb.items():
            setattr(fsf, "TERR2_%s_nb" % k, f)
        rk.hnew_func = orig_hnew
    rec.stdout = out.getvalue()
    rec.errors = errs
    if 0 in errs:
        raise RuntimeError("reference master rank failed: " + errs[0] + "\n" + rec.stdout[-3000:])
    return rec


def worker_roles(nranks, arrays):
    """(rank -> (lead, pole indices, eig indices)) from the reference's own
    ``partition_scheme3`` (Zandpack/mpi_splitter.py:582-654)."""
    mods = reference_modules()
    sp = mods["mpi_splitter"]
    noT_lead = sp.find_max_orbital_idx_per_lead(arrays["GG_P"], arrays["GL_P"], arrays["zero_tol"])
    NK = arrays["H_Ortho"].shape[0]
    NL, NX = int(arrays["psi_shape"][1]), int(arrays["psi_shape"][2])
    roles = {}
    for r in range(1, nranks):
        info = sp.partition_scheme3(r, nranks, NK, NL, NX, noT_lead)
        roles[r] = (int(info[2][0]), np.asarray(info[3]), np.asarray(info[4]))
    return roles, noT_lead


def run_psinought(workdir: str, file_dir: str, options=()):
    """Execute the reference ``cmdtools/psinought`` (the steady-state solver)
    in ``workdir`` (holding Initial.py/Bias.py) on ``file_dir/Arrays``; return
    (PSI, OMG, stdout) as saved in ``file_dir + '_save'``.  Extra stubs for
    modules the solver imports but that need absent packages:
    ``Zandpack.TimedependentTransport`` (only ``Q_nb``, used by the derivative
    printout, which these runs switch off), ``Zandpack.Louivillian`` (only with
    ``L_info``) and ``Zandpack.docstrings`` (banner strings)."""
    _install_stubs()
    for name, attrs in (("Zandpack.TimedependentTransport", {"Q_nb": None}),
                        ("Zandpack.Louivillian", {"Louivillian": None}),
                        ("Zandpack.docstrings", {"psi0_docstring": "", "CoolLine": ""})):
        if name not in sys.modules:
            m = types.ModuleType(name)
            for k, v in attrs.items():
                setattr(m, k, v)
            sys.modules[name] = m
    path = os.path.join(ZDIR, "cmdtools", "psinought")
    code = compile(open(path).read(), path, "exec")
    old = os.getcwd()
    saved_argv = sys.argv
    sys.path.insert(0, workdir)
    for m in ("Initial", "Bias"):
        sys.modules.pop(m, None)
    sys.argv = ["psinought", "Dir=" + workdir, "file=" + file_dir, "checkderivative=False",
                "printfile=None"] + list(options)
    out = io.StringIO()
    try:
        with contextlib.redirect_stdout(out):
            exec(code, {"__name__": "__psinought__", "__file__": path})
    finally:
        os.chdir(old)
        sys.path.remove(workdir)
        sys.argv = saved_argv
    save = os.path.join(workdir, file_dir + "_save")
    return np.load(os.path.join(save, "last_psi.npy")), np.load(os.path.join(save, "last_omg.npy")), out.getvalue()
