"""Fixtures of the reference's in-process stepper ``AdaptiveDOP``
(Zandpack/TimedependentTransport.py:3392-3560), run UNMODIFIED.

Usage (in a container that has the reference checkout; see ``refharness``):

    python tests/golden/make_inprocess_golden.py [mini2 mini3]

``TimedependentTransport.py`` imports packages absent here (sisl,
siesta_python, Gf_Module, Block_matrices, matplotlib through ``plot``); they
are replaced in ``sys.modules`` by empty stand-ins, which the stepper never
touches.  numba is stubbed as in ``refharness`` (its decorated ``PI_nb`` then
runs as the same arithmetic in plain Python).  The right-hand side handed to
the stepper is the oracle's ``zand`` stage body with h = 1
(``oracle.zand_np.Problem.rhs``), whose own parity with the reference is
pinned by the ``zand`` fixtures; these fixtures pin the stepper's loop: step
sizes, accept rule, the ``k7 = h * k6`` assignment, recorded times, density
matrices and currents.

For each case this writes ``tests/golden/inproc_<case>.npz`` with ``times``,
``dm`` (density matrix at the start of every accepted step), ``current_<a>``
per lead, and the run parameters.
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import refharness  # noqa: E402
from oracle import zand_np as zo  # noqa: E402

# The stepper's k7 = h * k6 leaves a first-order term in its error estimate, so
# its steps scale like eps; a loose eps keeps these runs to some dozens of steps.
CASES = {"mini2": dict(eps=1e-5, t1=0.05, h_guess=0.01), "mini3": dict(eps=1e-5, t1=0.05, h_guess=0.01)}


class _Absent(types.ModuleType):
    """Stand-in for a package the stepper does not use."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return lambda *a, **k: None


def _load_tdt():
    refharness._install_stubs()
    for m in ("sisl", "siesta_python", "siesta_python.siesta_python", "Gf_Module", "Gf_Module.Gf",
              "Block_matrices", "Block_matrices.Block_matrices", "Block_matrices.Croy", "plot"):
        sys.modules.setdefault(m, _Absent(m))
    import importlib
    return importlib.import_module("TimedependentTransport")


def make_case(name):
    from conftest import golden_callbacks, load_golden
    tdt = _load_tdt()
    z = load_golden(name)
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    NL = prob.NL

    def f(t, s, ps, o, dHf, delta_variant, dH_given=True):
        Ht = prob.H0 + dHf(t, s) if dH_given else dHf(t, s)
        ks, kp, ko, _, _ = prob.rhs(1.0, s, ps, o, Ht, [delta_variant(t, a) for a in range(NL)])
        return ks, kp, ko

    sig0, psi0, omg0 = prob.zero_state()
    sig0 = sig0 + np.asarray(z["DM_Ortho"])
    c = CASES[name]
    names = ["lead%d" % a for a in range(NL)]
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory(prefix="zinproc_") as d:
        os.chdir(d)
        try:
            times, data = tdt.AdaptiveDOP(f, sig0, psi0, omg0, c["eps"], 0.0, c["t1"], dH, bias,
                                          np.asarray(prob.Ixi), h_guess=c["h_guess"], elec_names=names)
        finally:
            os.chdir(cwd)
    out = dict(times=np.asarray(times), dm=np.asarray(data["density matrix"]),
               params=np.array(json.dumps(dict(case=name, t0=0.0, **c))))
    for a in range(NL):
        out["current_%d" % a] = np.asarray(data["current_" + names[a]])
    path = os.path.join(HERE, "inproc_%s.npz" % name)
    np.savez_compressed(path, **out)
    print("%s: %d accepted steps to t=%.4f -> %s" % (name, len(times), times[-1], path))


if __name__ == "__main__":
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    for c in sys.argv[1:] or list(CASES):
        make_case(c)
