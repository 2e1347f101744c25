"""Generate golden fixtures by running the UNMODIFIED reference ``zand`` (and,
for the ``nz_*`` cases, ``nozand`` on the same cases posed in a
non-orthogonal basis, ``make_nonorth_workload``).

Usage (in a container that has the reference checkout; see ``refharness``):

    python tests/golden/make_golden.py [c1 mini2 mini3 nz_mini2 nz_mini3]

For each case this writes ``tests/golden/<case>.npz`` holding

* the input ``Arrays`` (the exact bytes the reference consumed);
* the run parameters (t0, t1, eps, stepsize, hbar, bias/dH spec as JSON);
* ``h_hist, TE_hist``: every (h, TE) pair the controller saw, in order
  (rejected attempts included);
* ``times``, ``sig_traj`` (every ``keep_every``-th accepted complex128 sigma)
  and the lead ``currents`` at the start of every accepted step;
* for the attempts in ``KEEP``: the seven stage derivatives of sigma, psi and
  Omega (``ksig``, ``kpsi``, ``komg``; psi/Omega assembled from the worker
  slices into the padded ``(NL, NX, NOT, ...)`` layout, rows beyond a lead's
  ``noT`` zero as in the reference's global arrays) and the state the attempt
  started from (``y_sig``, ``y_psi``, ``y_omg``) plus its h and t.
"""
from __future__ import annotations

import json
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import refharness  # noqa: E402
from zandpack_gb300.workloads import make_kpoint_workload, make_nonorth_workload, make_workload  # noqa: E402
from zandpack_gb300.arrays_io import write_arrays  # noqa: E402

CASES = {
    # name: (t1, initial stepsize, attempts whose stages are kept, keep_every)
    # the large initial steps of the small cases force rejected attempts
    "c1": (1.0, 0.01, (0, 7), 4),
    # the n=20 chain over its full span, 0-50 fs (sigma kept every 40th step)
    "c1_50fs": (50.0, 0.01, (0,), 40),
    "mini2": (2.0, 0.3, (0, 1, 12), 1),
    "mini3": (1.0, 0.3, (0, 1, 9), 1),
    # the same cases posed in a non-orthogonal basis, run through ``nozand``
    "nz_mini2": (1.0, 0.3, (0, 1, 9), 1),
    "nz_mini3": (1.0, 0.3, (0, 1, 9), 1),
    # mini2 with two k-points (make_kpoint_workload)
    "k2_mini2": (1.0, 0.3, (0, 1, 9), 1),
}


def initial_py(w, t1, stepsize, saveevery=1):
    return "\n".join([
        "import numpy as np",
        "from Zandpack.Loader import load_dictionary",
        "hbar=%r" % w.hbar,
        "name='gold'",
        "t0=%r" % w.t0, "t1=%r" % t1, "eps=%r" % w.eps,
        "usesave=False", "LoadFromFull=False", "checkpoints=[]", "save_checkpoints=False",
        "print_timings=False", "stepsize=%r" % stepsize, "n_dm_compress=1", "save_PI=False",
        "saveevery=%d" % saveevery,
        "Arrs=load_dictionary('Arrays/')",
    ]) + "\n"


def make_case(name):
    t1, stepsize, keep, keep_every = CASES[name]
    nonorth = name.startswith("nz_")
    if nonorth:
        w = make_nonorth_workload(name[3:])
    elif name.startswith("k2_"):
        w = make_kpoint_workload(name[3:], nk=2)
    else:
        w = make_workload(name.split("_")[0])
    A = w.arrays
    L = int(A["psi_shape"][1])
    nranks = L + 1
    with tempfile.TemporaryDirectory(prefix="zgold_") as d:
        write_arrays(os.path.join(d, "Arrays"), A)
        with open(os.path.join(d, "Initial.py"), "w") as f:
            f.write(initial_py(w, t1, stepsize))
        with open(os.path.join(d, "Bias.py"), "w") as f:
            f.write(w.bias_source())
        rec = refharness.run_zand(d, nranks, keep_attempts=keep, script="nozand" if nonorth else "zand")
    roles, noT_lead = refharness.worker_roles(nranks, A)
    RK_N = 7
    NK, NL, NX, NOT, NO = (int(v) for v in A["psi_shape"])
    out = {k: v for k, v in A.items()}
    out["params"] = np.array(json.dumps(dict(
        t0=w.t0, t1=t1, eps=w.eps, stepsize=stepsize, hbar=w.hbar, bias=w.bias,
        hubbard_U=w.hubbard_U, nranks=nranks, keep=list(keep), keep_every=keep_every)))
    out["noT_lead"] = np.asarray(noT_lead)
    hh = np.array(rec.hnew)
    out["h_hist"] = hh[:, 0]
    out["TE_hist"] = hh[:, 1]
    # accepted-step outputs from the reference's own save files
    cur = {}
    times = None
    for fn, arr in rec.saves:
        b = os.path.basename(fn)
        m = re.match(r"current_(\d+)_(\d+)", b)
        if m:
            cur.setdefault(int(m.group(1)), {})[int(m.group(2))] = arr
        m = re.match(r"times(\d+)", b)
        if m:
            times = (times or {})
            times[int(m.group(1))] = arr
    steps = sorted(times)
    # times<step> holds the times of the DM list written at that save; with
    # saveevery=1 the first save holds [t0, t1] and later ones [t_step]
    tt = [np.asarray(times[s]).ravel() for s in steps]
    out["times"] = np.concatenate(tt)
    # (NL, steps) for one k-point, (NL, steps, NK) for several
    out["currents"] = np.stack([np.concatenate([np.asarray(cur[a][s]).reshape(-1, NK) for s in steps])
                                for a in range(NL)])
    if NK == 1:
        out["currents"] = out["currents"][..., 0]
    sig = np.array(rec.sig_states)  # (nsteps, NK, NO, NO)
    out["sig_traj_idx"] = np.arange(0, len(sig), keep_every)
    out["sig_traj"] = sig[::keep_every]
    out["sig_final"] = sig[-1]
    # stage derivatives and starting states of the kept attempts
    for a in keep:
        ks = rec.k.get(("sig", 0, a))
        if ks is None:
            raise RuntimeError("attempt %d not recorded" % a)
        kpsi = np.zeros((RK_N, NK, NL, NX, NOT, NO), complex)
        komg = np.zeros((RK_N, NK, NL, NX, NOT, NL, NX, NOT), complex)
        for r, (lead, px, ex) in roles.items():
            kp = rec.k[("psi", r, a)]
            ko = rec.k[("omg", r, a)]
            kpsi[:, :, lead][:, :, px[:, None], ex[None, :]] = kp[:, :, 0]
            komg[:, :, lead][:, :, px[:, None], ex[None, :]] = ko[:, :, 0]
        out["ksig_%d" % a] = ks
        out["kpsi_%d" % a] = kpsi
        out["komg_%d" % a] = komg
        ys = rec.ystate[("sig", 0, a)]
        yp = np.zeros((NK, NL, NX, NOT, NO), complex)
        yo = np.zeros((NK, NL, NX, NOT, NL, NX, NOT), complex)
        for r, (lead, px, ex) in roles.items():
            yp[:, lead][:, px[:, None], ex[None, :]] = rec.ystate[("psi", r, a)][:, 0]
            yo[:, lead][:, px[:, None], ex[None, :]] = rec.ystate[("omg", r, a)][:, 0]
        out["y_sig_%d" % a] = ys
        out["y_psi_%d" % a] = yp
        out["y_omg_%d" % a] = yo
        out["h_%d" % a] = np.array(hh[a, 0])
    # start time of every attempt: t advances on acceptance by the step size the
    # controller proposes next (Zandpack/mpi/zand:396-407,427)
    t = w.t0
    tstart = []
    for h, TE, eps in rec.hnew:
        tstart.append(t)
        if TE < eps:
            t += 0.9 * h * (eps / TE) ** 0.2
    out["t_attempt"] = np.array(tstart)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("%s: %d attempts, %d accepted steps, t_end=%.6f -> %s (%.0f KB)" % (
        name, len(hh), len(sig), out["times"][-1], path, os.path.getsize(path) / 1024))


def make_pade():
    """Poles and residues of the reference's ``Hu_poles`` (PadeDecomp.py:151-152)
    for the pole counts the workloads use."""
    pd = refharness.reference_modules()["PadeDecomp"]
    out = {}
    for N in (2, 3, 20, 30, 40):
        z, c = pd.Hu_poles(N)
        out["z_%d" % N] = np.asarray(z)
        out["c_%d" % N] = np.asarray(c)
    np.savez_compressed(os.path.join(HERE, "hu_poles.npz"), **out)


if __name__ == "__main__":
    args = sys.argv[1:] or list(CASES) + ["pade"]
    for c in args:
        if c == "pade":
            make_pade()
        else:
            make_case(c)
