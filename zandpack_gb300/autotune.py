"""Measured choice of kernels per trajectory class, kept across runs.

The mixed-precision path can compute its small complex products (the PI
partials, Omega xi, xi sigma^T) and dOmega/dt with FP32 SIMT kernels, with the
products on the tensor cores, or with both on the tensor cores in one or two
launches (``zg_set_impl``), and fork its second stream before or after psi H^T
(``zg_set_schedule``).  Which is fastest depends on the shapes (orbitals n, modes
N, sourced modes Ns, coupling width n_c, leads) and on the GPU, so it is
measured: ``zg_tune`` times one right-hand side of each, and the winner is
stored in a JSON file keyed by those shapes and the device name, so that later
trajectories of the same class (the serving loop admits many) reuse it without
measuring again.

The file is ``$ZG_TUNE_CACHE`` if set, else ``~/.cache/zandpack_gb300/tune.json``.
"""
from __future__ import annotations

import json
import os
import tempfile
import threading

from . import _lib

_MEM = {}
# one measurement at a time in this process (the serving loop tunes from its
# worker threads): a class is measured once, and the file is rewritten whole
_LOCK = threading.Lock()


def cache_path():
    p = os.environ.get("ZG_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "zandpack_gb300", "tune.json")


def class_key(layout, precision, device_name, coarse=False):
    """Key of a trajectory class: the shapes that decide the kernels' work.
    ``coarse``: orbitals, coupling width and leads only (the mode counts N and
    Ns left out), so that requests that differ only in their pole counts
    share one measurement."""
    L = layout
    if coarse:
        return "%s|%s|n=%d|nc=%d|L=%d|coarse" % (device_name, precision, L.n, L.nc, L.NL)
    return "%s|%s|n=%d|N=%d|Ns=%d|nc=%d|L=%d" % (device_name, precision, L.n, L.N, L.Ns, L.nc, L.NL)


def _load(path):
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(path, key, entry):
    d = _load(path)
    d[key] = entry
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    fd, tmp = tempfile.mkstemp(prefix=".tune", dir=os.path.dirname(os.path.abspath(path)))
    with os.fdopen(fd, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def device_name(device=0):
    import torch
    return torch.cuda.get_device_name(device).replace("|", "/")


def _name(impl, sched):
    return "%s/%s" % (_lib.IMPL_NAMES[impl], _lib.SCHED_NAMES[sched])


def _parse(name):
    impl, sched = name.split("/")
    return _lib.IMPL_NAMES.index(impl), _lib.SCHED_NAMES.index(sched)


def choose(traj, device=0, reps=5, path=None, retune=False, coarse=False):
    """Set the trajectory's kernels and stream schedule from the cache,
    measuring (and storing) the class's choice first when it is not there.
    ``coarse`` keys the class by orbitals, coupling width and leads only.
    Returns the entry: {"impl": "<kernels>/<schedule>", "ms": {name: ms per
    RHS}, "measured": bool}."""
    if traj.precision != "mixed":
        return {"impl": _name(_lib.ZG_IMPL_SIMT, _lib.ZG_SCHED_LATE), "ms": {}, "measured": False}
    path = path or cache_path()
    key = class_key(traj.layout, traj.precision, device_name(device), coarse)
    _, avail = traj.get_impl()
    with _LOCK:
        entry = None if retune else (_MEM.get(key) or _load(path).get(key))
        if entry is not None:
            try:
                impl, sched = _parse(entry["impl"])
            except (ValueError, KeyError):
                impl = -1
            if impl in avail:
                traj.set_impl(impl)
                traj.set_schedule(sched)
                _MEM[key] = entry
                return dict(entry, measured=False)
        (impl, sched), times = traj.tune(reps)
        entry = {"impl": _name(impl, sched), "ms": {_name(i, s): m for (i, s), m in sorted(times.items())}}
        _MEM[key] = entry
        try:
            _store(path, key, entry)
        except OSError:
            pass  # a read-only home: the choice still holds for this process
    return dict(entry, measured=True)
