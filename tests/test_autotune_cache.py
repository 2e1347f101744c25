"""The tuning cache (zandpack_gb300.autotune) on the CPU, with a stand-in
trajectory: the first trajectory of a class is measured and the choice
stored, later ones reuse it, a stored choice the trajectory cannot run is
measured again, and FP64 trajectories are never measured."""
import json
import types

from zandpack_gb300 import _lib, autotune


class _FakeTraj:
    def __init__(self, avail, best, precision="mixed"):
        self.precision = precision
        self.layout = types.SimpleNamespace(n=64, N=300, Ns=40, nc=8, NL=2)
        self.avail = avail
        self.best = best
        self.impl = _lib.ZG_IMPL_SIMT
        self.sched = _lib.ZG_SCHED_LATE
        self.tuned = 0

    def get_impl(self):
        return self.impl, list(self.avail)

    def set_impl(self, i):
        assert i in self.avail
        self.impl = i

    def set_schedule(self, s):
        self.sched = s

    def tune(self, reps=5):
        self.tuned += 1
        self.impl, self.sched = self.best, _lib.ZG_SCHED_EARLY
        return (self.best, _lib.ZG_SCHED_EARLY), {(i, s): 1.0 for i in self.avail for s in (0, 1)}


def test_measure_once_then_reuse(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "device_name", lambda device=0: "GB300")
    monkeypatch.setattr(autotune, "_MEM", {})
    path = str(tmp_path / "tune.json")
    a = _FakeTraj([0, 1, 2], best=2)
    e = autotune.choose(a, path=path)
    assert e["measured"] and e["impl"] == "tc_all/early" and a.tuned == 1
    stored = json.load(open(path))
    key = autotune.class_key(a.layout, "mixed", "GB300")
    assert stored[key]["impl"] == "tc_all/early"
    monkeypatch.setattr(autotune, "_MEM", {})  # a new process reads the file
    b = _FakeTraj([0, 1, 2], best=0)
    e = autotune.choose(b, path=path)
    assert not e["measured"] and b.tuned == 0 and b.impl == _lib.ZG_IMPL_TC_ALL
    assert b.sched == _lib.ZG_SCHED_EARLY
    # a class member that cannot run the stored choice is measured again
    c = _FakeTraj([0, 1], best=1)
    e = autotune.choose(c, path=path)
    assert e["measured"] and c.impl == 1


def test_fp64_is_not_measured(tmp_path):
    t = _FakeTraj([0], best=0, precision="f64")
    e = autotune.choose(t, path=str(tmp_path / "t.json"))
    assert t.tuned == 0 and not e["measured"]


def test_coarse_classes_share_one_measurement(tmp_path, monkeypatch):
    """Requests that differ only in their mode counts share a coarse class
    (the serving loop's default) and are measured apart in the full one."""
    monkeypatch.setattr(autotune, "device_name", lambda device=0: "GB300")
    monkeypatch.setattr(autotune, "_MEM", {})
    path = str(tmp_path / "tune.json")
    a = _FakeTraj([0, 1, 2], best=1)
    b = _FakeTraj([0, 1, 2], best=2)
    b.layout = types.SimpleNamespace(n=64, N=420, Ns=56, nc=8, NL=2)
    assert autotune.choose(a, path=path, coarse=True)["measured"]
    e = autotune.choose(b, path=path, coarse=True)
    assert not e["measured"] and b.tuned == 0 and b.impl == 1
    e = autotune.choose(b, path=path)
    assert e["measured"] and b.impl == 2
    keys = set(json.load(open(path)))
    assert keys == {autotune.class_key(a.layout, "mixed", "GB300", coarse=True),
                    autotune.class_key(b.layout, "mixed", "GB300")}
