"""Graph-launched attempts (zg_graph_*) against the host-driven zg_attempt.

Both run the same kernels on the same data; the graph keeps the controller
(t, h, TE, accept, next step size) and the bias on the device, where pow, exp,
sin and tanh may round differently from the host's libm in the last place.  So
the accept sequence must be identical; times and step sizes must agree to 1e-9
(relative), currents and the final sigma to 1e-10 (absolute), and error norms
to 1e-6 eps (absolute: TE is a difference of two nearly equal solutions, so
its relative rounding differences are amplified, while accept decisions only
see TE against eps).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_run(tr, w, b):
    t, h = w.t0, w.stepsize
    recs = []
    while t < w.t1:
        t_prev, h_prev = t, h
        TE, acc, t, h, J = tr.attempt_native(t, h, w.eps, b, w.hubbard_U)
        recs.append((t_prev, h_prev, TE, h, acc, J))
    return recs, t, h


def _graph_run(tr, w, b, batch):
    tr.graph_prepare(b, w.hubbard_U)
    tr.graph_set(w.t0, w.stepsize, w.eps, w.t1)
    recs, done = [], False
    while not done:
        r, t, h, done = tr.graph_run(batch)
        recs += [(x[0], x[1], x[2], x[3], x[4], x[6]) for x in r]
    return recs, t, h


def _fresh(w, precision):
    from zandpack_gb300.engine import Trajectory
    tr = Trajectory(w.arrays, w.hbar, precision=precision)
    tr.set_y(w.arrays["DM_Ortho"])
    return tr


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("name,precision,batch", [("mini2", "f64", 5), ("mini2", "mixed", 64),
                                                  ("c4", "mixed", 7), ("c4", "f64", 3)])
def test_graph_equals_host_attempts(name, precision, batch):
    from zandpack_gb300.engine import native_bias
    from zandpack_gb300.workloads import c4_requests, c4_workload, make_workload
    if name == "c4":
        req = [r for r in c4_requests(40, seed=5, t_span=0.4) if r["n"] == 64][0]
        w = c4_workload(req)
    else:
        w = make_workload(name)
    tr = _fresh(w, precision)
    b = native_bias(w.bias, tr.layout.NL)
    hr, ht, hh = _host_run(tr, w, b)
    s_host = tr.get_sigma()
    tr.close()
    tr = _fresh(w, precision)
    gr, gt, gh = _graph_run(tr, w, b, batch)
    s_graph = tr.get_sigma()
    tr.close()
    assert len(gr) == len(hr) > 2
    assert [r[4] for r in gr] == [r[4] for r in hr]
    for a, g in zip(hr, gr):
        assert _rel(a[0], g[0]) <= 1e-9 and _rel(a[1], g[1]) <= 1e-9
        assert abs(a[2] - g[2]) <= 1e-6 * w.eps and _rel(a[3], g[3]) <= 1e-9
        assert np.abs(a[5] - g[5]).max() <= 1e-10
    assert _rel(ht, gt) <= 1e-9 and _rel(hh, gh) <= 1e-9
    assert np.abs(s_host - s_graph).max() <= 1e-10


def test_graph_batches_past_the_end_change_nothing():
    """Attempts launched after t >= t1 are skipped on the device: one large
    batch gives the same records and state as single-attempt batches."""
    from zandpack_gb300.engine import native_bias
    from zandpack_gb300.workloads import make_workload
    w = make_workload("mini3")
    out = []
    for batch in (1, 200):
        tr = _fresh(w, "f64")
        b = native_bias(w.bias, tr.layout.NL)
        recs, t, h = _graph_run(tr, w, b, batch)
        out.append((recs, t, h, tr.get_sigma()))
        tr.close()
    (r1, t1, h1, s1), (r2, t2, h2, s2) = out
    assert len(r1) == len(r2) and t1 == t2 and h1 == h2
    assert all(a[:5] == b[:5] and np.array_equal(a[5], b[5]) for a, b in zip(r1, r2))
    assert np.array_equal(s1, s2)


def test_graph_counts_launches_and_recaptures_after_profile():
    """Each graph launch adds the captured kernel count to zg_launch_count;
    switching profiling on drops the graph and the next run captures it again
    with event nodes, whose regions are then reported."""
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import native_bias
    from zandpack_gb300.workloads import make_workload
    w = make_workload("mini2")
    tr = _fresh(w, "mixed")
    b = native_bias(w.bias, tr.layout.NL)
    tr.graph_prepare(b, w.hubbard_U)
    tr.graph_set(w.t0, w.stepsize, w.eps, w.t1)
    c0 = _lib.lib().zg_launch_count()
    tr.graph_run(1)
    per_attempt = _lib.lib().zg_launch_count() - c0
    assert per_attempt > 7 * 5
    c0 = _lib.lib().zg_launch_count()
    tr.graph_run(3)
    assert _lib.lib().zg_launch_count() - c0 == 3 * per_attempt
    import ctypes as C
    _lib.check(_lib.lib().zg_profile(tr._h, 1))
    recs, _, _, _ = tr.graph_run(2)
    ms = np.zeros(len(_lib.PROF_REGIONS))
    cnt = np.zeros(ms.size, np.int64)
    _lib.check(_lib.lib().zg_profile_read(tr._h, ms.ctypes.data_as(C.c_void_p), cnt.ctypes.data_as(C.c_void_p)))
    assert cnt[6] == 7 and ms[6] > 0.0  # the RHS region of the last attempt
    tr.close()
