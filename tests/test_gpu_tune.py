"""The implementations of the mixed path's small products and dOmega/dt
(FP32 SIMT; products on the tensor cores; products and dOmega/dt in one
tensor-core launch; products and dOmega/dt in two tensor-core launches, the
second on the second stream) against the oracle on one right-hand side, and
the measured
choice (zg_tune).  Tolerance: the mixed path's per-RHS bar, 2e-5 of the
magnitude of the products each array is made of."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


@pytest.mark.parametrize("case", ["mini3", "c2"])
def test_every_implementation_against_oracle(case):
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.workloads import make_workload
    w = make_workload(case)
    L = CompactLayout(w.arrays, w.hbar)
    rng = np.random.default_rng(17)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 1e-2
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2 + np.asarray(w.arrays["DM_Ortho"])
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    t, h = 2.0, 0.02
    delta = [w.bias_fn()(t, a) for a in range(L.NL)]
    prob = zo.Problem(w.arrays, w.hbar)
    Ht = prob.H0 + w.dH_fn()(t, ys)
    ref = prob.rhs(h, ys, yp, yo, Ht, delta)[:3]
    scales = (np.abs(Ht[0] @ ys[0]).max() * h / w.hbar, np.abs(yp.reshape(-1, L.n) @ Ht[0].T).max() * h / w.hbar, 0.0)
    tr = Trajectory(w.arrays, w.hbar, precision="mixed", layout=L)
    tr.set_slot(tr.stages, y)
    _, avail = tr.get_impl()
    assert _lib.ZG_IMPL_SIMT in avail and _lib.ZG_IMPL_TC_PRODUCTS in avail
    outs = {}
    mode = _lib.ZG_DH_HUBBARD if w.hubbard_U is not None else _lib.ZG_DH_NONE
    for impl in avail:
        tr.set_impl(impl)
        tr.stage_input(0)
        tr.rhs(0, t, h, delta, mode, w.hubbard_U or 0.0)
        got = L.unpack(tr.get_slot(0))
        for name, g, r, sc in zip(("sigma", "psi", "Omega"), got, ref, scales):
            err = np.abs(g - r).max() / max(np.abs(r).max(), sc, 1e-300)
            print("\n%s %s %s: %.2e" % (case, _lib.IMPL_NAMES[impl], name, err))
            assert err < 2e-5, (case, impl, name, err)
        outs[impl] = tr.get_slot(0)
    for impl in avail:  # the early fork gives the same numbers
        tr.set_impl(impl)
        tr.set_schedule(_lib.ZG_SCHED_EARLY)
        tr.stage_input(0)
        tr.rhs(0, t, h, delta, mode, w.hubbard_U or 0.0)
        assert np.array_equal(tr.get_slot(0), outs[impl])
        tr.set_schedule(_lib.ZG_SCHED_LATE)
    (best, sched), times = tr.tune(3)
    print("\n%s tuned: %s/%s, ms per RHS %s" % (case, _lib.IMPL_NAMES[best], _lib.SCHED_NAMES[sched], times))
    assert best in avail and {i for i, _ in times} == set(avail)
    assert tr.get_impl()[0] == best and tr.get_schedule() == sched
    tr.close()
