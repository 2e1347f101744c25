"""The dissipator term of the sigma equation, - hbar * dissipator(ts, sigma)
(Zandpack/mpi/zand:343), on the device against the oracle: per right-hand
side at 1e-12 (FP64 path), over a short adaptive run (same attempts, TE to
1e-9 relative, sigma to 1e-11), and the mixed path on the FP64 run's time grid
to 1e-6 in sigma at every step.  The dissipator is a sigma-dependent dephasing
gamma * (sigma - diag(sigma)), evaluated at every stage as the reference does.
"""
import numpy as np
import pytest

from conftest import golden_callbacks, load_golden

pytestmark = pytest.mark.gpu

GAMMA = 0.05


def dephasing(t, sig):
    s = np.asarray(sig)
    d = np.einsum("...ii->...i", s)
    out = s.copy()
    i = np.arange(s.shape[-1])
    out[..., i, i] -= d
    return GAMMA * (1.0 + 0.1 * np.sin(t)) * out


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_rhs_with_dissipator_matches_oracle():
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    z = load_golden("mini2")
    p = z["params"]
    prob = zo.Problem(z, p["hbar"])
    L = CompactLayout(z, p["hbar"])
    rng = np.random.default_rng(17)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    tr = Trajectory(z, p["hbar"], layout=L)
    tr.set_slot(tr.stages, y)
    delta = rng.uniform(-0.3, 0.3, L.NL)
    h, ts = 0.021, 0.37
    D = dephasing(ts, ys)
    tr.stage_input(0)
    tr.set_dissipator(D)
    tr.rhs(0, ts, h, delta)
    tr.set_dissipator(None)
    ks, kp, ko, _, _ = prob.rhs(h, ys, yp, yo, prob.H0, delta, D)
    g = L.unpack(tr.get_slot(0))
    for x, r in zip(g, (ks, kp, ko)):
        assert _rel(x, r) < 1e-12
    # and the term is really there: without it sigma's derivative differs
    tr.stage_input(0)
    tr.rhs(0, ts, h, delta)
    assert _rel(L.unpack(tr.get_slot(0))[0], ks) > 1e-6
    tr.close()


def _device_run(z, p, precision, t1, **replay):
    from zandpack_gb300.engine import Propagator
    bias, _ = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, dissipator=dephasing, hubbard_U=p["hubbard_U"], precision=precision)
    pr.set_state(z["DM_Ortho"])
    out = pr.run(p["t0"], t1, p["stepsize"], p["eps"], **replay)
    pr.traj.close()
    return out


def test_adaptive_run_with_dissipator_matches_oracle():
    from oracle import zand_np as zo
    z = load_golden("mini2")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    t1 = 0.9
    prob = zo.Problem(z, p["hbar"])
    ref = zo.propagate(prob, p["t0"], t1, p["stepsize"], p["eps"], bias, dH,
                       state=(np.asarray(z["DM_Ortho"]), None, None), dissipator=dephasing)
    out = _device_run(z, p, "f64", t1)
    assert len(out["TE_hist"]) == len(ref["TE_hist"]) > 2
    np.testing.assert_allclose(out["TE_hist"], ref["TE_hist"], rtol=1e-9)
    np.testing.assert_allclose(out["times"], ref["times"], rtol=0, atol=1e-10)
    assert np.abs(out["sig"][-1] - ref["sig"][-1][0]).max() < 1e-11
    # mixed precision on the FP64 run's time grid (its step sizes and accept decisions)
    replay_h = np.concatenate([out["h_hist"], [out["times"][-1] - out["times"][-2]]])
    mixed = _device_run(z, p, "mixed", t1, replay_h=replay_h, force_accept=out["accepted"])
    np.testing.assert_allclose(mixed["times"], out["times"], rtol=0, atol=1e-12)
    for a, b in zip(mixed["sig"], out["sig"]):
        assert np.abs(a - b).max() < 1e-6


def test_attempt_paths_refuse_a_set_dissipator():
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory, native_bias
    from zandpack_gb300.workloads import make_workload
    w = make_workload("mini3")
    tr = Trajectory(w.arrays, w.hbar)
    tr.set_y(w.arrays["DM_Ortho"])
    b = native_bias(w.bias, tr.layout.NL)
    tr.set_dissipator(np.eye(tr.layout.n) * 0.01)
    with pytest.raises(_lib.ZGInvalid):
        tr.attempt_native(0.0, 0.1, w.eps, b)
    with pytest.raises(_lib.ZGInvalid):
        tr.graph_prepare(b)
    tr.set_dissipator(None)
    tr.attempt_native(0.0, 0.1, w.eps, b)
    tr.close()
