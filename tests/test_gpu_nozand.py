"""Parity of the non-orthogonal-basis path (``nozand``) on the device.

* per-stage derivatives of recorded attempts against the unmodified
  reference ``nozand``'s own stage arrays at 1e-12 relative (FP64);
* a random dense state with a host dH matrix against the oracle at 1e-12;
* full adaptive runs against the reference (attempt sequence, time grid,
  final sigma', currents);
* the built-in Hubbard term equals the host dH callback, the graph-launched
  attempts equal host-driven ones, and the mixed path stays within 1e-6 of
  FP64 on sigma' and the currents.
"""
import numpy as np
import pytest

from conftest import golden_callbacks, load_golden

pytestmark = pytest.mark.gpu

RTOL_RHS = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from zandpack_gb300 import _lib
    _lib.lib()


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_nozand_stage_derivatives_match_reference(golden_nz):
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    case, z = golden_nz
    p = z["params"]
    bias, _ = golden_callbacks(p)
    for a in p["keep"]:
        ys, yp, yo = z["y_sig_%d" % a], z["y_psi_%d" % a], z["y_omg_%d" % a]
        tr = Trajectory(z, p["hbar"], psi0=yp, omg0=yo, nonorth=True)
        L = tr.layout
        tr.set_y(ys, yp, yo)
        h = float(z["h_%d" % a])
        t = float(z["t_attempt"][a])
        for i in range(7):
            tr.stage_input(i)
            ts = t + zo.A[i] * h
            delta = [bias(ts, l) for l in range(L.NL)]
            if p["hubbard_U"] is not None:
                tr.rhs(i, ts, h, delta, _lib.ZG_DH_HUBBARD, p["hubbard_U"])
            else:
                tr.rhs(i, ts, h, delta)
            ks, kp, ko = L.unpack(tr.get_slot(i))
            assert _rel(ks, z["ksig_%d" % a][i]) < RTOL_RHS, (case, a, i, "sig", _rel(ks, z["ksig_%d" % a][i]))
            assert _rel(kp, z["kpsi_%d" % a][i]) < RTOL_RHS, (case, a, i, "psi", _rel(kp, z["kpsi_%d" % a][i]))
            assert _rel(ko, z["komg_%d" % a][i]) < RTOL_RHS, (case, a, i, "omg", _rel(ko, z["komg_%d" % a][i]))
        tr.close()


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_nozand_rhs_against_oracle_random_state(golden_nz, precision):
    """Dense random state, host dH matrix (multiplied by S^-1 on the device):
    device k against the oracle at 1e-12 (FP64) or 1e-5 (mixed)."""
    from oracle import nozand_np as nz
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.nonorth import NonorthBasis
    case, z = golden_nz
    p = z["params"]
    prob = nz.NonorthProblem(z, p["hbar"])
    L = CompactLayout(NonorthBasis(z).arrays, p["hbar"])
    rng = np.random.default_rng(11)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    tr = Trajectory(z, p["hbar"], precision=precision, layout=L, nonorth=True)
    tr.set_slot(tr.stages, y)
    dHm = rng.standard_normal((L.n, L.n)) * 0.05
    dHm = (dHm + dHm.T).astype(complex)
    delta = rng.uniform(-0.3, 0.3, L.NL)
    h = 0.013
    tr.stage_input(0)
    tr.set_dH(dHm)
    J = tr.rhs(0, 0.1, h, delta, _lib.ZG_DH_MATRIX, 0.0, currents=True)
    ks, kp, ko, _, Jr = prob.rhs(h, ys, yp, yo, prob.H0 + dHm[None], delta)
    g = L.unpack(tr.get_slot(0))
    tol = RTOL_RHS if precision == "f64" else 1e-5
    for x, r, nm in zip(g, (ks, kp, ko), ("sig", "psi", "omg")):
        assert _rel(x, r) < tol, (nm, _rel(x, r))
    np.testing.assert_allclose(J, Jr[0], rtol=1e-11 if precision == "f64" else 1e-5, atol=1e-14)
    tr.close()


def test_nozand_trajectory_matches_reference(golden_nz):
    from zandpack_gb300.engine import Propagator
    case, z = golden_nz
    p = z["params"]
    bias, _ = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"], nonorth=True)
    pr.set_state(pr.traj.basis.sigma(z["DM_Ortho"]))
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"])
    TE = np.array(out["TE_hist"])
    assert len(TE) == len(z["TE_hist"])
    assert ((TE < p["eps"]) == (z["TE_hist"] < p["eps"])).all()
    np.testing.assert_allclose(TE, z["TE_hist"], rtol=1e-6)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-10)
    assert np.abs(out["sig"][-1] - z["sig_final"][0]).max() < 1e-11
    J = np.array(out["currents"]).T
    assert np.abs(J - z["currents"]).max() < 1e-10
    pr.traj.close()


def test_nozand_host_dH_callback_equals_device_hubbard():
    from zandpack_gb300.engine import Propagator
    z = load_golden("nz_mini2")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    outs = []
    for kw in (dict(hubbard_U=p["hubbard_U"]), dict(dH=dH)):
        pr = Propagator(z, p["hbar"], bias, nonorth=True, **kw)
        pr.set_state(pr.traj.basis.sigma(z["DM_Ortho"]))
        outs.append(pr.run(p["t0"], 0.3, p["stepsize"], p["eps"]))
        pr.traj.close()
    assert outs[0]["TE_hist"] == pytest.approx(outs[1]["TE_hist"], rel=1e-9)
    assert np.abs(outs[0]["sig"][-1] - outs[1]["sig"][-1]).max() < 1e-13


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_nozand_graph_attempts_equal_host_attempts(precision):
    """Graph-launched attempts (controller on the device) against host-driven
    zg_attempt, in the non-orthogonal basis (tolerances as in test_gpu_graph)."""
    import dataclasses
    from test_gpu_graph import _graph_run, _host_run, _rel
    from zandpack_gb300.engine import Trajectory, native_bias
    from zandpack_gb300.workloads import make_nonorth_workload
    w = dataclasses.replace(make_nonorth_workload("mini2"), t1=0.4)

    def fresh():
        tr = Trajectory(w.arrays, w.hbar, precision=precision, nonorth=True)
        tr.set_y(tr.basis.sigma(w.arrays["DM_Ortho"]))
        return tr
    tr = fresh()
    b = native_bias(w.bias, tr.layout.NL)
    hr, ht, hh = _host_run(tr, w, b)
    s_host = tr.get_sigma()
    tr.close()
    tr = fresh()
    gr, gt, gh = _graph_run(tr, w, b, 6)
    s_graph = tr.get_sigma()
    tr.close()
    assert len(gr) == len(hr) > 2
    assert [r[4] for r in gr] == [r[4] for r in hr]
    for a, g in zip(hr, gr):
        assert _rel(a[0], g[0]) <= 1e-9 and _rel(a[1], g[1]) <= 1e-9
        assert abs(a[2] - g[2]) <= 1e-6 * w.eps and _rel(a[3], g[3]) <= 1e-9
        assert np.abs(a[5] - g[5]).max() <= 1e-10
    assert np.abs(s_host - s_graph).max() <= 1e-10


def test_nozand_mixed_within_1e6_of_reference(golden_nz):
    """The mixed path on the reference nozand's own time grid (its step sizes
    replayed, its accept decisions forced): sigma' and the currents within
    1e-6 of the reference's FP64 trajectory."""
    from zandpack_gb300.engine import Propagator
    case, z = golden_nz
    p = z["params"]
    bias, _ = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"], precision="mixed", nonorth=True)
    pr.set_state(pr.traj.basis.sigma(z["DM_Ortho"]))
    acc = list(z["TE_hist"] < p["eps"])
    replay = np.concatenate([z["h_hist"], [z["times"][-1] - z["times"][-2]]])
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"], replay_h=replay, force_accept=acc)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-12)
    sig = np.array(out["sig"])[:, 0][z["sig_traj_idx"] + 1]
    dsig = np.abs(sig - z["sig_traj"][:, 0]).max()
    dJ = np.abs(np.array(out["currents"]).T - z["currents"]).max()
    print("\n%s mixed vs reference nozand: max|dsig| = %.2e, max|dJ| = %.2e" % (case, dsig, dJ))
    assert dsig <= 1e-6 and dJ <= 1e-6
    pr.traj.close()


@pytest.mark.parametrize("precision", ["f64", "mixed"])
@pytest.mark.parametrize("name", ["mini2", "mini3"])
def test_nozand_complex_overlap_against_oracle(name, precision):
    """A complex Hermitian overlap (S^-1 H(t) complex: the complex operand
    forms of the tensor-core products): one RHS from a dense random state with
    the Hubbard term on the device (mini2) or none (mini3), against the
    oracle (pinned to the reference nozand) at 1e-12 (FP64) / 1e-5 (mixed)."""
    from oracle import nozand_np as nz
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.nonorth import NonorthBasis
    from zandpack_gb300.workloads import make_nonorth_workload
    w = make_nonorth_workload(name, phases=True)
    prob = nz.NonorthProblem(w.arrays, w.hbar)
    assert np.abs(prob.Sm1.imag).max() > 1e-3
    L = CompactLayout(NonorthBasis(w.arrays).arrays, w.hbar)
    rng = np.random.default_rng(13)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    tr = Trajectory(w.arrays, w.hbar, precision=precision, layout=L, nonorth=True)
    tr.set_slot(tr.stages, y)
    delta = rng.uniform(-0.3, 0.3, L.NL)
    h = 0.011
    tr.stage_input(0)
    U = w.hubbard_U
    if U is not None:
        tr.rhs(0, 0.2, h, delta, _lib.ZG_DH_HUBBARD, U)
        dHm = w.dH_fn()(0.2, ys)
    else:
        tr.rhs(0, 0.2, h, delta)
        dHm = 0.0
    ks, kp, ko, _, _ = prob.rhs(h, ys, yp, yo, prob.H0 + dHm, delta)
    g = L.unpack(tr.get_slot(0))
    tol = RTOL_RHS if precision == "f64" else 1e-5
    for x, r, nm in zip(g, (ks, kp, ko), ("sig", "psi", "omg")):
        assert _rel(x, r) < tol, (nm, _rel(x, r))
    tr.close()


def test_overlap_switches_off_and_steady_state_refuses():
    """zg_set_overlap(NULL) returns a trajectory to the orthogonal equations
    (the same k as a trajectory that never had an overlap); the steady-state
    entry points refuse a trajectory with an overlap set."""
    import ctypes as C
    from zandpack_gb300 import _lib
    from zandpack_gb300._lib import ZGError, check, lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    z = load_golden("mini2")
    p = z["params"]
    L = CompactLayout(z, p["hbar"])
    rng = np.random.default_rng(17)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ks = []
    for switch in (False, True):
        tr = Trajectory(z, p["hbar"], layout=L)
        if switch:
            Sm1 = np.ascontiguousarray(np.eye(L.n, dtype=np.complex128) * 1.1)
            C0 = np.ascontiguousarray(np.ones((L.N, L.n), np.complex128))
            check(lib().zg_set_overlap(tr._h, Sm1.ctypes.data_as(C.c_void_p), C0.ctypes.data_as(C.c_void_p)))
            with pytest.raises(ZGError):
                check(lib().zg_stationary_setup(tr._h, 0.0, np.zeros(_lib.ZG_MAX_LEADS).ctypes.data_as(C.c_void_p),
                                                _lib.ZG_DH_NONE, 0.0, Sm1.ctypes.data_as(C.c_void_p),
                                                np.zeros(L.n).ctypes.data_as(C.c_void_p)))
            check(lib().zg_set_overlap(tr._h, None, None))
        tr.set_slot(tr.stages, y)
        tr.stage_input(0)
        tr.rhs(0, 0.1, 0.01, [0.1, -0.1], _lib.ZG_DH_HUBBARD, p["hubbard_U"])
        ks.append(tr.get_slot(0))
        tr.close()
    np.testing.assert_array_equal(ks[0], ks[1])
