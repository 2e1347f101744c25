"""Mixed-precision device path (3xTF32 tensor-core GEMMs, FP32 stage
arithmetic, FP64 state accumulation, error norm and currents) against the
FP64 reference.

Tolerances written here:
* one right-hand side: max-norm error <= 2e-5 per array (sigma, psi, Omega)
  relative to the larger of the result and the magnitude of the products it
  is made of (h/hbar |H sigma| for sigma, h/hbar |psi H^T| for psi), because
  near equilibrium H and sigma commute and k_sigma itself is roundoff;
* trajectories on the reference's own time grid (its step sizes replayed):
  max |delta sigma| <= 1e-6 and lead-current error <= 1e-6 at every
  recorded step, the mixed-precision bar of the target specification.
"""
import numpy as np
import pytest

from conftest import golden_callbacks, load_golden

pytestmark = pytest.mark.gpu

RTOL_RHS_MIXED = 2e-5
ATOL_TRAJ = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _rel(a, b, scale=0.0):
    return np.abs(a - b).max() / max(np.abs(b).max(), scale, 1e-300)


def _scales(h, hbar, Ht, sig, psi):
    """Magnitudes of the products inside k_sigma and k_psi."""
    hs = np.abs(Ht[0] @ sig[0]).max() * h / hbar
    hp = np.abs(psi.reshape(-1, Ht.shape[-1]) @ Ht[0].T).max() * h / hbar
    return hs, hp


@pytest.mark.parametrize("case", ["mini2", "mini3", "c1"])
def test_mixed_rhs_against_oracle(case):
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    z = load_golden(case)
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    for a in p["keep"]:
        ys, yp, yo = z["y_sig_%d" % a], z["y_psi_%d" % a], z["y_omg_%d" % a]
        tr = Trajectory(z, p["hbar"], precision="mixed", psi0=yp, omg0=yo)
        L = tr.layout
        tr.set_y(ys, yp, yo)
        h = float(z["h_%d" % a])
        t = float(z["t_attempt"][a])
        tr.stage_input(0)
        delta = [bias(t, l) for l in range(L.NL)]
        mode = _lib.ZG_DH_HUBBARD if p["hubbard_U"] is not None else _lib.ZG_DH_NONE
        J = tr.rhs(0, t, h, delta, mode, p["hubbard_U"] or 0.0, currents=True)
        Ht = prob.H0 + dH(t, ys)
        ks, kp, ko, _, Jr = prob.rhs(h, ys, yp, yo, Ht, delta)
        g = L.unpack(tr.get_slot(0))
        hs, hp = _scales(h, p["hbar"], Ht, ys, yp)
        assert _rel(g[0], ks, hs) < RTOL_RHS_MIXED, (case, a, "sig", _rel(g[0], ks, hs))
        assert _rel(g[1], kp, hp) < RTOL_RHS_MIXED, (case, a, "psi", _rel(g[1], kp, hp))
        if np.abs(ko).max() > 0:
            assert _rel(g[2], ko) < RTOL_RHS_MIXED, (case, a, "omg", _rel(g[2], ko))
        # stage-0 currents come from the FP64 state
        np.testing.assert_allclose(J, Jr[0], rtol=1e-11, atol=1e-15)
        tr.close()


@pytest.mark.parametrize("complex_dH", [False, True])
def test_mixed_rhs_random_dense_state(complex_dH):
    """All live entries nonzero and a dense host dH: mixed k vs oracle.  A
    real dH keeps H(t) real (the tensor-core products then skip Im H); a
    complex Hermitian dH takes the complex form of both products."""
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    z = load_golden("mini3")
    p = z["params"]
    prob = zo.Problem(z, p["hbar"])
    L = CompactLayout(z, p["hbar"])
    rng = np.random.default_rng(3)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    tr = Trajectory(z, p["hbar"], precision="mixed", layout=L)
    tr.set_slot(tr.stages, y)
    dHm = rng.standard_normal((L.n, L.n)) * 0.05
    if complex_dH:
        dHm = dHm + 1j * rng.standard_normal((L.n, L.n)) * 0.05
    dHm = ((dHm + dHm.conj().T) / 2).astype(complex)
    assert complex_dH == bool(np.abs(dHm.imag).max() > 0)
    delta = rng.uniform(-0.3, 0.3, L.NL)
    tr.stage_input(0)
    tr.set_dH(dHm)
    tr.rhs(0, 0.1, 0.013, delta, _lib.ZG_DH_MATRIX, 0.0)
    Ht = prob.H0 + dHm[None]
    ks, kp, ko, _, _ = prob.rhs(0.013, ys, yp, yo, Ht, delta)
    g = L.unpack(tr.get_slot(0))
    hs, hp = _scales(0.013, p["hbar"], Ht, ys, yp)
    for x, r, sc in zip(g, (ks, kp, ko), (hs, hp, 0.0)):
        assert _rel(x, r, sc) < RTOL_RHS_MIXED
    tr.close()


def test_mixed_vs_f64_at_n1024():
    """The n = 1024 workload (32x32 lattice, Hubbard dH, 4480 live modes):
    the FP64 device path, whose per-RHS parity with the reference is tested
    above, sets the time grid for 8 attempts; the mixed path replays it and
    sigma and the currents must stay within 1e-6 at every step."""
    from zandpack_gb300.engine import Propagator
    from zandpack_gb300.workloads import make_workload
    w = make_workload("c3")
    runs = {}
    for prec in ("f64", "mixed"):
        pr = Propagator(w.arrays, w.hbar, w.bias_fn(), hubbard_U=w.hubbard_U, precision=prec)
        pr.set_state(w.arrays["DM_Ortho"])
        if prec == "f64":
            out = pr.run(w.t0, 1e9, 0.05, w.eps, max_attempts=8)
        else:
            ref = runs["f64"]
            replay = list(ref["h_hist"]) + [ref["times"][-1] - ref["times"][-2]]
            out = pr.run(w.t0, ref["times"][-1] - 1e-12, 0.05, w.eps, replay_h=replay,
                         force_accept=ref["accepted"])
        runs[prec] = out
        pr.traj.close()
    a, b = runs["f64"], runs["mixed"]
    k = min(len(a["sig"]), len(b["sig"]))
    assert k >= 3
    dsig = max(np.abs(a["sig"][i] - b["sig"][i]).max() for i in range(k))
    m = min(len(a["currents"]), len(b["currents"]))
    dJ = max(np.abs(np.asarray(a["currents"][i]) - np.asarray(b["currents"][i])).max() for i in range(m))
    print("\nn=1024 mixed vs FP64 over %d steps: max|dsig| = %.2e, max|dJ| = %.2e" % (k - 1, dsig, dJ))
    assert dsig <= ATOL_TRAJ and dJ <= ATOL_TRAJ


@pytest.mark.parametrize("case", ["mini2", "mini3", "c1"])
def test_mixed_trajectory_on_reference_grid(case):
    """Replay the reference's step sizes; sigma and currents stay within 1e-6
    of the reference's FP64 run at every accepted step."""
    from zandpack_gb300.engine import Propagator
    z = load_golden(case)
    p = z["params"]
    bias, dH = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"], precision="mixed")
    pr.set_state(z["DM_Ortho"])
    # replaying h and forcing the reference's accept decisions reproduces its grid
    acc = list(z["TE_hist"] < p["eps"])
    replay = np.concatenate([z["h_hist"], [z["times"][-1] - z["times"][-2]]])
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"], replay_h=replay, force_accept=acc)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-12)
    sig = np.array(out["sig"])[:, 0][z["sig_traj_idx"] + 1]
    dsig = np.abs(sig - z["sig_traj"][:, 0]).max()
    J = np.array(out["currents"]).T
    dJ = np.abs(J - z["currents"]).max()
    print("\n%s mixed vs reference: max|dsig| = %.2e, max|dJ| = %.2e over %d steps" % (case, dsig, dJ, J.shape[1]))
    assert dsig <= ATOL_TRAJ
    assert dJ <= ATOL_TRAJ
    pr.traj.close()


def test_h_operands_after_a_full_dH_matrix():
    """The mixed path builds H0's tensor-core operands once and then rebuilds
    only their diagonal (Hubbard term); a stage with a full dH matrix
    overwrites them.  A Hubbard stage or a graph attempt that follows must
    give exactly what a fresh trajectory gives."""
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory, native_bias
    from zandpack_gb300.workloads import make_workload
    w = make_workload("mini2")
    U = w.hubbard_U
    trA = Trajectory(w.arrays, w.hbar, precision="mixed")
    trB = Trajectory(w.arrays, w.hbar, precision="mixed")
    n = trA.layout.n
    rng = np.random.default_rng(3)
    D = rng.standard_normal((n, n)) * 0.05
    D = (D + D.T).astype(complex)
    delta = [0.1, -0.1]
    for tr in (trA, trB):
        tr.set_y(w.arrays["DM_Ortho"])
    trA.stage_input(0)
    trA.set_dH(D)
    trA.rhs(0, 0.0, 0.02, delta, _lib.ZG_DH_MATRIX)
    for tr in (trA, trB):
        tr.stage_input(0)
        tr.rhs(0, 0.0, 0.02, delta, _lib.ZG_DH_HUBBARD, U)
    assert np.array_equal(trA.get_slot(0), trB.get_slot(0))
    trA.stage_input(0)
    trA.rhs(0, 0.0, 0.02, delta, _lib.ZG_DH_MATRIX)  # operands hold dH again
    b = native_bias(w.bias, trA.layout.NL)
    out = []
    for tr in (trA, trB):
        tr.graph_prepare(b, U)
        tr.graph_set(w.t0, w.stepsize, w.eps, w.t1)
        recs, _, _, _ = tr.graph_run(2)
        out.append([r[2] for r in recs])
        tr.close()
    assert out[0] == out[1] and len(out[0]) == 2


def test_mixed_c1_full_span_on_reference_grid():
    """The n=20 chain over 0-50 fs on the reference's own time grid (its
    5414 step sizes replayed): the mixed-precision path stays within 1e-6 of
    the unmodified ``zand`` in sigma and in the lead currents at every step,
    the final time included."""
    import os
    from conftest import GOLDEN
    from zandpack_gb300.engine import Propagator
    if not os.path.exists(os.path.join(GOLDEN, "c1_50fs.npz")):
        pytest.skip("fixture c1_50fs missing")
    z = load_golden("c1_50fs")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"], precision="mixed")
    pr.set_state(z["DM_Ortho"])
    acc = list(z["TE_hist"] < p["eps"])
    replay = np.concatenate([z["h_hist"], [z["times"][-1] - z["times"][-2]]])
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"], replay_h=replay, force_accept=acc)
    pr.traj.close()
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-10)
    sig = np.array(out["sig"])[:, 0][z["sig_traj_idx"] + 1]
    dsig = np.abs(sig - z["sig_traj"][:, 0]).max()
    dfin = np.abs(out["sig"][-1] - z["sig_final"][0]).max()
    J = np.array(out["currents"]).T
    dJ = np.abs(J - z["currents"]).max()
    dJfin = np.abs(J[:, -1] - z["currents"][:, -1]).max()
    print("\nc1 0-50 fs mixed vs reference: max|dsig| %.2e (final %.2e), max|dJ| %.2e (final %.2e)"
          % (dsig, dfin, dJ, dJfin))
    assert max(dsig, dfin) <= ATOL_TRAJ and dJ <= ATOL_TRAJ
