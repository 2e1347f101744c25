"""The device path beside the oracle at the workloads the metric is quoted on.

* One right-hand side of the n=256 ribbon (c2) and of the n=1024 lattice with
  the Hubbard dH(sigma) (c3), on a random dense state, against
  ``oracle.zand_np.Problem.rhs`` in the reference's padded layout.  These
  shapes take the large-problem code paths (split-K GEMM batches, multi-wave
  grids, 256-wide tensor-core tiles) that the small golden cases never reach.
  Tolerances: FP64 1e-12 relative (max norm per array, the per-RHS bar of the
  plain FP64 GPU path); mixed 2e-5 of the magnitude of the products each
  array is made of (h/hbar |H sigma|, h/hbar |psi H^T|), the per-RHS bar of the
  mixed path; stage-0 currents 1e-11 (both precisions compute them from the
  FP64 state).
* Trajectories, mixed against FP64 on the FP64 path's own time grid: c2 over
  its first 40 attempts and c3 over 10 fs (half a period of its 0.05 fs^-1
  sinusoidal bias, about 300 attempts).  Bar: max |delta sigma| <= 1e-6 and
  lead-current error <= 1e-6 at every step, the target specification's bar.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_RHS_F64 = 1e-12
RTOL_RHS_MIXED = 2e-5
ATOL_TRAJ = 1e-6

_ORACLE = {}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _rel(a, b, scale=0.0):
    return np.abs(a - b).max() / max(np.abs(b).max(), scale, 1e-300)


def _case(case):
    """Workload, compact layout, a seeded random dense state and the oracle's
    k for it (computed once per case)."""
    if case in _ORACLE:
        return _ORACLE[case]
    from oracle import zand_np as zo
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.workloads import make_workload
    w = make_workload(case)
    L = CompactLayout(w.arrays, w.hbar)
    rng = np.random.default_rng(11)
    y = ((rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 1e-2).astype(np.complex128)
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2 + np.asarray(w.arrays["DM_Ortho"])
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    t, h = 3.0, 0.02
    delta = [w.bias_fn()(t, a) for a in range(L.NL)]
    prob = zo.Problem(w.arrays, w.hbar)
    Ht = prob.H0 + w.dH_fn()(t, ys)
    ks, kp, ko, _, J = prob.rhs(h, ys, yp, yo, Ht, delta)
    hs = np.abs(Ht[0] @ ys[0]).max() * h / w.hbar
    hp = np.abs(yp.reshape(-1, L.n) @ Ht[0].T).max() * h / w.hbar
    del prob
    _ORACLE[case] = dict(w=w, L=L, y=y, t=t, h=h, delta=delta, k=(ks, kp, ko), J=J[0], scales=(hs, hp, 0.0))
    return _ORACLE[case]


@pytest.mark.parametrize("prec", ["f64", "mixed"])
@pytest.mark.parametrize("case", ["c2", "c3"])
def test_rhs_against_oracle_at_scale(case, prec):
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    c = _case(case)
    w, L = c["w"], c["L"]
    tr = Trajectory(w.arrays, w.hbar, precision=prec, layout=L)
    tr.set_slot(tr.stages, c["y"])
    tr.stage_input(0)
    if w.hubbard_U is not None:
        J = tr.rhs(0, c["t"], c["h"], c["delta"], _lib.ZG_DH_HUBBARD, w.hubbard_U, currents=True)
    else:
        J = tr.rhs(0, c["t"], c["h"], c["delta"], currents=True)
    got = L.unpack(tr.get_slot(0))
    tr.close()
    for name, g, r, sc in zip(("sigma", "psi", "Omega"), got, c["k"], c["scales"]):
        if prec == "f64":
            err = _rel(g, r)
            assert err < RTOL_RHS_F64, (case, prec, name, err)
        else:
            err = _rel(g, r, sc)
            assert err < RTOL_RHS_MIXED, (case, prec, name, err)
        print("\n%s %s %s: %.2e" % (case, prec, name, err))
    np.testing.assert_allclose(J, c["J"], rtol=1e-11, atol=1e-14)


def _mixed_vs_f64(case, t_end=None, attempts=None):
    """FP64 and mixed trajectories in lockstep: the FP64 path's error norm
    decides every accept and step size, the mixed path takes the same steps,
    and sigma and the stage-0 currents are compared after every accepted
    step."""
    from zandpack_gb300.engine import Propagator
    from zandpack_gb300.workloads import make_workload
    w = make_workload(case)
    pf, pm = (Propagator(w.arrays, w.hbar, w.bias_fn(), hubbard_U=w.hubbard_U, precision=p) for p in ("f64", "mixed"))
    for pr in (pf, pm):
        pr.set_state(w.arrays["DM_Ortho"])
    t, h = w.t0, w.stepsize
    t_end = 1e9 if t_end is None else t_end
    steps, tried, dsig, dJ = 0, 0, [], []
    while t < t_end and (attempts is None or tried < attempts):
        TEf, Jf, _ = pf.attempt(t, h)
        _, Jm, _ = pm.attempt(t, h)
        tried += 1
        h_next = pf.tab.hnew(h, TEf, w.eps)
        if TEf < w.eps:
            pf.step_fourth()
            pm.step_fourth()
            t += h_next
            steps += 1
            dJ.append(np.abs(np.asarray(Jf) - np.asarray(Jm)).max())
            dsig.append(np.abs(pf.get_sigma() - pm.get_sigma()).max())
        h = h_next
    for pr in (pf, pm):
        pr.traj.close()
    print("\n%s mixed vs FP64 over %d steps (%d attempts) to t = %.3f fs: max|dsig| = %.2e (final %.2e), "
          "max|dJ| = %.2e (final %.2e)" % (case, steps, tried, t, max(dsig), dsig[-1], max(dJ), dJ[-1]))
    return steps, dsig, dJ


def test_c2_mixed_vs_f64_trajectory():
    k, dsig, dJ = _mixed_vs_f64("c2", attempts=40)
    assert k >= 10
    assert max(dsig) <= ATOL_TRAJ and max(dJ) <= ATOL_TRAJ


def test_c3_mixed_vs_f64_over_10fs():
    k, dsig, dJ = _mixed_vs_f64("c3", t_end=10.0)
    assert k >= 100
    assert max(dsig) <= ATOL_TRAJ and max(dJ) <= ATOL_TRAJ
