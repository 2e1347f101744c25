"""Parity of the device path (libzandgpu, FP64) with the reference.

* per-stage derivatives of recorded attempts against the reference's own
  stage arrays (golden fixtures) at 1e-12 relative (max-norm per array), the
  tolerance the plain FP64 GPU path must meet per RHS call;
* full adaptive runs: same attempt count and accept/reject sequence, the
  reference's time grid, final sigma and lead currents;
* the array kernels behind the ``func_step_forward``/``mpi_funcs`` names
  against the oracle, including empty and ragged sizes.
"""
import numpy as np
import pytest

from conftest import golden_callbacks

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


def test_stage_derivatives_match_reference(golden):
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    case, z = golden
    p = z["params"]
    bias, dH = golden_callbacks(p)
    for a in p["keep"]:
        ys, yp, yo = z["y_sig_%d" % a], z["y_psi_%d" % a], z["y_omg_%d" % a]
        tr = Trajectory(z, p["hbar"], psi0=yp, omg0=yo)
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
            assert _rel(ks, z["ksig_%d" % a][i]) < RTOL_RHS, (case, a, i, "sig")
            assert _rel(kp, z["kpsi_%d" % a][i]) < RTOL_RHS, (case, a, i, "psi")
            assert _rel(ko, z["komg_%d" % a][i]) < RTOL_RHS, (case, a, i, "omg")
        tr.close()


def test_rhs_against_oracle_random_state(golden):
    """A dense random state (all live entries nonzero) and a host dH matrix:
    device k against the oracle's k at 1e-12."""
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    case, z = golden
    p = z["params"]
    prob = zo.Problem(z, p["hbar"])
    L = CompactLayout(z, p["hbar"])
    rng = np.random.default_rng(7)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2
    y = L.pack(ys, yp, yo)
    ys, yp, yo = L.unpack(y)
    tr = Trajectory(z, p["hbar"], layout=L)
    tr.set_slot(tr.stages, y)
    dHm = rng.standard_normal((L.n, L.n)) * 0.05
    dHm = (dHm + dHm.T).astype(complex)
    delta = rng.uniform(-0.3, 0.3, L.NL)
    h = 0.013
    tr.stage_input(0)
    tr.set_dH(dHm)
    J = tr.rhs(0, 0.1, h, delta, _lib.ZG_DH_MATRIX, 0.0, currents=True)
    ks, kp, ko, PI, Jr = prob.rhs(h, ys, yp, yo, prob.H0 + dHm[None], delta)
    g = L.unpack(tr.get_slot(0))
    for x, r in zip(g, (ks, kp, ko)):
        assert _rel(x, r) < RTOL_RHS
    np.testing.assert_allclose(J, Jr[0], rtol=1e-11, atol=1e-14)
    tr.close()


def test_trajectory_matches_reference(golden):
    from zandpack_gb300.engine import Propagator
    case, z = golden
    p = z["params"]
    bias, dH = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"])
    pr.set_state(z["DM_Ortho"])
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


def test_host_dH_callback_path():
    """The host-callback tier (sigma downloaded, dH(t, sigma) evaluated in
    Python, uploaded) gives the same trajectory as the built-in Hubbard term."""
    from conftest import load_golden
    from zandpack_gb300.engine import Propagator
    z = load_golden("mini2")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    outs = []
    for kw in (dict(hubbard_U=p["hubbard_U"]), dict(dH=dH)):
        pr = Propagator(z, p["hbar"], bias, **kw)
        pr.set_state(z["DM_Ortho"])
        outs.append(pr.run(p["t0"], 0.3, p["stepsize"], p["eps"]))
        pr.traj.close()
    assert outs[0]["TE_hist"] == pytest.approx(outs[1]["TE_hist"], rel=1e-9)
    assert np.abs(outs[0]["sig"][-1] - outs[1]["sig"][-1]).max() < 1e-13


@pytest.mark.parametrize("count", [0, 1, 7, 1000, 300001])
def test_array_kernels(count):
    import torch
    from oracle import zand_np as zo
    from zandpack_gb300 import func_step_forward as fsf
    from zandpack_gb300 import mpi_funcs as mf
    rng = np.random.default_rng(count)
    Y = rng.standard_normal((8, count)) + 1j * rng.standard_normal((8, count))
    Yd = torch.from_numpy(Y).cuda()
    b = rng.standard_normal(8)
    idx = np.array([0, 3, 1, 7])
    out = torch.zeros(count, dtype=torch.complex128, device="cuda")
    fsf.step_sig_forward_nb(Yd, b, out, idx)
    np.testing.assert_allclose(out.cpu().numpy(), zo.stage_combine(Y, b, idx), rtol=1e-14, atol=1e-14)
    ct = rng.standard_normal(7)
    e = mf.TERR2_psi(Yd[:7], ct)
    assert e == pytest.approx(zo.terr2(Y[:7], ct), rel=1e-12, abs=1e-300)
    ch = rng.standard_normal(8)
    Yc = Y.copy()
    zo.step_fourth(Yc, ch)
    mf.step_fourth_omg(Yd, ch)
    np.testing.assert_allclose(Yd.cpu().numpy(), Yc, rtol=1e-13, atol=1e-13)


def test_c1_full_span_matches_reference():
    """The n=20 chain over its whole span, 0-50 fs: the unmodified ``zand``
    took 5414 attempts (``c1_50fs``).  The FP64 device path must take the same
    attempts with the same accept decisions, land on the same time grid, and
    give the reference's sigma (every 40th step and the last) and currents."""
    import os
    from conftest import GOLDEN, load_golden
    from zandpack_gb300.engine import Propagator
    if not os.path.exists(os.path.join(GOLDEN, "c1_50fs.npz")):
        pytest.skip("fixture c1_50fs missing")
    z = load_golden("c1_50fs")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"])
    pr.set_state(z["DM_Ortho"])
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"])
    pr.traj.close()
    TE = np.array(out["TE_hist"])
    assert len(TE) == len(z["TE_hist"]) == 5414
    assert ((TE < p["eps"]) == (z["TE_hist"] < p["eps"])).all()
    np.testing.assert_allclose(TE, z["TE_hist"], rtol=1e-6)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-8)
    sig = np.array(out["sig"])[:, 0][z["sig_traj_idx"] + 1]
    dsig = np.abs(sig - z["sig_traj"][:, 0]).max()
    dfin = np.abs(out["sig"][-1] - z["sig_final"][0]).max()
    dJ = np.abs(np.array(out["currents"]).T - z["currents"]).max()
    print("\nc1 0-50 fs FP64 vs reference: %d attempts, t_end %.6f, max|dsig| %.2e, final %.2e, max|dJ| %.2e"
          % (len(TE), out["times"][-1], dsig, dfin, dJ))
    assert dsig < 1e-10 and dfin < 1e-10 and dJ < 1e-9


def test_kernel_name_shims():
    """``MM`` in its stage-combination form, ``OuterSubtraction_hard_opti`` and
    ``step_omg_forward_nb_fermi_opti`` on the device against the oracle's
    restatements, with ragged extents."""
    import torch
    from oracle import zand_np as zo
    from zandpack_gb300 import func_step_forward as fsf
    from zandpack_gb300 import mpi_funcs as mf
    rng = np.random.default_rng(9)

    def crand(*s):
        return rng.standard_normal(s) + 1j * rng.standard_normal(s)
    # MM(SIGS[idx].transpose(1, 2, 3, 0), B[i, idx], out), Zandpack/mpi/zand:306-313
    S = crand(8, 1, 7, 5)
    idx = [0, 1, 2, 7]
    b = rng.standard_normal(8)
    Sd = torch.from_numpy(S).cuda()
    out = torch.zeros((1, 7, 5), dtype=torch.complex128, device="cuda")
    mf.MM(Sd[idx].permute(1, 2, 3, 0), b[idx], out)
    np.testing.assert_allclose(out.cpu().numpy(), zo.stage_combine(S, b, idx), rtol=1e-14, atol=1e-14)
    # the general form stays a plain matmul
    Ad, Bd = torch.from_numpy(crand(2, 3, 4)).cuda(), torch.from_numpy(crand(2, 4, 6)).cuda()
    o2 = torch.empty((2, 3, 6), dtype=torch.complex128, device="cuda")
    mf.MM(Ad, Bd, o2)
    np.testing.assert_allclose(o2.cpu().numpy(), Ad.cpu().numpy() @ Bd.cpu().numpy(), rtol=1e-13)
    # OuterSubtraction_hard_opti
    nk, na, nx, noT, NA, NX, NO = 1, 3, 5, 2, 3, 5, 3
    A, B = crand(nk, na, nx, noT), crand(nk, NA, NX, NO)
    Cm, O = crand(nk, na, nx, noT, NA, NX, NO), crand(nk, na, nx, noT, NA, NX, NO)
    ref = O.copy()
    zo.outer_subtraction(A, B, Cm, ref)
    Od = torch.from_numpy(O).cuda()
    mf.OuterSubtraction_hard_opti(*(torch.from_numpy(x).cuda() for x in (A, B, Cm)), Od)
    np.testing.assert_allclose(Od.cpu().numpy(), ref, rtol=1e-14, atol=1e-14)
    # step_omg_forward_nb_fermi_opti: the Fermi x Fermi entries of out keep their value
    Y = crand(8, 1, 2, 6, 2, 2, 6, 2)
    fp = np.array([0, 0, 1, 1, 0, 1], bool)
    o0 = crand(1, 2, 6, 2, 2, 6, 2)
    ref = o0.copy()
    zo.combine_fermi_skip(Y, b, ref, idx, fp, fp)
    od = torch.from_numpy(o0).cuda()
    fsf.step_omg_forward_nb_fermi_opti(torch.from_numpy(Y).cuda(), b, od, idx, fp, fp)
    np.testing.assert_allclose(od.cpu().numpy(), ref, rtol=1e-14, atol=1e-14)
