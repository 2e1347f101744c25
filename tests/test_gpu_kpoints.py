"""Several k-points on the device against the unmodified reference ``zand``
run with two k-points (fixture ``k2_mini2``): one trajectory per k-point, the
error norm summed over them and the controller shared, as ``zand`` treats
the k axis.  Per-stage derivatives at 1e-12 (FP64), the adaptive run (attempt
sequence, time grid, final sigma of each k-point, per-k-point currents), the
``zand`` driver's output files, and the mixed path within 1e-6 on the
reference's grid."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_callbacks, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def k2():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    if not os.path.exists(os.path.join(GOLDEN, "k2_mini2.npz")):
        pytest.skip("fixture k2_mini2 missing")
    return load_golden("k2_mini2")


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_kpoint_stage_derivatives_match_reference(k2):
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory, kpoint_arrays
    z = k2
    p = z["params"]
    bias, _ = golden_callbacks(p)
    for a in p["keep"]:
        h = float(z["h_%d" % a])
        t = float(z["t_attempt"][a])
        for k in range(2):
            ys, yp, yo = (z["y_%s_%d" % (v, a)][k:k + 1] for v in ("sig", "psi", "omg"))
            tr = Trajectory(kpoint_arrays(z, k), p["hbar"], psi0=yp, omg0=yo)
            L = tr.layout
            tr.set_y(ys, yp, yo)
            for i in range(7):
                tr.stage_input(i)
                ts = t + zo.A[i] * h
                tr.rhs(i, ts, h, [bias(ts, l) for l in range(L.NL)], _lib.ZG_DH_HUBBARD, p["hubbard_U"])
                g = L.unpack(tr.get_slot(i))
                for x, nm in zip(g, ("ksig", "kpsi", "komg")):
                    ref = z["%s_%d" % (nm, a)][i][k:k + 1]
                    assert _rel(x, ref) < 1e-12, (a, k, i, nm, _rel(x, ref))
            tr.close()


def test_kpoint_trajectory_matches_reference(k2):
    from zandpack_gb300.engine import Propagator
    z = k2
    p = z["params"]
    bias, _ = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"])
    assert pr.NK == 2
    pr.set_state(z["DM_Ortho"])
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"])
    TE = np.array(out["TE_hist"])
    assert len(TE) == len(z["TE_hist"])
    assert ((TE < p["eps"]) == (z["TE_hist"] < p["eps"])).all()
    np.testing.assert_allclose(TE, z["TE_hist"], rtol=1e-6)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-10)
    assert np.abs(out["sig"][-1] - z["sig_final"]).max() < 1e-11
    J = np.array(out["currents"])  # (steps, NK, NL)
    assert np.abs(J.transpose(2, 0, 1) - z["currents"]).max() < 1e-10
    pr.close()


def test_kpoint_mixed_within_1e6_of_reference(k2):
    from zandpack_gb300.engine import Propagator
    z = k2
    p = z["params"]
    bias, _ = golden_callbacks(p)
    pr = Propagator(z, p["hbar"], bias, hubbard_U=p["hubbard_U"], precision="mixed")
    pr.set_state(z["DM_Ortho"])
    acc = list(z["TE_hist"] < p["eps"])
    replay = np.concatenate([z["h_hist"], [z["times"][-1] - z["times"][-2]]])
    out = pr.run(p["t0"], p["t1"], p["stepsize"], p["eps"], replay_h=replay, force_accept=acc)
    np.testing.assert_allclose(out["times"], z["times"], rtol=0, atol=1e-12)
    sig = np.array(out["sig"])[z["sig_traj_idx"] + 1]
    assert np.abs(sig - z["sig_traj"]).max() < 1e-6
    J = np.array(out["currents"]).transpose(2, 0, 1)
    assert np.abs(J - z["currents"]).max() < 1e-6
    pr.close()


def test_kpoint_zand_driver(tmp_path, k2):
    """The zand driver on the two-k-point run directory: time grid and
    per-k-point currents at 1e-10, sigma of both k-points (complex64 DM
    files) at 1e-6."""
    from test_zand_driver import _write_run
    from zandpack_gb300.mpi_tools import combine_currents, combine_dm
    from zandpack_gb300.zand import ZandRun
    z = k2
    _write_run(str(tmp_path), z, saveevery=1, device_dH=True)
    cwd = os.getcwd()
    try:
        ZandRun(str(tmp_path), log=lambda *a: None).run()
    finally:
        os.chdir(cwd)
    save = str(tmp_path / "run_save")
    T, C = combine_currents([save], n=2)
    np.testing.assert_allclose(T, z["times"][:-1], rtol=0, atol=1e-10)
    assert np.abs(np.stack(C) - z["currents"]).max() < 1e-10
    _, DM = combine_dm([save])
    assert DM.shape[1] == 2
    assert np.abs(DM[z["sig_traj_idx"] + 1] - z["sig_traj"]).max() < 1e-6
