"""The reference's in-process signatures on the device: ``make_f``'s
``f(t, old_sig, old_psi, old_omega, dH, delta_variant, dH_given=True)``
(Zandpack/TimedependentTransport.py:2754-2776) and ``AdaptiveDOP``
(:3392-3560), both through libzandgpu's C ABI, against the oracle
(``oracle.zand_np.Problem.rhs`` and ``oracle.zand_np.adaptive_dop``).
FP64 tolerances: f at 1e-12 relative (max norm per array); the stepper's
time grid at 1e-10, density matrices at 1e-11 and currents at 1e-10."""
import numpy as np
import pytest

from conftest import golden_callbacks, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _random_state(z, p, seed):
    from zandpack_gb300.layout import CompactLayout
    L = CompactLayout(z, p["hbar"])
    rng = np.random.default_rng(seed)
    y = (rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 0.1
    ys, yp, yo = L.unpack(y)
    ys = (ys + ys.conj().transpose(0, 2, 1)) / 2
    return L.unpack(L.pack(ys, yp, yo))


@pytest.mark.parametrize("case", ["mini2", "mini3", "c1"])
@pytest.mark.parametrize("dH_given", [True, False])
def test_make_f_against_oracle(case, dH_given):
    from oracle import zand_np as zo
    from zandpack_gb300.rhs import make_f
    z = load_golden(case)
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    ys, yp, yo = _random_state(z, p, 5)
    f = make_f(z, p["hbar"])
    t = 0.37
    if dH_given:
        cb = dH
    else:
        def cb(tt, s):  # H(t) itself
            return prob.H0 + dH(tt, s)
    Ds, Dp, Do = f(t, ys, yp, yo, cb, bias, dH_given=dH_given)
    Ht = prob.H0 + dH(t, ys)
    ks, kp, ko, _, _ = prob.rhs(1.0, ys, yp, yo, Ht, [bias(t, a) for a in range(prob.NL)])
    for g, r in zip((Ds, Dp, Do), (ks, kp, ko)):
        assert g.shape == r.shape
        assert _rel(g, r) < 1e-12
    f.close()


def test_make_f_refuses_states_it_cannot_hold():
    from zandpack_gb300.layout import LayoutError
    from zandpack_gb300.rhs import make_f
    z = load_golden("mini2")
    p = z["params"]
    bias, dH = golden_callbacks(p)
    f = make_f(z, p["hbar"])
    ys, yp, yo = _random_state(z, p, 6)
    L = f.trajs[0].layout
    a, x, c = L.modes[L.Ns]  # a source-free mode: its block with itself stays zero
    yo = yo.copy()
    yo[0, a, x, c, a, x, c] = 1e-3
    with pytest.raises(LayoutError):
        f(0.0, ys, yp, yo, dH, bias)
    f.close()


@pytest.mark.parametrize("case,faithful", [("mini2", True), ("mini3", True), ("mini2", False)])
def test_adaptive_dop_against_oracle(case, faithful, tmp_path, monkeypatch):
    """The parameters of the reference-stepper fixtures (inproc_<case>.npz);
    with the reference's k7 assignment the device run must also reproduce
    those fixtures."""
    import json
    import os
    from conftest import GOLDEN
    from oracle import zand_np as zo
    from zandpack_gb300.rhs import AdaptiveDOP, make_f
    monkeypatch.chdir(tmp_path)
    g = np.load(os.path.join(GOLDEN, "inproc_%s.npz" % case))
    c = json.loads(str(g["params"]))
    z = load_golden(case)
    p = z["params"]
    if not faithful:  # DOP54 proper takes long steps at the fixtures' loose tolerance
        c.update(eps=p["eps"], t1=0.4, h_guess=0.05)
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    sig0, psi0, omg0 = prob.zero_state()
    sig0 = sig0 + np.asarray(z["DM_Ortho"])
    ref = zo.adaptive_dop(prob, sig0, psi0, omg0, c["eps"], c["t0"], c["t1"], dH, bias, h_guess=c["h_guess"],
                          faithful_k7=faithful)
    f = make_f(z, p["hbar"])
    names = ["lead%d" % a for a in range(prob.NL)]
    times, data = AdaptiveDOP(f, sig0, psi0, omg0, c["eps"], c["t0"], c["t1"], dH, bias, z["Ixi"],
                              h_guess=c["h_guess"], elec_names=names, print_step=5, faithful_k7=faithful)
    f.close()
    assert len(times) == len(ref["times"]) >= 3
    np.testing.assert_allclose(times, ref["times"], rtol=0, atol=1e-10)
    assert np.abs(data["density matrix"] - ref["dm"]).max() < 1e-11
    for a in range(prob.NL):
        assert np.abs(np.array(data["current_lead%d" % a]) - ref["currents"][a]).max() < 1e-10
    if faithful:
        assert len(times) == len(g["times"])
        assert np.abs(data["density matrix"] - g["dm"]).max() < 1e-11
    assert (tmp_path / "Runge-Kutta.txt").exists() and (tmp_path / "Runge-Kutta_last_sig.npy").exists()
