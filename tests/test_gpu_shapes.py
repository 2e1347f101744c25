"""The larger workloads on the device: the n=256 ribbon (c2) and the n=2048,
4-lead, n_c=72 device (c5).  One right-hand side on a random dense state in
both precisions; the mixed result, in every kernel form the trajectory
supports, must agree with the FP64 one to 2e-5 of the magnitude of the
products (the per-RHS tolerance of the mixed path)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["c2", "c5"])
def test_mixed_vs_f64_rhs_large(case):
    import torch
    assert torch.cuda.is_available()
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.workloads import make_workload
    w = make_workload(case)
    L = CompactLayout(w.arrays, w.hbar)
    rng = np.random.default_rng(5)
    y = ((rng.standard_normal(L.size) + 1j * rng.standard_normal(L.size)) * 1e-2).astype(np.complex128)
    sig, psi, _, _ = L.views(y)
    sig[...] = (sig + sig.conj().T) / 2 + np.asarray(w.arrays["DM_Ortho"][0])
    delta = [w.bias_fn()(3.0, a) for a in range(L.NL)]
    tr = Trajectory(w.arrays, w.hbar, precision="f64", layout=L)
    tr.set_slot(tr.stages, y)
    tr.stage_input(0)
    Jf = tr.rhs(0, 3.0, 0.02, delta, currents=True)
    kf = tr.get_slot(0)
    tr.close()
    a = L.views(kf)
    H = np.asarray(w.arrays["H_Ortho"][0])
    scale_sig = np.abs(H @ sig).max() * 0.02 / w.hbar
    scale_psi = np.abs(psi @ H.T).max() * 0.02 / w.hbar
    # every kernel form of the mixed path the trajectory supports
    tr = Trajectory(w.arrays, w.hbar, precision="mixed", layout=L)
    tr.set_slot(tr.stages, y)
    _, avail = tr.get_impl()
    assert _lib.ZG_IMPL_TC_PRODUCTS in avail
    for impl in avail:
        tr.set_impl(impl)
        tr.stage_input(0)
        Jm = tr.rhs(0, 3.0, 0.02, delta, currents=True)
        b = L.views(tr.get_slot(0))
        for name, x, r, sc in zip(("sig", "psi", "omA", "omB"), b, a, (scale_sig, scale_psi, 0.0, 0.0)):
            err = np.abs(x - r).max() / max(np.abs(r).max(), sc, 1e-300)
            print("\n%s %s %s: %.2e" % (case, _lib.IMPL_NAMES[impl], name, err))
            assert err < 2e-5, (case, _lib.IMPL_NAMES[impl], name, err)
        np.testing.assert_allclose(Jm, Jf, rtol=1e-11, atol=1e-14)
    tr.close()
