"""Compact layout: exact pack/unpack round trips and term-by-term agreement of
the compact-layout equations with the padded oracle (CPU only)."""
import numpy as np
import pytest

from compact_model import rhs_compact
from conftest import golden_callbacks
from oracle import zand_np as zo
from zandpack_gb300.layout import CompactLayout, LayoutError


def test_roundtrip_and_rhs(golden):
    case, z = golden
    p = z["params"]
    bias, dH = golden_callbacks(p)
    prob = zo.Problem(z, p["hbar"])
    for a in p["keep"]:
        ys, yp, yo = z["y_sig_%d" % a], z["y_psi_%d" % a], z["y_omg_%d" % a]
        L = CompactLayout(z, p["hbar"], psi0=yp, omg0=yo)
        y = L.pack(ys, yp, yo)
        s2, p2, o2 = L.unpack(y)
        # exact round trip: every entry outside the layout is exactly zero
        assert np.array_equal(s2, ys) and np.array_equal(p2, yp) and np.array_equal(o2, yo)
        h = float(z["h_%d" % a]) * 0.7
        t = float(z["t_attempt"][a])
        delta = [bias(t, l) for l in range(prob.NL)]
        Ht = prob.H0 + dH(t, ys)
        ks, kp, ko, _, J = prob.rhs(h, ys, yp, yo, Ht, delta)
        k, Jc = rhs_compact(L, y, Ht[0], delta, h)
        ks2, kp2, ko2 = L.unpack(k)
        for g, r in ((ks2, ks), (kp2, kp), (ko2, ko)):
            assert np.abs(g - r).max() <= 1e-13 * max(np.abs(r).max(), 1e-300)
        np.testing.assert_allclose(Jc, J[0], rtol=1e-12, atol=1e-15)
        # the oracle's padded output has nothing outside the layout
        assert np.array_equal(L.unpack(L.pack(ks, kp, ko))[2], ko)


def test_mode_reduction_c3_sizes():
    from zandpack_gb300.workloads import make_workload
    w = make_workload("c3")
    L = CompactLayout(w.arrays, w.hbar)
    assert (L.N, L.Ns, L.nc, L.padded_modes) == (4480, 640, 32, 6400)
    assert L.size == 1024 ** 2 + 4480 * 1024 + 4480 * 640 + 640 * 3840


def test_rejects_unrepresentable_omega():
    from zandpack_gb300.workloads import make_workload
    w = make_workload("mini2")
    L = CompactLayout(w.arrays, w.hbar)
    _, psi, omg = L.unpack(np.zeros(L.size, complex))
    free = L.modes[L.Ns]
    omg[0, free[0], free[1], free[2], free[0], free[1], free[2]] = 1e-3
    with pytest.raises(LayoutError):
        CompactLayout(w.arrays, w.hbar, psi0=psi, omg0=omg)
