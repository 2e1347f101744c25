"""tcgen05 3xTF32 GEMM and the TF32 split against float64 references."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


def _split(x):
    import torch
    from zandpack_gb300._lib import check, lib
    hi = torch.empty_like(x)
    lo = torch.empty_like(x)
    check(lib().zg_split_tf32(_p(x), _p(hi), _p(lo), x.numel(), None))
    return hi, lo


def test_split_tf32():
    import torch
    x = torch.randn(100003, device="cuda", dtype=torch.float32) * 1e3
    hi, lo = _split(x)
    torch.cuda.synchronize()
    hb = hi.view(torch.int32).cpu().numpy()
    lb = lo.view(torch.int32).cpu().numpy()
    assert (hb & 0x1FFF == 0).all() and (lb & 0x1FFF == 0).all()
    xd = x.double().cpu().numpy()
    err = np.abs(hi.double().cpu().numpy() + lo.double().cpu().numpy() - xd) / np.abs(xd).max()
    assert err.max() < 2.0 ** -21


# the last two shapes take the 256-wide tiles (enough tiles to fill the GPU), the
# very last with partial tiles in M, N and K
@pytest.mark.parametrize("M,N,K", [(128, 256, 32), (128, 128, 64), (200, 96, 100), (1024, 2048, 2048),
                                   (4480, 2048, 2048), (4500, 2016, 1000)])
def test_gemm_tf32x3(M, N, K):
    import torch
    from zandpack_gb300._lib import check, lib
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    D = torch.full((M, N), float("nan"), device="cuda")
    check(lib().zg_gemm_tf32x3(_p(Ah), _p(Al), _p(Bh), _p(Bl), _p(D), M, N, K, None))
    ref = (Ah.double() + Al.double()) @ (Bh.double() + Bl.double()).T
    err = (D.double() - ref).abs().max().item() / ref.abs().max().item()
    assert err < 2e-6, err
    if M * N * K >= 1 << 32:
        # rough timing, printed for the log
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(2):
            check(lib().zg_gemm_tf32x3(_p(Ah), _p(Al), _p(Bh), _p(Bl), _p(D), M, N, K, None))
        e0.record()
        for _ in range(5):
            check(lib().zg_gemm_tf32x3(_p(Ah), _p(Al), _p(Bh), _p(Bl), _p(D), M, N, K, None))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5
        print("\nGEMM %dx%dx%d 3xTF32: %.3f ms, %.1f TFLOP/s (tensor flops %.1f)" % (
            M, N, K, ms, 2 * M * N * K / ms / 1e9, 6 * M * N * K / ms / 1e9))


def test_bounded_wait_gives_up_and_context_survives():
    """The bounded mbarrier wait of the tensor-core kernels, run on a barrier
    that nothing completes with a ~1 ms budget, records its code and returns
    (ZG_ETIMEOUT on the host); the context then still runs a GEMM."""
    import torch
    from zandpack_gb300 import _lib
    from zandpack_gb300._lib import check, lib
    assert lib().zg_wait_selftest(0, 2 * 1000 * 1000) == _lib.ZG_ETIMEOUT
    M, N, K = 128, 128, 64
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    Ah, Al = _split(A)
    Bh, Bl = _split(B)
    D = torch.empty((M, N), device="cuda")
    check(lib().zg_gemm_tf32x3(_p(Ah), _p(Al), _p(Bh), _p(Bl), _p(D), M, N, K, None))
    ref = (Ah.double() + Al.double()) @ (Bh.double() + Bl.double()).T
    assert (D.double() - ref).abs().max().item() / ref.abs().max().item() < 2e-6


def test_fp64_tensor_core_probe():
    """The DMMA (mma.sync m8n8k4 f64) probe runs and reports a rate beside
    the DFMA one (both printed for the record)."""
    import ctypes as C
    from zandpack_gb300 import _lib
    g = C.c_double()
    _lib.check(_lib.lib().zg_measure_fp64_mma(0, C.byref(g)))
    peaks = np.zeros(2)
    _lib.check(_lib.lib().zg_measure_peaks(0, peaks.ctypes.data_as(C.c_void_p)))
    print("\nFP64: DMMA %.1f GFLOP/s, DFMA %.1f GFLOP/s" % (g.value, peaks[0]))
    assert g.value > 0 and peaks[0] > 0
