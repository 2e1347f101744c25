"""zg_terr2_c128_noalloc: the error norm for callers that must not allocate
device memory while they run (a serving loop that reserved all of HBM at
start-up, a host whose device memory belongs to another allocator).

It must give the allocating entry point's result.  Two calls in a row, the
second on a smaller array, show that the shared static scratch carries nothing
over from the previous call.  This file sorts last so a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _terr2(fn, Y, ct):
    import torch
    res = np.zeros(1)
    ns, count = Y.shape[0], Y[0].numel()
    ctv = np.ascontiguousarray(ct, np.float64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = fn(C.c_void_p(Y.data_ptr()), count, ns, ctv.ctypes.data_as(C.c_void_p), count,
            res.ctypes.data_as(C.c_void_p), stream)
    return st, float(res[0])


def test_noalloc_error_norm_matches_allocating_entry_point():
    import torch
    assert torch.cuda.is_available(), "GPU test"
    from zandpack_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(2024)
    cases = []
    for count in (300001, 777):
        Y = rng.standard_normal((7, count)) + 1j * rng.standard_normal((7, count))
        ct = rng.standard_normal(7)
        cases.append((torch.from_numpy(Y).cuda(), ct))
    refs = []
    for Yd, ct in cases:
        st, r = _terr2(L.zg_terr2_c128, Yd, ct)
        _lib.check(st)
        refs.append(r)
    # two calls of the no-allocation entry point in a row
    for (Yd, ct), r in zip(cases, refs):
        st, v = _terr2(L.zg_terr2_c128_noalloc, Yd, ct)
        _lib.check(st)
        assert v == pytest.approx(r, rel=1e-12)
