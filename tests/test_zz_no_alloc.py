"""zg_terr2_c128_noalloc: the error norm for callers that must not allocate
device memory while they run (a serving loop that reserved all of HBM at
start-up, a host whose device memory belongs to another allocator).

It must give the allocating entry point's result and the oracle's
(``oracle.zand_np.terr2``), on two calls in a row, and it must not take memory
from the device's default stream-ordered pool, which the allocating entry
point uses for its partial sums (that entry point is the positive control of
the check).  This file sorts last so a run that stops at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7  # cuda.h, CUmemPool_attribute
CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8


def _terr2(fn, Y, ct):
    import torch
    res = np.zeros(1)
    ns, count = Y.shape[0], Y[0].numel()
    ctv = np.ascontiguousarray(ct, np.float64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = fn(C.c_void_p(Y.data_ptr()), count, ns, ctv.ctypes.data_as(C.c_void_p), count,
            res.ctypes.data_as(C.c_void_p), stream)
    return st, float(res[0])


class _DefaultPool:
    """High-water mark of the current device's default memory pool, through
    the driver API (the pool is a driver object, shared by every runtime in
    the process)."""

    def __init__(self):
        import torch
        self.cu = C.CDLL("libcuda.so.1")
        dev = C.c_int()
        assert self.cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def reset_high(self):
        z = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, C.byref(z)) == 0

    def _get(self, attr):
        v = C.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def high(self):
        return self._get(CU_MEMPOOL_ATTR_USED_MEM_HIGH)

    def used(self):
        return self._get(CU_MEMPOOL_ATTR_USED_MEM_CURRENT)


def test_noalloc_error_norm_matches_allocating_entry_point():
    import torch
    assert torch.cuda.is_available(), "GPU test"
    from oracle import zand_np as zo
    from zandpack_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(2024)
    cases = []
    for count in (300001, 777):
        Y = rng.standard_normal((7, count)) + 1j * rng.standard_normal((7, count))
        ct = rng.standard_normal(7)
        cases.append((Y, torch.from_numpy(Y).cuda(), ct))
    torch.cuda.synchronize()
    pool = _DefaultPool()
    # positive control: the allocating entry point draws its partial sums from the pool
    base = pool.used()
    pool.reset_high()
    refs = []
    for _, Yd, ct in cases:
        st, r = _terr2(L.zg_terr2_c128, Yd, ct)
        _lib.check(st)
        refs.append(r)
    assert pool.high() > base
    # two calls of the no-allocation entry point in a row: same results, no pool memory
    base = pool.used()
    pool.reset_high()
    for (Y, Yd, ct), r in zip(cases, refs):
        st, v = _terr2(L.zg_terr2_c128_noalloc, Yd, ct)
        _lib.check(st)
        assert v == pytest.approx(r, rel=1e-12)
        assert v == pytest.approx(zo.terr2(Y, ct), rel=1e-12)
    assert pool.high() <= base
