"""Host preparation of served requests in spawned worker processes (CPU only):
the pool's result equals the in-process preparation to 1e-12 (the workers run
single-threaded BLAS, whose sums may round differently in the last place)."""
import numpy as np


def test_prepare_in_pool_equals_in_process():
    from zandpack_gb300.serve import Server, c4_estimate, prepare
    from zandpack_gb300.workloads import c4_requests, c4_workload
    reqs = c4_requests(3, seed=11, t_span=0.1)
    srv = Server(c4_workload, c4_estimate, hbm_budget=1 << 40, prep_workers=2)
    pool = srv._start_pool()
    try:
        got = [pool.submit(prepare, c4_workload, r).result() for r in reqs]
    finally:
        pool.shutdown()
    for r, (w, L) in zip(reqs, got):
        w0, L0 = prepare(c4_workload, r)
        assert set(w.arrays) == {"DM_Ortho"}
        assert np.abs(w.arrays["DM_Ortho"] - w0.arrays["DM_Ortho"]).max() <= 1e-12
        assert (w.t1, w.eps, w.stepsize, w.bias) == (w0.t1, w0.eps, w0.stepsize, w0.bias)
        assert (L.n, L.N, L.Ns, L.nc) == (L0.n, L0.N, L0.Ns, L0.nc)
        for k in ("H0", "XI", "IXI", "XIS", "XIT2", "Xp", "Xm", "GLP", "dGP", "dGM", "lead_cols", "colmap"):
            a, b = getattr(L, k), getattr(L0, k)
            assert a.shape == b.shape and np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max()), k
