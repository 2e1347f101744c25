"""Run a few Dormand-Prince attempts of a synthetic workload, for profilers.

    python -m zandpack_gb300.profile_case --config c3 --precision mixed --attempts 2

Builds the workload, uploads the initial state, runs ``--warmup`` attempts and
then ``--attempts`` attempts, and exits; nothing else runs on the GPU.
"""
from __future__ import annotations

import argparse
import time


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c3")
    ap.add_argument("--precision", default="mixed", choices=["f64", "mixed"])
    ap.add_argument("--attempts", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--regions", action="store_true", help="print CUDA-event times per region of the timed attempts")
    ap.add_argument("--impl", default=None, choices=["simt", "tc_products", "tc_all", "tc_split"],
                    help="kernels of the small products and dOmega/dt (default: the trajectory's)")
    ap.add_argument("--nonorth", action="store_true",
                    help="the workload posed in a non-orthogonal basis, propagated as nozand does")
    args = ap.parse_args()
    import ctypes as C

    import numpy as np

    from ._lib import PROF_REGIONS, check, lib
    from .engine import Propagator
    from .workloads import make_nonorth_workload, make_workload
    w = make_nonorth_workload(args.config) if args.nonorth else make_workload(args.config)
    pr = Propagator(w.arrays, w.hbar, w.bias_fn(), hubbard_U=w.hubbard_U, precision=args.precision,
                    nonorth=args.nonorth)
    if args.impl is not None:
        from ._lib import IMPL_NAMES
        pr.traj.set_impl(IMPL_NAMES.index(args.impl))
    sig0 = w.arrays["DM_Ortho"]
    pr.set_state(pr.traj.basis.sigma(sig0) if args.nonorth else sig0)
    t, h = w.t0, w.stepsize
    for i in range(args.warmup + args.attempts):
        if args.regions and i == args.warmup:
            check(lib().zg_profile(pr.traj._h, 1))
        t0 = time.perf_counter()
        TE, _, _ = pr.attempt(t, h)
        hn = pr.tab.hnew(h, TE, w.eps)
        if TE < w.eps:
            pr.traj.step_fourth()
            t += hn
        h = hn
        print("attempt %d: TE=%.3e h=%.4g t=%.4g (%.2f ms host wall)" % (i, TE, h, t, (time.perf_counter() - t0) * 1e3))
    if args.regions:
        ms = np.zeros(len(PROF_REGIONS))
        cnt = np.zeros(len(PROF_REGIONS), np.int64)
        check(lib().zg_profile_read(pr.traj._h, ms.ctypes.data_as(C.c_void_p), cnt.ctypes.data_as(C.c_void_p)))
        for name, m, c in zip(PROF_REGIONS, ms, cnt):
            print("region %-8s %4d calls %9.4f ms/call %9.4f ms/attempt" % (name, c, m / max(c, 1), m / args.attempts))
    pr.traj.close()


if __name__ == "__main__":
    main()
