"""Serving many independent propagations on one GPU (continuous batching).

Requests arrive as a stream (their ``arrival`` times, seconds).  A request's
host input preparation (its Arrays and compact layout) starts when it arrives,
in a pool of worker processes when ``prep_workers`` > 0 (numpy work holds the
GIL, so threads alone serialise it).  The server admits a request as soon as a
slot is free and its estimated device footprint fits the HBM budget; an
admitted request is given its own trajectory on the device -- its own CUDA stream, state and step
size -- and propagated by a worker thread.  In the default ``graph`` mode the
worker captures one Dormand-Prince attempt as a CUDA graph with the step-size
controller on the device and launches batches of attempts with one host
synchronisation each (``zg_graph_run``); ``host`` mode calls one
``zg_attempt`` per attempt.  ctypes releases the Python GIL during each
call.  Trajectories therefore overlap on the GPU while requests that arrive
later wait for memory or a slot.  Each result is the final sigma, the last
lead currents, the number of attempts and the latency (completion minus
arrival).

Results do not depend on what else runs: trajectories share no device buffers
and every kernel is deterministic, so a trajectory computed in the mix is
identical to the same trajectory computed alone.
"""
from __future__ import annotations

import concurrent.futures as cf
import dataclasses
import math
import multiprocessing as mp
import os
import threading
import time
from typing import Callable, List, Optional

import numpy as np

from . import autotune
from .engine import Trajectory, native_bias
from .layout import CompactLayout


def footprint_bytes(n, N, Ns, nc, L, precision="mixed"):
    """Device bytes of one trajectory (state slots, stage buffers, operands and
    scratch) as zg_traj_create allocates them."""
    Nf = N - Ns
    S = n * n + N * n + N * Ns + Ns * Nf
    np_ = (n + 15) // 16 * 16
    const = 16 * (n * n + N * (5 + 5 * nc))
    if precision == "f64":
        state = 16 * S * 8 + 16 * S
        scratch = 16 * (3 * n * n + 3 * L * n * nc + N * L * nc + Ns * n + L * (N + Ns) * nc)
    else:
        state = 16 * S + 8 * S + 8 * S * 7 + 8 * (n * n + 2 * N * np_ + N * Ns + Ns * Nf)
        scratch = (4 * (2 * n * 2 * np_ + 4 * 4 * np_ * np_) + 8 * (n * np_ + N * np_)
                   + 8 * (3 * L * n * nc + N * L * nc + Ns * n + L * (N + Ns) * nc) + 16 * n * n)
    return int(1.15 * (const + state + scratch)) + (64 << 20)


@dataclasses.dataclass
class Result:
    id: int
    arrival: float
    admitted: float
    finished: float
    attempts: int
    accepted: int
    t_end: float
    sigma: Optional[np.ndarray]
    currents: Optional[np.ndarray]
    n: int
    modes: int
    error: Optional[str] = None

    @property
    def latency(self):
        return self.finished - self.arrival


class Server:
    def __init__(self, build: Callable, estimate: Callable, device=0, max_slots=16, hbm_budget=None,
                 precision="mixed", keep_sigma=True, attempt_mode="graph", max_batch=32, prep_workers=0,
                 tune=None):
        self.build, self.estimate = build, estimate
        # tune: the kernels of each trajectory chosen by measurement, once per
        # class (zandpack_gb300.autotune keeps the choice): "coarse" keys a
        # class by orbitals, coupling width and leads, so that requests that
        # differ in their pole counts share one measurement; "full" by every
        # shape (each distinct request is then measured, one at a time); None
        # (the default; both measured slower on the 512-request ensemble) or
        # False: the library's defaults
        if tune not in (None, False, "coarse", "full"):
            raise ValueError("tune must be 'coarse', 'full' or None")
        self.tune = tune
        self.device, self.max_slots = device, max_slots
        self.precision = precision
        self.keep_sigma = keep_sigma
        if attempt_mode not in ("graph", "host"):
            raise ValueError("attempt_mode must be 'graph' or 'host'")
        self.attempt_mode = attempt_mode
        self.max_batch = max_batch
        self.prep_workers = int(prep_workers)
        if hbm_budget is None:
            import torch
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget = int(0.8 * free)
        self.hbm_budget = hbm_budget
        self.lock = threading.Lock()
        self.in_use = 0
        self.peak_in_use = 0
        self.peak_slots = 0

    def _run_one(self, req, t_admit, fp, out: List[Result], done: threading.Semaphore, prepared=None):
        res = Result(id=req["id"], arrival=req["arrival"], admitted=t_admit, finished=0.0, attempts=0, accepted=0,
                     t_end=0.0, sigma=None, currents=None, n=req.get("n", 0), modes=0)
        tr = None
        try:
            w, L = prepared.result() if prepared is not None else prepare(self.build, req)
            res.modes = L.N
            tr = Trajectory(None, w.hbar, precision=self.precision, device=self.device, layout=L)
            tr.set_y(w.arrays["DM_Ortho"])
            if self.tune:
                autotune.choose(tr, self.device, coarse=self.tune == "coarse")
            b = native_bias(w.bias, L.NL)
            t, h = w.t0, w.stepsize
            J = None
            if self.attempt_mode == "graph":
                tr.graph_prepare(b, w.hubbard_U)
                tr.graph_set(t, h, w.eps, w.t1)
                finished = t >= w.t1
                while not finished:
                    # about as many attempts as the remaining span needs at the current step size
                    batch = int(min(self.max_batch, max(1, math.ceil((w.t1 - t) / h) + 1)))
                    recs, t, h, finished = tr.graph_run(batch)
                    for r in recs:
                        res.attempts += 1
                        if r[4]:
                            res.accepted += 1
                            J = r[6]
            else:
                while t < w.t1:
                    TE, acc, t, h, J0 = tr.attempt_native(t, h, w.eps, b, w.hubbard_U)
                    res.attempts += 1
                    if acc:
                        res.accepted += 1
                        J = J0
            res.t_end = t
            res.currents = J
            if self.keep_sigma:
                res.sigma = tr.get_sigma()
        except Exception as e:  # reported per request, the server keeps going
            res.error = repr(e)
        finally:
            if tr is not None:
                tr.close()
            res.finished = time.perf_counter() - self.t_start
            with self.lock:
                self.in_use -= fp
                out.append(res)
            done.release()

    def _start_pool(self):
        """Worker processes for host preparation, started (spawn: the parent
        already holds a CUDA context) and warmed before the request stream
        begins, each with single-threaded BLAS."""
        if self.prep_workers <= 0:
            return None
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in keys}
        for k in keys:
            os.environ[k] = "1"
        try:
            pool = cf.ProcessPoolExecutor(self.prep_workers, mp_context=mp.get_context("spawn"))
            for f in [pool.submit(_warm) for _ in range(self.prep_workers)]:
                f.result()
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        return pool

    def run(self, requests, time_scale=1.0):
        """Serve ``requests`` (dicts with ``id``, ``arrival``); arrivals are
        replayed in wall time scaled by ``time_scale``.  Returns the results
        in completion order and summary statistics."""
        reqs = sorted(requests, key=lambda r: r["arrival"])
        pool = self._start_pool()
        self.t_start = time.perf_counter()
        out: List[Result] = []
        slots = threading.Semaphore(self.max_slots)
        threads = []
        pending = list(reqs)
        prepared = {}
        if pool is not None:
            # each request's host preparation starts when it arrives, while it may still wait for admission
            prepared = {r["id"]: cf.Future() for r in reqs}

            def feed():
                for r in reqs:
                    wait = r["arrival"] * time_scale - (time.perf_counter() - self.t_start)
                    if wait > 0:
                        time.sleep(wait)
                    f = pool.submit(prepare, self.build, r)
                    f.add_done_callback(lambda f, dst=prepared[r["id"]]: _forward(f, dst))

            threading.Thread(target=feed, daemon=True).start()
        while pending:
            req = pending[0]
            due = req["arrival"] * time_scale
            now = time.perf_counter() - self.t_start
            if now < due:
                time.sleep(min(due - now, 0.01))
                continue
            fp = self.estimate(req, self.precision)
            if fp > self.hbm_budget:
                pending.pop(0)
                out.append(Result(id=req["id"], arrival=due, admitted=now, finished=now, attempts=0, accepted=0,
                                  t_end=0.0, sigma=None, currents=None, n=req.get("n", 0), modes=0,
                                  error="footprint %d B exceeds the HBM budget" % fp))
                continue
            slots.acquire()
            while True:
                with self.lock:
                    if self.in_use + fp <= self.hbm_budget:
                        self.in_use += fp
                        self.peak_in_use = max(self.peak_in_use, self.in_use)
                        break
                time.sleep(0.002)
            pending.pop(0)
            r = dict(req)
            r["arrival"] = due
            th = threading.Thread(target=self._run_one,
                                  args=(r, time.perf_counter() - self.t_start, fp, out, slots,
                                        prepared.get(r["id"])), daemon=True)
            th.start()
            threads.append(th)
            self.peak_slots = max(self.peak_slots, sum(t.is_alive() for t in threads))
        for th in threads:
            th.join()
        wall = time.perf_counter() - self.t_start
        if pool is not None:
            pool.shutdown(wait=True, cancel_futures=True)
        ok = [r for r in out if r.error is None]
        lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
        stats = dict(requests=len(reqs), completed=len(ok), failed=len(out) - len(ok), wall_s=wall,
                     throughput_traj_per_s=len(ok) / wall, simulated_fs=float(sum(r.t_end for r in ok)),
                     p50_latency_s=float(np.percentile(lat, 50)), p99_latency_s=float(np.percentile(lat, 99)),
                     mean_latency_s=float(lat.mean()), attempts=int(sum(r.attempts for r in ok)),
                     peak_hbm_reserved=int(self.peak_in_use), hbm_budget=int(self.hbm_budget),
                     max_slots=self.max_slots, prep_workers=self.prep_workers, attempt_mode=self.attempt_mode)
        stats["simulated_fs_per_s"] = stats["simulated_fs"] / wall
        return out, stats


def prepare(build, req):
    """Host input preparation of one request: its workload and compact layout.
    Only what the device run needs travels back (sigma_0 of the arrays)."""
    w = build(req)
    L = CompactLayout(w.arrays, w.hbar)
    slim = dataclasses.replace(w, arrays={"DM_Ortho": np.asarray(w.arrays["DM_Ortho"])})
    return slim, L


def _warm():
    time.sleep(0.2)  # keeps this worker busy so that every worker gets started
    return os.getpid()


def _forward(src, dst):
    if src.exception() is not None:
        dst.set_exception(src.exception())
    else:
        dst.set_result(src.result())


def c4_estimate(req, precision):
    from .workloads import c4_mode_estimate
    N, Ns, nc = c4_mode_estimate(req)
    return footprint_bytes(req["n"], N, Ns, nc, req["leads"], precision)
