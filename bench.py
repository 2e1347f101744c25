"""Throughput of the AME propagation: simulated femtoseconds per wall second.

Workload (default ``--config c3``): the n = 1024 case -- a 32 x 32 square
lattice (hopping -1 eV), two leads on opposite edges with 32 coupling orbitals
each, 40 rank-8 Lorentzians and 30 Pade poles per lead, the mean-field Hubbard
term U = 2 eV * (Re diag sigma - 0.5) rebuilt at every stage, sinusoidal bias
0.2 V sin(2 pi 0.05 t) split +-V/2.  Inputs are seeded synthetic ``Arrays``
(``zandpack_gb300.workloads``); the state starts from the isolated-device
Fermi density matrix with psi = Omega = 0.

A step is one Dormand-Prince 5(4) attempt of the reference controller (seven
right-hand sides, the embedded error norm, the accept test and, on
acceptance, the update), launched as the captured attempt graph with the
controller on the device (``zg_graph_run``, one launch and one host
synchronisation per attempt).  ``value`` = simulated fs advanced over the K
timed steps / their wall time measured with CUDA events on the trajectory's
stream.  ``e2e`` repeats it through the public C ABI with the initial state
uploaded from pinned host memory and every attempt's record plus sigma after
every accepted step read back, as ``zand`` records them.

``--impl reference`` times the CPU restatement of the reference (the oracle
port, NumPy/BLAS on all host cores) on the same workload; its step is one
attempt of its own controller from the initial state (seven stage
combinations and right-hand sides, the error norm and the update), and fs/s
is its own simulated advance over the wall time.  ``cpu_baseline`` in our
line is the same measurement on two attempts.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

# where the clock samples of a run are written (bench_clocks.csv)
OUT_DIR = os.environ.get("ZG_BENCH_OUT", os.path.join(HERE, "bench_out"))

# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the psi H^T tensor-core GEMM per (workload, H(t) form), taken from a separate
# ncu capture of that launch (ncu cannot run inside the timed region); reported
# with its source, never as a measurement of this run
NCU_TRAFFIC = {("c3", "real"): 83.8e6 + 8.6e6}
# the same for one launch of the complex-product kernel k_tcx per (workload,
# implementation): products and dOmega/dt in one launch at n=1024
NCU_TRAFFIC_TCX = {("c3", "tc_all"): 166.9e6 + 22.7e6}

METRIC = "simulated fs/s at n=1024"
WORKLOAD_DESC = {
    "c3": "n=1024 32x32 square lattice, 2 leads x 32 orbitals, 40 rank-8 Lorentzians + 30 Pade poles per lead, "
          "Hubbard dH(sigma) U=2 eV every stage, bias 0.2 V sin(2pi 0.05 t); eps=1e-6",
    "c2": "n=256 honeycomb ribbon, 2 leads x 16 orbitals, 32 rank-4 Lorentzians + 40 Pade poles, Gaussian pulse",
    "c1": "n=20 chain, 2 leads x 1 orbital, 16 Lorentzians + 20 Pade poles, exponential ramp",
    "c5": "n=2048 random sparse, 4 leads x 72 orbitals, 24 rank-8 Lorentzians + 40 Pade poles, step bias lead 0",
}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled during a region.

    Reads NVML in-process (libnvidia-ml through ctypes, read-only queries) from
    a thread every 5 ms, so that a timed region of tens of milliseconds still
    gets several samples; falls back to ``nvidia-smi -lms 200``.  Samples go to
    bench_clocks.csv in ``$ZG_BENCH_OUT`` (default ``bench_out/``)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40,
            "hw_power_brake_slowdown": 0x80}

    def __init__(self, index=0):
        self.index = index
        self.p = None
        self.nvml = None
        self.rows = []
        self.path = os.path.join(OUT_DIR, "bench_clocks.csv")

    def _nvml_open(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
            return None
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx)) != 0:
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        return lib, h, mx.value, reasons

    def _loop(self):
        import ctypes
        import time as _t
        lib, h, mx, reasons = self.nvml
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop:
            ok = lib.nvmlDeviceGetClockInfo(h, ctypes.c_int(1), ctypes.byref(clk)) == 0
            ok = ok and reasons(h, ctypes.byref(rs)) == 0
            if ok:
                self.rows.append((float(clk.value), float(mx), int(rs.value)))
            _t.sleep(0.005)

    def __enter__(self):
        import threading
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.nvml = self._nvml_open()
        except Exception:
            self.nvml = None
        if self.nvml is not None:
            self.stop = False
            self.th = threading.Thread(target=self._loop, daemon=True)
            self.th.start()
            return self
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.nvml is not None:
            self.stop = True
            self.th.join(timeout=5)
            with open(self.path, "w") as f:
                f.write("sm_mhz,sm_max_mhz,clocks_event_reasons\n")
                for c, m, r in self.rows:
                    f.write("%g,%g,0x%x\n" % (c, m, r))
            return
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if self.nvml is not None:
            if not self.rows:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
            reasons = sorted({k for _, _, r in self.rows for k, b in self.BITS.items() if r & b})
            return {"sm_mhz": float(np.median([r[0] for r in self.rows])), "sm_max_mhz": max(r[1] for r in self.rows),
                    "reasons": reasons, "samples": len(self.rows), "source": "NVML every 5 ms"}
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, fl in rows for i, v in enumerate(fl) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "source": "nvidia-smi -lms 200"}


def aggregate_ranks(ms, adv, device):
    """Replicas: the job's time is the slowest rank's, its simulated time the
    sum over ranks (each rank propagates its own trajectory)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms, adv], device=device, dtype=torch.float64)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    tsum = t.clone()
    dist.all_reduce(tsum)
    return float(tmax[0]), float(tsum[1])


def rhs_flops(L):
    """Algorithmic real flops of one right-hand side (structurally nonzero work)."""
    n, N, Ns, Nf, nc = L.n, L.N, L.Ns, L.Nf, L.nc
    gemm = 8 * n ** 3 + 8 * N * n * n + 8 * n * N * nc + 8 * Ns * nc * n + 8 * N * Ns * nc + 8 * Ns * Nf * nc
    omega = 8 * N * Ns * nc + 8 * Ns * Ns * nc + 8 * Ns * Nf * nc + 10 * (N * Ns + Ns * Nf)
    return gemm, omega


def run_ours(args):
    import ctypes

    import torch
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory, native_bias
    from zandpack_gb300.workloads import make_workload
    ws, rank = _dist()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w = make_workload(args.config)
    tr = Trajectory(w.arrays, w.hbar, precision=args.precision, device=dev)
    L = tr.layout
    stream = torch.cuda.ExternalStream(_lib.lib().zg_traj_stream(tr._h), device=dev)
    bias = native_bias(w.bias, L.NL)
    # one attempt = one launch of the captured attempt graph (controller on the device)
    tr.graph_prepare(bias, w.hubbard_U)
    tr.set_y(w.arrays["DM_Ortho"])
    # measured choice of the small-product / dOmega kernels for this workload class
    from zandpack_gb300 import autotune
    kernels = autotune.choose(tr, dev)
    tr.graph_set(w.t0, w.stepsize, w.eps, 1e30)

    def attempts(k):
        adv, n_acc = 0.0, 0
        for _ in range(k):
            recs, _, _, _ = tr.graph_run(1)
            for r in recs:
                if r[4]:
                    adv += r[3]
                    n_acc += 1
        return adv, n_acc

    attempts(args.warmup)
    # the e2e leg replays the timed attempts from this state, uploaded from pinned memory
    snap = torch.empty(2 * L.size, dtype=torch.float64).pin_memory()
    _lib.check(_lib.lib().zg_get_state(tr._h, tr.stages, ctypes.c_void_p(snap.data_ptr())))
    recs0, t0_, h0_, _ = tr.graph_run(0)
    state0 = (t0_, h0_)
    peaks = np.zeros(2)
    _lib.check(_lib.lib().zg_measure_peaks(dev, peaks.ctypes.data_as(ctypes.c_void_p)))
    dmma = ctypes.c_double()
    _lib.check(_lib.lib().zg_measure_fp64_mma(dev, ctypes.byref(dmma)))
    _lib.check(_lib.lib().zg_profile(tr._h, 1))
    tr.graph_run(0)  # recapture with the profiling event nodes before the timed region
    n0 = _lib.lib().zg_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        e0.record(stream)
        adv, n_acc = attempts(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = _lib.lib().zg_launch_count() - n0
    _, t_end, h_end, _ = tr.graph_run(0)
    state = (t_end, h_end)
    pms = np.zeros(len(_lib.PROF_REGIONS))
    pcnt = np.zeros(len(_lib.PROF_REGIONS), np.int64)
    _lib.check(_lib.lib().zg_profile_read(tr._h, pms.ctypes.data_as(ctypes.c_void_p), pcnt.ctypes.data_as(ctypes.c_void_p)))
    _lib.check(_lib.lib().zg_profile(tr._h, 0))
    tr.graph_run(0)  # recapture without event nodes, outside the e2e timed region
    if ws > 1:
        ms, adv_total = aggregate_ranks(ms, adv, "cuda")
    else:
        adv_total = adv
    value = adv_total / (ms / 1e3)
    # ---- e2e through the public API: pinned upload + per-step sigma/current readback
    e2e = run_e2e(tr, w, args, state0, snap, stream)
    reg = dict(zip(_lib.PROF_REGIONS, zip(pms.tolist(), pcnt.tolist())))
    # the update of a rejected attempt returns at once (its gate is off): its
    # time per call counts the accepted attempts only
    if "update" in reg and 0 < n_acc < reg["update"][1]:
        reg["update"] = (reg["update"][0], int(n_acc))
    gemm_f, omega_f = rhs_flops(L)
    g_ms, g_n = reg["gemm"]
    if args.precision == "f64":
        fp64_peak = peaks[0] / 1e3
        achieved = gemm_f / (g_ms / g_n / 1e3) / 1e12 if g_n else None
        roof = {"bound": "fp64", "kernel": "k_zgemm (batched FP64 complex GEMMs of one RHS)",
                "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": (achieved / fp64_peak) if achieved else None, "traffic": None,
                "peak_source": "live DFMA probe zg_measure_peaks (FP64 is not in MEASURED_PEAKS.json)",
                "algorithmic_flops_per_launch": gemm_f}
    else:
        tf32 = measure_tf32_peak()
        roof = mixed_roofline(args, w, L, reg, tr.stages, peaks, tf32, kernels["impl"].split("/")[0])
    roof["regions_ms_per_call"] = {k: (v[0] / v[1] if v[1] else None) for k, v in reg.items()}
    if args.precision == "mixed":
        roof["kernel_roofs"] = kernel_roofs(L, reg, tr.stages, peaks, tf32, kernels["impl"].split("/")[0])
    out = {
        "metric": METRIC, "value": value, "unit": "fs/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128" if args.precision == "f64" else "c64 tf32x3 compute, c128 state", "data": "synthetic",
        "config": {"workload": "%s: %s" % (args.config, WORKLOAD_DESC.get(args.config, "")),
                   "precision": args.precision, "layout": L.summary(),
                   "l2": "inputs larger than L2: %d state slots x %.0f MB" % (tr.stages + 1, L.size * 16 / 1e6),
                   "parallelism": "replicas" if ws > 1 else "single",
                   "kernels": kernels},
        "rhs_evals_per_s": tr.stages * args.steps * ws / (ms / 1e3),
        "simulated_fs": adv_total,
        "t_h_after": list(state),
        "roofline": roof,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "peaks_live_gflops": {"fp64": peaks[0], "fp32": peaks[1], "fp64_mma": dmma.value},
    }
    tr.close()
    if args.precision == "mixed" and not args.no_f64_ref:
        out["f64_path"] = f64_reference_timing(w, dev, state, value, ms / args.steps)
    if args.nonorth:
        out["nozand"] = run_nonorth(args, dev)
    if rank == 0:
        if args.ensemble > 0:
            out["ensemble"] = run_ensemble(args)
        if args.steady:
            out["steady_state"] = run_steady(args)
        if args.cpu:
            out["cpu_baseline"] = cpu_baseline(args, w, adv_total / (args.steps * ws))
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


def mixed_roofline(args, w, L, reg, stages, peaks, tf32, impl):
    """Roofline of the region that takes the most time per right-hand side,
    against MEASURED_PEAKS.json: the psi H^T tensor-core GEMM on algorithmic
    flops (8 N n^2, the count for a dense complex H(t)) against the bf16
    burst peak; the streaming regions on algorithmic bytes against the
    measured HBM copy rate."""
    pk = _peaks_file()
    bf16, hbm = pk.get("bf16_tflops"), pk.get("hbm_gbs")
    n, N, Ns, Nf, nc, NL = L.n, L.N, L.Ns, L.Nf, L.nc, L.NL
    np_ = (n + 15) // 16 * 16
    nb32 = (n + 31) // 32 * 32
    h_real = not np.any(np.asarray(w.arrays["H_Ortho"]).imag)  # the Hubbard term is real
    per_rhs = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in reg.items()}
    om = N * Ns + Ns * Nf
    cands = {
        "gemm": ("tensor", "k_gemm_tf32x3<256,4,16> (psi H(t)^T, tcgen05 kind::tf32, 3xTF32, %s H(t))"
                 % ("real" if h_real else "complex"), 8.0 * N * n * n, bf16, "TFLOP/s",
                 "MEASURED_PEAKS.json bf16_tflops (burst)"),
        # the small products read psi's hi/lo planes and the Omega blocks and write PI, Omega xi, xi sigma^T
        # (with dOmega/dt: the Omega blocks once more written, their second read not counted)
        "small": ("hbm", "k_tcx (PI partials, Omega xi, xi sigma^T%s on tcgen05)" % (
                  " and dOmega/dt" if impl == "tc_all" else "") if impl != "simt" else "k_zgemm<float> SIMT batch",
                  16.0 * N * np_ + 8.0 * om + 8.0 * (2 * NL * n * nc + NL * N * nc + NL * Ns * nc + Ns * n)
                  + (8.0 * om if impl == "tc_all" else 0.0), hbm, "GB/s", "MEASURED_PEAKS.json hbm_gbs"),
        "omega": ("hbm", "k_tcx<64> (dOmega/dt on tcgen05, second stream)" if impl == "tc_split"
                  else "k_omega<float> (dOmega/dt, SIMT)", 16.0 * om, hbm, "GB/s", "MEASURED_PEAKS.json hbm_gbs"),
        "final": ("hbm", "k_final_all_mixed (k_sigma and k_psi finalisation)",
                  8.0 * (4 * N * n + Ns * n) + 8.0 * 3 * n * n, hbm, "GB/s", "MEASURED_PEAKS.json hbm_gbs"),
    }
    name = max((k for k in cands if per_rhs.get(k, 0.0) > 0), key=lambda k: per_rhs[k])
    bound, kernel, amount, peak, unit, src = cands[name]
    t = per_rhs[name] / 1e3
    achieved = amount / t / (1e12 if unit == "TFLOP/s" else 1e9)
    roof = {"bound": bound, "kernel": kernel, "region": name, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak if peak else None, "peak_source": src,
            "algorithmic_%s_per_launch" % ("flops" if unit == "TFLOP/s" else "bytes"): amount,
            "ms_per_launch": per_rhs[name], "traffic": None,
            "regions_share_of_rhs": {k: v / sum(per_rhs[x] for x in cands) for k, v in per_rhs.items() if k in cands}}
    # psi H(t)^T beside it: executed 3xTF32 work against live cuBLAS TF32, and its ncu traffic
    g = per_rhs.get("gemm", 0.0) / 1e3
    tc_flops = 3 * 2 * (2 * N) * (nb32 if h_real else 2 * np_) * np_
    if g > 0:
        roof["psi_HT"] = {"algorithmic_tflops": 8.0 * N * n * n / g / 1e12,
                          "frac_of_bf16_burst": 8.0 * N * n * n / g / 1e12 / bf16 if bf16 else None,
                          "executed_tf32_tflops": tc_flops / g / 1e12, "live_cublas_tf32_tflops": tf32,
                          "frac_executed_of_tf32": tc_flops / g / 1e12 / tf32 if tf32 else None,
                          "ms_per_launch": g * 1e3}
        traffic = NCU_TRAFFIC.get((args.config, "real" if h_real else "complex"))
        if traffic is not None:
            roof["psi_HT"]["traffic"] = traffic
            roof["psi_HT"]["traffic_source"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one launch, "
                                                "separate ncu capture at this workload (not this run)")
            if name == "gemm":
                roof["traffic"] = traffic
                roof["traffic_source"] = roof["psi_HT"]["traffic_source"]
    if name == "small" and NCU_TRAFFIC_TCX.get((args.config, impl)) is not None:
        roof["traffic"] = NCU_TRAFFIC_TCX[(args.config, impl)]
        roof["traffic_source"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one launch, separate ncu "
                                  "capture at this workload (not this run); writes still in L2 at kernel end "
                                  "are not counted")
    return roof


def kernel_roofs(L, reg, stages, peaks, tf32, impl="simt"):
    """Roofline fraction of every region of the mixed attempt: algorithmic
    bytes (streaming regions, against the measured HBM copy rate of
    MEASURED_PEAKS.json) or flops (against the live FP32 / cuBLAS TF32 peaks)
    over the region's CUDA-event time per call."""
    hbm = _peaks_file().get("hbm_gbs")
    n, N, Ns, Nf, nc = L.n, L.N, L.Ns, L.Nf, L.nc
    np_ = (n + 15) // 16 * 16
    S = L.size
    # DOP54 stage inputs read y + the nonzero k slots of their row: 1, 2, 3, 4, 5, 6, 6 slots
    reads = [1, 2, 3, 4, 5, 6, 6][:stages]
    stage_out = n * n + 2 * N * np_ + N * Ns + Ns * Nf  # sigma, psi hi and lo (planar), Omega
    out = {}

    def put(name, amount, unit, peak, peak_src):
        ms, cnt = reg.get(name, (0.0, 0))
        if not cnt or not peak:
            return
        t = ms / cnt / 1e3
        ach = amount / t / (1e9 if unit == "GB/s" else 1e12)
        out[name] = {"achieved": ach, "unit": unit, "peak": peak, "frac": ach / peak, "per_call": amount,
                     "peak_source": peak_src}

    mp = "MEASURED_PEAKS.json hbm_gbs"
    put("combine", 8.0 * (sum(reads) * S + stages * stage_out) / stages, "GB/s", hbm, mp)
    put("error", 8.0 * 6 * S, "GB/s", hbm, mp)
    put("update", 8.0 * 5 * S + 16.0 * 2 * S + 8.0 * S, "GB/s", hbm, mp)
    # psi: hi, lo, R1 (planar) in, k out, plus R2 on the sourced rows; sigma: T in, k out, T^T re-read
    put("final", 8.0 * (4 * N * n + Ns * n) + 8.0 * 3 * n * n, "GB/s", hbm, mp)
    fp32 = peaks[1] / 1e3 if peaks is not None else None
    live = "live FFMA probe zg_measure_peaks"
    om = N * Ns + Ns * Nf
    if impl == "simt":
        put("small", 8.0 * (n * N * nc + Ns * nc * n + N * Ns * nc + Ns * Nf * nc), "TFLOP/s", fp32, live)
    else:  # on the tensor cores: bytes of psi's planes, the Omega blocks and the products
        put("small", 16.0 * N * np_ + 8.0 * om + 8.0 * (2 * L.NL * n * nc + L.NL * N * nc + L.NL * Ns * nc + Ns * n)
            + (8.0 * om if impl == "tc_all" else 0.0), "GB/s", hbm, mp)
    if impl != "tc_all":  # else dOmega/dt is part of the products' launch
        put("omega", 16.0 * om, "GB/s", hbm, mp)
    # executed tensor flops of H sigma with a real H(t) (the workloads' Hamiltonians and Hubbard term)
    put("gemm2", 3 * 2.0 * ((n + 31) // 32 * 32) * 2 * np_ * np_, "TFLOP/s", tf32, "live cuBLAS TF32")
    return out


def _peaks_file():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def measure_tf32_peak():
    """cuBLAS TF32 throughput (TFLOP/s) of an 8192^3 GEMM, best of 5."""
    import torch
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(8192, 8192, device="cuda")
        b = torch.randn(8192, 8192, device="cuda")
        for _ in range(2):
            torch.matmul(a, b)
        best = 0.0
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = max(best, 2 * 8192 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
        del a, b
        return best
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old


def f64_reference_timing(w, dev, state, mixed_value, mixed_ms, attempts=6):
    """The plain FP64 device path on the same workload, at the mixed run's
    controller state: one warm-up and `attempts` timed attempts, each a launch
    of the FP64 attempt graph (the mixed run's launch mode) with the step size
    reset to the mixed run's before every attempt, for the mixed/FP64 ratio of
    the target specification."""
    import torch
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory, native_bias
    tr = Trajectory(w.arrays, w.hbar, precision="f64", device=dev)
    tr.graph_prepare(native_bias(w.bias, tr.layout.NL), w.hubbard_U)
    tr.set_y(w.arrays["DM_Ortho"])
    t, h = state
    stream = torch.cuda.ExternalStream(_lib.lib().zg_traj_stream(tr._h), device=dev)
    tr.graph_set(t, h, w.eps, 1e30)
    tr.graph_run(1)
    times = []
    for _ in range(attempts):
        tr.graph_set(t, h, w.eps, 1e30)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        tr.graph_run(1)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    tr.close()
    ms = float(np.median(times))
    return {"ms_per_step": ms, "ms_per_step_min_max": [min(times), max(times)], "attempts": attempts,
            "value_same_h": mixed_value * mixed_ms / ms, "unit": "fs/s", "mixed_over_f64": ms / mixed_ms,
            "note": "median FP64 attempt (graph launch) at the mixed run's step size; "
                    "value_same_h = mixed value x time ratio"}


def run_e2e(tr, w, args, state0, pinned, stream):
    """The timed attempts again through the public C ABI: the state they start
    from is uploaded from pinned host memory and the controller set inside the
    timed region, each attempt's record (error norm, step sizes, stage-0
    currents) comes back to the host, and sigma after every accepted step, as
    zand records them."""
    import ctypes

    import torch
    from zandpack_gb300._lib import check, lib
    L = tr.layout
    sig_host = torch.empty((L.n, L.n * 2), dtype=torch.float64).pin_memory()
    rec_bytes = ctypes.sizeof(__import__("zandpack_gb300._lib", fromlist=["zg_attempt_rec"]).zg_attempt_rec)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    check(lib().zg_set_state(tr._h, tr.stages, ctypes.c_void_p(pinned.data_ptr())))
    tr.graph_set(state0[0], state0[1], w.eps, 1e30)
    adv = 0.0
    d2h = 0
    for _ in range(args.steps):
        recs, _, _, _ = tr.graph_run(1)
        d2h += rec_bytes
        for r in recs:
            if r[4]:
                check(lib().zg_get_sigma(tr._h, tr.stages, ctypes.c_void_p(sig_host.data_ptr())))
                d2h += L.n * L.n * 16
                adv += r[3]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"value": adv / (ms / 1e3), "unit": "fs/s", "h2d_bytes_per_step": int(L.size * 16 / args.steps),
            "d2h_bytes_per_step": int(d2h / args.steps),
            "api": "zg_set_state (pinned host) + zg_graph_set + zg_graph_run per attempt + zg_get_sigma per "
                   "accepted step",
            "note": "the timed attempts repeated from their starting state, uploaded once from pinned memory "
                    "(bytes amortised over the steps); attempt records and sigma read back as zand records them"}


def _oracle_stages(w, nstages, warm_stages=0):
    """Run the oracle's controller stage by stage; returns (wall s, simulated fs
    attributed to the timed stages, stages timed)."""
    from oracle import zand_np as zo
    prob = zo.Problem(w.arrays, w.hbar)
    bias, dH = w.bias_fn(), w.dH_fn()
    s0, p0, o0 = prob.zero_state()
    SIGS = np.zeros((8,) + s0.shape, complex)
    PSIS = np.zeros((8,) + p0.shape, complex)
    OMGS = np.zeros((8,) + o0.shape, complex)
    SIGS[-1] = w.arrays["DM_Ortho"]
    t, h = w.t0, w.stepsize
    wall, sim = 0.0, 0.0
    timed_in_attempt = 0
    for k in range(warm_stages + nstages):
        i = k % 7
        if i == 0:
            timed_in_attempt = 0
        t_start = time.perf_counter()
        if i == 0:
            ys, yp, yo = SIGS[-1], PSIS[-1], OMGS[-1]
        else:
            ix = zo.idxholder[i]
            ys, yp, yo = (zo.stage_combine(Y, zo.B[i], ix) for Y in (SIGS, PSIS, OMGS))
        ts = t + zo.A[i] * h
        ks, kp, ko, _, _ = prob.rhs(h, ys, yp, yo, prob.H0 + dH(ts, ys), [bias(ts, a) for a in range(prob.NL)])
        SIGS[i], PSIS[i], OMGS[i] = ks, kp, ko
        adv = None
        if i == 6:
            TE = math.sqrt(sum(zo.terr2(Y[:7], zo.CT) for Y in (SIGS, PSIS, OMGS)))
            hn = float(zo.hnew_func(h, TE, w.eps))
            adv = 0.0
            if TE < w.eps:
                for Y in (SIGS, PSIS, OMGS):
                    zo.step_fourth(Y, zo.CH)
                t += hn
                adv = hn
            h_used, h = h, hn
        dt = time.perf_counter() - t_start
        if k >= warm_stages:
            wall += dt
            timed_in_attempt += 1
        if adv is not None:
            # the attempt's advance is shared evenly over its seven stages
            sim += adv * timed_in_attempt / 7
            timed_in_attempt = 0
    # an attempt cut off by the end of the sample counts at the step it uses
    sim += h * timed_in_attempt / 7
    return wall, sim, nstages


def cpu_baseline(args, w, adv_per_attempt):
    """The reference arm's measurement on a bounded sample: the oracle port
    (NumPy restatement of the reference's stage body and controller, BLAS on
    the host cores) runs one warm-up attempt and two timed attempts of its own
    controller from the initial state (~20 s); fs/s = its own simulated
    advance / wall.  The same protocol as ``--impl reference``, whose step is
    one attempt too."""
    try:
        wall, sim, done = _oracle_stages(w, 14, 7)
    except MemoryError:
        return {"value": None, "unit": "fs/s", "cores": os.cpu_count(), "kind": "port",
                "sample": "oracle out of host memory"}
    return {"value": sim / wall if wall > 0 else None, "unit": "fs/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "2 attempts (14 stages: stage combination + RHS, error norm, update) of %s after one warm-up "
                      "attempt, the oracle's own controller from the initial state; NumPy/BLAS default threads. "
                      "The port, not the unmodified zand (numba and mpi4py are absent on the GPU box)" % args.config,
            "s_per_rhs": wall / done, "simulated_fs": sim,
            "gpu_fs_per_attempt_for_reference": adv_per_attempt}


def run_ensemble(args):
    """The serving ensemble (512 independent trajectories, Poisson arrivals at
    50/s, sizes n in {64..512}, 2-3 leads, each with its own step size), served
    with continuous batching; p50/p99 latency from arrival to completion."""
    from zandpack_gb300.serve import Server, c4_estimate
    from zandpack_gb300.workloads import c4_requests, c4_workload
    span = args.ensemble_fs if args.ensemble_fs == "pulse" else float(args.ensemble_fs)
    reqs = c4_requests(args.ensemble, rate=50.0, seed=1004, t_span=span)
    srv = Server(c4_workload, c4_estimate, max_slots=args.slots, precision=args.precision, keep_sigma=False,
                 prep_workers=args.prep_workers)
    res, stats = srv.run(reqs)
    stats["t_span_fs"] = args.ensemble_fs if span != "pulse" else "pulse centre + 3 widths (%.1f-%.1f fs, mean %.1f)" % (
        min(r["t1"] for r in reqs), max(r["t1"] for r in reqs), float(np.mean([r["t1"] for r in reqs])))
    stats["rate_per_s"] = 50.0
    stats["errors"] = sorted({r.error for r in res if r.error})[:3]
    if args.capacity:
        # capacity: the same requests all present at t = 0
        srv2 = Server(c4_workload, c4_estimate, max_slots=args.slots, precision=args.precision, keep_sigma=False,
                      prep_workers=args.prep_workers)
        _, burst = srv2.run(reqs, time_scale=0.0)
        stats["capacity"] = {k: burst[k] for k in ("wall_s", "throughput_traj_per_s", "simulated_fs_per_s",
                                                   "p50_latency_s", "p99_latency_s", "completed")}
    return stats


def run_nonorth(args, dev):
    """The same workload posed in a non-orthogonal basis and propagated as the
    reference's nozand does (overlap 1 + 0.08 x the bonds of H): attempts as
    graph launches from its initial state, CUDA events on the trajectory's
    stream; ms per attempt beside the orthogonal run's."""
    import torch
    from zandpack_gb300 import _lib
    from zandpack_gb300.engine import Trajectory, native_bias
    from zandpack_gb300.workloads import make_nonorth_workload
    w = make_nonorth_workload(args.config)
    tr = Trajectory(w.arrays, w.hbar, precision=args.precision, device=dev, nonorth=True)
    stream = torch.cuda.ExternalStream(_lib.lib().zg_traj_stream(tr._h), device=dev)
    tr.graph_prepare(native_bias(w.bias, tr.layout.NL), w.hubbard_U)
    tr.set_y(tr.basis.sigma(w.arrays["DM_Ortho"]))
    tr.graph_set(w.t0, w.stepsize, w.eps, 1e30)
    adv = 0.0
    for _ in range(max(3, args.warmup)):
        tr.graph_run(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        recs, _, _, _ = tr.graph_run(1)
        adv += sum(r[3] for r in recs if r[4])
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    tr.close()
    return {"workload": "%s posed with an overlap (nozand)" % args.config, "precision": args.precision,
            "ms_per_step": ms / args.steps, "value": adv / (ms / 1e3), "unit": "fs/s", "steps": args.steps}


def run_steady(args):
    """The steady state (psinought) of a workload at its initial density matrix:
    GMRES on the device to a relative residual of 1e-8, as the reference's
    default steptol; wall time of the solve (operator and preconditioner in
    libzandgpu, FP64)."""
    from zandpack_gb300.layout import CompactLayout
    from zandpack_gb300.psinought import steady_state
    from zandpack_gb300.workloads import make_workload
    w = make_workload(args.steady)
    L = CompactLayout(w.arrays, w.hbar)
    # the first solve also loads the complex vector kernels the GMRES uses; time the second
    steady_state(w.arrays, w.hbar, w.bias_fn(), w.dH_fn(), t0=w.t0, tol=1e-8, layout=L, maxiter=2)
    res = steady_state(w.arrays, w.hbar, w.bias_fn(), w.dH_fn(), t0=w.t0, tol=1e-8, layout=L)
    return {"workload": args.steady, "n": L.n, "modes": L.N, "unknowns_complex": L.N * L.n,
            "iterations": res.iterations, "relative_residual": res.residual, "converged": res.converged,
            "seconds": res.seconds}


def run_reference(args):
    """The reference arm: the oracle port (the reference's stage body and
    controller restated in NumPy, pinned to the unmodified zand's outputs) on
    the host cores.  A step is one Dormand-Prince attempt of its own controller
    from the initial state, like a step of our arm; `--warmup` attempts are
    untimed."""
    ws, rank = _dist()
    if rank != 0:
        return
    from zandpack_gb300.workloads import make_workload
    w = make_workload(args.config)
    wall, sim, done = _oracle_stages(w, 7 * args.steps, 7 * args.warmup)
    value = sim / wall if wall > 0 else None
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "fs/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
           "config": {"workload": "%s: %s" % (args.config, WORKLOAD_DESC.get(args.config, "")),
                      "precision": "f64", "layout": "reference padded (NL, NX, NOT)"},
           "cpu_baseline": {"value": value, "unit": "fs/s", "cores": os.cpu_count(), "kind": "port",
                            "sample": "%d attempts (%d stages) of the oracle port's controller after %d warm-up "
                                      "attempts, NumPy/BLAS on the host cores; the port, not the unmodified zand "
                                      "(numba and mpi4py are absent on the GPU box)" % (args.steps, done, args.warmup),
                            "s_per_rhs": wall / done},
           "e2e": {"value": value, "unit": "fs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3")
    ap.add_argument("--precision", default="mixed", choices=["f64", "mixed"])
    ap.add_argument("--no-f64-ref", action="store_true", help="skip timing the FP64 path beside the mixed one")
    ap.add_argument("--ensemble", type=int, default=512, help="requests of the serving ensemble (0: skip)")
    ap.add_argument("--ensemble-fs", default="pulse",
                    help="simulated span per ensemble trajectory: 'pulse' (its pulse centre + 3 widths) or fs")
    ap.add_argument("--slots", type=int, default=32, help="concurrent trajectories of the ensemble")
    ap.add_argument("--cpu", type=int, default=1,
                    help="time the CPU baseline (the oracle port; 0 for workloads too large for host memory, c5)")
    ap.add_argument("--capacity", action="store_true",
                    help="also serve the ensemble with every request present at t = 0")
    ap.add_argument("--prep-workers", type=int, default=max(1, min(12, (os.cpu_count() or 4) - 4)),
                    help="worker processes preparing ensemble requests on the host")
    ap.add_argument("--nonorth", type=int, default=1, help="also time the workload posed with an overlap (nozand)")
    ap.add_argument("--steady", default="c2", help="workload of the steady-state (psinought) timing ('' to skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
