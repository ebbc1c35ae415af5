"""Benchmark: VKDE kernel-point pairs/s (d=16, N=8192, Student-t nu=3, banana).

One step = one eval_m2lnp pass of 8192 points over the 8192 prepared kernels
(6.71e7 pairs).  `value` times the mixed-precision form on device-resident
points with CUDA events on the library's stream (L2 flushed between steps by
writing a 512 MiB buffer); `e2e` times the same step through the C-ABI call a
user makes with pinned host buffers (host->device copy of the points and
device->host copy of the 8192 results inside the timed region).  The plain
FP64 form is timed the same way and reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--no-cpu] [--no-extra] [--serve-rate HZ] [--serve-steps S]

At N=1 the same JSON line also carries the other workloads of the path:
`interp` (prepare_interp, Gaussian VKDE d=12 N=4096 on a 3-component mixture,
FP64 and mixed NNLS), `batch` (256 uneven problems in one persistent launch)
and `serving` (64 concurrent APES chains, Poisson arrivals, p50/p99 step
latency).  Under torchrun (N>1) every rank evaluates its own 8192 points
against the same kernels (weak scaling, no collective on the data path);
rank 0 prints.
`--impl reference` times NumCosmo's FP64 CPU algorithm (the oracle restatement;
the reference itself cannot be built without GLib/GSL/LAPACK) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

PEAKS_PATH = os.path.join(HERE, "MEASURED_PEAKS.json")
D, N, M, NU = 16, 8192, 8192, 3.0
FLOP_PER_PAIR = D * D + 3 * D          # triangular whitening d^2, difference d, dot 2d
METRIC = "VKDE kernel·point pairs/s (d=16,N=8192)"


def _peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """SM clock and throttle reasons sampled every millisecond during the timed
    region through NVML (read-only queries of libnvidia-ml), else nvidia-smi."""

    # nvmlClocksEventReasons bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.max_mhz = None
        self.reasons = set()
        self._stop = None
        self._th = None
        self._nv = None
        self._dev = None
        self._smi = None

    def _nvml(self):
        import ctypes as C

        nv = C.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit")
        dev = C.c_void_p()
        if nv.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(dev)) != 0:
            raise OSError("nvmlDeviceGetHandleByIndex")
        mx = C.c_uint()
        if nv.nvmlDeviceGetMaxClockInfo(dev, C.c_int(1), C.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        return nv, dev

    def _loop(self):
        import ctypes as C

        clk, rs = C.c_uint(), C.c_ulonglong()
        get_r = getattr(self._nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(self._nv, "nvmlDeviceGetCurrentClocksThrottleReasons")
        while not self._stop.is_set():
            if self._nv.nvmlDeviceGetClockInfo(self._dev, C.c_int(1), C.byref(clk)) == 0:
                self.samples.append(float(clk.value))
            if get_r(self._dev, C.byref(rs)) == 0:
                for bit, name in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(name)
            time.sleep(0.001)

    def __enter__(self):
        import threading

        try:
            self._nv, self._dev = self._nvml()
            self._stop = threading.Event()
            self._th = threading.Thread(target=self._loop, daemon=True)
            self._th.start()
        except Exception:
            self._nv = None
            fd, path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            try:
                self._smi = (path, subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                                      "--format=csv,noheader,nounits", "-lms", "20"],
                                                     stdout=open(path, "w"), stderr=subprocess.DEVNULL))
            except Exception:
                self._smi = None
        return self

    def __exit__(self, *a):
        if self._th is not None:
            self._stop.set()
            self._th.join(timeout=2)
        if self._smi is not None:
            path, proc = self._smi
            proc.terminate()
            try:
                proc.wait(timeout=5)
            except Exception:
                proc.kill()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            try:
                for line in open(path):
                    f = [x.strip() for x in line.split(",")]
                    if len(f) < 6:
                        continue
                    try:
                        self.samples.append(float(f[0]))
                        self.max_mhz = float(f[1])
                    except ValueError:
                        continue
                    for nm, v in zip(names, f[2:6]):
                        if v.lower() in ("active", "1", "true"):
                            self.reasons.add(nm)
                os.remove(path)
            except Exception:
                pass

    def summary(self):
        return {"sm_mhz": statistics.median(self.samples) if self.samples else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(self.samples),
                "source": "nvml" if self._nv is not None else "nvidia-smi"}


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_points(rank: int, m: int = M, d: int = D):
    """The points one rank evaluates against the (replicated) kernels: rank 0
    the workload's own points, rank r > 0 its own seeded draw from the same
    law (weak scaling: per-rank work is fixed, no data exchange)."""
    from numcosmo_gb300 import workloads as wl

    return wl.config2().points[:m] if rank == 0 else wl.banana(m, d, 2002 + 1000 * rank)


def max_over_ranks(values, dist=None, device="cpu"):
    """Element-wise maximum over ranks of per-rank timings: the slowest rank
    sets the job's time.  Without a process group, the values themselves."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    tt = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return [float(v) for v in tt]


def job_rate(units_per_rank: float, steps: int, world: int, seconds: float) -> float:
    """Whole-job throughput: the units every rank processed over the job time."""
    return world * units_per_rank * steps / seconds


def cpu_baseline(seconds: float = 8.0, threads: int | None = None):
    """Oracle (NumCosmo's FP64 algorithm restated in C) on the host cores, a bounded sample of points."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import numpy as np

    import oracle as O
    from numcosmo_gb300 import workloads as wl

    if not os.path.exists(O.LIB_PATH):
        O.build()
    threads = threads or os.cpu_count()
    p = wl.config2()
    sd = O.OracleStatsDist(O.VKDE, O.ST, D, nu=NU, nthreads=threads)
    sd.set_sample(p.centres)
    assert sd.prepare() == 0
    m = 64
    t = 0.0
    while True:
        t0 = time.perf_counter()
        sd.eval_m2lnp(p.points[:m])
        t = time.perf_counter() - t0
        if t > seconds / 4 or m >= M:
            break
        m = min(M, m * 4)
    reps = max(1, int(seconds / max(t, 1e-3)))
    ts = []
    for _ in range(min(reps, 5)):
        t0 = time.perf_counter()
        sd.eval_m2lnp(p.points[:m])
        ts.append(time.perf_counter() - t0)
    tmed = statistics.median(ts)
    return {"value": m * N / tmed, "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"eval_m2lnp of {m} of the 8192 points over all 8192 prepared kernels, median of {len(ts)}",
            "seconds_per_sample": tmed}


def bench_config(world: int) -> dict:
    """The workload both arms run (identical keys and values in either arm's line)."""
    return {"workload": "vkde_st3_d16_n8192_banana: eval_m2lnp, 8192 points x 8192 prepared kernels",
            "kernels": N, "points_per_gpu": M, "dim": D, "kernel": "student-t nu=3", "local_frac": 0.05,
            "l2": "flushed between timed steps (512 MiB write)",
            "parallelism": f"points sharded, {world} replica(s)"}


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    import numpy as np

    cb = cpu_baseline(seconds=max(2.0, 20.0 / max(1, args.steps)))
    vals = []
    for _ in range(args.steps):
        c = cpu_baseline(seconds=2.0) if args.steps > 1 else cb
        vals.append(c["value"])
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * (N * N) / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(ws),
            "implementation": "oracle/ncg_oracle.c (NumCosmo FP64 CPU algorithm restated; the reference itself "
                              "needs GLib/GSL/LAPACK, absent here)",
            "cpu_baseline": {**cb, "value": v},
            "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_gpu(args):
    import numpy as np
    import torch

    import numcosmo_gb300 as ng
    from numcosmo_gb300 import workloads as wl

    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    p = wl.config2()
    kern = ng.StatsDistKernelST(D, NU)
    sd = ng.StatsDistVKDE(kern, ng.StatsDistCV.NONE, device=local)
    stream = torch.cuda.Stream()
    sd.set_stream(stream.cuda_stream)
    sd.set_sample(p.centres)
    t0 = time.perf_counter()
    sd.prepare()
    prep_s = time.perf_counter() - t0

    # each rank evaluates its own 8192 points (weak scaling)
    pts = rank_points(rank)
    xq = torch.tensor(pts, dtype=torch.float64, device="cuda")
    out = torch.empty(M, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    kernel_ms = []

    def timed(precision, steps, warm, kernel_time=False):
        sd.set_precision(precision)
        sd.set_kernel_timing(kernel_time)
        with torch.cuda.stream(stream):
            for _ in range(warm):
                sd.eval_m2lnp_device(xq.data_ptr(), M, out.data_ptr())
        stream.synchronize()
        times = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sd.eval_m2lnp_device(xq.data_ptr(), M, out.data_ptr())
                e1.record(stream)
            stream.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
            if kernel_time:
                kernel_ms.append(sd.get_kernel_time())
        sd.set_kernel_timing(False)
        return times

    # plain FP64 form (the comparison bar), fewer steps: it is ~100x slower
    t64 = timed(ng.Precision.FP64, max(3, args.steps // 4), args.warmup)
    ref64 = out.cpu().numpy().copy()

    # FP32 CUDA-core mixed form (reported beside the tensor-core form)
    tsimt = timed(ng.Precision.MIXED_SIMT, max(3, args.steps // 2), args.warmup)
    err_simt = float(np.max(np.abs(out.cpu().numpy() - ref64) / np.maximum(np.abs(ref64), 1.0)))

    # tensor-core mixed form: the headline, with clocks sampled during the timed region
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        tmx = timed(ng.Precision.MIXED, args.steps, args.warmup, kernel_time=True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    gotmx = out.cpu().numpy()
    err_mx = float(np.max(np.abs(gotmx - ref64) / np.maximum(np.abs(ref64), 1.0)))
    path_info = sd.get_eval_path()

    tot_mx, tot_64 = max_over_ranks([sum(tmx), sum(t64) * args.steps / len(t64)], dist, "cuda")
    pairs = float(N) * M
    value = job_rate(pairs, args.steps, ws, tot_mx)
    v64 = job_rate(pairs, args.steps, ws, tot_64)

    # e2e: C-ABI call with pinned host buffers (H2D points, D2H results inside the timed region)
    sd.set_precision(ng.Precision.MIXED)
    hx = torch.empty((M, D), dtype=torch.float64, pin_memory=True).numpy()
    hx[:] = pts
    ho = torch.empty(M, dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(args.warmup):
        sd.eval_m2lnp_into(hx, ho)
    e2e_t = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        stream.synchronize()
        t0 = time.perf_counter()
        sd.eval_m2lnp_into(hx, ho)
        e2e_t.append(time.perf_counter() - t0)
    (e2e_tot,) = max_over_ranks([sum(e2e_t)], dist, "cuda")
    e2e_v = job_rate(pairs, args.steps, ws, e2e_tot)

    peaks, src = _peaks()
    fp64_peak = ng.measure_fp64_peak(local)
    dur = 1e-3 * statistics.mean(kernel_ms) if kernel_ms else statistics.mean(tmx)
    achieved = pairs * FLOP_PER_PAIR / dur / 1e12
    peak = float(peaks["bf16_tflops"])
    traffic = None
    tpath = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("eval_tc_bytes_per_launch")
        except Exception:
            traffic = None
    launches_per_eval = 2  # tensor core: point-tile build + eval (merge fused); SIMT: eval + merge

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    cb = cpu_baseline(seconds=8.0) if ws == 1 and not args.no_cpu else None
    if cb is not None:
        one = cpu_baseline(seconds=2.0, threads=1)
        cb["single_core"] = {"value": one["value"], "unit": one["unit"], "sample": one["sample"]}
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_mx / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp16x3/f32 (mixed)", "data": "synthetic",
        "config": bench_config(ws),
        "fp64": {"value": v64, "unit": "pairs/s", "ms_per_step": 1e3 * tot_64 / args.steps,
                 "speedup_mixed_over_fp64": value / v64,
                 "roofline": {"bound": "fp64", "achieved": v64 / ws * FLOP_PER_PAIR / 1e12, "peak": fp64_peak,
                              "unit": "TFLOP/s", "frac": v64 / ws * FLOP_PER_PAIR / 1e12 / fp64_peak,
                              "note": "peak = FP64 FMA rate measured on this device (ncg_measure_fp64_peak)"}},
        "mixed_simt": {"value": ws * pairs * len(tsimt) / sum(tsimt), "unit": "pairs/s",
                       "ms_per_step": 1e3 * sum(tsimt) / len(tsimt), "max_rel_err_vs_fp64": err_simt},
        "mixed_max_rel_err_vs_fp64": err_mx,
        "mixed_path": dict(zip(("arithmetic", "whitening_cond_max"), path_info)),
        "prepare_s": prep_s,
        "e2e": {"value": e2e_v, "unit": "pairs/s", "h2d_bytes_per_step": M * D * 8, "d2h_bytes_per_step": M * 8},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel_ms": 1e3 * dur,
                     "note": f"algorithmic {FLOP_PER_PAIR} flop/pair x {N * M} pairs per launch / mean CUDA-event "
                             f"time of the tensor-core kernel (events on the library stream around that launch "
                             f"only); peak = {src} dense bf16 (the kernel's kind::f16 MMAs run at that rate)"},
        "cpu_baseline": cb,
        "clocks": clk.summary(),
        "gpu_launches": launches_per_eval * args.steps,
    }
    if ws == 1 and not args.no_extra:
        line["config1"] = bench_config1(ng)
        line["interp"] = bench_interp(ng)
        line["batch"] = bench_batch(ng, torch)
        line["serving"] = bench_serving(ng, args.serve_rate, args.serve_steps)
        if args.serve_sweep:
            line["serving_sweep"] = {}
            for r in (float(x) for x in args.serve_sweep.split(",")):
                o = bench_serving(ng, r, args.serve_steps, small_chains=False)
                line["serving_sweep"][str(r)] = {k: o[k] for k in ("p50_ms", "p99_ms", "mean_ms", "completed",
                                                                  "failed", "pairs_per_s", "by_n")}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def bench_config1(ng):
    """Plain KDE, Gaussian kernel, FP64 (d=4, N=1000 centres, 1000 fresh points,
    1000 samples): prepare, eval_m2lnp and sample times through the C-ABI with
    host buffers (parity with the oracle: tests/test_gpu_parity.py)."""
    from numcosmo_gb300 import workloads as wl

    p = wl.config1()
    sd = ng.StatsDistKDE(ng.StatsDistKernelGauss(p.d), ng.StatsDistCV.NONE)
    sd.set_sample(p.centres)
    t0 = time.perf_counter()
    sd.prepare()
    tp = time.perf_counter() - t0
    sd.eval_m2lnp(p.points)
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        got = sd.eval_m2lnp(p.points)
    te = (time.perf_counter() - t0) / reps
    del got
    rng = ng.RNG(p.meta["sample_seed"])
    u, z, _ = rng.sample_stream(ng.StatsDistKernelGauss(p.d), 1000)
    sd.sample(u, z, None)
    t0 = time.perf_counter()
    for _ in range(reps):
        sd.sample(u, z, None)
    ts = (time.perf_counter() - t0) / reps
    out = {"workload": "kde_gauss_d4_n1000: eval_m2lnp at 1000 points, 1000 samples, FP64",
           "prepare_s": tp, "eval_s": te, "eval_pairs_per_s": 1000 * 1000 / te, "sample_s": ts}
    return out


def bench_interp(ng):
    """prepare_interp, Gaussian VKDE d=12 N=4096 (3-component mixture): FP64 NNLS
    against the mixed one (FP32 factorisation, FP64 refinement)."""
    import numpy as np

    from numcosmo_gb300 import workloads as wl

    p = wl.config3()
    out = {"workload": "prepare_interp, gauss vkde d=12 n=4096, 3-component gmm, target = exact -2lnp"}
    res = {}
    for name, prec in (("fp64", ng.Precision.FP64), ("mixed", ng.Precision.MIXED)):
        sd = ng.StatsDistVKDE(ng.StatsDistKernelGauss(12), ng.StatsDistCV.NONE)
        sd.set_sample(p.centres)
        sd.set_precision(prec)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            sd.prepare_interp(p.m2lnp)
            ts.append(time.perf_counter() - t0)
        sd.set_precision(ng.Precision.FP64)
        res[name] = (min(ts), sd.peek_weights(), sd.get_rnorm(), sd.get_interp_stats(), sd.eval_m2lnp(p.points[:2048]),
                     sd.get_interp_branch())
    (t0, w0, r0, s0, e0, b0), (t1, w1, r1, s1, e1, b1) = res["fp64"], res["mixed"]
    out.update({
        "fp64_s": t0, "mixed_s": t1, "speedup": t0 / t1, "branch": b0,
        "pairs": 4096 * 4096, "nnls": {"fp64": s0, "mixed": s1},
        "rnorm": {"fp64": r0, "mixed": r1},
        "mixed_weights_max_abs_diff_over_max": float(np.max(np.abs(w1 - w0)) / np.max(w0)),
        "mixed_weights_m2lnp_max_rel_err": float(np.max(np.abs(e1 - e0) / np.maximum(np.abs(e0), 1.0))),
    })
    return out


def bench_batch(ng, torch):
    """256 uneven problems (d 2..32, N 256..16384, KDE/VKDE, Gauss/ST) in one
    persistent launch replayed from a CUDA graph, against the same evals one
    problem at a time."""
    import numpy as np

    from numcosmo_gb300 import workloads as wl

    probs = wl.config4(256)

    def handles():
        out = []
        for p in probs:
            k = ng.StatsDistKernelST(p.d, 3.0) if p.kernel else ng.StatsDistKernelGauss(p.d)
            sd = (ng.StatsDistVKDE if p.kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
            sd.set_sample(p.centres)
            out.append(sd)
        return out

    sds = handles()
    t0 = time.perf_counter()
    for sd in sds:
        sd.prepare()
    prep = time.perf_counter() - t0
    # the same prepares issued at once (ncg_batch_prepare), on fresh handles
    sds_b = handles()
    bp = ng.Batch()
    for sd, p in zip(sds_b, probs):
        bp.add(sd, p.points.shape[0])
    t0 = time.perf_counter()
    bp.prepare()
    prep_b = time.perf_counter() - t0
    # prepare_interp (mixed NNLS) of the problems with N <= 1024: one at a
    # time against ncg_batch_prepare_interp (the full set takes minutes: the
    # low-dimensional fits run hundreds of active-set solves)
    sub = [i for i, p in enumerate(probs) if p.centres.shape[0] <= 1024]
    bi = ng.Batch()
    for i in sub:
        sds_b[i].set_precision(ng.Precision.MIXED)
        bi.add(sds_b[i], 64)
    t0 = time.perf_counter()
    bi.prepare_interp([probs[i].m2lnp for i in sub])
    interp_b = time.perf_counter() - t0
    sds_c = {}
    for i in sub:
        p = probs[i]
        k = ng.StatsDistKernelST(p.d, 3.0) if p.kernel else ng.StatsDistKernelGauss(p.d)
        sds_c[i] = (ng.StatsDistVKDE if p.kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
        sds_c[i].set_sample(p.centres)
        sds_c[i].prepare()
        sds_c[i].set_precision(ng.Precision.MIXED)
    t0 = time.perf_counter()
    for i in sub:
        sds_c[i].prepare_interp(probs[i].m2lnp)
    interp_s = time.perf_counter() - t0
    interp_same = all(np.array_equal(sds_c[i].peek_weights(), sds_b[i].peek_weights()) for i in sub)
    del sds_c, bi, bp, sds_b
    b = ng.Batch()
    for sd, p in zip(sds, probs):
        b.add(sd, p.points.shape[0])
    X = torch.from_numpy(b.pack([p.points for p in probs])).cuda()
    xo, oo, _, ot = b.layout()
    out = torch.empty(ot, dtype=torch.float64, device="cuda")
    pairs = sum(p.centres.shape[0] * p.points.shape[0] for p in probs)
    s = torch.cuda.current_stream()

    def ev_time(fn, reps):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return min(ts)

    t64 = ev_time(lambda: b.eval_m2lnp_device(X.data_ptr(), out.data_ptr(), ng.Precision.FP64, s.cuda_stream), 1)
    o64 = out.cpu().numpy().copy()
    tune_ms = b.autotune(ng.Precision.MIXED, reps=1)
    tmx = ev_time(lambda: b.eval_m2lnp_device(X.data_ptr(), out.data_ptr(), ng.Precision.MIXED, s.cuda_stream), 5)
    omx = out.cpu().numpy().copy()

    def one_at_a_time():
        for sd, p, x0, y0 in zip(sds, probs, xo, oo):
            sd.set_precision(ng.Precision.MIXED)
            sd.eval_m2lnp_device(X.data_ptr() + 8 * int(x0), p.points.shape[0], out.data_ptr() + 8 * int(y0))

    one_at_a_time()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    one_at_a_time()
    torch.cuda.synchronize()
    t1 = time.perf_counter() - t0
    st = b.get_stats(ng.Precision.MIXED)
    return {
        "workload": "256 problems: d U{2..32}, N log-U(256..16384), KDE/VKDE and Gauss/ST(3) 50/50, M = N points",
        "pairs": pairs, "prepare_all_s": prep, "prepare_all_batched_s": prep_b,
        "prepare_interp_n_le_1024": {"problems": len(sub), "one_at_a_time_s": interp_s, "batched_s": interp_b,
                                     "same_weights": interp_same},
        "mixed": {"value": pairs / tmx, "unit": "pairs/s", "ms": 1e3 * tmx, "params": b.get_params(ng.Precision.MIXED),
                  "autotune_best_ms": tune_ms, "launches": st["launches"], "items": st["items"],
                  "problems_on_fp64_tiles": st["fp64_problems"], "problems_on_tensor_cores": st["tc_problems"],
                  "graph_launches": st["graph_launches"]},
        "fp64": {"value": pairs / t64, "unit": "pairs/s", "ms": 1e3 * t64},
        "mixed_one_problem_at_a_time": {"value": pairs / t1, "unit": "pairs/s", "ms": 1e3 * t1,
                                        "note": "each handle's own launch on its own stream (wall clock)"},
        "mixed_max_rel_err_vs_fp64": float(np.max(np.abs(omx - o64) / np.maximum(np.abs(o64), 1.0))),
    }


def bench_serving(ng, rate, steps, small_chains=True):
    """64 concurrent APES chains (d U{4..32}, N in {512, 2048, 8192, 16384},
    VKDE Student-t 3, 2N walkers each), one step = one APES half-move:
    prepare_interp of the other half (N kernels) + N proposals + eval at 2N
    points + accept; Poisson arrivals; 40 GB budget; 4 slots."""
    import numpy as np

    from numcosmo_gb300 import workloads as wl

    chains = wl.config5_chains(64)

    def start(srv, subset):
        ids = {}
        for i in subset:
            c = chains[i]
            rng = np.random.default_rng(c["seed"])
            X0 = rng.standard_normal((2 * c["n"], c["d"])) @ np.linalg.cholesky(c["cov"]).T * 1.3
            ids[i] = srv.add_chain(X0, c["cov"], kind=1, kernel=1, nu=3.0, seed=c["seed"])
        return ids

    srv = ng.Server(slots=4, precision=ng.Precision.MIXED, hbm_budget=40 << 30)
    ids = start(srv, range(64))
    sched = ng.poisson_arrivals(64, steps, rate_hz=rate, seed=5005)
    reqs = ng.run_schedule(srv, [(t, ids[c]) for t, c in sched])
    srv.drain()
    st = srv.stats()
    chain_of = {v: k for k, v in ids.items()}
    by_n = {}
    for r in (srv.result(q) for q in reqs):
        c = chains[chain_of[r["chain"]]]
        by_n.setdefault(c["n"], []).append((1e3 * (r["t_done"] - r["t_start"]), 1e3 * (r["t_done"] - r["t_arrive"]),
                                           c["d"]))
    srv.close()
    out = {"workload": f"64 chains, {steps} step(s) each, Poisson {rate}/s, 4 slots, 40 GB budget, mixed",
           "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
           "completed": st["completed"], "failed": st["failed"], "pairs_per_s": st["pairs"] / st["span_s"],
           "peak_reserved_gb": st["peak_reserved_bytes"] / 2 ** 30, "evicted": st["evicted"],
           "by_n": {str(n): {"steps": len(v), "service_ms_median": float(np.median([a for a, _, _ in v])),
                             "service_ms_max": max(a for a, _, _ in v),
                             "latency_ms_max": max(b for _, b, _ in v),
                             "d_of_slowest": max(v)[2]}
                    for n, v in sorted(by_n.items())}}

    if not small_chains:
        return out

    # like for like on the chains the FP64 form finishes in seconds (N <= 2048):
    # one step each, the plain FP64 form one at a time against the mixed
    # server with all of them submitted at once
    small = [i for i in range(64) if chains[i]["n"] <= 2048]
    res = {}
    for name, prec, slots in (("fp64_one_at_a_time", ng.Precision.FP64, 1), ("mixed_4_slots", ng.Precision.MIXED, 4)):
        srv = ng.Server(slots=slots, precision=prec, hbm_budget=40 << 30)
        ids = start(srv, small)
        t0 = time.perf_counter()
        for i in small:
            srv.submit(ids[i])
        srv.drain()
        wall = time.perf_counter() - t0
        s2 = srv.stats()
        srv.close()
        res[name] = {"pairs_per_s": s2["pairs"] / wall, "wall_s": wall, "p50_ms": s2["p50_ms"],
                     "p99_ms": s2["p99_ms"], "completed": s2["completed"]}
    out["small_chains"] = {"chains": len(small), **res,
                           "speedup": res["mixed_4_slots"]["pairs_per_s"] / res["fp64_one_at_a_time"]["pairs_per_s"]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true", help="headline eval only (no interp / batch / serving)")
    ap.add_argument("--serve-rate", type=float, default=0.6, help="Poisson arrival rate of APES steps (1/s)")
    ap.add_argument("--serve-steps", type=int, default=1, help="steps per chain in the serving run")
    ap.add_argument("--serve-sweep", default="", help="extra Poisson rates (comma list) of the serving stream")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
