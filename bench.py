"""Benchmark: VKDE kernel-point pairs/s (d=16, N=8192, Student-t nu=3, banana).

One step = one eval_m2lnp pass of 8192 points over the 8192 prepared kernels
(6.71e7 pairs).  `value` times the mixed-precision form on device-resident
points with CUDA events on the library's stream (L2 flushed between steps by
writing a 512 MiB buffer); `e2e` times the same step through the C-ABI call a
user makes with pinned host buffers (host->device copy of the points and
device->host copy of the 8192 results inside the timed region).  The plain
FP64 form is timed the same way and reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N>1) every rank evaluates its own 8192 points against the
same kernels (weak scaling, no collective on the data path); rank 0 prints.
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
    """nvidia-smi sampling in the background during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "25"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() in ("active", "1", "true"):
                        reasons.add(nm)
            os.remove(self.path)
        except Exception:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
            "config": {"workload": "vkde_st3_d16_n8192_banana (eval_m2lnp, 8192 points x 8192 kernels)",
                       "kernels": N, "points": M, "dim": D, "kernel": "student-t nu=3",
                       "implementation": "oracle/ncg_oracle.c (NumCosmo FP64 CPU algorithm restated; the "
                                         "reference itself needs GLib/GSL/LAPACK, absent here)"},
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
    pts = p.points if rank == 0 else wl.banana(M, D, 2002 + 1000 * rank)
    xq = torch.tensor(pts, dtype=torch.float64, device="cuda")
    out = torch.empty(M, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(precision, steps, warm):
        sd.set_precision(precision)
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
        tmx = timed(ng.Precision.MIXED, args.steps, args.warmup)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    gotmx = out.cpu().numpy()
    err_mx = float(np.max(np.abs(gotmx - ref64) / np.maximum(np.abs(ref64), 1.0)))
    path_info = sd.get_eval_path()

    tot_mx = sum(tmx)
    tot_64 = sum(t64) * args.steps / len(t64)
    if dist is not None:
        tt = torch.tensor([tot_mx, tot_64], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tot_mx, tot_64 = float(tt[0]), float(tt[1])
    pairs = float(N) * M
    value = ws * pairs * args.steps / tot_mx
    v64 = ws * pairs * args.steps / tot_64

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
    e2e_tot = sum(e2e_t)
    if dist is not None:
        tt = torch.tensor([e2e_tot], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_tot = float(tt[0])
    e2e_v = ws * pairs * args.steps / e2e_tot

    peaks, src = _peaks()
    dur = statistics.mean(tmx)
    achieved = pairs * FLOP_PER_PAIR / dur / 1e12
    peak = float(peaks["bf16_tflops"])
    traffic = None
    tpath = os.path.join(HERE, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("eval_mixed_bytes_per_launch")
        except Exception:
            traffic = None

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    cb = cpu_baseline(seconds=8.0) if ws == 1 and not args.no_cpu else None
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_mx / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3/f32 (mixed)", "data": "synthetic",
        "config": {"workload": "vkde_st3_d16_n8192_banana: eval_m2lnp, 8192 points x 8192 prepared kernels",
                   "kernels": N, "points_per_gpu": M, "dim": D, "kernel": "student-t nu=3", "local_frac": 0.05,
                   "l2": "flushed between timed steps (512 MiB write)", "parallelism": f"points sharded, {ws} replica(s)"},
        "fp64": {"value": v64, "unit": "pairs/s", "ms_per_step": 1e3 * tot_64 / args.steps,
                 "speedup_mixed_over_fp64": value / v64},
        "mixed_simt": {"value": ws * pairs * len(tsimt) / sum(tsimt), "unit": "pairs/s",
                       "ms_per_step": 1e3 * sum(tsimt) / len(tsimt), "max_rel_err_vs_fp64": err_simt},
        "mixed_max_rel_err_vs_fp64": err_mx,
        "mixed_path": dict(zip(("arithmetic", "whitening_cond_max"), path_info)),
        "prepare_s": prep_s,
        "e2e": {"value": e2e_v, "unit": "pairs/s", "h2d_bytes_per_step": M * D * 8, "d2h_bytes_per_step": M * 8},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "note": f"algorithmic {FLOP_PER_PAIR} flop/pair x {N * M} pairs per launch / CUDA-event time "
                             f"of the eval launch; peak = {src} dense bf16"},
        "cpu_baseline": cb,
        "clocks": clk.summary(),
        "gpu_launches": 2 * args.steps,
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
