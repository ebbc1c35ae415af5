"""Named single-GPU workloads for profiling runs (``python tests/profile_cases.py``).

    interp N d        mixed prepare_interp of a VKDE Student-t(3) handle on N
                      seeded Gaussian walkers in d dimensions, the target their
                      exact Gaussian -2 ln L (one call; prints time and NNLS
                      counters)
    eval_tc d N M     VKDE Student-t(3) with N kernels on seeded Gaussian data,
                      mixed eval_m2lnp_device at M points: three calls, then one
                      timed by the library's CUDA events (prints the kernel time)
    prepare4 COUNT    prepare of the first COUNT problems of the 256-problem
                      uneven mix, one at a time (prints the slowest problems)
    robust KIND COV N d
                      prepare of a Student-t(3) KDE (KIND 0) or VKDE (KIND 1)
                      with cov-type COV (0 SAMPLE, 2 ROBUST_DIAG, 3 ROBUST)
                      on N seeded correlated Gaussian rows in d dimensions
                      (one untimed prepare, then the median of three)

The profile summaries under ``profiles/`` name the case and arguments they ran.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from numcosmo_gb300 import Precision, StatsDistCV, StatsDistKernelST, StatsDistVKDE  # noqa: E402


def _gaussian_walkers(n: int, d: int, seed: int = 3):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    cov = A @ A.T
    L = np.linalg.cholesky(cov)
    X = rng.standard_normal((n, d)) @ L.T * 1.3
    m2 = np.sum(np.linalg.solve(L, X.T) ** 2, axis=0)
    return X, m2


def interp(n: int, d: int) -> dict:
    X, m2 = _gaussian_walkers(n, d)
    sd = StatsDistVKDE(StatsDistKernelST(d, 3.0))
    sd.set_sample(X)
    sd.set_precision(Precision.MIXED)
    t0 = time.perf_counter()
    sd.prepare_interp(m2)
    return {"case": "interp", "n": n, "d": d, "seconds": time.perf_counter() - t0, "nnls": sd.get_interp_stats()}


def eval_tc(d: int, n: int, m: int) -> dict:
    import torch

    rng = np.random.default_rng(32)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    X = rng.standard_normal((n, d)) @ A.T
    P = rng.standard_normal((m, d)) @ A.T
    sd = StatsDistVKDE(StatsDistKernelST(d, 3.0), StatsDistCV.NONE)
    st = torch.cuda.Stream()
    sd.set_stream(st.cuda_stream)
    sd.set_sample(X)
    sd.prepare()
    sd.set_precision(Precision.MIXED)
    xq = torch.tensor(P, device="cuda")
    out = torch.empty(m, dtype=torch.float64, device="cuda")
    for _ in range(3):
        sd.eval_m2lnp_device(xq.data_ptr(), m, out.data_ptr())
    sd.set_kernel_timing(True)
    sd.eval_m2lnp_device(xq.data_ptr(), m, out.data_ptr())
    ms = sd.get_kernel_time()
    return {"case": "eval_tc", "d": d, "n": n, "m": m, "path": sd.get_eval_path(), "kernel_ms": ms,
            "pairs_per_s": n * m / (ms * 1e-3)}


def prepare4(count: int) -> dict:
    from numcosmo_gb300 import StatsDistKDE, StatsDistKernelGauss
    from numcosmo_gb300 import workloads as wl

    times = []
    t_all = time.perf_counter()
    for i, p in enumerate(wl.config4(256)[:count]):
        k = StatsDistKernelST(p.d, 3.0) if p.kernel else StatsDistKernelGauss(p.d)
        sd = (StatsDistVKDE if p.kind else StatsDistKDE)(k, StatsDistCV.NONE)
        sd.set_sample(p.centres)
        t0 = time.perf_counter()
        sd.prepare()
        times.append((time.perf_counter() - t0, i, p.kind, p.d, p.centres.shape[0]))
    times.sort(reverse=True)
    return {"case": "prepare4", "count": count, "total_s": time.perf_counter() - t_all,
            "prepare_s": sum(t for t, *_ in times), "slowest (s, problem, kind, d, N)": times[:12]}


def robust(kind: int, cov: int, n: int, d: int) -> dict:
    from numcosmo_gb300 import StatsDistKDE, StatsDistKDECovType

    rng = np.random.default_rng(8)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    X = rng.standard_normal((n, d)) @ A.T + 1.5
    sd = (StatsDistVKDE if kind else StatsDistKDE)(StatsDistKernelST(d, 3.0), StatsDistCV.NONE)
    sd.set_cov_type(StatsDistKDECovType(cov))
    sd.set_sample(X)
    times = []
    for _ in range(4):
        t0 = time.perf_counter()
        sd.prepare()
        times.append(time.perf_counter() - t0)
    return {"case": "robust", "kind": kind, "cov_type": cov, "n": n, "d": d,
            "prepare_ms": 1e3 * float(np.median(times[1:])), "first_ms": 1e3 * times[0]}


def main(argv: list[str]) -> int:
    cases = {"interp": (interp, 2), "eval_tc": (eval_tc, 3), "prepare4": (prepare4, 1), "robust": (robust, 4)}
    if len(argv) < 1 or argv[0] not in cases or len(argv) != 1 + cases[argv[0]][1]:
        print(__doc__)
        return 2
    fn, _ = cases[argv[0]]
    print(fn(*(int(a) for a in argv[1:])))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
