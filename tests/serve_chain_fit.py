"""One APES fit (prepare_interp, mixed precision) of config-5 serving chains,
as the serving step runs it: the fit of the other half of the chain's 2N
seeded walkers (N kernels, VKDE Student-t 3) to the Gaussian target's -2 ln L;
prints the prepare and fit times and the NNLS counters.  The profiling
workload of profiles/interp_serving_chain12_vkde_st3_d11_n16384.md.

    python tests/serve_chain_fit.py <chain index> [...]
"""
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def fit(cid: int) -> dict:
    import numcosmo_gb300 as ng
    from numcosmo_gb300 import workloads as wl

    c = wl.config5_chains(64)[cid]
    rng = np.random.default_rng(c["seed"])
    L = np.linalg.cholesky(c["cov"])
    X0 = rng.standard_normal((2 * c["n"], c["d"])) @ L.T * 1.3     # the bench's initial walkers
    X = X0[c["n"]:]                                                 # the half the first step fits
    y = np.linalg.solve(L, X.T)
    m2 = np.sum(y * y, axis=0) + 2 * np.sum(np.log(np.diag(L)))
    sd = ng.StatsDistVKDE(ng.StatsDistKernelST(c["d"], 3.0), ng.StatsDistCV.NONE)
    sd.set_precision(ng.Precision.MIXED)
    sd.set_sample(X)
    sd.prepare()
    t0 = time.perf_counter()
    sd.prepare()
    tp = time.perf_counter() - t0
    t0 = time.perf_counter()
    sd.prepare_interp(m2)
    ti = time.perf_counter() - t0
    return {"chain": cid, "d": c["d"], "n": c["n"], "prepare_s": tp, "interp_s": ti, "stats": sd.get_interp_stats()}


if __name__ == "__main__":
    for a in sys.argv[1:]:
        print(fit(int(a)), flush=True)
