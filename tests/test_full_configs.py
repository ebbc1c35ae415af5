"""The workload configurations at their full sizes against the oracle, through
fixtures the oracle produced on the CPU (tests/golden/make_golden.py config3 |
config4 | config5), so the GPU run does not wait for the O(N^3) CPU fits.

Tolerances: FP64 -2 ln p <= 1e-10 relative, FP64 weights <= 1e-10 of the
largest weight, mixed -2 ln p <= 1e-6 relative (|ref| floored at 1), mixed
weights <= 1e-7 of the largest weight, serving steps <= 1e-9 (walkers and
-2 ln L, relative to their largest magnitude).
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, golden, rel_err

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def test_config3_full_size(gpu):
    """prepare_interp, Gaussian VKDE d=12, N=4096, 3-component mixture."""
    ng = gpu
    from numcosmo_gb300 import workloads as wl

    p = wl.config3()
    g = golden("vkde_gauss_interp_d12_n4096")
    sd = ng.StatsDistVKDE(ng.StatsDistKernelGauss(12), ng.StatsDistCV.NONE)
    sd.set_sample(p.centres)
    sd.prepare_interp(p.m2lnp)
    assert sd.get_interp_branch() == int(g["branch"])
    w = sd.peek_weights()
    assert np.max(np.abs(w - g["weights"])) <= 1e-10 * np.max(g["weights"])
    assert sd.get_rnorm() == pytest.approx(float(g["rnorm"]), rel=1e-10)
    assert rel_err(sd.eval_m2lnp(p.points[:512]), g["m2lnp"]) < 1e-10

    sdm = ng.StatsDistVKDE(ng.StatsDistKernelGauss(12), ng.StatsDistCV.NONE)
    sdm.set_sample(p.centres)
    sdm.set_precision(ng.Precision.MIXED)
    sdm.prepare_interp(p.m2lnp)
    assert np.max(np.abs(sdm.peek_weights() - g["weights"])) <= 1e-7 * np.max(g["weights"])
    assert rel_err(sdm.eval_m2lnp(p.points[:512]), g["m2lnp"], floor=1.0) < 1e-6


def test_config4_all_problems(gpu):
    """All 256 uneven problems: each handle's FP64 eval, the FP64 batch and the
    mixed batch at the first 64 points of every problem against the oracle.

    A VKDE problem whose neighbourhoods hold fewer points than its dimension
    (k = 0.05 N < d) has singular local covariances that the nearPD repair
    makes definite with eigenvalues of the size of rounding, which decide
    -2 ln p (1e14 and more) in any implementation; for those the number of
    repaired factors must match the oracle's (a factor at the very edge of
    definiteness may go either way), and the batch must equal the handle's
    own evaluation."""
    import torch

    ng = gpu
    from numcosmo_gb300 import workloads as wl

    probs = wl.config4(256)
    g = golden("config4_m2lnp_64pts")
    want = g["m2lnp"].reshape(256, 64)
    sds, exact = [], []
    for j, p in enumerate(probs):
        k = ng.StatsDistKernelST(p.d, 3.0) if p.kernel else ng.StatsDistKernelGauss(p.d)
        sd = (ng.StatsDistVKDE if p.kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
        sd.set_sample(p.centres)
        sd.prepare()
        fo, fg = int(g["chol_fallbacks"][j]), sd.get_chol_fallbacks()
        # a factor at the edge of definiteness may fail in one implementation only
        assert (fg == 0) if fo == 0 else abs(fg - fo) <= max(2, fo // 100), p.name
        exact.append(fo == 0)
        if exact[j]:
            assert rel_err(sd.eval_m2lnp(p.points[:64]), want[j]) < 1e-10, p.name
        sds.append(sd)
    assert sum(exact) >= 150
    own = [sd.eval_m2lnp(p.points[:64]) for sd, p in zip(sds, probs)]

    b = ng.Batch()
    for sd in sds:
        b.add(sd, 64)
    X = torch.from_numpy(b.pack([p.points[:64] for p in probs])).cuda()
    xo, oo, _, ot = b.layout()
    out = torch.empty(ot, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    b.eval_m2lnp_device(X.data_ptr(), out.data_ptr(), ng.Precision.FP64, s.cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for j in range(256):
        ref = want[j] if exact[j] else own[j]
        assert rel_err(got[oo[j]:oo[j] + 64], ref) < 1e-10, probs[j].name
    b.eval_m2lnp_device(X.data_ptr(), out.data_ptr(), ng.Precision.MIXED, s.cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    for j in range(256):
        ref = want[j] if exact[j] else own[j]
        assert rel_err(got[oo[j]:oo[j] + 64], ref, floor=1.0) < 1e-6, probs[j].name
    # each handle's own mixed eval too (the tensor-core kernel where it applies)
    for j, (sd, p) in enumerate(zip(sds, probs)):
        sd.set_precision(ng.Precision.MIXED)
        ref = want[j] if exact[j] else own[j]
        assert rel_err(sd.eval_m2lnp(p.points[:64]), ref, floor=1.0) < 1e-6, p.name


@pytest.fixture(scope="module")
def config5_golden():
    return golden("config5_steps")


@pytest.mark.parametrize("d", [4, 16, 32])
@pytest.mark.parametrize("n", [512, 2048])
def test_config5_step(gpu, config5_golden, d, n):
    """One FP64 APES half-move of a chain of config 5's kind (2n walkers, VKDE
    Student-t 3 fit of n) against its CPU restatement on the oracle."""
    import make_golden as mg

    ng = gpu
    S, X0, seed = mg.config5_chain(d, n)
    srv = ng.Server(slots=1, precision=ng.Precision.FP64)
    c = srv.add_chain(X0, S, kind=1, kernel=1, nu=3.0, seed=seed)
    srv.submit(c)
    srv.drain()
    assert srv.stats()["failed"] == 0
    X, m2 = srv.chain_state(c)
    srv.close()
    Xo, mo = config5_golden[f"X_d{d}_n{n}"], config5_golden[f"m2_d{d}_n{n}"]
    assert not np.array_equal(Xo, X0)
    assert np.max(np.abs(X - Xo)) <= 1e-9 * max(1.0, np.max(np.abs(Xo)))
    assert np.max(np.abs(m2 - mo)) <= 1e-9 * max(1.0, np.max(np.abs(mo)))
