"""The multi-problem launch (ncg_batch_*): uneven problems in one persistent
launch give each problem's own result.

Tolerances: FP64 batch against the FP64 oracle <= 1e-10 relative (the plain
form's bar) and against the handle's own one-problem eval <= 1e-13 relative
(the two differ only in how the kernel range is sliced, i.e. in the order of
the log-sum-exp merge); mixed batch against the oracle <= 1e-6 relative with
|ref| floored at 1.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
SLICE_TOL = 1e-13
MIXED_TOL = 1e-6

# (kind, kernel, d, n, m)
SHAPES = [
    (0, 0, 2, 300, 1), (1, 1, 3, 450, 130), (0, 1, 5, 700, 257), (1, 0, 8, 520, 128),
    (1, 1, 12, 900, 300), (0, 0, 16, 1100, 64), (1, 1, 16, 1300, 513), (1, 0, 19, 800, 200),
    (0, 1, 24, 1000, 77), (1, 1, 27, 1500, 129), (1, 0, 32, 1700, 260), (0, 0, 32, 400, 50),
]


def _problem(ng, kind, kernel, d, n, m, seed, precision=0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    X = rng.standard_normal((n, d)) @ A.T + 1.0
    P = rng.standard_normal((m, d)) @ A.T + 1.0
    k = ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
    sd.set_sample(X)
    sd.set_precision(ng.Precision(precision))
    sd.prepare()
    return sd, X, P


@pytest.fixture(scope="module")
def problems(gpu):
    ng = gpu
    return [_problem(ng, *s, seed=700 + i) for i, s in enumerate(SHAPES)]


def test_batch_fp64_matches_single_and_oracle(gpu, oracle, problems):
    ng = gpu
    b = ng.Batch()
    for sd, X, P in problems:
        b.add(sd, P.shape[0])
    outs = b.eval_m2lnp([P for _, _, P in problems], ng.Precision.FP64)
    st = b.get_stats(ng.Precision.FP64)
    assert st["launches"] in (1, 2) and st["graph_launches"] >= 1 and st["captures"] >= 1
    for (sd, X, P), (kind, kernel, d, n, m), got in zip(problems, SHAPES, outs):
        assert rel_err(got, sd.eval_m2lnp(P)) < SLICE_TOL
        o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0)
        o.set_sample(X)
        assert o.prepare() == 0
        assert rel_err(got, o.eval_m2lnp(P)) < FP64_TOL


def test_batch_mixed_matches_oracle(gpu, oracle, problems):
    ng = gpu
    b = ng.Batch()
    for sd, X, P in problems:
        b.add(sd, P.shape[0])
    outs = b.eval_m2lnp([P for _, _, P in problems], ng.Precision.MIXED)
    for (sd, X, P), (kind, kernel, d, n, m), got in zip(problems, SHAPES, outs):
        o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0)
        o.set_sample(X)
        assert o.prepare() == 0
        assert rel_err(got, o.eval_m2lnp(P), floor=1.0) < MIXED_TOL


def test_batch_alone_and_in_the_mix(gpu, problems):
    """A problem's result does not depend on what else is in the launch."""
    ng = gpu
    pts = [P for _, _, P in problems]
    mix = ng.Batch()
    for sd, X, P in problems:
        mix.add(sd, P.shape[0])
    for prec in (ng.Precision.FP64, ng.Precision.MIXED):
        together = mix.eval_m2lnp(pts, prec)
        for i in (0, 4, 10):
            alone = ng.Batch()
            alone.add(problems[i][0], pts[i].shape[0])
            got = alone.eval_m2lnp([pts[i]], prec)[0]
            tol = SLICE_TOL if prec == ng.Precision.FP64 else MIXED_TOL
            assert rel_err(got, together[i], floor=1.0) < tol


def test_batch_autotune_split_and_replan(gpu, problems):
    ng = gpu
    b = ng.Batch()
    for sd, X, P in problems:
        b.add(sd, P.shape[0])
    pts = [P for _, _, P in problems]
    ref = b.eval_m2lnp(pts, ng.Precision.MIXED)
    ms = b.autotune(ng.Precision.MIXED, reps=1)
    assert ms > 0.0
    tuned = b.eval_m2lnp(pts, ng.Precision.MIXED)
    for a, c in zip(tuned, ref):
        assert rel_err(a, c, floor=1.0) < MIXED_TOL
    b.set_params(ng.Precision.MIXED, split=1, order=0, items_per_cta=3.0, tc=1)
    split = b.eval_m2lnp(pts, ng.Precision.MIXED)
    assert b.get_stats(ng.Precision.MIXED)["launches"] == 2
    for a, c in zip(split, ref):
        assert rel_err(a, c, floor=1.0) < MIXED_TOL
    # refitting one handle's weights re-plans the batch on the next call
    sd0, X0, P0 = problems[1]
    sd0.prepare_interp(np.sum(X0 * X0, axis=1))
    after = b.eval_m2lnp(pts, ng.Precision.FP64)
    assert rel_err(after[1], sd0.eval_m2lnp(P0)) < SLICE_TOL
    sd0.prepare()


@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
def test_batch_branch_schedule_equals_each_problem_alone(gpu, problems, prec):
    """tc = 2: every problem is one launch of the kernel its own eval uses,
    spread over parallel graph branches -- so each result is bit-identical to
    that problem's own eval_m2lnp, and no persistent launch runs."""
    ng = gpu
    precision = getattr(ng.Precision, prec)
    b = ng.Batch()
    for sd, X, P in problems:
        b.add(sd, P.shape[0])
    b.set_params(precision, tc=2)
    pts = [P for _, _, P in problems]
    outs = b.eval_m2lnp(pts, precision)
    outs2 = b.eval_m2lnp(pts, precision)          # graph replay
    st = b.get_stats(precision)
    assert st["launches"] == 0 and st["items"] == 0 and st["graph_launches"] >= 2
    for (sd, X, P), got, again in zip(problems, outs, outs2):
        sd.set_precision(precision)
        assert np.array_equal(got, sd.eval_m2lnp(P))
        assert np.array_equal(got, again)
        sd.set_precision(ng.Precision.FP64)


def test_batch_device_entry(gpu, problems):
    import torch

    ng = gpu
    b = ng.Batch()
    for sd, X, P in problems[:6]:
        b.add(sd, P.shape[0])
    pts = [P for _, _, P in problems[:6]]
    X = torch.from_numpy(b.pack(pts)).cuda()
    _, _, _, ot = b.layout()
    out = torch.empty(ot, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    b.eval_m2lnp_device(X.data_ptr(), out.data_ptr(), ng.Precision.FP64, stream=s.cuda_stream)
    s.synchronize()
    want = b.eval_m2lnp(pts, ng.Precision.FP64)
    for g, w in zip(b.unpack(out.cpu().numpy()), want):
        assert np.array_equal(g, w)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_prepare_and_interp_equal_one_at_a_time(gpu, precision):
    """ncg_batch_prepare / ncg_batch_prepare_interp (every problem from a pool
    of host threads, each handle on its own stream) leave each handle as its
    own prepare / prepare_interp does: identical -2 ln p and weights."""
    ng = gpu
    shapes = SHAPES[:8]
    alone, batched = [], []
    b = ng.Batch()
    for i, (kind, kernel, d, n, m) in enumerate(shapes):
        rng = np.random.default_rng(900 + i)
        X = rng.standard_normal((n, d)) * np.linspace(1.0, 2.0, d)
        P = rng.standard_normal((m, d)) * np.linspace(1.0, 2.0, d)
        m2 = np.sum((X / np.linspace(1.0, 2.0, d)) ** 2, axis=1)
        k = ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)
        one = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
        one.set_sample(X)
        one.set_precision(ng.Precision(precision))
        one.prepare()
        e0 = one.eval_m2lnp(P)
        one.prepare_interp(m2)
        alone.append((e0, one.peek_weights(), one.eval_m2lnp(P)))
        sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
        sd.set_sample(X)
        sd.set_precision(ng.Precision(precision))
        b.add(sd, m)
        batched.append((sd, P, m2))
    b.prepare(nthreads=4)
    e_b = [sd.eval_m2lnp(P) for sd, P, _ in batched]
    b.prepare_interp([m2 for _, _, m2 in batched], nthreads=4)
    for (sd, P, _), (e0, w0, e1), eb in zip(batched, alone, e_b):
        assert np.array_equal(eb, e0)
        assert np.array_equal(sd.peek_weights(), w0)
        assert np.array_equal(sd.eval_m2lnp(P), e1)
