"""GPU parity of the C-ABI against the oracle and the golden fixtures.

Tolerances (written per assertion): FP64 form -2lnp, eval, factors and
sampled points <= 1e-10 relative; interpolation weights <= 1e-10 relative to
the largest weight; sampled kernel indices bit-exact; mixed-precision -2lnp
<= 1e-6 relative, with |ref| floored at 1 (a density near p = 1 has -2lnp
near 0, where a relative error is meaningless; there the bound is 1e-6
absolute).  Mixed-precision interpolation weights (FP32 factorisation, FP64
conjugate-gradient refinement) <= 1e-7 relative to the largest weight.
"""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-6
MIXED_W_TOL = 1e-7


def _gpu_dist(ng, kind, kernel, d, nu=3.0, X=None, precision=0, **props):
    k = ng.StatsDistKernelST(d, nu) if kernel == 1 else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind == 1 else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
    for name, v in props.items():
        getattr(sd, "set_" + name)(v)
    if X is not None:
        sd.set_sample(X)
    sd.set_precision(ng.Precision(precision))
    return sd


def _orc_dist(oracle, kind, kernel, d, nu=3.0, X=None, **kw):
    sd = oracle.OracleStatsDist(kind, kernel, d, nu=nu, **kw)
    if X is not None:
        sd.set_sample(X)
    return sd


def test_kde_config1_full(gpu, oracle):
    ng = gpu
    g = golden("kde_gauss_d4_n1000")
    sd = _gpu_dist(ng, 0, 0, 4, X=g["centres"])
    sd.prepare()
    assert sd.get_href() == pytest.approx(float(g["href"]), rel=1e-15)
    assert rel_err(sd.peek_full_cov(), g["cov"], floor=1e-3) < 1e-13
    assert rel_err(np.triu(sd.peek_full_cov_decomp()), np.triu(g["U"]), floor=1e-3) < 1e-13
    m2 = sd.eval_m2lnp(g["points"])
    assert rel_err(m2, g["m2lnp"]) < FP64_TOL
    assert rel_err(sd.eval(g["points"][:64]), g["p"]) < FP64_TOL
    x, idx = sd.sample(g["u"], g["z"])
    assert np.array_equal(idx, g["idx"])
    assert np.max(np.abs(x - g["x"])) <= FP64_TOL * max(1.0, np.max(np.abs(g["x"])))
    sd.set_precision(ng.Precision.MIXED)
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"], floor=1.0) < MIXED_TOL


def test_vkde_st3_golden(gpu, oracle):
    ng = gpu
    g = golden("vkde_st3_d16_n1024")
    sd = _gpu_dist(ng, 1, 1, 16, nu=3.0, X=g["centres"])
    sd.prepare()
    assert sd.get_knn_k() == 51
    assert sd.get_href() == 1.0
    assert rel_err(np.triu(sd.peek_cov_decomp(0)), np.triu(g["U0"]), floor=1e-2) < 1e-12
    assert rel_err(np.triu(sd.peek_cov_decomp(7)), np.triu(g["U7"]), floor=1e-2) < 1e-12
    lnn = np.array([sd.get_lnnorm(i) for i in (0, 1, 500, 1023)])
    assert rel_err(lnn, g["lnnorms"][[0, 1, 500, 1023]], floor=1.0) < 1e-12
    m2 = sd.eval_m2lnp(g["points"])
    assert rel_err(m2, g["m2lnp"]) < FP64_TOL
    x, idx = sd.sample(g["u"], g["z"], g["chisq"])
    assert np.array_equal(idx, g["idx"])
    assert np.max(np.abs(x - g["x"])) <= FP64_TOL * max(1.0, np.max(np.abs(g["x"])))
    sd.set_precision(ng.Precision.MIXED)
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"], floor=1.0) < MIXED_TOL


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("kernel,nu", [(0, 0.0), (1, 3.0), (1, 1.0), (1, 5.5)])
@pytest.mark.parametrize("d", [1, 2, 3, 5, 8, 13, 16, 21, 32])
def test_eval_parity_grid(gpu, oracle, kind, kernel, nu, d):
    ng = gpu
    n = 60 * d + 100
    rng = np.random.default_rng(1000 * d + 10 * kind + kernel)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    X = rng.standard_normal((n, d)) @ A.T + 3.0
    P = rng.standard_normal((97, d)) @ A.T + 3.0
    o = _orc_dist(oracle, kind, kernel, d, nu=nu or 3.0, X=X)
    assert o.prepare() == 0
    want = o.eval_m2lnp(P)
    sd = _gpu_dist(ng, kind, kernel, d, nu=nu or 3.0, X=X)
    sd.prepare()
    assert sd.get_href() == pytest.approx(o.href, rel=1e-15)
    assert rel_err(sd.eval_m2lnp(P), want) < FP64_TOL
    assert rel_err(sd.eval(P[:16]), o.eval(P[:16])) < FP64_TOL
    assert sd.eval_m2lnp(P[3]) == pytest.approx(want[3], rel=FP64_TOL)
    sd.set_precision(ng.Precision.MIXED)
    assert rel_err(sd.eval_m2lnp(P), want, floor=1.0) < MIXED_TOL


def test_vkde_config2_full_kernels(gpu, oracle):
    """N = 8192 kernels of the banana at d=16 (1024 of the 8192 points checked against the oracle)."""
    ng = gpu
    from numcosmo_gb300 import workloads as wl

    p = wl.config2()
    o = _orc_dist(oracle, 1, 1, 16, nu=3.0, X=p.centres)
    assert o.prepare() == 0
    sd = _gpu_dist(ng, 1, 1, 16, nu=3.0, X=p.centres)
    sd.prepare()
    assert sd.get_knn_k() == 409 == o.k
    sub = p.points[:1024]
    want = o.eval_m2lnp(sub)
    got = sd.eval_m2lnp(p.points)
    assert rel_err(got[:1024], want) < FP64_TOL
    sd.set_precision(ng.Precision.MIXED)
    gotm = sd.eval_m2lnp(p.points)
    assert rel_err(gotm[:1024], want, floor=1.0) < MIXED_TOL
    assert rel_err(gotm, got, floor=1.0) < MIXED_TOL
    for i in (0, 4095, 8191):
        assert sd.get_lnnorm(i) == pytest.approx(o.lnnorms()[i], rel=1e-12)


def test_interp_golden(gpu, oracle):
    ng = gpu
    g = golden("vkde_gauss_interp_d12_n512")
    sd = _gpu_dist(ng, 1, 0, 12, X=g["centres"])
    sd.prepare_interp(g["target"])
    assert sd.get_interp_branch() == 0
    w = sd.peek_weights()
    assert np.max(np.abs(w - g["weights"])) <= FP64_TOL * np.max(np.abs(g["weights"]))
    assert sd.get_rnorm() == pytest.approx(float(g["rnorm"]), rel=1e-10)
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"]) < FP64_TOL


@pytest.mark.parametrize("kind,kernel", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_interp_parity(gpu, oracle, kind, kernel):
    ng = gpu
    rng = np.random.default_rng(40 + kind * 2 + kernel)
    d, n = 5, 700
    X = rng.standard_normal((n, d)) * np.linspace(0.5, 2.0, d)
    m2 = np.sum((X / np.linspace(0.5, 2.0, d)) ** 2, axis=1) + 0.3 * np.sin(X[:, 0])
    o = _orc_dist(oracle, kind, kernel, d, nu=4.0, X=X)
    assert o.prepare_interp(m2) == 0
    sd = _gpu_dist(ng, kind, kernel, d, nu=4.0, X=X)
    sd.prepare_interp(m2)
    w, wo = sd.peek_weights(), o.weights()
    assert np.max(np.abs(w - wo)) <= FP64_TOL * np.max(wo)
    assert sd.get_rnorm() == pytest.approx(o.rnorm, rel=1e-10)
    IM = sd.compute_IM()
    assert rel_err(IM, o.compute_IM(), floor=1e-300) < FP64_TOL
    u = rng.uniform(size=4000)
    assert np.array_equal(sd.kernel_choose(u), o.kernel_choose(u))


@pytest.mark.parametrize("kind,kernel", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_interp_mixed_parity(gpu, oracle, kind, kernel):
    """Mixed NNLS: the same active-set decisions, weights within MIXED_W_TOL."""
    ng = gpu
    rng = np.random.default_rng(40 + kind * 2 + kernel)
    d, n = 5, 700
    X = rng.standard_normal((n, d)) * np.linspace(0.5, 2.0, d)
    m2 = np.sum((X / np.linspace(0.5, 2.0, d)) ** 2, axis=1) + 0.3 * np.sin(X[:, 0])
    o = _orc_dist(oracle, kind, kernel, d, nu=4.0, X=X)
    assert o.prepare_interp(m2) == 0
    sd = _gpu_dist(ng, kind, kernel, d, nu=4.0, X=X, precision=1)
    sd.prepare_interp(m2)
    st = sd.get_interp_stats()
    assert st["solves"] > 0 and st["fp64"] == 0 and 0 < st["cg_iters"] <= 5 * st["solves"]
    w, wo = sd.peek_weights(), o.weights()
    assert np.max(np.abs(w - wo)) <= MIXED_W_TOL * np.max(wo)
    assert sd.get_rnorm() == pytest.approx(o.rnorm, rel=1e-8)
    pts = rng.standard_normal((300, d))
    sd.set_precision(ng.Precision.FP64)
    assert rel_err(sd.eval_m2lnp(pts), o.eval_m2lnp(pts), floor=1.0) < MIXED_TOL


def test_interp_mixed_golden(gpu):
    ng = gpu
    g = golden("vkde_gauss_interp_d12_n512")
    sd = _gpu_dist(ng, 1, 0, 12, X=g["centres"], precision=1)
    sd.prepare_interp(g["target"])
    assert sd.get_interp_branch() == 0
    assert sd.get_interp_stats()["fp64"] == 0
    w = sd.peek_weights()
    assert np.max(np.abs(w - g["weights"])) <= MIXED_W_TOL * np.max(np.abs(g["weights"]))
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"], floor=1.0) < MIXED_TOL


def test_interp_config3_mixed_vs_fp64(gpu):
    """Gauss VKDE d=12, N=4096 from the 3-component mixture: the mixed fit
    against the FP64 fit of the same handle type (itself pinned to the oracle
    at smaller sizes)."""
    ng = gpu
    from numcosmo_gb300 import workloads as wl

    p = wl.config3()
    res = {}
    for prec in (0, 1):
        sd = _gpu_dist(ng, 1, 0, 12, X=p.centres, precision=prec)
        sd.prepare_interp(p.m2lnp)
        res[prec] = (sd.peek_weights(), sd.get_rnorm(), sd.get_interp_stats(), sd.eval_m2lnp(p.points[:2048]))
    w0, r0, s0, e0 = res[0]
    w1, r1, s1, e1 = res[1]
    assert s1["fp64"] == 0 and s0["solves"] == s1["solves"]
    # a good FP32 preconditioner: a few conjugate-gradient iterations per solve
    assert s1["cg_iters"] <= 4 * s1["solves"] and s1["shifted"] == 0
    assert np.max(np.abs(w1 - w0)) <= MIXED_W_TOL * np.max(w0)
    assert r1 == pytest.approx(r0, rel=1e-8)
    assert rel_err(e1, e0, floor=1.0) < MIXED_TOL


def test_interp_range_cut_branches(gpu, oracle):
    ng = gpu
    g = golden("kde_st4_interp_cut_d3_n300")
    for tag, key in (("heur", "m2_heur"), ("cut", "m2_cut")):
        sd = _gpu_dist(ng, 0, 1, 3, nu=4.0, X=g["centres"])
        sd.prepare_interp(g[key])
        assert sd.get_interp_branch() == int(g[f"{tag}_branch"])
        assert sd.get_sample_size() == int(g[f"{tag}_n"])
        w = sd.peek_weights()
        assert np.max(np.abs(w - g[f"{tag}_weights"])) <= FP64_TOL * np.max(g[f"{tag}_weights"])
        assert rel_err(sd.eval_m2lnp(g["centres"][:50]), g[f"{tag}_m2lnp"]) < FP64_TOL


def test_nearpd_fallback_high_dim(gpu, oracle):
    """d=32, N=512: k = 25 neighbours < d, so every local covariance is singular."""
    ng = gpu
    rng = np.random.default_rng(91)
    d, n = 32, 512
    X = rng.standard_normal((n, d))
    o = _orc_dist(oracle, 1, 0, d, X=X)
    assert o.prepare() == 0
    assert o.chol_fallbacks > 0
    sd = _gpu_dist(ng, 1, 0, d, X=X)
    sd.prepare()
    assert sd.get_chol_fallbacks() == o.chol_fallbacks
    # The repaired covariances keep eigenvalues of order eps * lambda_min, which
    # rounding decides in any implementation (and so does -2lnp, ~1e15 here):
    # compare the repaired matrices U^T U relative to their norm instead.
    for i in (0, 17, 255, 511):
        Ug, Uo = np.triu(sd.peek_cov_decomp(i)), np.triu(o.Ui(i))
        Sg, So = Ug.T @ Ug, Uo.T @ Uo
        assert np.max(np.abs(Sg - So)) <= 1e-9 * np.max(np.abs(So))
        assert np.all(np.diag(Ug) > 0)


def test_sample_indices_bit_exact(gpu, oracle):
    ng = gpu
    rng = np.random.default_rng(5)
    X = rng.standard_normal((3000, 6))
    for kind, kernel in ((0, 1), (1, 0)):
        o = _orc_dist(oracle, kind, kernel, 6, nu=3.0, X=X)
        assert o.prepare() == 0
        sd = _gpu_dist(ng, kind, kernel, 6, nu=3.0, X=X)
        sd.prepare()
        k = ng.StatsDistKernelST(6, 3.0) if kernel else ng.StatsDistKernelGauss(6)
        u, z, cs = ng.RNG(11 + kind).sample_stream(k, 20000)
        x, idx = sd.sample(u, z, cs)
        xo, io = o.sample(u, z, cs)
        assert np.array_equal(idx, io)
        assert np.max(np.abs(x - xo)) <= FP64_TOL * np.max(np.abs(xo))


def test_errors_are_status_codes(gpu):
    ng = gpu
    sd = _gpu_dist(ng, 1, 0, 4)
    with pytest.raises(ng.NcgError) as e:
        sd.eval_m2lnp(np.zeros(4))
    assert e.value.name == "NCG_ERR_NOT_PREPARED"
    sd.set_sample(np.random.default_rng(0).standard_normal((4, 4)))
    with pytest.raises(ng.NcgError) as e:
        sd.prepare()
    assert e.value.name == "NCG_ERR_SAMPLE_TOO_SMALL"
    sd.set_sample(np.random.default_rng(0).standard_normal((30, 4)))
    with pytest.raises(ng.NcgError) as e:
        sd.prepare()
    assert e.value.name == "NCG_ERR_TOO_FEW_LOCAL"
    with pytest.raises(ng.NcgError) as e:
        sd.add_obs(np.array([0.0, np.nan, 0.0, 0.0]))
    assert e.value.name == "NCG_ERR_NONFINITE"
    sd.set_sample(np.random.default_rng(0).standard_normal((200, 4)))
    sd.prepare()
    with pytest.raises(ng.NcgError) as e:
        sd.eval_m2lnp(np.array([[0.0, 0.0, np.inf, 0.0]]))
    assert e.value.name == "NCG_ERR_NONFINITE"


def test_run_twice_identical(gpu):
    ng = gpu
    g = golden("vkde_st3_d16_n1024")
    outs = []
    for prec in (0, 0, 1, 1):
        sd = _gpu_dist(ng, 1, 1, 16, nu=3.0, X=g["centres"], precision=prec)
        sd.prepare()
        outs.append(sd.eval_m2lnp(g["points"]))
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[2], outs[3])


def test_device_pointer_entry(gpu):
    import torch

    ng = gpu
    g = golden("vkde_st3_d16_n1024")
    sd = _gpu_dist(ng, 1, 1, 16, nu=3.0, X=g["centres"])
    sd.prepare()
    s = torch.cuda.Stream()
    sd.set_stream(s.cuda_stream)
    xq = torch.tensor(g["points"], dtype=torch.float64, device="cuda")
    out = torch.empty(xq.shape[0], dtype=torch.float64, device="cuda")
    with torch.cuda.stream(s):
        sd.eval_m2lnp_device(xq.data_ptr(), xq.shape[0], out.data_ptr())
    s.synchronize()
    assert rel_err(out.cpu().numpy(), g["m2lnp"]) < FP64_TOL


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("n,m", [(1000, 1000), (4099, 257), (1000, 1), (350, 130), (8192, 8192)])
def test_tensor_core_eval(gpu, oracle, kernel, n, m):
    """The tcgen05 TF32x3 form (VKDE, d=16) against the FP64 form, the FP32 SIMT form
    and the oracle, with ragged point and kernel counts."""
    ng = gpu
    from numcosmo_gb300 import workloads as wl

    X = wl.banana(n, 16, 3100 + n)
    P = wl.banana(m, 16, 3200 + m)
    sd = _gpu_dist(ng, 1, kernel, 16, nu=3.0, X=X)
    sd.prepare()
    f64 = sd.eval_m2lnp(P)
    sd.set_precision(ng.Precision.MIXED)
    tc = sd.eval_m2lnp(P)
    path, kappa = sd.get_eval_path()
    sd.set_precision(ng.Precision.MIXED_SIMT)
    simt = sd.eval_m2lnp(P)
    assert rel_err(tc, f64, floor=1.0) < MIXED_TOL
    assert rel_err(simt, f64, floor=1.0) < MIXED_TOL
    if n == 350:
        # k = 17 neighbours in d = 16: nearly singular local covariances, the
        # FP32 whitening is too ill-conditioned and the mixed request runs FP64
        assert kappa > 1000 and path == "fp64"
        assert np.array_equal(tc, f64)
    else:
        assert kappa < 1000 and path == "tensor_core"
    if n * m <= 2_000_000:
        o = _orc_dist(oracle, 1, kernel, 16, nu=3.0, X=X)
        assert o.prepare() == 0
        assert rel_err(f64, o.eval_m2lnp(P)) < FP64_TOL
    # repeated calls give identical bits
    sd.set_precision(ng.Precision.MIXED)
    assert np.array_equal(sd.eval_m2lnp(P), tc)


@pytest.mark.parametrize("kind,kernel", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_cov_fixed_parity(gpu, oracle, kind, kernel):
    """cov-type FIXED (ncm_stats_dist_kde.c:414-421, 825-845): the given matrix
    is the global covariance (and the VKDE whitening), factored as given;
    -2lnp, factors and interpolation weights against the oracle; a matrix
    that is not positive definite is an error on both sides."""
    ng = gpu
    rng = np.random.default_rng(70 + 2 * kind + kernel)
    d, n = 4, 900
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    X = rng.standard_normal((n, d)) @ A.T + 1.0
    F = 1.3 * A @ A.T + 0.2 * np.eye(d)
    P = rng.standard_normal((64, d)) @ A.T + 1.0
    props = dict(cov_type=ng.StatsDistKDECovType.FIXED, cov_fixed=F)
    sd = _gpu_dist(ng, kind, kernel, d, nu=3.5, X=X, **props)
    sd.prepare()
    o = _orc_dist(oracle, kind, kernel, d, nu=3.5, X=X, cov_type=1)
    o.set_cov_fixed(F)
    assert o.prepare() == 0
    assert np.array_equal(sd.peek_full_cov(), F)
    assert rel_err(np.triu(sd.peek_full_cov_decomp()), o.U(), floor=1e-3) < 1e-12
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < FP64_TOL
    if kind == 1:
        for i in (0, 17, n - 1):
            Ug, Uo = np.triu(sd.peek_cov_decomp(i)), np.triu(o.Ui(i))
            assert rel_err(Ug, Uo, floor=1e-3 * np.max(np.abs(Uo))) < FP64_TOL
    m2 = np.sum(np.linalg.solve(A, (X - 1.0).T) ** 2, axis=0)
    sd.prepare_interp(m2)
    assert o.prepare_interp(m2) == 0
    w, wo = sd.peek_weights(), o.weights()
    assert np.max(np.abs(w - wo)) <= FP64_TOL * np.max(wo)
    bad = np.diag([1.0, 1.0, -1.0, 1.0])
    sd_bad = _gpu_dist(ng, kind, kernel, d, nu=3.5, X=X, cov_type=ng.StatsDistKDECovType.FIXED, cov_fixed=bad)
    with pytest.raises(ng.NcgError) as e:
        sd_bad.prepare()
    assert e.value.name == "NCG_ERR_NOT_PD"
    o_bad = _orc_dist(oracle, kind, kernel, d, nu=3.5, X=X, cov_type=1)
    o_bad.set_cov_fixed(bad)
    assert o_bad.prepare() == 4
