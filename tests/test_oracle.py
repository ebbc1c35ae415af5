"""Pinning of the CPU oracle (no GPU).

* kNN against NumCosmo's own kd-tree (numcosmo/external/misc/kdtree.c), live when
  oracle/_ref is built and through the stored fixture otherwise;
* kernel formulas against the closed forms of the reference's own tests
  (tests/c/ncm/stats/test_ncm_stats_dist_kernel.c:179-202 bandwidth,
  :204-256 lnnorm and unnormalised kernel, :314-428 sum0/sum1 gamma/lambda);
* Welford covariance, Cholesky, NNLS and eval against independent numpy/scipy
  computations (parity of these pieces with NumCosmo itself is unpinned: the
  reference cannot be built here);
* the stored golden fixtures (regression across machines).
"""
import numpy as np
import pytest
import scipy.optimize
import scipy.special
from scipy.special import gammaln

from conftest import golden, rel_err


def test_knn_matches_reference_kdtree_fixture(oracle):
    g = golden("kdtree_ref_knn")
    for d in (1, 3, 8, 16):
        Y = g[f"Y_d{d}"]
        want = g[f"knn_d{d}"]
        got = oracle.knn(Y, want.shape[1])
        assert np.array_equal(got, want), f"d={d}"


def test_knn_matches_reference_kdtree_live(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("reference kd-tree not built (NumCosmo sources absent)")
    rng = np.random.default_rng(5)
    for d, n, k in ((2, 300, 15), (5, 800, 40), (12, 1500, 75), (16, 2000, 100)):
        Y = rng.standard_normal((n, d)) * rng.uniform(0.5, 3.0, d)
        Y[10:14] = Y[3]            # exact duplicates: ties broken by index
        assert np.array_equal(oracle.knn(Y, k), oracle.ref_knn(Y, k)), (d, n, k)


@pytest.mark.parametrize("kernel,nu", [(0, 0.0), (1, 3.0), (1, 4.7), (1, 1.5)])
@pytest.mark.parametrize("d", [1, 2, 3, 7, 16])
def test_kernel_bandwidth_and_lnnorm_closed_forms(oracle, kernel, nu, d):
    rng = np.random.default_rng(d * 10 + kernel)
    n = rng.uniform(1.0, 200.0)
    h = oracle.lib().orc_kernel_rot_bandwidth(kernel, nu, d, n)
    if kernel == 0:
        want = (4.0 / (n * (d + 2.0))) ** (1.0 / (d + 4.0))
    else:
        nuc = max(nu, 3.0)
        want = (16.0 * (nuc - 2) ** 2 * (1.0 + d + nuc) * (3.0 + d + nuc)
                / ((2.0 + d) * (d + nuc) * (2.0 + d + nuc) * (d + 2.0 * nuc) * (2.0 + d + 2.0 * nuc) * n)) ** (1.0 / (d + 4.0))
    assert abs(h - want) <= 1e-14 * abs(want)

    A = rng.standard_normal((d, d))
    S = A @ A.T + d * np.eye(d)
    U, info = oracle.cholesky_upper(S)
    assert info == 0
    lndet = np.linalg.slogdet(S)[1]
    got = oracle.lib().orc_kernel_lnnorm(kernel, nu, d, oracle.dptr(np.ascontiguousarray(np.triu(U))))
    if kernel == 0:
        want = 0.5 * (d * np.log(2 * np.pi) + lndet)
    else:
        want = gammaln(nu / 2) - gammaln((nu + d) / 2) + 0.5 * lndet + (d / 2.0) * (np.log(np.pi) + np.log(nu))
    assert abs(got - want) <= 1e-13 * max(1.0, abs(want))

    for chi2 in rng.uniform(0, 100, 20):
        got = oracle.lib().orc_kernel_eval_unnorm(kernel, nu, d, chi2)
        want = np.exp(-0.5 * chi2) if kernel == 0 else (1 + chi2 / nu) ** (-0.5 * (nu + d))
        assert abs(got - want) <= 1e-15 * max(want, 1e-300) + 1e-300


@pytest.mark.parametrize("kernel,nu", [(0, 3.0), (1, 3.0), (1, 4.2)])
def test_kernel_sum_gamma_lambda(oracle, kernel, nu):
    """tests/c/ncm/stats/test_ncm_stats_dist_kernel.c:314-428 restated."""
    rng = np.random.default_rng(11)
    d = 3
    n = int(rng.integers(5, 100))
    w = rng.uniform(1.0, 200.0, n)
    lnu = rng.uniform(1.0, 200.0, n)
    chi2 = rng.uniform(1.0, 200.0, n)
    lnnorm = rng.uniform(1.0, 200.0)
    kappa = -0.5 * (nu + d)
    t = -0.5 * chi2 if kernel == 0 else kappa * np.log1p(chi2 / nu)
    lnt0 = t - lnu + np.log(w)
    lnt1 = t + np.log(w)
    g0, l0 = oracle.kernel_sum(kernel, nu, d, chi2, w, lnu=lnu)
    g1, l1 = oracle.kernel_sum(kernel, nu, d, chi2, w, lnnorm=lnnorm)
    i0, i1 = int(np.argmax(lnt0)), int(np.argmax(lnt1))
    assert g0 == pytest.approx(lnt0[i0], rel=1e-15)
    assert g1 == pytest.approx(lnt1[i1] - lnnorm, rel=1e-15)
    want0 = np.sum(np.exp(np.delete(lnt0, i0) - lnt0[i0]))
    want1 = np.sum(np.exp(np.delete(lnt1, i1) - lnt1[i1]))
    assert l0 == pytest.approx(want0, rel=1e-13, abs=1e-300)
    assert l1 == pytest.approx(want1, rel=1e-13, abs=1e-300)


def test_welford_cov_and_cholesky(oracle):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((700, 6)) @ rng.standard_normal((6, 6)) + 5.0
    c = oracle.welford_cov(X)
    assert rel_err(c, np.cov(X.T), floor=1e-3) < 1e-12
    rows = rng.permutation(700)[:50]
    c2 = oracle.welford_cov(X, rows)
    assert rel_err(c2, np.cov(X[rows].T), floor=1e-3) < 1e-12
    U, info = oracle.cholesky_upper(c)
    U = np.triu(U)
    assert info == 0
    assert rel_err(U.T @ U, c, floor=1e-3) < 1e-13
    assert oracle.lndet(U) == pytest.approx(np.linalg.slogdet(c)[1], rel=1e-13)


def test_cholesky_fallbacks(oracle):
    # rank-deficient covariance: Cholesky fails, nearPD repairs it
    rng = np.random.default_rng(4)
    B = rng.standard_normal((5, 3))
    S = B @ B.T
    U, r = oracle.cholesky_decomp_fallback(S, 200)
    assert r in (1, 2)
    assert np.all(np.diag(U) > 0)
    if r == 1:
        # the repaired matrix keeps the original diagonal (Higham's unit-diagonal projection)
        assert np.allclose(np.diag(U.T @ U), np.diag(S), rtol=1e-10)
    # zero covariance: nothing can repair it
    U, r = oracle.cholesky_decomp_fallback(np.zeros((3, 3)), 10)
    assert r == -1


def test_nnls_matches_scipy(oracle):
    rng = np.random.default_rng(8)
    for m, n in ((40, 30), (120, 80), (200, 200)):
        A = np.abs(rng.standard_normal((m, n))) + 0.1 * np.eye(m, n)
        f = rng.standard_normal(m) + 1.0
        x, rn = oracle.nnls(A, f)
        xs, rns = scipy.optimize.nnls(A, f, maxiter=50 * n)
        assert rn == pytest.approx(rns, rel=1e-10)
        assert np.max(np.abs(x - xs)) <= 1e-9 * max(1.0, np.max(np.abs(xs)))
        assert np.all(x >= 0)


@pytest.mark.parametrize("cov_type", [0, 1, 2, 3])
@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("kernel", [0, 1])
def test_eval_m2lnp_direct_restatement(oracle, kind, kernel, cov_type):
    """-2 ln p as the log-sum-exp of the kernels written out in numpy from the
    oracle's factors, for every covariance type (SAMPLE, FIXED, ROBUST_DIAG,
    ROBUST); the KDE's factor is the Cholesky factor of the type's matrix."""
    rng = np.random.default_rng(21 + 2 * kind + kernel)
    d, n, nu = 3, 300, 3.5
    X = rng.standard_normal((n, d)) * [1.0, 3.0, 0.5]
    sd = oracle.OracleStatsDist(kind, kernel, d, nu=nu, cov_type=cov_type)
    F = np.diag([1.2, 8.0, 0.3]) + 0.1
    if cov_type == 1:
        sd.set_cov_fixed(F)
    sd.set_sample(X)
    assert sd.prepare() == 0
    want_cov = {0: np.cov(X.T), 1: F}.get(cov_type)
    if want_cov is not None:
        assert rel_err(sd.cov(), want_cov, floor=1e-3) < 1e-13
    assert rel_err(sd.U().T @ sd.U(), sd.cov(), floor=1e-3) < 1e-13
    xq = rng.standard_normal((9, d))
    got = sd.eval_m2lnp(xq)
    h, w = sd.href, sd.weights()
    want = []
    for x in xq:
        lnt = []
        for i in range(n):
            Ui = sd.Ui(i)
            y = np.linalg.solve(Ui.T, x - X[i])
            chi2 = y @ y / h ** 2
            t = -0.5 * chi2 if kernel == 0 else -0.5 * (nu + d) * np.log1p(chi2 / nu)
            lnu = sd.lnnorms()[i]
            lnt.append(t - lnu + np.log(w[i]))
        want.append(-2.0 * (scipy.special.logsumexp(lnt) - d * np.log(h)))
    assert rel_err(got, want) < 1e-13
    assert rel_err(sd.eval(xq), np.exp(-0.5 * np.asarray(want))) < 1e-12


def test_kde_prepare_bits(oracle):
    g = golden("kde_gauss_d4_n1000")
    sd = oracle.OracleStatsDist(0, 0, 4)
    sd.set_sample(g["centres"])
    assert sd.prepare() == 0
    n, d = 1000, 4
    assert sd.href == pytest.approx((4.0 / (n * (d + 2.0))) ** (1.0 / (d + 4.0)), rel=1e-15)
    assert rel_err(sd.cov(), g["cov"], floor=1e-3) < 1e-13
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"]) < 1e-12


def test_golden_vkde_st3(oracle):
    g = golden("vkde_st3_d16_n1024")
    sd = oracle.OracleStatsDist(1, 1, 16, nu=3.0)
    sd.set_sample(g["centres"])
    assert sd.prepare() == 0
    assert sd.k == 51
    assert np.array_equal(sd.knn(), g["knn_ref"])
    assert rel_err(sd.lnnorms(), g["lnnorms"], floor=1.0) < 1e-12
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"]) < 1e-12
    x, idx = sd.sample(g["u"], g["z"], g["chisq"])
    assert np.array_equal(idx, g["idx"])
    assert np.max(np.abs(x - g["x"])) < 1e-11


def test_golden_interp(oracle):
    g = golden("vkde_gauss_interp_d12_n512")
    sd = oracle.OracleStatsDist(1, 0, 12)
    sd.set_sample(g["centres"])
    assert sd.prepare_interp(g["target"]) == 0
    assert sd.interp_branch == int(g["branch"]) == 0
    w = sd.weights()
    assert np.max(np.abs(w - g["weights"])) <= 1e-10 * np.max(np.abs(g["weights"]))
    assert sd.rnorm == pytest.approx(float(g["rnorm"]), rel=1e-10)
    assert abs(w.sum() - 1.0) < 1e-12


def test_golden_interp_range_cut(oracle):
    g = golden("kde_st4_interp_cut_d3_n300")
    for tag, key in (("heur", "m2_heur"), ("cut", "m2_cut")):
        sd = oracle.OracleStatsDist(0, 1, 3, nu=4.0)
        sd.set_sample(g["centres"])
        assert sd.prepare_interp(g[key]) == 0
        assert sd.interp_branch == int(g[f"{tag}_branch"])
        assert sd.n == int(g[f"{tag}_n"])
        assert np.max(np.abs(sd.weights() - g[f"{tag}_weights"])) <= 1e-10 * np.max(g[f"{tag}_weights"])
    assert int(g["heur_branch"]) == 1 and int(g["cut_branch"]) == 2 and int(g["cut_n"]) == 260


def test_prepare_errors(oracle):
    sd = oracle.OracleStatsDist(1, 0, 5)
    sd.set_sample(np.random.default_rng(0).standard_normal((5, 5)))
    assert sd.prepare() == 2                      # n <= d
    sd = oracle.OracleStatsDist(1, 0, 2, local_frac=0.05)
    sd.set_sample(np.random.default_rng(0).standard_normal((30, 2)))
    assert sd.prepare() == 3                      # local_frac * n < 2


def test_kernel_choose_binary_search(oracle):
    rng = np.random.default_rng(2)
    X = rng.standard_normal((50, 2))
    sd = oracle.OracleStatsDist(0, 0, 2)
    sd.set_sample(X)
    assert sd.prepare() == 0
    u = rng.uniform(size=2000)
    idx = sd.kernel_choose(u)
    # equal weights: index = floor(u * n) up to the rounding of the cumulative table
    assert np.mean(idx == np.floor(u * 50)) > 0.99


def _qn_brute(x):
    """Qn by enumerating every pairwise difference (Rousseeuw & Croux 1993)."""
    x = np.sort(np.asarray(x, dtype=np.float64))
    m = x.size
    diffs = np.sort(np.concatenate([x[j + 1:] - x[j] for j in range(m - 1)]))
    h = m // 2 + 1
    k = h * (h - 1) // 2
    small = {2: 0.399, 3: 0.994, 4: 0.512, 5: 0.844, 6: 0.611, 7: 0.857, 8: 0.669, 9: 0.872}
    dn = small[m] if m <= 9 else (m / (m + 1.4) if m % 2 else m / (m + 3.8))
    return 2.21914 * dn * diffs[k - 1]


@pytest.mark.parametrize("m", [4, 5, 6, 7, 8, 9, 10, 11, 31, 64, 101, 409])
def test_qn_matches_enumeration(oracle, m):
    rng = np.random.default_rng(77 + m)
    for x in (rng.standard_normal(m) * 3.0 + 1.0, rng.integers(0, 5, m).astype(float),
              rng.standard_cauchy(m)):
        assert oracle.qn(x) == _qn_brute(x)


def test_qn_scale_of_a_gaussian(oracle):
    x = np.random.default_rng(5).standard_normal(20000) * 2.5
    assert abs(oracle.qn(x) / 2.5 - 1.0) < 0.02


def test_robust_covariances(oracle):
    rng = np.random.default_rng(11)
    d, n = 5, 4000
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    S = A @ A.T
    X = rng.standard_normal((n, d)) @ np.linalg.cholesky(S).T
    diag = oracle.cov_robust(X, ogk=False)
    assert np.array_equal(diag, np.diag(np.diag(diag)))
    assert np.allclose(np.diag(diag), [oracle.qn(X[:, i]) ** 2 for i in range(d)], rtol=0, atol=0)
    ogk = oracle.cov_robust(X, ogk=True)
    assert np.array_equal(ogk, ogk.T)
    assert np.all(np.linalg.eigvalsh(ogk) > 0)
    assert np.max(np.abs(ogk - S)) / np.max(np.abs(S)) < 0.1
    # 5 % gross outliers barely move the robust estimate, unlike the sample covariance
    Xo = X.copy()
    Xo[: n // 20] += 50.0
    ogk_o = oracle.cov_robust(Xo, ogk=True)
    assert np.max(np.abs(ogk_o - S)) / np.max(np.abs(S)) < 0.5
    assert np.max(np.abs(np.cov(Xo.T) - S)) / np.max(np.abs(S)) > 10.0
    # the row subset form (a VKDE neighbourhood) equals the estimate of the gathered rows
    rows = rng.permutation(n)[:300].astype(np.int32)
    assert np.array_equal(oracle.cov_robust(X, ogk=True, rows=rows), oracle.cov_robust(X[rows], ogk=True))


@pytest.mark.parametrize("kind", [0, 1])
def test_cov_fixed(oracle, kind):
    """cov-type FIXED (ncm_stats_dist_kde.c:414-421, 825-845): the global
    covariance is the given matrix with its plain Cholesky factor, whatever
    the sample; VKDE neighbourhoods keep their sample covariances
    (ncm_stats_dist_vkde.c:462-476); no nearPD repair (a matrix that is not
    positive definite is an error), no robust minimum of 4 rows, and FIXED
    without a matrix is an error."""
    rng = np.random.default_rng(5)
    X = rng.standard_normal((400, 3)) @ np.diag([1.0, 2.0, 0.5])
    F = np.array([[2.0, 0.3, 0.1], [0.3, 1.0, -0.2], [0.1, -0.2, 0.5]])
    o = oracle.OracleStatsDist(kind, 1, 3, local_frac=0.05, cov_type=1)
    o.set_sample(X)
    assert o.prepare() == 7
    o.set_cov_fixed(F)
    assert o.prepare() == 0
    assert np.array_equal(o.cov(), F)
    assert rel_err(o.U(), np.linalg.cholesky(F).T, floor=1e-3) < 1e-15
    s = oracle.OracleStatsDist(kind, 1, 3, local_frac=0.05, cov_type=0)
    s.set_sample(X)
    assert s.prepare() == 0
    if kind == 1:
        # the neighbourhoods are found in the fixed whitening, their covariances are sample ones
        Ui = o.Ui(11)
        nb = X[o.knn()[11]]
        assert rel_err(Ui.T @ Ui, np.cov(nb.T), floor=1e-3) < 1e-12
    else:
        assert not np.allclose(o.eval_m2lnp(X[:8]), s.eval_m2lnp(X[:8]))
    bad = oracle.OracleStatsDist(kind, 0, 3, local_frac=0.05, cov_type=1)
    bad.set_sample(X)
    bad.set_cov_fixed(np.diag([1.0, -1.0, 1.0]))
    assert bad.prepare() == 4
    few = oracle.OracleStatsDist(0, 0, 2, cov_type=1)
    few.set_sample(X[:3, :2])
    few.set_cov_fixed(np.eye(2))
    assert few.prepare() == 0


@pytest.mark.parametrize("cov_type", [2, 3])
def test_robust_prepare_errors(oracle, cov_type):
    X = np.random.default_rng(3).standard_normal((60, 3))
    o = oracle.OracleStatsDist(1, 0, 3, local_frac=0.05, cov_type=cov_type)   # k = 3 neighbours
    o.set_sample(X)
    assert o.prepare() == 2
    o = oracle.OracleStatsDist(1, 0, 3, local_frac=0.1, cov_type=cov_type)
    o.set_sample(X)
    assert o.prepare() == 0


def test_robust_ogk_reference_scenario(oracle):
    """The scenario of the reference's own robust test
    (tests/c/ncm/stats/test_ncm_stats_vec.c:363-436: 80 % correlated Gaussian rows
    of scale sigma, 20 % rows clustered at 1 with a tenth of the scale); that test
    only runs the estimator, so the check here is the estimator's purpose: the OGK
    variances stay far closer to sigma^2 than the sample variances (the cluster
    sits about 3 sigma out, so it still widens Qn somewhat)."""
    rng = np.random.default_rng(363)
    sigma, dim, ntests = 0.3, 4, 5000
    def rows(count, centre, scale):
        z = rng.standard_normal((count, dim)) * scale + centre
        x = z.copy()
        x[:, 1:] = (z[:, :1] + z[:, 1:]) / np.sqrt(2.0)
        return x
    X = np.vstack([rows(ntests, 0.0, sigma), rows(int(ntests * 0.2), 1.0, sigma / 10.0)])
    var_n = np.var(X, axis=0, ddof=1)
    var_r = np.diag(oracle.cov_robust(X, ogk=True))
    err_r, err_n = np.abs(var_r / sigma ** 2 - 1.0), np.abs(var_n / sigma ** 2 - 1.0)
    assert np.all(err_r < 0.6) and np.all(err_n > 1.0) and np.all(err_r < 0.4 * err_n)


def test_lm_restatement_pinned_to_reference_levmar(oracle):
    """The oracle's one-parameter dlevmar_dif (the CV_SPLIT bandwidth fit,
    ncm_stats_dist.c:1018-1066) against the reference's own levmar
    (numcosmo/external/levmar, stored by tests/golden/make_golden.py levmar):
    bit-identical iterates and iteration counts up to 1024 measurements (the
    same summation order), within 4 ulps above (levmar's blocked J^T J)."""
    from conftest import golden

    g = golden("levmar_ref")
    for n in (40, 700, 1500):
        a, b = g[f"a_n{n}"], g[f"b_n{n}"]
        f = (lambda a, b: (lambda p: np.exp(-a * np.exp(p)) - b))(a, b)
        for j, p0 in enumerate(g["p0"]):
            p, it = oracle.lm1_oracle(f, float(p0), n, g["opts"])
            assert it == g[f"it_n{n}"][j]
            if n <= 1024:
                assert p == g[f"p_n{n}"][j]
            else:
                assert abs(p - g[f"p_n{n}"][j]) <= 4 * np.spacing(abs(p))
            live = oracle.lm1_reference(f, float(p0), n, g["opts"])
            if live is not None:
                assert live == (g[f"p_n{n}"][j], g[f"it_n{n}"][j])
