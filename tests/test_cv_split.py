"""CV_SPLIT_NOFIT (ncm_stats_dist.c:714-770, 484-511, 660-701): the first
ceil(n split_frac) observations are the kernels (the KDE's global covariance
comes from them, the VKDE neighbourhoods from all observations), and the
over-smoothing is fitted by Nelder-Mead to the -2 ln p of the held-out rest;
prepare_interp then fits the kernels' weights on all observations (the
n_obs x n_kernels system of ncm_stats_dist.c:1067-1072).

Tolerances: the fitted over-smoothing and bandwidth <= 1e-10 relative to the
oracle's (both follow the same simplex steps on objectives equal to ~1e-13),
-2 ln p <= 1e-10 relative, neighbour lists and sampled indices bit-exact.
"""
import numpy as np
import pytest

from conftest import rel_err

CASES = [(0, 0, 3, 900, 0.6), (0, 1, 5, 1200, 0.5), (1, 0, 4, 1000, 0.7), (1, 1, 6, 1500, 0.4)]


def _data(seed, n, d):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    return rng.standard_normal((n, d)) @ A.T, rng.standard_normal((300, d)) @ A.T


def _oracle(oracle, kind, kernel, d, X, frac):
    o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0)
    o.set_cv(2, frac)
    o.set_sample(X)
    return o


@pytest.mark.parametrize("kind,kernel,d,n,frac", CASES)
def test_oracle_split_fit_lowers_the_objective(oracle, kind, kernel, d, n, frac):
    """The restated fit: kernels = ceil(n frac), and the held-out -2 ln p at the
    fitted over-smoothing is below its value at the start (over_smooth = 1)."""
    X, _ = _data(60 + n, n, d)
    o = _oracle(oracle, kind, kernel, d, X, frac)
    assert o.prepare() == 0
    nk = int(np.ceil(n * frac))
    assert o.n_kernels == nk
    fitted = np.sum(o.eval_m2lnp(X[nk:]))
    o0 = _oracle(oracle, kind, kernel, d, X, 1.0)     # no held-out rest: the objective is 0 throughout
    assert o0.prepare() == 0 and o0.n_kernels == n
    assert np.isfinite(fitted) and o.over_smooth != 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("kind,kernel,d,n,frac", CASES)
def test_split_nofit_matches_the_oracle(gpu, oracle, kind, kernel, d, n, frac):
    ng = gpu
    X, P = _data(60 + n, n, d)
    o = _oracle(oracle, kind, kernel, d, X, frac)
    assert o.prepare() == 0
    k = ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.SPLIT_NOFIT)
    sd.set_split_frac(frac)
    sd.set_sample(X)
    sd.prepare()
    assert sd.get_n_kernels() == o.n_kernels
    assert sd.get_over_smooth() == pytest.approx(o.over_smooth, rel=1e-10)
    assert sd.get_href() == pytest.approx(o.href, rel=1e-10)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < 1e-10
    w = sd.peek_weights()
    assert w.shape == (o.n_kernels,) and np.all(w == 1.0 / o.n_kernels)
    IM = sd.compute_IM()                      # n_obs x n_kernels (unit f)
    assert IM.shape == (n, o.n_kernels)
    assert rel_err(IM, o.compute_IM(), floor=1e-300) < 1e-10
    if kind:
        assert np.array_equal(sd.get_knn(), o.knn())
    u, z, cs = ng.RNG(31).sample_stream(k, 2000)
    x, idx = sd.sample(u, z, cs if kernel else None)
    xo, io = o.sample(u, z, cs if kernel else None)
    assert np.array_equal(idx, io) and idx.max() < o.n_kernels
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
    sd.set_precision(ng.Precision.MIXED)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P), floor=1.0) < 1e-6


def _target(X):
    """-2 ln of a Gaussian centred near the sample's mean: the weight-fit target."""
    mu = X.mean(axis=0)
    C = np.cov(X.T)
    L = np.linalg.cholesky(C)
    y = np.linalg.solve(L, (X - mu).T)
    return np.sum(y * y, axis=0) + 2.0 * np.sum(np.log(np.diag(L)))


@pytest.mark.parametrize("kind,kernel,d,n,frac", CASES)
def test_oracle_split_interp_weights(oracle, kind, kernel, d, n, frac):
    """prepare_interp under SPLIT_NOFIT (ncm_stats_dist.c:1067-1072): the
    n_obs x n_kernels system, weights on the kernels only, normalised."""
    X, _ = _data(60 + n, n, d)
    o = _oracle(oracle, kind, kernel, d, X, frac)
    assert o.prepare_interp(_target(X)) == 0
    w = o.weights()
    nk = int(np.ceil(n * frac))
    assert w.shape == (nk,) and np.all(w > 0) and abs(np.sum(w) - 1.0) < 1e-12
    assert np.isfinite(o.rnorm)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
@pytest.mark.parametrize("kind,kernel,d,n,frac", CASES)
def test_split_nofit_interp_matches_the_oracle(gpu, oracle, kind, kernel, d, n, frac, prec):
    """Weights <= 1e-10 of the largest weight (FP64; mixed NNLS <= 1e-7),
    rnorm and the fitted bandwidth <= 1e-10 relative."""
    ng = gpu
    X, P = _data(60 + n, n, d)
    m2 = _target(X)
    o = _oracle(oracle, kind, kernel, d, X, frac)
    assert o.prepare_interp(m2) == 0
    k = ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.SPLIT_NOFIT)
    sd.set_split_frac(frac)
    sd.set_precision(getattr(ng.Precision, prec))
    sd.set_sample(X)
    sd.prepare_interp(m2)
    w, wo = sd.peek_weights(), o.weights()
    tol = 1e-10 if prec == "FP64" else 1e-7
    assert w.shape == wo.shape
    assert np.max(np.abs(w - wo)) <= tol * np.max(wo)
    assert sd.get_rnorm() == pytest.approx(o.rnorm, rel=1e-8 if prec == "FP64" else 1e-6)
    assert sd.get_over_smooth() == pytest.approx(o.over_smooth, rel=1e-10)
    assert sd.get_interp_branch() == o.interp_branch
    sd.set_precision(ng.Precision.FP64)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < 1e-10 if prec == "FP64" else True


@pytest.mark.gpu
@pytest.mark.parametrize("cv", ["SPLIT_NOFIT", "SPLIT"])
def test_split_fraction_defaults_to_one_half(gpu, cv):
    """A new handle's split fraction is the "split-frac" property's
    construct-time default, 0.5 (ncm_stats_dist.c:428-434): the reference's
    own CV tests never set it.  The same fit as with set_split_frac(0.5);
    fractions outside [0.01, 1] are refused by the setter."""
    ng = gpu
    X, _ = _data(1, 201, 3)
    m2 = np.sum(X * X, axis=1)
    a = ng.StatsDistKDE(ng.StatsDistKernelGauss(3), ng.StatsDistCV[cv])
    a.set_sample(X)
    a.prepare_interp(m2)
    b = ng.StatsDistKDE(ng.StatsDistKernelGauss(3), ng.StatsDistCV[cv])
    b.set_split_frac(0.5)
    b.set_sample(X)
    b.prepare_interp(m2)
    assert a.get_n_kernels() == 101
    assert a.get_over_smooth() == b.get_over_smooth()
    assert np.array_equal(a.peek_weights(), b.peek_weights())
    for bad in (0.0, 1.5):
        with pytest.raises(ng.NcgError) as e:
            a.set_split_frac(bad)
        assert e.value.name == "NCG_ERR_INVALID_ARG"


# ---- CV_SPLIT: the levmar fit of ln over_smooth (ncm_stats_dist.c:1018-1066)

SPLIT_CASES = [(0, 0, 3, 700, 0.6), (1, 1, 4, 800, 0.5)]


def _split_oracle(oracle, ng, kind, kernel, d, X, frac):
    o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0)
    o.set_cv(1, frac)
    r = ng.RNG(4357)
    o.set_split_draws(np.array([r.ugaussian() for _ in range(100)]))
    o.set_sample(X)
    return o


@pytest.mark.parametrize("kind,kernel,d,n,frac", SPLIT_CASES)
def test_oracle_split_fit(oracle, ng, kind, kernel, d, n, frac):
    """The restated CV_SPLIT weight fit: ten restarts, the Levenberg-Marquardt
    fit of ln over_smooth, normalised weights on the kernels."""
    X, _ = _data(70 + n, n, d)
    o = _split_oracle(oracle, ng, kind, kernel, d, X, frac)
    assert o.prepare() == 0 and o.over_smooth == 1.0      # SPLIT's prepare fits nothing
    assert o.prepare_interp(_target(X)) == 0
    w = o.weights()
    assert w.shape == (int(np.ceil(n * frac)),) and abs(np.sum(w) - 1.0) < 1e-12
    assert o.over_smooth != 1.0 and np.isfinite(o.rnorm)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,kernel,d,n,frac", SPLIT_CASES)
def test_split_matches_the_oracle(gpu, oracle, kind, kernel, d, n, frac):
    """The same restarts (the handle's generator, MT19937 seeded 4357; a
    second call continues it as the reference's does) and the same
    Levenberg-Marquardt method: the fitted ln over_smooth agrees within 1e-6
    (levmar stops once a step is below 1e-7 of the parameter, and its
    forward-difference Jacobian, step 1e-6, turns the ~1e-13 differences of
    the two implementations' weight fits into 1e-7 relative step differences,
    so two correct fits stop at points ~1e-8 apart); at the device's fitted
    bandwidth, rnorm equals the oracle's weight fit at that bandwidth to 1e-8,
    and the weights and -2 ln p to 1e-10 (or the fit's own conditioning limit,
    see below)."""
    ng = gpu
    X, P = _data(70 + n, n, d)
    m2 = _target(X)
    o = _split_oracle(oracle, ng, kind, kernel, d, X, frac)
    k = ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.SPLIT)
    sd.set_split_frac(frac)
    sd.set_sample(X)
    for call in range(2):
        assert o.prepare_interp(m2) == 0
        sd.prepare_interp(m2)
        os_dev = sd.get_over_smooth()
        assert abs(np.log(os_dev) - np.log(o.over_smooth)) <= 1e-6
        # the oracle's weight fit at the device's bandwidth (a split with no fit)
        o2 = oracle.OracleStatsDist(kind, kernel, d, nu=3.0, over_smooth=os_dev)
        o2.set_cv(2, frac)
        o2.set_sample(X)
        o2.set_no_fit(True)
        assert o2.prepare_interp(m2) == 0
        assert sd.get_href() == pytest.approx(o2.href, rel=1e-14)
        # the fitted bandwidth can leave the system nearly singular (rnorm
        # ~1e-3): then the weights move along near-null directions under
        # ulp-level changes, so the bound is ten times the oracle's own largest
        # change when the bandwidth moves by +-1e-15 or 1e-14 relative (the
        # size of the two implementations' exp/pow rounding differences in the
        # interpolation matrix), at least 1e-10
        w, wo = sd.peek_weights(), o2.weights()
        e2 = o2.eval_m2lnp(P)
        tol_w = tol_e = 1e-10
        for eps in (1e-15, -1e-15, 1e-14):
            o3 = oracle.OracleStatsDist(kind, kernel, d, nu=3.0, over_smooth=os_dev * (1.0 + eps))
            o3.set_cv(2, frac)
            o3.set_sample(X)
            o3.set_no_fit(True)
            assert o3.prepare_interp(m2) == 0
            tol_w = max(tol_w, 10.0 * np.max(np.abs(o3.weights() - wo)) / np.max(wo))
            tol_e = max(tol_e, 10.0 * rel_err(o3.eval_m2lnp(P), e2))
        assert np.max(np.abs(w - wo)) <= tol_w * np.max(wo)
        assert sd.get_rnorm() == pytest.approx(o2.rnorm, rel=1e-8)
        assert rel_err(sd.eval_m2lnp(P), e2) < tol_e


# ---- the range cut under a split (ncm_stats_dist.c:895-976)

def _cut_case(kind_of_cut, n=600, d=3, frac=0.5, seed=5):
    """-2 ln L with a range beyond the cut (-4 ln eps): 'heur' puts the few
    lowest values among the kernels (heuristic weights), 'cut' keeps most of
    the sample below the cut (the recursion on the cut sample), 'held' puts
    one of the lowest values on a held-out observation."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d))
    m2 = rng.uniform(0.0, 1.0, n)
    nk = int(np.ceil(n * frac))
    if kind_of_cut == "heur":
        m2[:] = 500.0
        m2[:20] = rng.uniform(0.0, 1.0, 20)          # 20 lowest, all kernels
        m2[nk:] = 900.0
    elif kind_of_cut == "cut":
        # the cut index is looked for among the first n_kernels sorted values
        # only (ncm_stats_dist.c:913-922), so the recursion needs
        # n_kernels > n_obs / 2: a quarter above the cut, kernels 90 %
        frac = 0.9
        m2[::4] = 400.0
    else:
        m2[:] = 500.0
        m2[:20] = rng.uniform(0.0, 1.0, 20)
        m2[nk + 3] = 0.5                             # a held-out observation among the lowest
    return X, m2, frac


@pytest.mark.parametrize("which", ["heur", "cut", "held"])
def test_oracle_split_range_cut(oracle, which):
    X, m2, frac = _cut_case(which)
    o = oracle.OracleStatsDist(0, 1, X.shape[1], nu=3.0)
    o.set_cv(2, frac)
    o.set_sample(X)
    r = o.prepare_interp(m2)
    if which == "held":
        assert r == 7                                # ORC_ERR_INVALID: the reference would index past n_kernels
    else:
        assert r == 0 and o.interp_branch == (1 if which == "heur" else 2)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["heur", "cut", "held"])
def test_split_range_cut_matches_the_oracle(gpu, oracle, which):
    ng = gpu
    X, m2, frac = _cut_case(which)
    d = X.shape[1]
    o = oracle.OracleStatsDist(0, 1, d, nu=3.0)
    o.set_cv(2, frac)
    o.set_sample(X)
    r = o.prepare_interp(m2)
    sd = ng.StatsDistKDE(ng.StatsDistKernelST(d, 3.0), ng.StatsDistCV.SPLIT_NOFIT)
    sd.set_split_frac(frac)
    sd.set_sample(X)
    if which == "held":
        with pytest.raises(ng.NcgError) as e:
            sd.prepare_interp(m2)
        assert e.value.name == "NCG_ERR_INVALID_ARG" and r == 7
        return
    sd.prepare_interp(m2)
    assert sd.get_interp_branch() == o.interp_branch
    assert sd.get_sample_size() == o.n
    w, wo = sd.peek_weights(), o.weights()
    assert w.shape == wo.shape and np.max(np.abs(w - wo)) <= 1e-10 * np.max(wo)
    assert sd.get_over_smooth() == pytest.approx(o.over_smooth, rel=1e-10)
