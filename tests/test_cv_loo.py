"""CV_LOO (ncm_stats_dist.c:703-789 with :760-765): every observation is a
kernel, and the over-smoothing is fitted by Nelder-Mead to the AMISE -- in
closed form for the Gaussian KDE (_ncm_stats_dist_amise_kde_gauss,
:513-557), otherwise minus twice the off-diagonal interpolation-matrix mean
plus a Monte Carlo mean of the density over antithetic pairs
(_ncm_stats_dist_amise, :561-658; ncm_stats_dist_sample2, :1633-1651) from a
generator reseeded at every evaluation, run to a relative standard error
below 1e-2.  prepare_interp then fits the weights on the square system.

The device draws its pairs from MT19937 seeded as GSL seeds 0 (4357); the
oracle consumes the same pairs (ncg_rng_sample2_stream), so both run the same
Monte Carlo.  Tolerances: fitted over-smoothing <= 1e-10 relative (the same
simplex steps on objectives equal to ~1e-14), -2 ln p <= 1e-10 relative,
weights <= 1e-10 of the largest weight, or ten times the oracle's own weight
change under a 1e-15 relative bandwidth change where the fit is that
ill-conditioned (_weight_tol).
"""
import numpy as np
import pytest

from conftest import rel_err

CASES = [(0, 0, 3, 600), (0, 1, 3, 500), (1, 0, 4, 600), (1, 1, 3, 500)]
NPAIRS = 200000


def _data(seed, n, d):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    return rng.standard_normal((n, d)) @ A.T, rng.standard_normal((300, d)) @ A.T


def _kernel(ng, kernel, d):
    return ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)


def _oracle(oracle, ng, kind, kernel, d, X):
    o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0)
    o.set_cv(3)
    o.set_loo_draws(*ng.RNG(4357).sample2_stream(_kernel(ng, kernel, d), NPAIRS))
    o.set_sample(X)
    return o


def _target(X):
    mu = X.mean(axis=0)
    L = np.linalg.cholesky(np.cov(X.T))
    y = np.linalg.solve(L, (X - mu).T)
    return np.sum(y * y, axis=0) + 2.0 * np.sum(np.log(np.diag(L)))


@pytest.mark.parametrize("kind,kernel,d,n", CASES)
def test_oracle_loo_fit(oracle, ng, kind, kernel, d, n):
    """The restated fit ends inside its draws and moves the bandwidth; the
    closed-form Gaussian-KDE AMISE equals its direct numpy evaluation."""
    X, _ = _data(80 + n, n, d)
    o = _oracle(oracle, ng, kind, kernel, d, X)
    assert o.prepare() == 0 and not o.loo_short
    assert o.n_kernels == n and o.over_smooth != 1.0
    if kind == 0 and kernel == 0:
        # AMISE at the fitted bandwidth from the matrix itself: the minimum of
        # the simplex is within its size (1e-3 in ln over_smooth) of the optimum
        def amise(os_):
            o2 = oracle.OracleStatsDist(0, 0, d, over_smooth=os_)
            o2.set_sample(X)
            assert o2.prepare() == 0
            h = o2.href
            o3 = oracle.OracleStatsDist(0, 0, d, over_smooth=os_ * np.sqrt(2.0))
            o3.set_sample(X)
            assert o3.prepare() == 0
            a = np.sum(o3.compute_IM()) / n ** 2
            M = o2.compute_IM()
            assert o2.href == h
            return a - 2.0 * (np.sum(M) - np.trace(M)) / (n * (n - 1))
        f0 = amise(o.over_smooth)
        assert f0 <= amise(o.over_smooth * np.exp(0.05)) and f0 <= amise(o.over_smooth * np.exp(-0.05))


@pytest.mark.gpu
@pytest.mark.parametrize("kind,kernel,d,n", CASES)
def test_loo_matches_the_oracle(gpu, oracle, kind, kernel, d, n):
    ng = gpu
    X, P = _data(80 + n, n, d)
    o = _oracle(oracle, ng, kind, kernel, d, X)
    assert o.prepare() == 0
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(_kernel(ng, kernel, d), ng.StatsDistCV.LOO)
    sd.set_sample(X)
    sd.prepare()
    assert sd.get_over_smooth() == pytest.approx(o.over_smooth, rel=1e-10)
    assert sd.get_href() == pytest.approx(o.href, rel=1e-10)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["FP64", "MIXED"])
@pytest.mark.parametrize("kind,kernel,d,n", CASES)
def test_loo_interp_matches_the_oracle(gpu, oracle, kind, kernel, d, n, prec):
    """FP64: as above; mixed (FP32-preconditioned FP64 conjugate gradients):
    weights within 1e-7 of the largest weight (or the fit's conditioning
    limit), rnorm 1e-6."""
    ng = gpu
    X, _ = _data(90 + n, n, d)
    m2 = _target(X)
    o = _oracle(oracle, ng, kind, kernel, d, X)
    assert o.prepare_interp(m2) == 0
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(_kernel(ng, kernel, d), ng.StatsDistCV.LOO)
    sd.set_precision(getattr(ng.Precision, prec))
    sd.set_sample(X)
    sd.prepare_interp(m2)
    w, wo = sd.peek_weights(), o.weights()
    tol = _weight_tol(oracle, kind, kernel, d, X, m2, o)
    if prec == "MIXED":
        tol = max(tol, 1e-7)
    assert np.max(np.abs(w - wo)) <= tol * np.max(wo)
    assert sd.get_over_smooth() == pytest.approx(o.over_smooth, rel=1e-10)
    assert sd.get_rnorm() == pytest.approx(o.rnorm, rel=1e-8 if prec == "FP64" else 1e-6)


def _weight_tol(oracle, kind, kernel, d, X, m2, o):
    """1e-10, or ten times the oracle's own weight change when its fitted
    bandwidth moves by 1e-15 relative (a few ulps), whichever is larger: a
    fitted bandwidth can leave the NNLS system so ill-conditioned that
    ulp-level differences in the interpolation matrix (the device's exp and
    pow against the C library's) move the weights beyond 1e-10."""
    wo = o.weights()
    o2 = oracle.OracleStatsDist(kind, kernel, d, nu=3.0, over_smooth=o.over_smooth * (1.0 + 1e-15))
    o2.set_sample(X)
    assert o2.prepare_interp(m2) == 0
    sens = np.max(np.abs(o2.weights() - wo)) / np.max(wo)
    return max(1e-10, 10.0 * sens)
