"""The FP64 NNLS solve's fallbacks (ncm_nnls.c:573-638, dispatch :640-666):
duplicated sample points make identical kernels, identical columns of the
interpolation matrix and exactly singular normal equations, so the Cholesky
solve fails, the symmetric LU solve meets an exactly zero pivot and the
least-squares QR solve runs -- in the oracle and on the device alike.

Tolerances: how the weight of a group of identical kernels is split is not
determined by the fit (any split gives the same density), so the checks are
on what is: the weights of the other kernels and the summed weight of each
group <= 1e-10 of the largest weight, rnorm <= 1e-10 relative, -2 ln p at
fresh points <= 1e-10 relative.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _with_duplicates(seed, n, d, groups):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d)) * np.linspace(1.0, 2.0, d)
    for g in groups:
        X[list(g[1:])] = X[g[0]]
    return X


@pytest.mark.parametrize("kind,kernel,d,n,groups", [
    (1, 0, 3, 300, [(5, 17), (40, 41), (100, 250, 251)]),
    (1, 1, 5, 400, [(1, 2), (3, 4)]),
    (0, 0, 4, 350, [(0, 349), (10, 20, 30)]),
])
def test_fallbacks_on_duplicate_kernels(gpu, oracle, kind, kernel, d, n, groups):
    ng = gpu
    X = _with_duplicates(17 + n, n, d, groups)
    m2 = np.sum(X * X / np.linspace(1.0, 2.0, d) ** 2, axis=1)
    o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0)
    o.set_sample(X)
    assert o.prepare_interp(m2) == 0
    ofb = oracle.nnls_fallbacks()
    assert ofb["lu"] > 0 and ofb["qr"] > 0

    k = ng.StatsDistKernelST(d, 3.0) if kernel else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
    sd.set_sample(X)
    sd.prepare_interp(m2)
    gfb = sd.get_interp_fallbacks()
    assert gfb["lu"] > 0 and gfb["qr"] > 0

    w, wo = sd.peek_weights(), o.weights()
    tol = 1e-10 * np.max(wo)
    grouped = np.zeros(n, dtype=bool)
    for g in groups:
        grouped[list(g)] = True
        assert abs(w[list(g)].sum() - wo[list(g)].sum()) <= tol
    assert np.max(np.abs(w[~grouped] - wo[~grouped])) <= tol
    assert sd.get_rnorm() == pytest.approx(o.rnorm, rel=1e-10)
    P = np.random.default_rng(5).standard_normal((200, d)) * np.linspace(1.0, 2.0, d)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < 1e-10
