"""Robust covariance types (cov-type ROBUST_DIAG and ROBUST / OGK) on the GPU
against the oracle: the global covariance (KDE and the VKDE whitening) and
each VKDE kernel's neighbourhood covariance, through the C-ABI.

The Qn selections are exact on both sides (the same differences of the same
values); the OGK eigenvectors come from two Jacobi orderings, so factors and
-2lnp agree to rounding: 1e-10 relative, as the FP64 form.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def _data(d, n, seed, outliers=0.0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    X = rng.standard_normal((n, d)) @ A.T + 1.5
    if outliers:
        X[: int(outliers * n)] += 40.0
    P = rng.standard_normal((64, d)) @ A.T + 1.5
    return X, P


def _pair(ng, oracle, kind, kernel, d, X, cov_type, local_frac=0.05):
    k = ng.StatsDistKernelST(d, 3.0) if kernel == 1 else ng.StatsDistKernelGauss(d)
    sd = (ng.StatsDistVKDE if kind == 1 else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
    sd.set_cov_type(ng.StatsDistKDECovType(cov_type))
    if kind == 1:
        sd.set_local_frac(local_frac)
    sd.set_sample(X)
    sd.prepare()
    o = oracle.OracleStatsDist(kind, kernel, d, nu=3.0, local_frac=local_frac, cov_type=cov_type)
    o.set_sample(X)
    assert o.prepare() == 0
    return sd, o


@pytest.mark.parametrize("cov_type", [2, 3])
@pytest.mark.parametrize("kind,kernel", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("d", [1, 3, 8])
def test_robust_parity(gpu, oracle, cov_type, kind, kernel, d):
    X, P = _data(d, 40 * d + 300, 100 * d + 10 * kind + kernel + cov_type, outliers=0.03)
    sd, o = _pair(gpu, oracle, kind, kernel, d, X, cov_type)
    # ROBUST_DIAG: the same Qn selections, so the same bits; OGK: rounding of the eigenvectors
    cov_tol = 0.0 if cov_type == 2 else FP64_TOL
    assert rel_err(sd.peek_full_cov(), o.cov(), floor=1e-3 * np.max(np.abs(o.cov()))) <= cov_tol
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < FP64_TOL
    if kind == 1:
        for i in (0, 7, X.shape[0] - 1):
            Ug, Uo = np.triu(sd.peek_cov_decomp(i)), np.triu(o.Ui(i))
            assert rel_err(Ug, Uo, floor=1e-3 * np.max(np.abs(Uo))) < 1e-10
        assert rel_err([sd.get_lnnorm(i) for i in range(0, X.shape[0], 17)],
                       o.lnnorms()[:: 17], floor=1.0) < 1e-12


def test_robust_vkde_d16_banana(gpu, oracle):
    """OGK on the d=16 banana with k = 51 neighbours per kernel (N = 1024)."""
    from numcosmo_gb300 import workloads as wl

    X = wl.banana(1024, 16, 2001)
    P = wl.banana(128, 16, 2002)
    sd, o = _pair(gpu, oracle, 1, 1, 16, X, 3)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < FP64_TOL
    sd.set_precision(gpu.Precision.MIXED)
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P), floor=1.0) < 1e-6


def test_robust_errors(gpu):
    ng = gpu
    X, _ = _data(3, 60, 1)
    sd = ng.StatsDistVKDE(ng.StatsDistKernelGauss(3), ng.StatsDistCV.NONE)
    sd.set_cov_type(ng.StatsDistKDECovType.ROBUST)
    sd.set_local_frac(0.05)   # k = 3 < 4 neighbours
    sd.set_sample(X)
    with pytest.raises(ng.NcgError) as e:
        sd.prepare()
    assert e.value.status == 2


@pytest.mark.parametrize("values", ["integers", "offset", "tiny", "huge"])
@pytest.mark.parametrize("kind,n", [(0, 1500), (1, 600)])
def test_robust_qn_decision_band(gpu, oracle, values, kind, n):
    """Sets whose Qn counts sit in or beyond the FP32 decision band: exact
    ties of values and of differences (integers), a spread far below the
    values (offset), values in the FP32 subnormal range (tiny) and values
    past 2^100 from their median (huge: every test in FP64).  KDE at
    n = 1500 runs the CTA selection, VKDE's 180-row neighbourhoods the warp
    one; ROBUST_DIAG gives the same bits as the oracle, OGK agrees to
    rounding."""
    d = 3
    rng = np.random.default_rng({"integers": 1, "offset": 2, "tiny": 3, "huge": 4}[values] + 10 * kind)
    Z = rng.standard_normal((n, d)) @ np.array([[1.0, 0.0, 0.0], [0.4, 1.0, 0.0], [0.2, -0.3, 1.0]]).T
    if values == "integers":
        X = np.floor(4.0 * Z)
    elif values == "offset":
        X = 1.0e6 + Z
    elif values == "tiny":
        X = 1.0e-40 * Z
    else:
        X = 2.0 ** 101 * Z
    P = X[rng.choice(n, 16, replace=False)] + 0.1 * np.std(X, axis=0)
    # integer data gives coinciding Qn values in the OGK correlation matrix, so
    # repeated eigenvalues whose eigenvectors are not unique: ROBUST_DIAG only
    # OGK projects on eigenvectors that two Jacobi orderings give to ~1e-15:
    # the projections move by 1e-15 |x| against a spread std(x), and their Qn
    # with them (1e-9 relative at the 1e6 offset)
    ogk_tol = max(FP64_TOL, 1e-13 * np.max(np.abs(X)) / np.min(np.std(X, axis=0)))
    for cov_type in ((2,) if values == "integers" else (2, 3)):
        sd, o = _pair(gpu, oracle, kind, 0, d, X, cov_type, local_frac=0.3)
        cov_tol = 0.0 if cov_type == 2 else ogk_tol
        assert rel_err(sd.peek_full_cov(), o.cov(), floor=1e-3 * np.max(np.abs(o.cov()))) <= cov_tol
        tol = FP64_TOL if cov_type == 2 else ogk_tol
        if kind == 1:
            # OGK: the eigenvector rounding spreads over the whole factor, so
            # normwise (relative to its largest element)
            for i in (0, 11, n - 1):
                Ug, Uo = np.triu(sd.peek_cov_decomp(i)), np.triu(o.Ui(i))
                floor = (1e-3 if cov_type == 2 else 1.0) * np.max(np.abs(Uo))
                assert rel_err(Ug, Uo, floor=floor) < tol
        assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P), floor=1.0) < tol


@pytest.mark.parametrize("cov_type", [2, 3])
def test_robust_vkde_large_neighbourhoods(gpu, oracle, cov_type):
    """Neighbourhoods of 550 rows (local-frac 0.5 at N = 1100): the warp
    selection at its largest padded size (1024 slots), whose CTAs carry fewer
    warps when the shared memory of eight would leave one CTA per SM."""
    X, P = _data(3, 1100, 77)
    sd, o = _pair(gpu, oracle, 1, 1, 3, X, cov_type, local_frac=0.5)
    assert sd.get_knn_k() > 512
    for i in (0, 500, X.shape[0] - 1):
        Ug, Uo = np.triu(sd.peek_cov_decomp(i)), np.triu(o.Ui(i))
        assert rel_err(Ug, Uo, floor=1e-3 * np.max(np.abs(Uo))) < FP64_TOL
    assert rel_err(sd.eval_m2lnp(P), o.eval_m2lnp(P)) < FP64_TOL
