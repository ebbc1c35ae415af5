"""The drop-in boundary beyond eval/sample: ncm_stats_dist_get_Ki, the VKDE
neighbour lists checked directly against the reference kd-tree (ties
included), and the failure path of the bounded device waits.

Tolerances: neighbour lists bit-exact; get_Ki's location bit-exact, its
covariance, normalisation and weight <= 1e-12 relative to the oracle's
factor-derived values; after an injected wait timeout the handle's next fit
equals an undisturbed fit to 1e-10 relative to the largest weight.
"""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu


def _vkde(ng, kernel, d, X, nu=3.0):
    k = ng.StatsDistKernelST(d, nu) if kernel == 1 else ng.StatsDistKernelGauss(d)
    sd = ng.StatsDistVKDE(k, ng.StatsDistCV.NONE)
    sd.set_sample(X)
    return sd


def test_knn_equals_reference_kdtree(gpu):
    """The device's kNN sets against NumCosmo's own kd-tree (numcosmo/external/misc/kdtree.c)
    run on the oracle's whitened sample: config 2 at N = 1024 (k = 51)."""
    g = golden("vkde_st3_d16_n1024")
    sd = _vkde(gpu, 1, 16, g["centres"])
    sd.prepare()
    got = sd.get_knn()
    assert got.shape == g["knn_ref"].shape
    assert np.array_equal(got, g["knn_ref"])


@pytest.mark.parametrize("d", [2, 5, 16])
def test_knn_ties_equal_reference_kdtree(gpu, d):
    """Duplicated sample points: groups of exactly equal distances are ordered
    by index, as rb_knn_list_compare orders them (rb_knn_list.c:32-40)."""
    g = golden("vkde_knn_ties")
    X = g[f"X_d{d}"]
    sd = _vkde(gpu, 0, d, X)
    sd.prepare()
    got = sd.get_knn()
    want = g[f"knn_d{d}"]
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    # the neighbourhood decides the local covariance bit for bit
    assert np.array_equal(np.triu(sd.peek_cov_decomp(3)), np.triu(g[f"U3_d{d}"]))


def test_knn_launch_at_the_default_shared_memory_limit(gpu, oracle):
    """N = 5300 in d = 3 with local-frac 0.05: k = 265 neighbours, so the
    kNN kernel's dynamic shared memory (48552 B) is under 48 KiB and only
    its static arrays take the launch past that default; the sets equal the
    oracle's."""
    X = np.random.default_rng(53).standard_normal((5300, 3))
    sd = _vkde(gpu, 0, 3, X)
    sd.set_local_frac(0.05)
    sd.prepare()
    assert 256 < sd.get_knn_k() <= 512
    o = oracle.OracleStatsDist(1, 0, 3, nu=3.0, local_frac=0.05)
    o.set_sample(X)
    assert o.prepare() == 0
    assert np.array_equal(sd.get_knn(), o.knn())


def test_knn_on_kde_is_unsupported(gpu):
    ng = gpu
    sd = ng.StatsDistKDE(ng.StatsDistKernelGauss(3), ng.StatsDistCV.NONE)
    sd.set_sample(np.random.default_rng(1).standard_normal((50, 3)))
    sd.prepare()
    with pytest.raises(ng.NcgError) as e:
        sd.get_knn()
    assert e.value.name == "NCG_ERR_UNSUPPORTED"


@pytest.mark.parametrize("kind", [0, 1])
def test_get_Ki(gpu, oracle, kind):
    """ncm_stats_dist_get_Ki (ncm_stats_dist.c:1811-1829) after a weight fit:
    y_i = the sample point, cov_i = href^2 U_i^T U_i, n_i = exp(lnnorm_i), w_i."""
    ng = gpu
    g = golden("vkde_gauss_interp_d12_n512")
    k = ng.StatsDistKernelGauss(12)
    sd = (ng.StatsDistVKDE if kind else ng.StatsDistKDE)(k, ng.StatsDistCV.NONE)
    sd.set_sample(g["centres"])
    sd.prepare_interp(g["target"])
    o = oracle.OracleStatsDist(kind, oracle.GAUSS, 12)
    o.set_sample(g["centres"])
    assert o.prepare_interp(g["target"]) == 0
    X = o.sample_array()
    w = o.weights()
    h = o.href
    for i in (0, 17, 511):
        y, cov, ni, wi = sd.get_Ki(i)
        U = np.triu(o.Ui(i) if kind else o.U())
        assert np.array_equal(y, X[i])
        assert rel_err(cov, U.T @ U * h * h, floor=1e-3) < 1e-12
        lnn = (o.lnnorms()[i] if kind else o.kernel_lnnorm) + 12 * np.log(h)
        assert ni == pytest.approx(np.exp(lnn), rel=1e-12)
        assert wi == pytest.approx(w[i], rel=1e-10, abs=1e-10 * w.max())


def test_chain_wait_timeout_reports_and_recovers(gpu):
    """A chained triangular solve whose dependent wait never sees its value:
    the wait gives up after its poll limit, the launch ends, prepare_interp
    returns NCG_ERR_TIMEOUT, and the same handle's next fit is undisturbed."""
    ng = gpu
    from numcosmo_gb300 import _lib

    L = _lib.load()
    g = golden("vkde_gauss_interp_d12_n512")

    ref = _vkde(ng, 0, 12, g["centres"])
    ref.set_precision(ng.Precision.MIXED)
    ref.prepare_interp(g["target"])
    w_ref = ref.peek_weights()

    sd = _vkde(ng, 0, 12, g["centres"])
    sd.set_precision(ng.Precision.MIXED)
    _lib.check(L.ncg_debug_inject_wait_fault(2), "ncg_debug_inject_wait_fault")
    with pytest.raises(ng.NcgError) as e:
        sd.prepare_interp(g["target"])
    assert e.value.name == "NCG_ERR_TIMEOUT"

    # the hook is one-shot and the context stays usable
    sd.prepare_interp(g["target"])
    w = sd.peek_weights()
    assert np.max(np.abs(w - w_ref)) <= 1e-10 * np.max(w_ref)
    assert rel_err(sd.eval_m2lnp(g["points"]), g["m2lnp"], floor=1.0) < 1e-6


def test_eval_tc_wait_timeout_reports_and_recovers(gpu):
    """The tensor-core eval with its copy warp idle: the MMA warp's first
    mbarrier wait runs out (1.5 s of %globaltimer), every role of the CTA stops,
    TMEM is freed, and the call returns NCG_ERR_TIMEOUT; the next call is exact."""
    ng = gpu
    from numcosmo_gb300 import _lib

    L = _lib.load()
    g = golden("vkde_st3_d16_n1024")
    sd = _vkde(ng, 1, 16, g["centres"])
    sd.prepare()
    sd.set_precision(ng.Precision.MIXED)
    want = sd.eval_m2lnp(g["points"])            # builds the operand and passes its check
    assert sd.get_eval_path()[0] == "tensor_core"
    _lib.check(L.ncg_debug_inject_wait_fault(1), "ncg_debug_inject_wait_fault")
    with pytest.raises(ng.NcgError) as e:
        sd.eval_m2lnp(g["points"])
    assert e.value.name == "NCG_ERR_TIMEOUT"
    got = sd.eval_m2lnp(g["points"])
    assert np.array_equal(got, want)
    assert rel_err(got, g["m2lnp"], floor=1.0) < 1e-6
