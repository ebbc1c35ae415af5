"""ctypes wrapper over the CPU oracle (oracle/_build/libncg_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the checker.  It restates NumCosmo's
FP64 CPU path for NcmStatsDistKDE / NcmStatsDistVKDE (see ncg_oracle.c for
the file:line of every piece).  The optional reference kd-tree
(oracle/_ref/libkdtree_ref.so, compiled from NumCosmo's own
numcosmo/external/misc/kdtree.c) pins the oracle's exact kNN.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libncg_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libkdtree_ref.so")
REF_LM_PATH = os.path.join(HERE, "_ref", "liblevmar_ref.so")

KDE, VKDE = 0, 1
GAUSS, ST = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


# The NumCosmo source tree whose kd-tree and levmar pin the oracle: the
# NUMCOSMO_SRC environment variable, else the checkout's usual location.
DEFAULT_NUMCOSMO_SRC = "/root/reference"


def numcosmo_src() -> str | None:
    """The NumCosmo source tree if it is present on this machine, else None."""
    src = os.environ.get("NUMCOSMO_SRC") or DEFAULT_NUMCOSMO_SRC
    return src if os.path.isfile(os.path.join(src, "numcosmo", "external", "misc", "kdtree.c")) else None


def build(numcosmo: str | None = None) -> None:
    """Compile the oracle (and the reference kd-tree when the NumCosmo sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    src = numcosmo or numcosmo_src()
    if src is not None:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"NUMCOSMO_SRC={src}"], check=True)


_lib = None
_ref = None
_ref_lm = None


LM_FN = C.CFUNCTYPE(None, C.c_double, C.POINTER(C.c_double), C.c_int, C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        sig = {
            "orc_kernel_rot_bandwidth": (C.c_double, [C.c_int, C.c_double, C.c_int, C.c_double]),
            "orc_kernel_lnnorm": (C.c_double, [C.c_int, C.c_double, C.c_int, _dp]),
            "orc_kernel_eval_unnorm": (C.c_double, [C.c_int, C.c_double, C.c_int, C.c_double]),
            "orc_kernel_sum0": (None, [C.c_int, C.c_double, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]),
            "orc_kernel_sum1": (None, [C.c_int, C.c_double, C.c_int, C.c_int, _dp, _dp, C.c_double, _dp, _dp, _dp]),
            "orc_welford_cov": (None, [_dp, _ip, C.c_int, C.c_int, _dp]),
            "orc_cholesky_upper": (C.c_int, [_dp, C.c_int]),
            "orc_cholesky_lndet": (C.c_double, [_dp, C.c_int]),
            "orc_nearPD": (C.c_int, [_dp, C.c_int, C.c_int]),
            "orc_cholesky_decomp_fallback": (C.c_int, [_dp, _dp, C.c_int, C.c_int]),
            "orc_sym_eigen": (C.c_int, [_dp, C.c_int, _dp, _dp]),
            "orc_qn": (C.c_double, [_dp, C.c_int]),
            "orc_cov_robust_diag": (None, [_dp, _ip, C.c_int, C.c_int, _dp]),
            "orc_cov_robust_ogk": (None, [_dp, _ip, C.c_int, C.c_int, _dp]),
            "orc_knn": (None, [_dp, C.c_int, C.c_int, C.c_int, _ip, C.c_int]),
            "orc_nnls_fallbacks": (None, [_ip, _ip]),
            "orc_sd_set_cv": (None, [C.c_void_p, C.c_int, C.c_double]),
            "orc_sd_set_loo_draws": (None, [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp, _dp]),
            "orc_sd_get_loo_short": (C.c_int, [C.c_void_p]),
            "orc_sd_set_split_draws": (None, [C.c_void_p, C.c_long, _dp]),
            "orc_sd_set_no_fit": (None, [C.c_void_p, C.c_int]),
            "orc_lm1_dif": (C.c_int, [LM_FN, _dp, C.c_int, C.c_int, _dp, C.c_void_p]),
            "orc_sd_get_nk": (C.c_int, [C.c_void_p]),
            "orc_sd_get_over_smooth": (C.c_double, [C.c_void_p]),
            "orc_knn_q": (None, [_dp, C.c_int, C.c_int, C.c_int, C.c_int, _ip, C.c_int]),
            "orc_nnls_solve": (C.c_double, [_dp, C.c_int, C.c_int, _dp, _dp, C.c_int]),
            "orc_sd_new": (C.c_void_p, [C.c_int, C.c_int, C.c_double, C.c_int]),
            "orc_sd_free": (None, [C.c_void_p]),
            "orc_sd_set_params": (None, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]),
            "orc_sd_set_threads": (None, [C.c_void_p, C.c_int]),
            "orc_sd_set_cov_type": (None, [C.c_void_p, C.c_int]),
            "orc_sd_set_cov_fixed": (None, [C.c_void_p, _dp]),
            "orc_sd_set_sample": (None, [C.c_void_p, _dp, C.c_int]),
            "orc_sd_prepare": (C.c_int, [C.c_void_p]),
            "orc_sd_prepare_interp": (C.c_int, [C.c_void_p, _dp]),
            "orc_sd_eval_m2lnp": (C.c_double, [C.c_void_p, _dp]),
            "orc_sd_eval_m2lnp_batch": (None, [C.c_void_p, _dp, C.c_int, _dp]),
            "orc_sd_eval": (C.c_double, [C.c_void_p, _dp]),
            "orc_sd_eval_batch": (None, [C.c_void_p, _dp, C.c_int, _dp]),
            "orc_sd_compute_IM": (C.c_int, [C.c_void_p, _dp]),
            "orc_sd_kernel_choose": (C.c_int, [C.c_void_p, C.c_double]),
            "orc_sd_sample": (C.c_int, [C.c_void_p, C.c_double, _dp, C.c_double, _dp]),
            "orc_sd_sample_batch": (None, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _ip]),
            "orc_sd_get_n": (C.c_int, [C.c_void_p]),
            "orc_sd_get_k": (C.c_int, [C.c_void_p]),
            "orc_sd_get_href": (C.c_double, [C.c_void_p]),
            "orc_sd_get_rnorm": (C.c_double, [C.c_void_p]),
            "orc_sd_get_kernel_lnnorm": (C.c_double, [C.c_void_p]),
            "orc_sd_get_interp_branch": (C.c_int, [C.c_void_p]),
            "orc_sd_get_chol_fallbacks": (C.c_int, [C.c_void_p]),
            "orc_sd_get_weights": (None, [C.c_void_p, _dp]),
            "orc_sd_get_sample": (None, [C.c_void_p, _dp]),
            "orc_sd_get_cov": (None, [C.c_void_p, _dp]),
            "orc_sd_get_U": (None, [C.c_void_p, _dp]),
            "orc_sd_get_invUsample": (None, [C.c_void_p, _dp]),
            "orc_sd_get_Ui": (None, [C.c_void_p, C.c_int, _dp]),
            "orc_sd_get_lnnorms": (None, [C.c_void_p, _dp]),
            "orc_sd_get_knn": (None, [C.c_void_p, _ip]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ref_lib():
    """The reference kd-tree, or None when it was not built (no NumCosmo sources)."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = C.CDLL(REF_PATH)
        R.ref_kdtree_knn.restype = None
        R.ref_kdtree_knn.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _ip]
        _ref = R
    return _ref


def ref_levmar():
    """The reference levmar driver, or None when it was not built."""
    global _ref_lm
    if _ref_lm is None and os.path.exists(REF_LM_PATH):
        R = C.CDLL(REF_LM_PATH)
        R.ref_levmar_dif1.restype = C.c_int
        R.ref_levmar_dif1.argtypes = [LM_FN, _dp, C.c_int, C.c_int, _dp, C.c_void_p, _dp]
        _ref_lm = R
    return _ref_lm


def lm1_oracle(f, p0: float, n: int, opts, itmax: int = 10000):
    """The oracle's one-parameter dlevmar_dif restatement on f(p) -> n values."""
    cb = LM_FN(lambda p, hx, nn, ctx: _lm_fill(f, p, hx, nn))
    p = np.array([p0], dtype=np.float64)
    o = _f64(opts)
    it = lib().orc_lm1_dif(cb, dptr(p), n, itmax, dptr(o), None)
    return float(p[0]), int(it)


def lm1_reference(f, p0: float, n: int, opts, itmax: int = 10000):
    """The reference's dlevmar_dif (compiled from its sources) on the same f;
    returns (p, iterations) or None when it was not built."""
    R = ref_levmar()
    if R is None:
        return None
    cb = LM_FN(lambda p, hx, nn, ctx: _lm_fill(f, p, hx, nn))
    p = np.array([p0], dtype=np.float64)
    o = _f64(opts)
    info = np.zeros(10)
    R.ref_levmar_dif1(cb, dptr(p), n, itmax, dptr(o), None, dptr(info))
    return float(p[0]), int(info[5])


def _lm_fill(f, p, hx, n):
    v = np.asarray(f(p), dtype=np.float64)
    for i in range(n):
        hx[i] = v[i]


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


# ---- building blocks -------------------------------------------------------

def welford_cov(X, rows=None) -> np.ndarray:
    X = _f64(X)
    n, d = X.shape
    cov = np.zeros((d, d))
    if rows is None:
        lib().orc_welford_cov(dptr(X), None, n, d, dptr(cov))
    else:
        r = np.ascontiguousarray(rows, dtype=np.int32)
        lib().orc_welford_cov(dptr(X), iptr(r), len(r), d, dptr(cov))
    return cov


def qn(x) -> float:
    """Qn scale estimator (the statistic of GSL's gsl_stats_Qn_from_sorted_data)."""
    v = _f64(np.array(x, dtype=np.float64).ravel())
    return lib().orc_qn(dptr(v), v.size)


def cov_robust(X, ogk: bool, rows=None) -> np.ndarray:
    """ROBUST (OGK) or ROBUST_DIAG covariance of X's rows (all, or the given ones)."""
    X = _f64(X)
    n, d = X.shape
    r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
    cov = np.zeros((d, d))
    f = lib().orc_cov_robust_ogk if ogk else lib().orc_cov_robust_diag
    f(dptr(X), None if r is None else iptr(r), n if r is None else r.size, d, dptr(cov))
    return cov


def cholesky_upper(A) -> tuple[np.ndarray, int]:
    U = _f64(A).copy()
    info = lib().orc_cholesky_upper(dptr(U), U.shape[0])
    return U, info


def cholesky_decomp_fallback(cov, maxiter=200) -> tuple[np.ndarray, int]:
    cov = _f64(cov)
    U = np.zeros_like(cov)
    r = lib().orc_cholesky_decomp_fallback(dptr(cov), dptr(U), cov.shape[0], maxiter)
    return U, r


def lndet(U) -> float:
    U = _f64(U)
    return lib().orc_cholesky_lndet(dptr(U), U.shape[0])


def knn(Y, k, nthreads=os.cpu_count()) -> np.ndarray:
    Y = _f64(Y)
    n, d = Y.shape
    out = np.zeros((n, k), dtype=np.int32)
    lib().orc_knn(dptr(Y), n, d, k, iptr(out), nthreads)
    return out


def ref_knn(Y, k) -> np.ndarray:
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference kd-tree not built")
    Y = _f64(Y)
    n, d = Y.shape
    out = np.zeros((n, k), dtype=np.int32)
    R.ref_kdtree_knn(dptr(Y), n, d, k, iptr(out))
    return out


def nnls(A, f, nthreads=os.cpu_count()) -> tuple[np.ndarray, float]:
    A = _f64(A)
    f = _f64(f)
    x = np.zeros(A.shape[1])
    rn = lib().orc_nnls_solve(dptr(A), A.shape[0], A.shape[1], dptr(f), dptr(x), nthreads)
    return x, rn


def nnls_fallbacks() -> dict:
    """Solves of the last NNLS fit that took the LU and the QR fallback."""
    lu, qr = C.c_int(), C.c_int()
    lib().orc_nnls_fallbacks(C.byref(lu), C.byref(qr))
    return {"lu": lu.value, "qr": qr.value}


def kernel_sum(kernel, nu, d, chi2, w, lnu=None, lnnorm=None):
    chi2, w = _f64(chi2), _f64(w)
    n = len(chi2)
    lnK = np.zeros(n)
    g, lam = C.c_double(), C.c_double()
    if lnu is not None:
        lnu = _f64(lnu)
        lib().orc_kernel_sum0(kernel, nu, d, n, dptr(chi2), dptr(w), dptr(lnu), dptr(lnK), C.byref(g), C.byref(lam))
    else:
        lib().orc_kernel_sum1(kernel, nu, d, n, dptr(chi2), dptr(w), lnnorm, dptr(lnK), C.byref(g), C.byref(lam))
    return g.value, lam.value


# ---- StatsDist -------------------------------------------------------------

class OracleStatsDist:
    """Mirror of NcmStatsDistKDE / NcmStatsDistVKDE on the CPU (every CV and covariance type)."""

    def __init__(self, kind: int, kernel: int, d: int, nu: float = 3.0, over_smooth=1.0,
                 shrink=0.01, local_frac=0.05, use_rot_href=False, nearPD_maxiter=200,
                 nthreads: int | None = None, cov_type: int = 0):
        self.kind, self.kernel, self.d, self.nu = kind, kernel, d, float(nu)
        self._h = lib().orc_sd_new(kind, kernel, float(nu), d)
        lib().orc_sd_set_params(self._h, over_smooth, shrink, local_frac, int(use_rot_href), nearPD_maxiter)
        lib().orc_sd_set_threads(self._h, nthreads or os.cpu_count())
        lib().orc_sd_set_cov_type(self._h, int(cov_type))

    def set_cov_fixed(self, cov) -> None:
        """ncm_stats_dist_kde_set_cov_fixed: the global covariance of cov-type FIXED."""
        self._cov_fixed = _f64(cov).reshape(self.d, self.d)
        lib().orc_sd_set_cov_fixed(self._h, dptr(self._cov_fixed))

    def set_cv(self, cv_type: int, split_frac: float = 0.5) -> None:
        """NcmStatsDistCV and the split fraction (NONE = 0, SPLIT = 1, SPLIT_NOFIT = 2,
        LOO = 3; the fraction's default is the reference property's, 0.5)."""
        lib().orc_sd_set_cv(self._h, int(cv_type), float(split_frac))

    def set_loo_draws(self, u, z1, c1, z2, c2) -> None:
        """The LOO Monte Carlo's draw pairs (ncm_stats_dist_sample2 order); c1, c2
        are None for the Gaussian kernel."""
        u, z1, z2 = _f64(u), _f64(z1), _f64(z2)
        c1 = None if c1 is None else _f64(c1)
        c2 = None if c2 is None else _f64(c2)
        self._loo = (u, z1, c1, z2, c2)
        lib().orc_sd_set_loo_draws(self._h, len(u), dptr(u), dptr(z1), None if c1 is None else dptr(c1),
                                   dptr(z2), None if c2 is None else dptr(c2))

    def set_no_fit(self, on: bool) -> None:
        """Skip the CV type's bandwidth fit (the weight fit at the set over-smoothing)."""
        lib().orc_sd_set_no_fit(self._h, int(bool(on)))

    def set_split_draws(self, g) -> None:
        """CV_SPLIT's restart draws (unit gaussians, consumed in order across calls)."""
        g = _f64(g)
        lib().orc_sd_set_split_draws(self._h, len(g), dptr(g))

    @property
    def loo_short(self) -> bool:
        return bool(lib().orc_sd_get_loo_short(self._h))

    @property
    def n_kernels(self) -> int:
        return lib().orc_sd_get_nk(self._h)

    @property
    def over_smooth(self) -> float:
        return lib().orc_sd_get_over_smooth(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_sd_free(self._h)
            self._h = None

    def set_sample(self, X):
        X = _f64(X)
        assert X.shape[1] == self.d
        lib().orc_sd_set_sample(self._h, dptr(X), X.shape[0])

    def prepare(self) -> int:
        return lib().orc_sd_prepare(self._h)

    def prepare_interp(self, m2lnp) -> int:
        m = _f64(m2lnp)
        return lib().orc_sd_prepare_interp(self._h, dptr(m))

    def eval_m2lnp(self, X) -> np.ndarray:
        X = _f64(np.atleast_2d(X))
        out = np.zeros(X.shape[0])
        lib().orc_sd_eval_m2lnp_batch(self._h, dptr(X), X.shape[0], dptr(out))
        return out

    def eval(self, X) -> np.ndarray:
        X = _f64(np.atleast_2d(X))
        out = np.zeros(X.shape[0])
        lib().orc_sd_eval_batch(self._h, dptr(X), X.shape[0], dptr(out))
        return out

    def compute_IM(self) -> np.ndarray:
        """The interpolation matrix with unit f, n_obs x n_kernels."""
        n = self.n
        IM = np.zeros((n, self.n_kernels))
        lib().orc_sd_compute_IM(self._h, dptr(IM))
        return IM

    def kernel_choose(self, u) -> np.ndarray:
        return np.array([lib().orc_sd_kernel_choose(self._h, float(x)) for x in np.atleast_1d(u)], dtype=np.int32)

    def sample(self, u, z, chisq=None):
        u = _f64(np.atleast_1d(u))
        n = len(u)
        z = _f64(z).reshape(n, self.d)
        x = np.zeros((n, self.d))
        idx = np.zeros(n, dtype=np.int32)
        cs = _f64(chisq) if chisq is not None else None
        lib().orc_sd_sample_batch(self._h, n, dptr(u), dptr(z), dptr(cs) if cs is not None else None,
                                  dptr(x), iptr(idx))
        return x, idx

    @property
    def n(self) -> int:
        return lib().orc_sd_get_n(self._h)

    @property
    def k(self) -> int:
        return lib().orc_sd_get_k(self._h)

    @property
    def href(self) -> float:
        return lib().orc_sd_get_href(self._h)

    @property
    def rnorm(self) -> float:
        return lib().orc_sd_get_rnorm(self._h)

    @property
    def kernel_lnnorm(self) -> float:
        return lib().orc_sd_get_kernel_lnnorm(self._h)

    @property
    def interp_branch(self) -> int:
        return lib().orc_sd_get_interp_branch(self._h)

    @property
    def chol_fallbacks(self) -> int:
        return lib().orc_sd_get_chol_fallbacks(self._h)

    def weights(self) -> np.ndarray:
        w = np.zeros(self.n_kernels)
        lib().orc_sd_get_weights(self._h, dptr(w))
        return w

    def sample_array(self) -> np.ndarray:
        X = np.zeros((self.n, self.d))
        lib().orc_sd_get_sample(self._h, dptr(X))
        return X

    def cov(self) -> np.ndarray:
        c = np.zeros((self.d, self.d))
        lib().orc_sd_get_cov(self._h, dptr(c))
        return c

    def U(self) -> np.ndarray:
        c = np.zeros((self.d, self.d))
        lib().orc_sd_get_U(self._h, dptr(c))
        return c

    def invUsample(self) -> np.ndarray:
        Y = np.zeros((self.n, self.d))
        lib().orc_sd_get_invUsample(self._h, dptr(Y))
        return Y

    def Ui(self, i: int) -> np.ndarray:
        c = np.zeros((self.d, self.d))
        lib().orc_sd_get_Ui(self._h, i, dptr(c))
        return c

    def lnnorms(self) -> np.ndarray:
        v = np.zeros(self.n_kernels)
        lib().orc_sd_get_lnnorms(self._h, dptr(v))
        return v

    def knn(self) -> np.ndarray:
        out = np.zeros((self.n_kernels, self.k), dtype=np.int32)
        lib().orc_sd_get_knn(self._h, iptr(out))
        return out
