"""Python mirror of NumCosmo's StatsDist interface over libncg.so.

Names follow the reference's GObject-Introspection API
(numcosmo_py/interpolation/stats_dist.py:57-112 builds them as
``Ncm.StatsDistVKDE.new(Ncm.StatsDistKernelST.new(dim, nu), Ncm.StatsDistCV.NONE)``):
StatsDistKernelGauss / StatsDistKernelST, StatsDistKDE / StatsDistVKDE with
set_over_smooth, set_shrink, add_obs, reset, prepare, prepare_interp,
eval_m2lnp, eval, kernel_choose, sample, get_href, get_rnorm, peek_weights,
peek_cov_decomp, peek_full_cov, get_lnnorm.  Batched forms take 2-D arrays.
Every call goes through the C-ABI; errors raise NcgError.
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np

from . import _lib
from ._lib import NcgError, call, load

__all__ = [
    "NcgError", "StatsDistCV", "StatsDistKDECovType", "Precision", "StatsDistKernelGauss",
    "StatsDistKernelST", "StatsDistKDE", "StatsDistVKDE", "RNG",
]


class StatsDistCV(IntEnum):
    NONE = 0
    SPLIT = 1
    SPLIT_NOFIT = 2
    LOO = 3


class StatsDistKDECovType(IntEnum):
    SAMPLE = 0
    FIXED = 1
    ROBUST_DIAG = 2
    ROBUST = 3


class Precision(IntEnum):
    FP64 = 0
    MIXED = 1          # FP16x3 tensor cores where the operand passes its check, else FP32 SIMT
    MIXED_SIMT = 2     # FP32 CUDA-core form (hi/lo-split differences)


KDE, VKDE = 0, 1
GAUSS, ST = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_dp)


def measure_fp64_peak(device: int = 0) -> float:
    """Measured FP64 FMA rate of the device in TFLOP/s (ncg_measure_fp64_peak)."""
    v = C.c_double()
    call("ncg_measure_fp64_peak", device, C.byref(v))
    return v.value


class StatsDistKernelGauss:
    """ncm_stats_dist_kernel_gauss_new (numcosmo/ncm/stats/ncm_stats_dist_kernel_gauss.c:365-373)."""

    kernel_type = GAUSS

    def __init__(self, dim: int):
        self.dim = int(dim)
        self.nu = 0.0

    @classmethod
    def new(cls, dim: int):
        return cls(dim)


class StatsDistKernelST:
    """ncm_stats_dist_kernel_st_new (numcosmo/ncm/stats/ncm_stats_dist_kernel_st.c:426-435)."""

    kernel_type = ST

    def __init__(self, dim: int, nu: float = 3.0):
        self.dim = int(dim)
        self.nu = float(nu)

    @classmethod
    def new(cls, dim: int, nu: float):
        return cls(dim, nu)


class _StatsDist:
    kind = -1

    def __init__(self, kernel, cv_type: StatsDistCV = StatsDistCV.NONE, precision: Precision = Precision.FP64,
                 device: int = 0):
        L = load()
        cfg = _lib.ncg_sd_config_t()
        L.ncg_sd_config_init(C.byref(cfg))
        cfg.cv_type = int(cv_type)
        cfg.precision = int(precision)
        cfg.device = int(device)
        h = C.c_void_p()
        call("ncg_sd_new", self.kind, kernel.kernel_type, kernel.dim, kernel.nu, C.byref(cfg), C.byref(h))
        self._h = h
        self.kernel = kernel
        self.dim = kernel.dim

    @classmethod
    def new(cls, kernel, cv_type: StatsDistCV = StatsDistCV.NONE):
        return cls(kernel, cv_type)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                load().ncg_sd_free(h)
            except Exception:
                pass
            self._h = None

    # ---- properties -------------------------------------------------------
    def set_over_smooth(self, v: float):
        call("ncg_sd_set_over_smooth", self._h, float(v))

    def set_split_frac(self, v: float):
        """Fraction of the sample used as kernels under a split cross-validation (default 0.5)."""
        call("ncg_sd_set_split_frac", self._h, float(v))

    def get_over_smooth(self) -> float:
        v = C.c_double()
        call("ncg_sd_get_over_smooth", self._h, C.byref(v))
        return v.value

    def set_shrink(self, v: float):
        call("ncg_sd_set_shrink", self._h, float(v))

    def set_nearPD_maxiter(self, v: int):
        call("ncg_sd_set_nearPD_maxiter", self._h, int(v))

    def set_cov_type(self, t: StatsDistKDECovType):
        call("ncg_sd_set_cov_type", self._h, int(t))

    def set_cov_fixed(self, cov):
        c = _f64(cov)
        call("ncg_sd_set_cov_fixed", self._h, _p(c))

    def set_precision(self, p: Precision):
        call("ncg_sd_set_precision", self._h, int(p))

    def set_stream(self, cuda_stream: int | None):
        call("ncg_sd_set_stream", self._h, C.c_void_p(cuda_stream or 0))

    def synchronize(self):
        call("ncg_sd_synchronize", self._h)

    # ---- sample ------------------------------------------------------------
    def reset(self):
        call("ncg_sd_reset", self._h)

    def add_obs(self, y):
        y = _f64(y)
        if y.ndim == 1:
            call("ncg_sd_add_obs", self._h, _p(y))
        else:
            call("ncg_sd_add_obs_batch", self._h, _p(y), y.shape[0])

    def set_sample(self, X):
        self.reset()
        self.add_obs(_f64(X).reshape(-1, self.dim))

    # ---- prepare -----------------------------------------------------------
    def prepare(self):
        call("ncg_sd_prepare", self._h)

    def prepare_interp(self, m2lnp):
        m = _f64(m2lnp)
        call("ncg_sd_prepare_interp", self._h, _p(m))

    # ---- evaluation ----------------------------------------------------------
    def eval_m2lnp(self, x):
        x = _f64(x)
        if x.ndim == 1:
            out = C.c_double()
            call("ncg_sd_eval_m2lnp", self._h, _p(x), C.byref(out))
            return out.value
        out = np.empty(x.shape[0])
        call("ncg_sd_eval_m2lnp_batch", self._h, _p(x), x.shape[0], _p(out))
        return out

    def eval_m2lnp_into(self, x: np.ndarray, out: np.ndarray):
        """eval_m2lnp of the rows of x into the preallocated out (both C-contiguous float64, host)."""
        assert x.dtype == np.float64 and out.dtype == np.float64 and x.flags.c_contiguous
        call("ncg_sd_eval_m2lnp_batch", self._h, _p(x), x.shape[0], _p(out))

    def eval_m2lnp_device(self, d_x: int, m: int, d_out: int):
        """Device pointers (e.g. torch tensor .data_ptr()), asynchronous on the handle's stream."""
        call("ncg_sd_eval_m2lnp_device", self._h, C.c_void_p(d_x), m, C.c_void_p(d_out))

    def eval(self, x):
        x = _f64(x)
        if x.ndim == 1:
            out = C.c_double()
            call("ncg_sd_eval", self._h, _p(x), C.byref(out))
            return out.value
        out = np.empty(x.shape[0])
        call("ncg_sd_eval_batch", self._h, _p(x), x.shape[0], _p(out))
        return out

    def kernel_choose(self, u):
        u = _f64(np.atleast_1d(u))
        idx = np.empty(len(u), dtype=np.int32)
        call("ncg_sd_kernel_choose_batch", self._h, _p(u), len(u), idx.ctypes.data_as(_ip))
        return idx

    def sample(self, u, z, chisq=None):
        """Draws from the replay stream (u[n], z[n, dim], chisq[n] for Student-t)."""
        u = _f64(np.atleast_1d(u))
        n = len(u)
        z = _f64(z).reshape(n, self.dim)
        cs = _f64(chisq) if chisq is not None else None
        x = np.empty((n, self.dim))
        idx = np.empty(n, dtype=np.int32)
        call("ncg_sd_sample_batch", self._h, _p(u), _p(z), _p(cs), n, _p(x), idx.ctypes.data_as(_ip))
        return x, idx

    def sample_rng(self, rng: "RNG", n: int):
        """n calls of ncm_stats_dist_sample with the stream drawn from rng."""
        u, z, cs = rng.sample_stream(self.kernel, n)
        return self.sample(u, z, cs)

    # ---- getters -------------------------------------------------------------
    def get_dim(self) -> int:
        return self.dim

    def get_sample_size(self) -> int:
        v = C.c_uint64()
        call("ncg_sd_get_sample_size", self._h, C.byref(v))
        return v.value

    def get_n_kernels(self) -> int:
        """Kernels of the last prepare (the sample size unless a split cross-validation is set)."""
        v = C.c_uint64()
        call("ncg_sd_get_n_kernels", self._h, C.byref(v))
        return v.value

    def get_href(self) -> float:
        v = C.c_double()
        call("ncg_sd_get_href", self._h, C.byref(v))
        return v.value

    def get_rnorm(self) -> float:
        v = C.c_double()
        call("ncg_sd_get_rnorm", self._h, C.byref(v))
        return v.value

    def peek_weights(self) -> np.ndarray:
        w = np.empty(self.get_n_kernels())
        call("ncg_sd_get_weights", self._h, _p(w))
        return w

    def peek_sample_array(self) -> np.ndarray:
        X = np.empty((self.get_sample_size(), self.dim))
        call("ncg_sd_get_sample", self._h, _p(X))
        return X

    def peek_cov_decomp(self, i: int) -> np.ndarray:
        U = np.empty((self.dim, self.dim))
        call("ncg_sd_get_cov_decomp", self._h, int(i), _p(U))
        return U

    def peek_full_cov_decomp(self) -> np.ndarray:
        U = np.empty((self.dim, self.dim))
        call("ncg_sd_get_full_cov_decomp", self._h, _p(U))
        return U

    def peek_full_cov(self) -> np.ndarray:
        c = np.empty((self.dim, self.dim))
        call("ncg_sd_get_full_cov", self._h, _p(c))
        return c

    def get_lnnorm(self, i: int) -> float:
        v = C.c_double()
        call("ncg_sd_get_lnnorm", self._h, int(i), C.byref(v))
        return v.value

    def get_interp_branch(self) -> int:
        v = C.c_int32()
        call("ncg_sd_get_interp_branch", self._h, C.byref(v))
        return v.value

    def get_chol_fallbacks(self) -> int:
        v = C.c_uint64()
        call("ncg_sd_get_chol_fallbacks", self._h, C.byref(v))
        return v.value

    def get_eval_path(self) -> tuple[str, float]:
        """("fp64" | "tensor_core" | "simt", largest condition number of the mixed whitening)."""
        v = C.c_int32()
        k = C.c_double()
        call("ncg_sd_get_eval_path", self._h, C.byref(v), C.byref(k))
        return ("fp64", "tensor_core", "simt")[v.value], k.value

    def get_tc_check(self) -> float:
        """Measured error of the tensor-core operand on the kernel centres (-1: not checked)."""
        v = C.c_double()
        call("ncg_sd_get_tc_check", self._h, C.byref(v))
        return v.value

    def set_kernel_timing(self, on: bool) -> None:
        call("ncg_sd_set_kernel_timing", self._h, 1 if on else 0)

    def get_kernel_time(self) -> float:
        """Milliseconds of the main kernel of the last tensor-core eval (timing on)."""
        v = C.c_double()
        call("ncg_sd_get_kernel_time", self._h, C.byref(v))
        return v.value

    def get_interp_stats(self) -> dict:
        """Counters of the last prepare_interp NNLS fit."""
        v = (C.c_int32 * 4)()
        call("ncg_sd_get_interp_stats", self._h, v)
        return dict(solves=v[0], cg_iters=v[1], shifted=v[2], fp64=v[3])

    def get_knn_k(self) -> int:
        v = C.c_uint32()
        call("ncg_sd_get_knn_k", self._h, C.byref(v))
        return v.value

    def get_interp_fallbacks(self) -> dict:
        """Solves of the last fit that took the LU and the QR fallback."""
        lu, qr = C.c_int32(), C.c_int32()
        call("ncg_sd_get_interp_fallbacks", self._h, C.byref(lu), C.byref(qr))
        return {"lu": lu.value, "qr": qr.value}

    def get_knn(self) -> np.ndarray:
        """Neighbour lists of the VKDE local covariances, n_kernels x k (int32)."""
        n, k = self.get_n_kernels(), self.get_knn_k()
        idx = np.empty((n, k), dtype=np.int32)
        call("ncg_sd_get_knn", self._h, idx.ctypes.data_as(C.POINTER(C.c_int32)))
        return idx

    def get_Ki(self, i: int):
        """ncm_stats_dist_get_Ki: (y_i, cov_i, n_i, w_i) of kernel i."""
        d = self.dim
        y = np.empty(d)
        cov = np.empty((d, d))
        ni, wi = C.c_double(), C.c_double()
        call("ncg_sd_get_Ki", self._h, int(i), _p(y), _p(cov), C.byref(ni), C.byref(wi))
        return y, cov, ni.value, wi.value

    def compute_IM(self) -> np.ndarray:
        """The interpolation matrix with unit f: n_obs x n_kernels (square but under a split)."""
        IM = np.empty((self.get_sample_size(), self.get_n_kernels()))
        call("ncg_sd_compute_IM", self._h, _p(IM))
        return IM


class StatsDistKDE(_StatsDist):
    """ncm_stats_dist_kde_new (numcosmo/ncm/stats/ncm_stats_dist_kde.c:694-702)."""

    kind = KDE


class StatsDistVKDE(_StatsDist):
    """ncm_stats_dist_vkde_new (numcosmo/ncm/stats/ncm_stats_dist_vkde.c:743-751)."""

    kind = VKDE

    def set_local_frac(self, v: float):
        call("ncg_sd_set_local_frac", self._h, float(v))

    def set_use_rot_href(self, v: bool):
        call("ncg_sd_set_use_rot_href", self._h, int(bool(v)))


class RNG:
    """NcmRNG stand-in (MT19937 + transforms) producing replay streams for sample()."""

    def __init__(self, seed: int = 0):
        h = C.c_void_p()
        call("ncg_rng_new", C.c_uint32(seed & 0xFFFFFFFF), C.byref(h))
        self._h = h

    @classmethod
    def seeded_new(cls, algo, seed: int):
        return cls(seed)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().ncg_rng_free(h)
            self._h = None

    def get_u32(self) -> int:
        return load().ncg_rng_get_u32(self._h)

    def uniform(self) -> float:
        return load().ncg_rng_uniform(self._h)

    def uniform_pos(self) -> float:
        return load().ncg_rng_uniform_pos(self._h)

    def ugaussian(self) -> float:
        return load().ncg_rng_ugaussian(self._h)

    def chisq(self, nu: float) -> float:
        return load().ncg_rng_chisq(self._h, float(nu))

    def sample_stream(self, kernel, n: int):
        d = kernel.dim
        u = np.empty(n)
        z = np.empty((n, d))
        cs = np.empty(n) if kernel.kernel_type == ST else None
        call("ncg_rng_sample_stream", self._h, kernel.kernel_type, d, float(kernel.nu), n, _p(u), _p(z), _p(cs))
        return u, z, cs

    def sample2_stream(self, kernel, n: int):
        """The draws of n ncm_stats_dist_sample2 calls: u, z1, c1, z2, c2."""
        d = kernel.dim
        u = np.empty(n)
        z1, z2 = np.empty((n, d)), np.empty((n, d))
        st = kernel.kernel_type == ST
        c1, c2 = (np.empty(n), np.empty(n)) if st else (None, None)
        call("ncg_rng_sample2_stream", self._h, kernel.kernel_type, d, float(kernel.nu), n, _p(u), _p(z1), _p(c1),
             _p(z2), _p(c2))
        return u, z1, c1, z2, c2
