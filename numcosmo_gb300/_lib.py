"""ctypes binding of libncg.so (the C-ABI declared in include/ncg.h).

The library is built in-tree by numcosmo_gb300.build; loading fails loudly
when it is missing, there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)

STATUS = {
    0: "NCG_OK", 1: "NCG_ERR_INVALID_ARG", 2: "NCG_ERR_SAMPLE_TOO_SMALL", 3: "NCG_ERR_TOO_FEW_LOCAL",
    4: "NCG_ERR_NOT_PD", 5: "NCG_ERR_NOT_PREPARED", 6: "NCG_ERR_NONFINITE", 7: "NCG_ERR_UNSUPPORTED",
    8: "NCG_ERR_CUDA", 9: "NCG_ERR_OUT_OF_MEMORY", 10: "NCG_ERR_TIMEOUT", 11: "NCG_ERR_BAD_WEIGHTS",
    12: "NCG_ERR_BUSY",
}


class NcgError(RuntimeError):
    """A non-OK ncg_status_t; .status is the code, .name its enum name."""

    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        self.name = STATUS.get(status, str(status))
        super().__init__(f"{where}: {self.name}: {detail}")


class ncg_sd_config_t(C.Structure):
    _fields_ = [
        ("over_smooth", C.c_double), ("shrink", C.c_double), ("local_frac", C.c_double),
        ("use_rot_href", C.c_int32), ("nearPD_maxiter", C.c_int32), ("cv_type", C.c_int32),
        ("cov_type", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32),
    ]


# name: (restype, argtypes); restype None means ncg_status_t checked
_SIGS = {
    "ncg_status_string": (C.c_char_p, [C.c_int]),
    "ncg_last_error": (C.c_char_p, []),
    "ncg_version": (C.c_char_p, []),
    "ncg_sd_config_init": ("void", [C.POINTER(ncg_sd_config_t)]),
    "ncg_sd_new": (None, [C.c_int, C.c_int, C.c_uint32, C.c_double, C.POINTER(ncg_sd_config_t), C.POINTER(C.c_void_p)]),
    "ncg_sd_free": (None, [C.c_void_p]),
    "ncg_sd_set_stream": (None, [C.c_void_p, C.c_void_p]),
    "ncg_sd_synchronize": (None, [C.c_void_p]),
    "ncg_sd_set_over_smooth": (None, [C.c_void_p, C.c_double]),
    "ncg_sd_set_shrink": (None, [C.c_void_p, C.c_double]),
    "ncg_sd_set_local_frac": (None, [C.c_void_p, C.c_double]),
    "ncg_sd_set_use_rot_href": (None, [C.c_void_p, C.c_int32]),
    "ncg_sd_set_nearPD_maxiter": (None, [C.c_void_p, C.c_int32]),
    "ncg_sd_set_cov_type": (None, [C.c_void_p, C.c_int]),
    "ncg_sd_set_cov_fixed": (None, [C.c_void_p, _dp]),
    "ncg_sd_set_precision": (None, [C.c_void_p, C.c_int]),
    "ncg_sd_reset": (None, [C.c_void_p]),
    "ncg_sd_add_obs": (None, [C.c_void_p, _dp]),
    "ncg_sd_add_obs_batch": (None, [C.c_void_p, _dp, C.c_uint64]),
    "ncg_sd_prepare": (None, [C.c_void_p]),
    "ncg_sd_prepare_interp": (None, [C.c_void_p, _dp]),
    "ncg_sd_eval_m2lnp": (None, [C.c_void_p, _dp, _dp]),
    "ncg_sd_eval_m2lnp_batch": (None, [C.c_void_p, _dp, C.c_uint64, _dp]),
    "ncg_sd_eval_m2lnp_device": (None, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ncg_sd_eval_m2lnp_device_noalloc": (None, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "ncg_sd_eval": (None, [C.c_void_p, _dp, _dp]),
    "ncg_sd_eval_batch": (None, [C.c_void_p, _dp, C.c_uint64, _dp]),
    "ncg_sd_kernel_choose_batch": (None, [C.c_void_p, _dp, C.c_uint64, _ip]),
    "ncg_sd_sample_batch": (None, [C.c_void_p, _dp, _dp, _dp, C.c_uint64, _dp, _ip]),
    "ncg_sd_get_dim": (None, [C.c_void_p, _u32p]),
    "ncg_sd_get_sample_size": (None, [C.c_void_p, _u64p]),
    "ncg_sd_get_n_kernels": (None, [C.c_void_p, _u64p]),
    "ncg_sd_get_href": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_rnorm": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_weights": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_sample": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_cov_decomp": (None, [C.c_void_p, C.c_uint32, _dp]),
    "ncg_sd_get_full_cov_decomp": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_full_cov": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_lnnorm": (None, [C.c_void_p, C.c_uint32, _dp]),
    "ncg_sd_get_interp_branch": (None, [C.c_void_p, _ip]),
    "ncg_sd_get_chol_fallbacks": (None, [C.c_void_p, _u64p]),
    "ncg_sd_get_knn_k": (None, [C.c_void_p, _u32p]),
    "ncg_sd_get_interp_stats": (None, [C.c_void_p, _ip]),
    "ncg_sd_get_eval_path": (None, [C.c_void_p, _ip, _dp]),
    "ncg_sd_compute_IM": (None, [C.c_void_p, _dp]),
    "ncg_rng_new": (None, [C.c_uint32, C.POINTER(C.c_void_p)]),
    "ncg_rng_free": (None, [C.c_void_p]),
    "ncg_rng_get_u32": (C.c_uint32, [C.c_void_p]),
    "ncg_rng_uniform": (C.c_double, [C.c_void_p]),
    "ncg_rng_uniform_pos": (C.c_double, [C.c_void_p]),
    "ncg_rng_ugaussian": (C.c_double, [C.c_void_p]),
    "ncg_rng_chisq": (C.c_double, [C.c_void_p, C.c_double]),
    "ncg_rng_sample_stream": (None, [C.c_void_p, C.c_int, C.c_uint32, C.c_double, C.c_uint64, _dp, _dp, _dp]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load libncg.so; raise if it is not built (no silent fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(f"libncg.so not built at {path}; run numcosmo_gb300.build.build()")
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        if res is None:
            f.restype = C.c_int
        elif res == "void":
            f.restype = None
        else:
            f.restype = res
    _lib = L
    return L


def check(status: int, where: str) -> None:
    if status != 0:
        L = load()
        detail = L.ncg_last_error().decode() or L.ncg_status_string(status).decode()
        raise NcgError(status, where, detail)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def exported_symbols() -> list[str]:
    return sorted(_SIGS)
