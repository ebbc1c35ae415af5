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
        ("cov_type", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32), ("async_alloc", C.c_int32),
    ]


class ncg_batch_params_t(C.Structure):
    _fields_ = [
        ("items_per_cta", C.c_double), ("ctas_per_sm", C.c_int32), ("order", C.c_int32), ("split", C.c_int32),
        ("tc", C.c_int32),
    ]


_i64p = C.POINTER(C.c_int64)


class ncg_server_config_t(C.Structure):
    _fields_ = [("device", C.c_int32), ("slots", C.c_int32), ("precision", C.c_int32), ("pad_", C.c_int32),
                ("hbm_budget", C.c_uint64)]


class ncg_chain_desc_t(C.Structure):
    _fields_ = [("kind", C.c_int32), ("kernel", C.c_int32), ("dim", C.c_uint32), ("pad_", C.c_int32),
                ("n", C.c_uint64), ("nu", C.c_double), ("over_smooth", C.c_double), ("local_frac", C.c_double),
                ("seed", C.c_uint32), ("pad2_", C.c_int32), ("X0", C.POINTER(C.c_double)),
                ("target_L", C.POINTER(C.c_double)), ("random_walk_prob", C.c_double), ("exploration", C.c_uint32),
                ("pad3_", C.c_int32), ("lb", C.POINTER(C.c_double)), ("ub", C.POINTER(C.c_double))]


class ncg_step_result_t(C.Structure):
    _fields_ = [("request", C.c_int64), ("chain", C.c_int32), ("status", C.c_int32), ("step", C.c_uint64),
                ("accepted", C.c_uint64), ("pairs", C.c_uint64), ("mean_m2lnL", C.c_double),
                ("state_sum", C.c_double), ("t_arrive", C.c_double), ("t_start", C.c_double),
                ("t_done", C.c_double), ("detail", C.c_char * 128)]


class ncg_server_stats_t(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("admitted", C.c_uint64), ("evicted", C.c_uint64), ("reserved_bytes", C.c_uint64),
                ("peak_reserved_bytes", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("span_s", C.c_double), ("pairs", C.c_double)]

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
    "ncg_sd_get_knn": (None, [C.c_void_p, _ip]),
    "ncg_sd_set_split_frac": (None, [C.c_void_p, C.c_double]),
    "ncg_sd_get_over_smooth": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_interp_fallbacks": (None, [C.c_void_p, _ip, _ip]),
    "ncg_debug_inject_wait_fault": (None, [C.c_int32]),
    "ncg_sd_get_Ki": (None, [C.c_void_p, C.c_uint32, _dp, _dp, _dp, _dp]),
    "ncg_sd_get_interp_stats": (None, [C.c_void_p, _ip]),
    "ncg_sd_set_kernel_timing": (None, [C.c_void_p, C.c_int32]),
    "ncg_measure_fp64_peak": (None, [C.c_int32, _dp]),
    "ncg_sd_get_tc_check": (None, [C.c_void_p, _dp]),
    "ncg_sd_get_kernel_time": (None, [C.c_void_p, _dp]),
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
    "ncg_rng_sample2_stream": (None, [C.c_void_p, C.c_int, C.c_uint32, C.c_double, C.c_uint64, _dp, _dp, _dp, _dp,
                                       _dp]),
    "ncg_batch_params_init": (None, [C.POINTER(ncg_batch_params_t)]),
    "ncg_batch_new": (None, [C.c_int, C.POINTER(C.c_void_p)]),
    "ncg_batch_free": ("void", [C.c_void_p]),
    "ncg_batch_add": (None, [C.c_void_p, C.c_void_p, C.c_uint64, _ip]),
    "ncg_batch_clear": (None, [C.c_void_p]),
    "ncg_batch_layout": (None, [C.c_void_p, _i64p, _i64p, _i64p]),
    "ncg_batch_set_params": (None, [C.c_void_p, C.c_int32, C.POINTER(ncg_batch_params_t)]),
    "ncg_batch_get_params": (None, [C.c_void_p, C.c_int32, C.POINTER(ncg_batch_params_t)]),
    "ncg_batch_autotune": (None, [C.c_void_p, C.c_int32, C.c_int32, _dp]),
    "ncg_batch_eval_m2lnp_device": (None, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ncg_batch_eval_m2lnp": (None, [C.c_void_p, C.c_int32, _dp, _dp]),
    "ncg_batch_get_stats": (None, [C.c_void_p, C.c_int32, _i64p]),
    "ncg_batch_prepare": (None, [C.c_void_p, C.c_int32]),
    "ncg_batch_prepare_interp": (None, [C.c_void_p, _dp, C.c_int32]),
    "ncg_sd_sample_batch_device": (None, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                          C.c_void_p]),
    "ncg_sd_workspace_bytes": (None, [C.c_void_p, C.c_uint64, C.POINTER(C.c_size_t)]),
    "ncg_sd_set_workspace": (None, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "ncg_server_config_init": (None, [C.POINTER(ncg_server_config_t)]),
    "ncg_server_new": (None, [C.POINTER(ncg_server_config_t), C.POINTER(C.c_void_p)]),
    "ncg_server_free": ("void", [C.c_void_p]),
    "ncg_server_add_chain": (None, [C.c_void_p, C.POINTER(ncg_chain_desc_t), _ip]),
    "ncg_server_submit": (None, [C.c_void_p, C.c_int32, _i64p]),
    "ncg_server_wait": (None, [C.c_void_p, C.c_int64, C.POINTER(ncg_step_result_t)]),
    "ncg_server_drain": (None, [C.c_void_p]),
    "ncg_server_get_stats": (None, [C.c_void_p, C.POINTER(ncg_server_stats_t)]),
    "ncg_server_get_chain": (None, [C.c_void_p, C.c_int32, _dp, _dp]),
    "ncg_server_clock": (C.c_double, [C.c_void_p]),
    "ncg_server_checkpoint": (None, [C.c_void_p, C.c_char_p]),
    "ncg_server_restore": (None, [C.c_void_p, C.c_char_p, _ip, _ip]),
    "ncg_server_get_chain_info": (None, [C.c_void_p, C.c_int32, C.POINTER(ncg_chain_desc_t), _u64p]),
    "ncg_rng_state_bytes": (C.c_size_t, []),
    "ncg_rng_get_state": (None, [C.c_void_p, C.c_void_p]),
    "ncg_rng_set_state": (None, [C.c_void_p, C.c_void_p]),
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
