"""Many StatsDist problems in one launch (the ncg_batch_* C-ABI).

A Batch borrows prepared StatsDistKDE / StatsDistVKDE objects together with
the number of points each is evaluated at, and evaluates -2 ln p of all of
them in one persistent-kernel launch replayed from a captured CUDA graph.
The reference has no such object (APES evaluates one NcmStatsDist at a time);
each problem's result equals its own eval_m2lnp with the same arithmetic up
to the slicing of its kernel range.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import call, load, ncg_batch_params_t
from .stats_dist import Precision, _StatsDist

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)


class Batch:
    def __init__(self, device: int = 0):
        load()
        h = C.c_void_p()
        call("ncg_batch_new", int(device), C.byref(h))
        self._h = h
        self._members: list[tuple[_StatsDist, int]] = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            load().ncg_batch_free(h)
            self._h = None

    def add(self, sd: _StatsDist, m: int) -> int:
        slot = C.c_int32()
        call("ncg_batch_add", self._h, sd._h, int(m), C.byref(slot))
        self._members.append((sd, int(m)))
        return slot.value

    def clear(self) -> None:
        call("ncg_batch_clear", self._h)
        self._members.clear()

    def __len__(self) -> int:
        return len(self._members)

    def layout(self) -> tuple[np.ndarray, np.ndarray, int, int]:
        n = len(self._members)
        xo = np.zeros(max(n, 1), dtype=np.int64)
        oo = np.zeros(max(n, 1), dtype=np.int64)
        tot = np.zeros(2, dtype=np.int64)
        call("ncg_batch_layout", self._h, xo.ctypes.data_as(_i64p), oo.ctypes.data_as(_i64p), tot.ctypes.data_as(_i64p))
        return xo[:n], oo[:n], int(tot[0]), int(tot[1])

    def pack(self, points: list[np.ndarray]) -> np.ndarray:
        """Concatenate per-problem point arrays (m_i x dim_i) in the batch layout."""
        xo, _, xt, _ = self.layout()
        X = np.empty(xt)
        for (sd, m), off, P in zip(self._members, xo, points):
            P = np.ascontiguousarray(P, dtype=np.float64)
            if P.shape != (m, sd.get_dim()):
                raise ValueError(f"points of shape {P.shape}, batch slot wants {(m, sd.get_dim())}")
            X[off:off + P.size] = P.ravel()
        return X

    def unpack(self, out: np.ndarray) -> list[np.ndarray]:
        _, oo, _, _ = self.layout()
        return [out[o:o + m] for (sd, m), o in zip(self._members, oo)]

    def eval_m2lnp(self, points: list[np.ndarray] | np.ndarray, precision: Precision = Precision.FP64):
        """-2 ln p of every problem at its points (list, or the packed array)."""
        X = points if isinstance(points, np.ndarray) and points.ndim == 1 else self.pack(points)
        X = np.ascontiguousarray(X, dtype=np.float64)
        _, _, _, ot = self.layout()
        out = np.empty(ot)
        call("ncg_batch_eval_m2lnp", self._h, int(precision), X.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
        return self.unpack(out)

    def eval_m2lnp_device(self, d_X: int, d_out: int, precision: Precision = Precision.FP64, stream: int = 0):
        """Device-pointer form (e.g. torch tensors' data_ptr()), ordered on `stream`."""
        call("ncg_batch_eval_m2lnp_device", self._h, int(precision), C.c_void_p(d_X), C.c_void_p(d_out),
             C.c_void_p(stream))

    def prepare(self, nthreads: int = 0) -> None:
        """Prepare every problem's handle at once (their samples set)."""
        call("ncg_batch_prepare", self._h, int(nthreads))

    def prepare_interp(self, m2lnp: list[np.ndarray], nthreads: int = 0) -> None:
        """prepare_interp of every problem at once, one -2 ln L array per problem."""
        flat = np.ascontiguousarray(np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in m2lnp]))
        call("ncg_batch_prepare_interp", self._h, flat.ctypes.data_as(_dp), int(nthreads))

    def autotune(self, precision: Precision = Precision.MIXED, reps: int = 2) -> float:
        ms = C.c_double()
        call("ncg_batch_autotune", self._h, int(precision), int(reps), C.byref(ms))
        return ms.value

    def get_params(self, precision: Precision = Precision.MIXED) -> dict:
        p = ncg_batch_params_t()
        call("ncg_batch_get_params", self._h, int(precision), C.byref(p))
        return dict(items_per_cta=p.items_per_cta, ctas_per_sm=p.ctas_per_sm, order=p.order, split=p.split, tc=p.tc)

    def set_params(self, precision: Precision = Precision.MIXED, **kw) -> None:
        p = ncg_batch_params_t()
        call("ncg_batch_get_params", self._h, int(precision), C.byref(p))
        for k, v in kw.items():
            setattr(p, k, v)
        call("ncg_batch_set_params", self._h, int(precision), C.byref(p))

    def get_stats(self, precision: Precision = Precision.MIXED) -> dict:
        s = np.zeros(7, dtype=np.int64)
        call("ncg_batch_get_stats", self._h, int(precision), s.ctypes.data_as(_i64p))
        keys = ("items", "launches", "fp64_problems", "pairs", "captures", "graph_launches", "tc_problems")
        return dict(zip(keys, (int(v) for v in s)))
