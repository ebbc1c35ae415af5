"""The serving loop (ncg_server_* C-ABI): concurrent APES chains on one GPU.

Server(slots, precision, hbm_budget) owns worker threads in the native
library; add_chain registers a walker ensemble with its Gaussian target;
submit queues one APES step of a chain and returns at once; wait / drain
block for results; stats reports p50/p99 step latency (arrival to
completion) and pairs.  `poisson_arrivals` builds a seeded arrival schedule
and `run_schedule` replays it against a server in real time.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from ._lib import (NcgError, call, load, ncg_chain_desc_t, ncg_server_config_t, ncg_server_stats_t,
                   ncg_step_result_t)
from .stats_dist import Precision

_dp = C.POINTER(C.c_double)


class Server:
    def __init__(self, slots: int = 4, precision: Precision = Precision.MIXED, hbm_budget: int = 40 << 30,
                 device: int = 0):
        L = load()
        cfg = ncg_server_config_t()
        call("ncg_server_config_init", C.byref(cfg))
        cfg.device, cfg.slots, cfg.precision, cfg.hbm_budget = int(device), int(slots), int(precision), int(hbm_budget)
        h = C.c_void_p()
        call("ncg_server_new", C.byref(cfg), C.byref(h))
        self._h = h
        self._L = L
        self._dims: list[tuple[int, int]] = []

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.ncg_server_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def add_chain(self, X0: np.ndarray, target_cov: np.ndarray, kind: int = 1, kernel: int = 1, nu: float = 3.0,
                  seed: int = 0, over_smooth: float = 1.0, local_frac: float = 0.05, random_walk_prob: float = 0.0,
                  exploration: int = 0, lb=None, ub=None) -> int:
        X0 = np.ascontiguousarray(X0, dtype=np.float64)
        Lt = np.ascontiguousarray(np.linalg.cholesky(np.asarray(target_cov, dtype=np.float64)))
        n, d = X0.shape
        desc = ncg_chain_desc_t()
        desc.kind, desc.kernel, desc.dim, desc.n = int(kind), int(kernel), int(d), int(n)
        desc.nu, desc.over_smooth, desc.local_frac, desc.seed = float(nu), float(over_smooth), float(local_frac), int(seed)
        desc.X0 = X0.ctypes.data_as(_dp)
        desc.target_L = Lt.ctypes.data_as(_dp)
        desc.random_walk_prob, desc.exploration = float(random_walk_prob), int(exploration)
        bounds = [None if b is None else np.ascontiguousarray(np.broadcast_to(b, (d,)), dtype=np.float64)
                  for b in (lb, ub)]
        desc.lb = bounds[0].ctypes.data_as(_dp) if bounds[0] is not None else None
        desc.ub = bounds[1].ctypes.data_as(_dp) if bounds[1] is not None else None
        cid = C.c_int32()
        call("ncg_server_add_chain", self._h, C.byref(desc), C.byref(cid))
        self._dims.append((n, d))
        return cid.value

    def submit(self, chain: int) -> int:
        rid = C.c_int64()
        call("ncg_server_submit", self._h, int(chain), C.byref(rid))
        return rid.value

    def wait(self, request: int) -> dict:
        out = self.result(request)
        if out["status"] != 0:
            raise NcgError(out["status"], "ncg_server_wait", out["detail"])
        return out

    def result(self, request: int) -> dict:
        """Like wait, but returns a failed step's status instead of raising."""
        r = ncg_step_result_t()
        st = self._L.ncg_server_wait(self._h, int(request), C.byref(r))
        out = {f: getattr(r, f) for f, _ in ncg_step_result_t._fields_}
        out["status"] = int(st)
        out["detail"] = r.detail.decode(errors="replace")
        return out

    def drain(self) -> None:
        call("ncg_server_drain", self._h)

    def stats(self) -> dict:
        s = ncg_server_stats_t()
        call("ncg_server_get_stats", self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in ncg_server_stats_t._fields_}

    def chain_state(self, chain: int) -> tuple[np.ndarray, np.ndarray]:
        n, d = self._dims[chain]
        X = np.empty((n, d))
        m2 = np.empty(n)
        call("ncg_server_get_chain", self._h, int(chain), X.ctypes.data_as(_dp), m2.ctypes.data_as(_dp))
        return X, m2

    def clock(self) -> float:
        return self._L.ncg_server_clock(self._h)

    def checkpoint(self, path: str) -> None:
        """Save every chain's state (the server must be idle)."""
        call("ncg_server_checkpoint", self._h, os.fsencode(path))

    def restore(self, path: str) -> list[int]:
        """Add the chains of a checkpoint; returns their ids."""
        first, count = C.c_int32(-1), C.c_int32(0)
        call("ncg_server_restore", self._h, os.fsencode(path), C.byref(first), C.byref(count))
        ids = list(range(first.value, first.value + count.value))
        for c in ids:
            self._dims.append(self._chain_dims(c))
        return ids

    def chain_info(self, chain: int) -> dict:
        desc, steps = ncg_chain_desc_t(), C.c_uint64()
        call("ncg_server_get_chain_info", self._h, int(chain), C.byref(desc), C.byref(steps))
        out = {f: getattr(desc, f) for f, _ in ncg_chain_desc_t._fields_
               if f not in ("X0", "target_L", "lb", "ub") and not f.startswith("pad")}
        out["steps"] = steps.value
        return out

    def _chain_dims(self, chain: int) -> tuple[int, int]:
        i = self.chain_info(chain)
        return i["n"], i["dim"]


def poisson_arrivals(nchains: int, steps_per_chain: int, rate_hz: float, seed: int) -> list[tuple[float, int]]:
    """(time, chain) for every step: each chain's steps in order, the merged
    stream a Poisson process of `rate_hz` requests per second."""
    rng = np.random.default_rng(seed)
    order = np.repeat(np.arange(nchains), steps_per_chain)
    rng.shuffle(order)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=order.size))
    return list(zip(t.tolist(), order.tolist()))


def run_schedule(server: Server, schedule: list[tuple[float, int]]) -> list[int]:
    """Submit each request at its arrival time (real time) and return the ids."""
    t0 = time.perf_counter()
    ids = []
    for t, c in schedule:
        dt = t - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        ids.append(server.submit(c))
    return ids


__all__ = ["Server", "poisson_arrivals", "run_schedule", "NcgError"]
