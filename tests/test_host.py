"""Host-side helpers that need no GPU: the seeded arrival schedule of the
serving benchmark and the synthetic workload generators."""
import numpy as np

from numcosmo_gb300 import workloads as wl
from numcosmo_gb300.serve import poisson_arrivals


def test_poisson_arrivals():
    a = poisson_arrivals(64, 3, rate_hz=2.0, seed=11)
    assert a == poisson_arrivals(64, 3, rate_hz=2.0, seed=11)
    assert a != poisson_arrivals(64, 3, rate_hz=2.0, seed=12)
    t = np.array([x for x, _ in a])
    c = np.array([y for _, y in a])
    assert len(a) == 192 and np.all(np.diff(t) > 0)
    assert np.array_equal(np.bincount(c, minlength=64), np.full(64, 3))
    # mean gap of an exponential process of 2/s (192 gaps: a loose 5-sigma band)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 0.5) < 5 * 0.5 / np.sqrt(192)


def test_serving_chains():
    ch = wl.config5_chains(64)
    assert len(ch) == 64
    assert {c["n"] for c in ch} <= {512, 2048, 8192, 16384}
    for c in ch:
        assert 4 <= c["d"] <= 32
        np.linalg.cholesky(c["cov"])           # SPD
    again = wl.config5_chains(64)
    assert all(np.array_equal(x["cov"], y["cov"]) and x["seed"] == y["seed"] for x, y in zip(ch, again))


def test_benchmark_configs_shapes():
    p1 = wl.config1()
    assert p1.centres.shape == (1000, 4) and p1.points.shape == (1000, 4)
    ev = np.linalg.eigvalsh(p1.meta["cov"])
    assert abs(ev.max() / ev.min() - 100.0) < 1e-8
    p3 = wl.config3(512)
    assert p3.centres.shape == (512, 12) and p3.m2lnp.shape == (512,)
    x = wl.banana(2000, 16, 1)
    assert x.shape == (2000, 16) and abs(np.mean(x[:, 1])) < 1.0
