"""The serving loop (ncg_server_*): concurrent APES chains.

Each chain's trajectory must be the same whether its steps run alone or
interleaved with other chains' steps on other slots, and whether or not the
memory budget forces the chain out of device memory between steps: the
comparison is exact (np.array_equal), since every kernel on the path has a
fixed reduction order and each chain draws from its own RNG stream.
"""
import numpy as np
import pytest

from serve_restatement import oracle_chain as _oracle_chain

pytestmark = pytest.mark.gpu

# (kind, kernel, d, walkers); each step moves one half with the fit of the other
CHAINS = [(1, 1, 4, 1024), (0, 0, 3, 600), (1, 0, 8, 1400), (1, 1, 12, 2048), (0, 1, 6, 512), (1, 1, 16, 1280)]
STEPS = 4


def _chain_inputs(i, kind, kernel, d, n):
    rng = np.random.default_rng(900 + i)
    A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
    cov = A @ A.T
    X0 = rng.standard_normal((n, d)) @ np.linalg.cholesky(cov).T * 1.3
    return X0, cov


def _add_all(srv, chains=CHAINS):
    ids = []
    for i, (kind, kernel, d, n) in enumerate(chains):
        X0, cov = _chain_inputs(i, kind, kernel, d, n)
        ids.append(srv.add_chain(X0, cov, kind=kind, kernel=kernel, nu=3.0, seed=77 + i))
    return ids


def _final(srv, ids):
    return [srv.chain_state(c) for c in ids]


@pytest.mark.parametrize("precision", [0, 1])
def test_alone_and_in_the_mix(gpu, precision):
    ng = gpu
    mix = ng.Server(slots=4, precision=ng.Precision(precision))
    ids = _add_all(mix)
    reqs = [mix.submit(c) for _ in range(STEPS) for c in ids]
    mix.drain()
    res_mix = [mix.wait(r) for r in reqs]
    st = mix.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert 0.0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    fin_mix = _final(mix, ids)
    mix.close()

    alone = ng.Server(slots=1, precision=ng.Precision(precision))
    ids2 = _add_all(alone)
    res_alone = {}
    for c in ids2:
        rr = [alone.submit(c) for _ in range(STEPS)]
        alone.drain()
        res_alone[c] = [alone.wait(r) for r in rr]
    fin_alone = _final(alone, ids2)
    alone.close()

    for (Xa, ma), (Xb, mb) in zip(fin_mix, fin_alone):
        assert np.array_equal(Xa, Xb) and np.array_equal(ma, mb)
    for r in res_mix:
        b = res_alone[r["chain"]][r["step"]]
        assert r["accepted"] == b["accepted"] and r["state_sum"] == b["state_sum"]
    assert any(r["accepted"] > 0 for r in res_mix)


def test_budget_admission_and_eviction(gpu):
    ng = gpu
    big = ng.Server(slots=2, precision=ng.Precision.MIXED)
    ids = _add_all(big)
    reqs = [big.submit(c) for _ in range(2) for c in ids]
    big.drain()
    peak = big.stats()["peak_reserved_bytes"]
    fin_big = _final(big, ids)
    big.close()

    small = ng.Server(slots=2, precision=ng.Precision.MIXED, hbm_budget=int(peak * 0.8))
    ids2 = _add_all(small)
    reqs = [small.submit(c) for _ in range(2) for c in ids2]
    small.drain()
    st = small.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["evicted"] > 0 and st["peak_reserved_bytes"] <= int(peak * 0.8)
    for (Xa, ma), (Xb, mb) in zip(_final(small, ids2), fin_big):
        assert np.array_equal(Xa, Xb) and np.array_equal(ma, mb)
    small.close()


def test_request_larger_than_budget_fails(gpu):
    ng = gpu
    srv = ng.Server(slots=1, precision=ng.Precision.MIXED, hbm_budget=1 << 20)
    (c,) = _add_all(srv, CHAINS[:1])
    r = srv.result(srv.submit(c))
    assert r["status"] == 9    # NCG_ERR_OUT_OF_MEMORY
    assert srv.stats()["failed"] == 1
    srv.close()


def test_poisson_schedule(gpu):
    ng = gpu
    srv = ng.Server(slots=3, precision=ng.Precision.MIXED)
    ids = _add_all(srv)
    sched = ng.poisson_arrivals(len(ids), 2, rate_hz=200.0, seed=5)
    reqs = ng.run_schedule(srv, [(t, ids[c]) for t, c in sched])
    srv.drain()
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["pairs"] == sum(3 * (CHAINS[c][3] // 2) ** 2 for _, c in sched)
    srv.close()


def test_checkpoint_resume(gpu, tmp_path):
    """Two steps, checkpoint, a fresh server, restore, two more steps: the same
    trajectories as four steps in one server; a damaged file is refused."""
    ng = gpu
    chains = CHAINS[:3]

    a = ng.Server(slots=2, precision=ng.Precision.MIXED)
    ids = _add_all(a, chains)
    for _ in range(4):
        for c in ids:
            a.submit(c)
    a.drain()
    fin_a = _final(a, ids)
    a.close()

    b = ng.Server(slots=2, precision=ng.Precision.MIXED)
    ids_b = _add_all(b, chains)
    for _ in range(2):
        for c in ids_b:
            b.submit(c)
    b.drain()
    path = str(tmp_path / "chains.ckpt")
    b.checkpoint(path)
    b.close()

    c = ng.Server(slots=3, precision=ng.Precision.MIXED)
    ids_c = c.restore(path)
    assert len(ids_c) == len(chains)
    assert [c.chain_info(i)["steps"] for i in ids_c] == [2] * len(chains)
    assert [c.chain_info(i)["dim"] for i in ids_c] == [ch[2] for ch in chains]
    for _ in range(2):
        for i in ids_c:
            c.submit(i)
    c.drain()
    for (Xa, ma), (Xc, mc) in zip(fin_a, _final(c, ids_c)):
        assert np.array_equal(Xa, Xc) and np.array_equal(ma, mc)

    raw = bytearray(open(path, "rb").read())
    raw[200] ^= 0x01
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(ng.NcgError):
        c.restore(bad)
    open(bad, "wb").write(bytes(raw[: len(raw) // 2]))
    with pytest.raises(ng.NcgError):
        c.restore(bad)
    c.close()


def _gauss_chain(seed, n, d, cov, scale=1.5):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, d)) @ np.linalg.cholesky(cov).T * scale


def test_walker_options_alone_and_in_the_mix(gpu):
    """Random-walk mixture, bounds and exploration: every walker stays inside
    its bounds, and each trajectory is the same alone and interleaved."""
    ng = gpu
    specs = []
    for i, (kind, kernel, d, n) in enumerate(CHAINS[:4]):
        cov = np.eye(d) * (1.0 + 0.1 * i)
        X0 = np.abs(_gauss_chain(40 + i, n, d, cov)) * 0.5 + 0.1
        lb = np.zeros(d)
        ub = np.full(d, np.inf)
        ub[0] = 2.0
        X0[:, 0] = np.minimum(X0[:, 0], 1.9)
        specs.append(dict(X0=X0, target_cov=cov, kind=kind, kernel=kernel, nu=3.0, seed=500 + i,
                          random_walk_prob=0.25 if i % 2 == 0 else 0.0, exploration=2 if i < 2 else 0,
                          lb=lb, ub=ub))

    def run(slots, one_by_one):
        srv = ng.Server(slots=slots, precision=ng.Precision.MIXED)
        ids = [srv.add_chain(**sp) for sp in specs]
        if one_by_one:
            for c in ids:
                for _ in range(STEPS):
                    srv.submit(c)
                srv.drain()
        else:
            for _ in range(STEPS):
                for c in ids:
                    srv.submit(c)
            srv.drain()
        assert srv.stats()["failed"] == 0
        out = _final(srv, ids)
        srv.close()
        return out

    mix, alone = run(4, False), run(1, True)
    for sp, (Xa, ma), (Xb, mb) in zip(specs, mix, alone):
        assert np.array_equal(Xa, Xb) and np.array_equal(ma, mb)
        assert np.all(Xa >= sp["lb"]) and np.all(Xa <= sp["ub"])
        assert not np.array_equal(Xa, sp["X0"])


@pytest.mark.parametrize("rw", [0.0, 0.4])
def test_mixture_chain_reaches_the_target(gpu, rw):
    """With the random-walk mixture on or off, 2000 walkers started 1.5x too
    wide and shifted settle on the Gaussian target: mean within 0.1 sigma,
    covariance within 15 %; a bounded coordinate settles on the truncated
    normal's mean."""
    ng = gpu
    d, n = 3, 2000
    cov = np.diag([1.0, 2.0, 0.5])
    X0 = _gauss_chain(7, n, d, cov) + 0.5
    lb = np.array([-np.inf, -np.inf, -0.5])
    X0[:, 2] = np.abs(X0[:, 2])
    srv = ng.Server(slots=1, precision=ng.Precision.MIXED)
    c = srv.add_chain(X0, cov, kind=1, kernel=1, nu=3.0, seed=99, random_walk_prob=rw, lb=lb)
    for _ in range(40):
        srv.submit(c)
    srv.drain()
    X, _ = srv.chain_state(c)
    srv.close()
    sd = np.sqrt(np.diag(cov))
    assert np.all(np.abs(X[:, :2].mean(axis=0)) < 0.1 * sd[:2])
    C = np.cov(X[:, :2].T)
    assert np.all(np.abs(np.diag(C) / np.diag(cov)[:2] - 1.0) < 0.15)
    from math import erf, exp, pi, sqrt
    a = -0.5 / sd[2]
    want = sd[2] * exp(-0.5 * a * a) / sqrt(2 * pi) / (0.5 * (1.0 - erf(a / sqrt(2))))
    assert np.all(X[:, 2] >= -0.5)
    assert abs(X[:, 2].mean() - want) < 0.1 * sd[2]


@pytest.mark.parametrize("p,explore,bounded", [(0.0, 0, False), (0.0, 0, True), (0.3, 1, True)])
def test_step_matches_the_oracle(gpu, oracle, p, explore, bounded):
    """FP64 serving steps against their CPU restatement with the oracle's fit,
    sampling and eval on the same draws: walkers and -2 ln L to 1e-9."""
    ng = gpu
    d, nw, seed, steps = 3, 400, 4242, 3
    rng = np.random.default_rng(17)
    cov = np.array([[1.0, 0.3, 0.0], [0.3, 2.0, 0.2], [0.0, 0.2, 0.5]])
    lb = np.array([-np.inf, -np.inf, -0.4]) if bounded else np.full(d, -np.inf)
    ub = np.array([np.inf, 2.5, np.inf]) if bounded else np.full(d, np.inf)
    X0 = rng.standard_normal((4 * nw, d)) @ np.linalg.cholesky(cov).T * 1.3
    X0 = X0[np.all((X0 > lb) & (X0 < ub), axis=1)][:nw]     # walkers inside the bounds
    srv = ng.Server(slots=1, precision=ng.Precision.FP64)
    c = srv.add_chain(X0, cov, kind=1, kernel=1, nu=3.0, seed=seed, random_walk_prob=p, exploration=explore,
                      lb=lb if bounded else None, ub=ub if bounded else None)
    for _ in range(steps):
        srv.submit(c)
    srv.drain()
    assert srv.stats()["failed"] == 0
    Xg, mg = srv.chain_state(c)
    srv.close()
    Xo, mo = _oracle_chain(ng, oracle, X0, cov, seed, steps, p, explore, lb, ub)
    assert not np.array_equal(Xo, X0)
    assert np.max(np.abs(Xg - Xo)) <= 1e-9 * max(1.0, np.max(np.abs(Xo)))
    assert np.max(np.abs(mg - mo)) <= 1e-9 * max(1.0, np.max(np.abs(mo)))
