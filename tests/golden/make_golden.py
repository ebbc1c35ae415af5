"""Generate the golden fixtures under tests/golden/ (run from the repo root).

Inputs are the seeded workloads of numcosmo_gb300.workloads at reduced sizes;
outputs come from the CPU oracle (oracle/ncg_oracle.c, a restatement of
NumCosmo's FP64 path) and, for the kNN neighbour lists, from NumCosmo's own
kd-tree (numcosmo/external/misc/kdtree.c compiled by `make -C oracle ref`).
The reference's kd-tree exists only where the NumCosmo sources are present,
so its result is stored here for the machines that lack them; so are the
iterates of the reference's vendored levmar (`python tests/golden/make_golden.py
levmar`), which pin the oracle's Levenberg-Marquardt restatement.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from numcosmo_gb300 import workloads as wl  # noqa: E402
from numcosmo_gb300.stats_dist import RNG, StatsDistKernelGauss, StatsDistKernelST  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def _save(name: str, **arrs) -> str:
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrs)
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _dist(kind, kernel, prob, **kw) -> O.OracleStatsDist:
    sd = O.OracleStatsDist(kind, kernel, prob.d, nu=prob.nu or 3.0, **kw)
    sd.set_sample(prob.centres)
    return sd


LM_OPTS = [1e-3, 1e-7, 1e-7, 1e-10, 1e-6]     # the options CV_SPLIT passes (ncm_stats_dist.c:1034-1038)


def levmar_ref() -> str:
    """The reference's own dlevmar_dif (numcosmo/external/levmar compiled by
    `make -C oracle ref`) on one-parameter problems f_i(p) = exp(-a_i e^p) - b_i:
    the fitted p and the iteration count from three starts, for n below and
    above levmar's small-problem size (1024 measurements)."""
    cases = {"opts": np.array(LM_OPTS), "p0": np.array([0.0, 2.0, -1.5])}
    for n in (40, 700, 1500):
        rng = np.random.default_rng(500 + n)
        a = rng.uniform(0.2, 2.0, n)
        b = np.exp(-a * 1.7) + rng.normal(0.0, 1e-3, n)
        f = (lambda a, b: (lambda p: np.exp(-a * np.exp(p)) - b))(a, b)
        res = [O.lm1_reference(f, p0, n, LM_OPTS) for p0 in cases["p0"]]
        assert all(r is not None for r in res), "the reference levmar was not built (NUMCOSMO_SRC)"
        cases[f"a_n{n}"], cases[f"b_n{n}"] = a, b
        cases[f"p_n{n}"] = np.array([r[0] for r in res])
        cases[f"it_n{n}"] = np.array([r[1] for r in res])
    return _save("levmar_ref", **cases)


def config3_full() -> str:
    """Config 3 at full size (Gaussian VKDE d=12, N=4096, 3-component mixture):
    the oracle's weights, rnorm and branch.  The oracle's O(N^3) NNLS takes
    tens of minutes here, so this fixture has its own entry point:
        python tests/golden/make_golden.py config3"""
    p = wl.config3()
    sd = _dist(O.VKDE, O.GAUSS, p)
    assert sd.prepare_interp(p.m2lnp) == 0
    return _save("vkde_gauss_interp_d12_n4096", weights=sd.weights(), rnorm=sd.rnorm, branch=sd.interp_branch,
                 m2lnp=sd.eval_m2lnp(p.points[:512]))


def config4_all() -> str:
    """All 256 uneven problems of config 4 (d 2..32, N 256..16384, KDE/VKDE,
    Gauss/ST(3)): the oracle's -2 ln p at the first 64 of each problem's points.
        python tests/golden/make_golden.py config4"""
    m2, fb = [], []
    for p in wl.config4(256):
        sd = _dist(p.kind, p.kernel, p)
        assert sd.prepare() == 0, p.name
        m2.append(sd.eval_m2lnp(p.points[:64]))
        fb.append(sd.chol_fallbacks)
    return _save("config4_m2lnp_64pts", m2lnp=np.concatenate(m2), chol_fallbacks=np.array(fb, dtype=np.int64))


CONFIG5_CASES = [(d, n) for d in (4, 16, 32) for n in (512, 2048)]


def config5_chain(d: int, n: int):
    """One APES chain of config 5's kind: 2n walkers of a seeded random-SPD
    Gaussian target in d dimensions, started 1.3 sigma wide."""
    rng = np.random.default_rng(5100 + 100 * d + n)
    S = wl.random_spd(d, rng)
    X0 = rng.standard_normal((2 * n, d)) @ np.linalg.cholesky(S).T * 1.3
    return S, X0, 5100 + 100 * d + n


def config5_steps() -> str:
    """One FP64 APES half-move (VKDE Student-t 3 fit of n walkers) for d in
    {4, 16, 32} and n in {512, 2048}, by the CPU restatement of the serving
    step on the oracle.
        python tests/golden/make_golden.py config5"""
    sys.path.insert(0, os.path.dirname(OUT))
    import numcosmo_gb300 as ng
    from serve_restatement import oracle_chain

    out = {}
    for d, n in CONFIG5_CASES:
        S, X0, seed = config5_chain(d, n)
        X, m2 = oracle_chain(ng, O, X0, S, seed, 1, 0.0, 0, np.full(d, -np.inf), np.full(d, np.inf))
        out[f"X_d{d}_n{n}"] = X
        out[f"m2_d{d}_n{n}"] = m2
    return _save("config5_steps", **out)


def main() -> None:
    O.build()
    if O.ref_lib() is None:
        raise SystemExit("reference kd-tree not built (NumCosmo sources missing)")
    manifest = {}

    # config 1 at full size: KDE, Gaussian kernel, d=4, N=M=1000, 1000 draws
    p = wl.config1()
    sd = _dist(O.KDE, O.GAUSS, p)
    assert sd.prepare() == 0
    kern = StatsDistKernelGauss(p.d)
    u, z, cs = RNG(1003).sample_stream(kern, 1000)
    x, idx = sd.sample(u, z)
    manifest["kde_gauss_d4_n1000"] = _save(
        "kde_gauss_d4_n1000", centres=p.centres, points=p.points, m2lnp=sd.eval_m2lnp(p.points),
        p=sd.eval(p.points[:64]), cov=sd.cov(), U=sd.U(), href=sd.href, kernel_lnnorm=sd.kernel_lnnorm,
        u=u, z=z, x=x, idx=idx)

    # config 2 reduced: VKDE, Student-t nu=3, banana, d=16, N=1024, M=256
    p = wl.config2(n=1024, m=256)
    sd = _dist(O.VKDE, O.ST, p)
    assert sd.prepare() == 0
    Y = sd.invUsample()
    knn = sd.knn()
    knn_ref = O.ref_knn(Y, sd.k)
    assert np.array_equal(knn, knn_ref), "oracle kNN differs from the reference kd-tree"
    kern = StatsDistKernelST(p.d, 3.0)
    u, z, cs = RNG(2003).sample_stream(kern, 512)
    x, idx = sd.sample(u, z, cs)
    manifest["vkde_st3_d16_n1024"] = _save(
        "vkde_st3_d16_n1024", centres=p.centres, points=p.points, m2lnp=sd.eval_m2lnp(p.points),
        lnnorms=sd.lnnorms(), knn_ref=knn_ref, U0=sd.Ui(0), U7=sd.Ui(7), href=sd.href,
        u=u, z=z, chisq=cs, x=x, idx=idx)

    # config 3 reduced: Gaussian VKDE prepare_interp, d=12, N=512 (3-component GMM)
    p = wl.config3(n=512, d=12, m=128)
    sd = _dist(O.VKDE, O.GAUSS, p)
    assert sd.prepare_interp(p.m2lnp) == 0
    manifest["vkde_gauss_interp_d12_n512"] = _save(
        "vkde_gauss_interp_d12_n512", centres=p.centres, target=p.m2lnp, points=p.points,
        weights=sd.weights(), rnorm=sd.rnorm, branch=sd.interp_branch, m2lnp=sd.eval_m2lnp(p.points))

    # range-cut branches of prepare_interp on a small KDE (heuristic and refit)
    rng = np.random.default_rng(77)
    X = rng.standard_normal((300, 3))
    m2 = np.sum(X * X, axis=1)
    m2_heur = m2.copy()
    m2_heur[:200] += 400.0          # more than half above the cut: heuristic weights
    m2_cut = m2.copy()
    m2_cut[:40] += 400.0            # a few above the cut: drop them and refit
    res = {}
    for tag, mm in (("heur", m2_heur), ("cut", m2_cut)):
        sd = O.OracleStatsDist(O.KDE, O.ST, 3, nu=4.0)
        sd.set_sample(X)
        assert sd.prepare_interp(mm) == 0
        res[f"{tag}_weights"] = sd.weights()
        res[f"{tag}_branch"] = sd.interp_branch
        res[f"{tag}_n"] = sd.n
        res[f"{tag}_m2lnp"] = sd.eval_m2lnp(X[:50])
    manifest["kde_st4_interp_cut_d3_n300"] = _save("kde_st4_interp_cut_d3_n300", centres=X, m2_heur=m2_heur,
                                                    m2_cut=m2_cut, **res)

    # reference kd-tree neighbour lists in several dimensions, with duplicated points (ties)
    cases = {}
    for d, n, k in ((1, 200, 10), (3, 500, 25), (8, 700, 35), (16, 1200, 60)):
        Y = np.random.default_rng(100 + d).standard_normal((n, d))
        Y[n // 2:n // 2 + 5] = Y[0]
        cases[f"Y_d{d}"] = Y
        cases[f"knn_d{d}"] = O.ref_knn(Y, k)
    manifest["kdtree_ref_knn"] = _save("kdtree_ref_knn", **cases)

    # VKDE neighbour lists with exact ties: duplicated sample points (whole
    # groups of equal distances), the reference kd-tree run on the oracle's
    # whitened sample; the device's lists must equal them bit for bit
    cases = {}
    for d, n in ((2, 400), (5, 600), (16, 1100)):
        rng = np.random.default_rng(300 + d)
        A = rng.standard_normal((d, d)) / np.sqrt(d) + np.eye(d)
        X = rng.standard_normal((n, d)) @ A.T
        X[100:106] = X[7]            # six copies of one point
        X[200:203] = X[300]          # three of another
        X[-4:] = X[5]
        sd = O.OracleStatsDist(O.VKDE, O.GAUSS, d)
        sd.set_sample(X)
        assert sd.prepare() == 0
        Y = sd.invUsample()
        knn_ref = O.ref_knn(Y, sd.k)
        assert np.array_equal(sd.knn(), knn_ref), "oracle kNN differs from the reference kd-tree"
        cases[f"X_d{d}"] = X
        cases[f"knn_d{d}"] = knn_ref
        cases[f"U3_d{d}"] = sd.Ui(3)
    manifest["vkde_knn_ties"] = _save("vkde_knn_ties", **cases)

    with open(os.path.join(OUT, "MANIFEST.json"), "w") as f:
        json.dump({"sha256": manifest,
                   "generator": "tests/golden/make_golden.py",
                   "oracle": "oracle/ncg_oracle.c (CPU restatement of NumCosmo's FP64 path)",
                   "knn_reference": "numcosmo/external/misc/kdtree.c via oracle/_ref"}, f, indent=1, sort_keys=True)
    print(json.dumps(manifest, indent=1))


if __name__ == "__main__":
    extra = {"config3": ("vkde_gauss_interp_d12_n4096", config3_full), "config4": ("config4_m2lnp_64pts", config4_all),
             "config5": ("config5_steps", config5_steps), "levmar": ("levmar_ref", levmar_ref)}
    if sys.argv[1:2] and sys.argv[1] in extra:
        O.build()
        name, fn = extra[sys.argv[1]]
        sha = fn()
        path = os.path.join(OUT, "MANIFEST.json")
        man = json.load(open(path))
        man["sha256"][name] = sha
        with open(path, "w") as f:
            json.dump(man, f, indent=1, sort_keys=True)
        print(sha)
    else:
        main()
