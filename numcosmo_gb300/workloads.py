"""Seeded synthetic workloads for the KDE/VKDE proposal path.

The reference publishes no dataset for this path; these generators give the
shapes and value distributions of the five benchmark configurations:

1. KDE, Gaussian kernel: d=4, N=1000 centres from N(0, Sigma), Sigma a seeded
   random SPD matrix with condition number 100; 1000 evaluation points; 1000 draws.
2. VKDE, Student-t nu=3, local_frac 0.05: d=16, N=M=8192 centres and points from
   a banana law (x1 = 10 z1, x2 = z2 + 0.1 (x1^2 - 100), the rest z).
3. prepare_interp: Gaussian VKDE, d=12, N=4096 centres from a 3-component Gaussian
   mixture (weights 0.5/0.3/0.2, means 3 sigma apart); target -2 ln p exact.
4. 256 independent problems with d in 2..32 and N log-uniform in 256..16384.
5. A stream of APES steps from 64 chains (d in 4..32, N in {512,2048,8192,16384}).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def random_spd(d: int, rng: np.random.Generator, cond: float = 100.0) -> np.ndarray:
    """Q diag(logspace(0, log10 cond, d)) Q^T with Q from the QR of a N(0,1) matrix."""
    Q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    ev = np.logspace(0.0, np.log10(cond), d) if d > 1 else np.array([1.0])
    S = (Q * ev) @ Q.T
    return 0.5 * (S + S.T)


@dataclass
class Problem:
    kind: int            # 0 KDE, 1 VKDE
    kernel: int          # 0 Gauss, 1 Student-t
    d: int
    nu: float
    centres: np.ndarray  # N x d
    points: np.ndarray   # M x d
    m2lnp: np.ndarray | None = None   # target -2 ln p at the centres (prepare_interp)
    local_frac: float = 0.05
    over_smooth: float = 1.0
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.centres.shape[0]

    @property
    def m(self) -> int:
        return self.points.shape[0]

    @property
    def pairs(self) -> int:
        return self.n * self.m


def config1(n: int = 1000, m: int = 1000, d: int = 4) -> Problem:
    S = random_spd(d, np.random.default_rng(1001))
    L = np.linalg.cholesky(S)
    X = np.random.default_rng(1001 + 10_000).standard_normal((n, d)) @ L.T
    P = np.random.default_rng(1002).standard_normal((m, d)) @ L.T
    return Problem(0, 0, d, 0.0, X, P, name=f"kde_gauss_d{d}_n{n}", meta={"cov": S, "sample_seed": 1003})


def banana(n: int, d: int, seed: int) -> np.ndarray:
    z = np.random.default_rng(seed).standard_normal((n, d))
    x = z.copy()
    x[:, 0] = 10.0 * z[:, 0]
    if d > 1:
        x[:, 1] = z[:, 1] + 0.1 * (x[:, 0] ** 2 - 100.0)
    return x


def config2(n: int = 8192, m: int = 8192, d: int = 16) -> Problem:
    return Problem(1, 1, d, 3.0, banana(n, d, 2001), banana(m, d, 2002), name=f"vkde_st3_d{d}_n{n}_banana")


def gmm(d: int, seeds=(3001, 3002, 3003), weights=(0.5, 0.3, 0.2)):
    covs = [random_spd(d, np.random.default_rng(s)) for s in seeds]
    sig = max(float(np.sqrt(np.max(np.diag(c)))) for c in covs)
    means = [np.zeros(d), np.zeros(d), np.zeros(d)]
    means[1][0] = 3.0 * sig
    means[2][min(1, d - 1)] += 3.0 * sig
    return np.array(weights), means, covs


def gmm_sample(n: int, d: int, seed: int = 3004):
    w, mu, covs = gmm(d)
    rng = np.random.default_rng(seed)
    comp = rng.choice(3, size=n, p=w)
    X = np.empty((n, d))
    for k in range(3):
        sel = comp == k
        X[sel] = rng.multivariate_normal(mu[k], covs[k], size=int(sel.sum()))
    return X


def gmm_m2lnp(X: np.ndarray) -> np.ndarray:
    d = X.shape[1]
    w, mu, covs = gmm(d)
    terms = []
    for k in range(3):
        L = np.linalg.cholesky(covs[k])
        y = np.linalg.solve(L, (X - mu[k]).T)
        lndet = 2.0 * np.sum(np.log(np.diag(L)))
        terms.append(np.log(w[k]) - 0.5 * (np.sum(y * y, axis=0) + lndet + d * np.log(2 * np.pi)))
    T = np.array(terms)
    mx = T.max(axis=0)
    return -2.0 * (mx + np.log(np.exp(T - mx).sum(axis=0)))


def config3(n: int = 4096, d: int = 12, m: int | None = None) -> Problem:
    X = gmm_sample(n, d, 3004)
    P = gmm_sample(m or n, d, 3005)
    return Problem(1, 0, d, 0.0, X, P, m2lnp=gmm_m2lnp(X), name=f"vkde_gauss_interp_d{d}_n{n}_gmm3")


def config4(count: int = 256, nmin: int = 256, nmax: int = 16384, dmin: int = 2, dmax: int = 32):
    out = []
    for j in range(count):
        rng = np.random.default_rng(4000 + j)
        d = int(rng.integers(dmin, dmax + 1))
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        n = max(n, 2 * d + 2, int(np.ceil(2.0 / 0.05)) + 1)
        kernel = int(rng.integers(0, 2))
        kind = int(rng.integers(0, 2))
        S = random_spd(d, rng)
        L = np.linalg.cholesky(S)
        X = rng.standard_normal((n, d)) @ L.T
        P = rng.standard_normal((n, d)) @ L.T
        y = np.linalg.solve(L, X.T)
        m2 = np.sum(y * y, axis=0)
        out.append(Problem(kind, kernel, d, 3.0 if kernel else 0.0, X, P, m2lnp=m2,
                           name=f"batch{j}_{'vkde' if kind else 'kde'}_{'st3' if kernel else 'gauss'}_d{d}_n{n}"))
    return out


def config5_chains(count: int = 64, ns=(512, 2048, 8192, 16384)):
    chains = []
    for c in range(count):
        rng = np.random.default_rng(5000 + c)
        d = int(rng.integers(4, 33))
        n = int(ns[int(rng.integers(0, len(ns)))])
        S = random_spd(d, rng)
        chains.append({"chain": c, "d": d, "n": n, "cov": S, "seed": 5000 + c})
    return chains
