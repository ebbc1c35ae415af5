"""The APES serving step restated on the CPU (test infrastructure): the fit of
one half by the oracle, the chain's draws from the same MT19937 stream in the
reference's order, the random-walk mixture densities, bounds and the
acceptance test of ncm_fit_esmcmc_walker_apes.c:646-919, written out in
numpy.  Used by tests/test_serve.py and by the fixture generator."""
import numpy as np


def _mix2(m_sd, m_rw, p):
    """-2 ln of (1 - p) q + p rw, combined as the reference combines it."""
    m_rw = m_rw - 2.0 * np.log(p)
    m_sd = m_sd - 2.0 * np.log1p(-p)
    return np.where(m_sd < m_rw, m_sd - 2.0 * np.log1p(np.exp(-0.5 * (m_rw - m_sd))),
                    m_rw - 2.0 * np.log1p(np.exp(-0.5 * (m_sd - m_rw))))


def _log_ngi(zl, zu):
    """ncm_util_log_normal_gaussian_integral, restated with scipy's erf / erfc."""
    from scipy.special import erf, erfc

    ul, uu = np.minimum(zl, zu) / np.sqrt(2.0), np.maximum(zl, zu) / np.sqrt(2.0)
    if ul > 3.0:
        return np.log(abs(0.5 * (erfc(ul) - erfc(uu))))
    if uu < -3.0:
        return np.log(abs(0.5 * (erfc(-ul) - erfc(-uu))))
    if uu > 3.0 and ul < -3.0:
        return np.log1p(-0.5 * (erfc(uu) + erfc(-ul)))
    return np.log(abs(0.5 * (erf(uu) - erf(ul))))


def _m2lnp_rw(frm, to, std, lb, ub):
    m = 0.0
    for i in range(len(std)):
        ln_norm = 0.5 * np.log(2.0 * np.pi) + np.log(std[i]) + _log_ngi((lb[i] - frm[i]) / std[i],
                                                                          (ub[i] - frm[i]) / std[i])
        m += ((to[i] - frm[i]) / std[i]) ** 2 + 2.0 * ln_norm
    return m


def oracle_chain(ng, oracle, X0, cov, seed, steps, p, explore, lb, ub):
    """The serving step restated on the CPU: the fit of one half by the oracle,
    the chain's draws from the same MT19937 stream in the reference's order
    (walker by walker, each redrawn until inside the bounds), the random-walk
    mixture and bounds, the acceptance test."""
    from scipy.linalg import solve_triangular

    L = np.linalg.cholesky(cov)
    target = lambda X: np.sum(solve_triangular(L, X.T, lower=True) ** 2, axis=0)
    X = X0.copy()
    m2 = target(X)
    nw, d = X.shape
    n = nw // 2
    rng = ng.RNG(seed)
    kern = ng.StatsDistKernelST(d, 3.0)
    for step in range(steps):
        h, o = step & 1, 1 - (step & 1)
        Xh, Xo = X[h * n:(h + 1) * n], X[o * n:(o + 1) * n]
        orc = oracle.OracleStatsDist(1, 1, d, nu=3.0)
        orc.set_sample(Xo)
        assert orc.prepare_interp(m2[o * n:(o + 1) * n]) == 0
        std = 0.25 * np.sqrt(np.diag(orc.cov()))
        prop = np.empty((n, d))
        for j in range(n):
            # walker by walker, as _ncm_fit_esmcmc_walker_apes_sample draws
            # (ncm_fit_esmcmc_walker_apes.c:717-737): redrawn until inside
            while True:
                if p > 0.0 and rng.uniform_pos() < p:
                    for i in range(d):
                        while True:
                            x = rng.ugaussian() * std[i] + Xh[j, i]
                            if lb[i] <= x <= ub[i]:
                                break
                        prop[j, i] = x
                    break
                u, z, cs = rng.sample_stream(kern, 1)
                x, _ = orc.sample(u, z, cs)
                if np.all(x[0] >= lb) and np.all(x[0] <= ub):
                    prop[j] = x[0]
                    break
        uacc = np.array([rng.uniform_pos() for _ in range(n)])
        q = orc.eval_m2lnp(np.vstack([prop, Xh]))
        qs, qc = q[:n], q[n:]
        if p > 0.0:
            qs = np.array([_mix2(qs[j], _m2lnp_rw(Xh[j], prop[j], std, lb, ub), p) for j in range(n)])
            qc = np.array([_mix2(qc[j], _m2lnp_rw(prop[j], Xh[j], std, lb, ub), p) for j in range(n)])
        m2s, m2h = target(prop), m2[h * n:(h + 1) * n]
        lnr = -0.5 * (m2s - m2h) if step < explore else -0.5 * (m2s - m2h) + 0.5 * (qs - qc)
        acc = np.log(uacc) < lnr
        Xh[acc] = prop[acc]
        m2h[acc] = m2s[acc]
    return X, m2
