"""The FP32 decision band of the robust covariance's Qn counts, on the CPU.

The device decides each count test fl64(x_b - x_a) <= t (x sorted, b > a)
on FP32 copies y = fl32(x - c) of the values less their median c: with
b = y_a, tf = fl32(t) and e = 2^-19 (|b| + tf) + 2^-100,

    y_b <= (b + tf) - e   ->  true,
    y_b >  (b + tf) + e   ->  false,

and in FP64 otherwise (and for every test of a set with some |x - c| >= 2^100).
This restates that arithmetic in numpy float32 (IEEE single, round to
nearest, as the CUDA float operations; an FMA for e rounds once instead of
twice, which only shrinks its error) and checks that no decided test
contradicts the FP64 comparison, over sets built to sit on the band's edge:
thresholds equal to or one ulp beside exact differences, integer ties,
ulp-spaced values, FP32-subnormal magnitudes, large offsets and magnitudes
up to 2^99 around offsets of 2^120.
"""
import numpy as np

E_REL = np.float32(2.0 ** -19)
E_ABS = np.float32(2.0 ** -100)


def _band(y_a, y_b, tf):
    c = (y_a + tf).astype(np.float32)
    e = (E_REL * (np.abs(y_a) + tf).astype(np.float32) + E_ABS).astype(np.float32)
    lo = (c - e).astype(np.float32)
    hi = (c + e).astype(np.float32)
    return y_b <= lo, y_b > hi


def _sets(rng, mode, m):
    if mode == "scaled":
        return (rng.random(m) - 0.5) * 2.0 ** int(rng.integers(-100, 100))
    if mode == "integers":
        return np.floor((rng.random(m) - 0.3) * 64.0)
    if mode == "tiny":
        x = (rng.random(m) - 0.5) * 1e-40
        x[rng.random(m) < 0.3] = 0.0
        return x
    if mode == "ulp":
        return 1.0 + rng.integers(0, 16, m) * 2.0 ** -52
    if mode == "offset":
        return 1.0e6 + rng.standard_normal(m)
    if mode == "huge":
        return (rng.random(m) - 0.5) * 2.0 ** 99 + 2.0 ** 120
    return np.ldexp(rng.random(m) - 0.5, rng.integers(-150, 150, m))


def test_qn_band_never_contradicts_fp64():
    rng = np.random.default_rng(2024)
    decided = wrong = 0
    for mode in ("scaled", "integers", "tiny", "ulp", "offset", "huge", "exponents"):
        for _ in range(36):
            m = int(rng.integers(8, 300))
            v = np.sort(_sets(rng, mode, m))
            c = v[m >> 1]
            if not (abs(v[0] - c) < 2.0 ** 100 and abs(v[-1] - c) < 2.0 ** 100):
                continue                        # the device takes every test in FP64
            y = (v - c).astype(np.float32)
            # thresholds: exact differences, their neighbours, and uniform ones
            ia = rng.integers(0, m, 64)
            ib = np.minimum(m - 1, ia + rng.integers(0, m, 64))
            dif = v[ib] - v[ia]
            t = np.concatenate([dif, np.nextafter(dif, np.inf), np.maximum(np.nextafter(dif, -np.inf), 0.0),
                                (v[-1] - v[0]) * rng.random(64)])
            t = np.maximum(t, 0.0)
            tf = t.astype(np.float32)
            a, b = np.triu_indices(m, 1)
            for k in range(t.size):
                yes, no = _band(y[a], y[b], tf[k])
                truth = (v[b] - v[a]) <= t[k]
                decided += int(yes.sum() + no.sum())
                wrong += int(np.sum(yes & ~truth) + np.sum(no & truth))
    assert decided > 1_000_000
    assert wrong == 0


def test_qn_band_decides_most_tests_on_gaussian_sets():
    """On Gaussian sets the band leaves well under 1 % of the tests to FP64."""
    rng = np.random.default_rng(7)
    amb = tot = 0
    for _ in range(20):
        v = np.sort(1.5 + rng.standard_normal(409))
        y = (v - v[204]).astype(np.float32)
        a, b = np.triu_indices(409, 1)
        d = v[b] - v[a]
        t = float(np.quantile(d, 0.25))
        yes, no = _band(y[a], y[b], np.float32(t))
        amb += int(np.sum(~yes & ~no))
        tot += d.size
    assert amb / tot < 0.01
