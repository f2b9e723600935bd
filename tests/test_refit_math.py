"""Arithmetic invariants of the VB refit kernel (k_vb_fin), restated on the CPU.

1. The digamma / trigamma asymptotic series (kernel_functions.cuh:1006-1022) are
   evaluated on the device by Horner's rule in r = 1/x; the term-by-term form
   the reference writes agrees with it to rounding.
2. The Gauss-Jordan pivot search runs as a warp reduction over integer keys of
   |entry| (NaN below every number, ties to the lower row, a NaN diagonal entry
   kept); it picks the row the reference's serial "v > best" scan picks.
"""
import numpy as np


def psi_terms(x):
    return (np.log(x) - 1.0 / (2.0 * x) - 1.0 / (12.0 * x**2) + 1.0 / (120.0 * x**4)
            - 1.0 / (252.0 * x**6) + 1.0 / (240.0 * x**8) - 5.0 / (660.0 * x**10)
            + 691.0 / (32760.0 * x**12) - 1.0 / (12.0 * x**14))


def psi1_terms(x):
    return (1.0 / x + 1.0 / (2.0 * x**2) + 1.0 / (6.0 * x**3) - 1.0 / (30.0 * x**5)
            + 1.0 / (42.0 * x**7) - 1.0 / (30.0 * x**9))


def psi_horner(x):
    r = 1.0 / x
    t = r * r
    s = t * (-1.0 / 12.0 + t * (1.0 / 120.0 + t * (-1.0 / 252.0 + t * (
        1.0 / 240.0 + t * (-5.0 / 660.0 + t * (691.0 / 32760.0 + t * (-1.0 / 12.0)))))))
    return np.log(x) - 0.5 * r + s


def psi1_horner(x):
    r = 1.0 / x
    t = r * r
    return r + 0.5 * t + t * r * (1.0 / 6.0 + t * (-1.0 / 30.0 + t * (1.0 / 42.0 + t * (-1.0 / 30.0))))


def test_digamma_series_forms_agree():
    # the Newton iterate's argument n/2 over the range the filter visits
    x = np.logspace(np.log10(0.75), 5, 4000)
    np.testing.assert_allclose(psi_horner(x), psi_terms(x), rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(psi1_horner(x), psi1_terms(x), rtol=1e-13, atol=0)


def pivot_serial(col, k):
    """The reference's scan: best = k, then the first row with a strictly larger |v|."""
    best, bv = k, abs(col[k])
    for r in range(k + 1, len(col)):
        v = abs(col[r])
        if v > bv:
            best, bv = r, v
    return best


def pivot_key(v):
    b = np.float64(v).view(np.int64) & np.int64(0x7FFFFFFFFFFFFFFF)
    return np.int64(-1) if b > np.int64(0x7FF0000000000000) else b


def pivot_warp(col, k):
    """Lane l takes row l (and rows l + 32, ...) at or below k; a butterfly over
    32 lanes keeps the larger key, ties to the lower row; a NaN diagonal stays."""
    pj = len(col)
    key = [np.int64(-2)] * 32
    idx = [k] * 32
    for lane in range(32):
        if k <= lane < pj:
            key[lane], idx[lane] = pivot_key(col[lane]), lane
        for r in range(lane + 32, pj, 32):
            if r < k:
                continue
            kr = pivot_key(col[r])
            if kr > key[lane]:
                key[lane], idx[lane] = kr, r
    o = 16
    while o:
        nk, ni = list(key), list(idx)
        for lane in range(32):
            ko, io = key[lane ^ o], idx[lane ^ o]
            if ko > key[lane] or (ko == key[lane] and io < idx[lane]):
                nk[lane], ni[lane] = ko, io
        key, idx = nk, ni
        o >>= 1
    assert len(set(idx)) == 1
    return k if np.isnan(col[k]) else idx[0]


def test_pivot_key_reduction_matches_serial_scan():
    rng = np.random.default_rng(20261203)
    specials = [0.0, -0.0, np.inf, -np.inf, np.nan, 1e-300, 5e-324]
    for trial in range(3000):
        pj = int(rng.integers(1, 65))
        col = rng.standard_normal(pj)
        if trial % 2:  # ties
            col = np.round(col, 1)
        for _ in range(int(rng.integers(0, 4))):
            col[int(rng.integers(0, pj))] = specials[int(rng.integers(0, len(specials)))]
        k = int(rng.integers(0, pj))
        assert pivot_warp(col, k) == pivot_serial(col, k), (col, k)
