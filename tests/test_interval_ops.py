"""The FP32 screen's interval square, square root and quotient (no GPU).

The device computes them branch-free: it selects operands first and runs one
instruction sequence for every sign case.  This test emulates that form and the
per-case form (one branch per sign case) with the same IEEE operations and
requires identical results on random intervals, including zeros, signed zeros,
degenerate intervals and NaN.
"""
import numpy as np

F32 = np.float32
NINF, PINF = F32(-np.inf), F32(np.inf)


def rd(x):
    f = x.astype(F32)
    return np.where(f.astype(np.float64) > x, np.nextafter(f, NINF), f)


def ru(x):
    f = x.astype(F32)
    return np.where(f.astype(np.float64) < x, np.nextafter(f, PINF), f)


def mul_rd(a, b):
    return rd(a.astype(np.float64) * b.astype(np.float64))


def mul_ru(a, b):
    return ru(a.astype(np.float64) * b.astype(np.float64))


def f_dn(x):   # the device's f_dn: toward -inf, 0 -> -2^-149, infinities kept
    return np.where(np.isinf(x), x, np.nextafter(x, NINF))


def f_up(x):
    return np.where(np.isinf(x), x, np.nextafter(x, PINF))


def isqr_cases(lo, hi):
    c1, c2 = lo >= 0, (~(lo >= 0)) & (hi <= 0)
    l = np.where(c1, mul_rd(lo, lo), np.where(c2, mul_rd(hi, hi), F32(0)))
    h = np.where(c1, mul_ru(hi, hi), np.where(c2, mul_ru(lo, lo), np.maximum(mul_ru(lo, lo), mul_ru(hi, hi))))
    return l, h


def isqr_select(lo, hi):
    m = np.where(lo >= 0, lo, np.where(hi <= 0, -hi, F32(0)))
    return mul_rd(m, m), np.maximum(mul_ru(lo, lo), mul_ru(hi, hi))


def isqrt_cases(lo, hi):
    with np.errstate(invalid="ignore"):
        l = np.where(lo > 0, f_dn(np.sqrt(np.where(lo > 0, lo, F32(1)))), F32(0))
        return np.where(l > 0, l, F32(0)), f_up(np.sqrt(hi))


def isqrt_select(lo, hi):
    with np.errstate(invalid="ignore"):
        sl = np.sqrt(np.fmax(lo, F32(0)))
        l = np.where(lo > 0, f_dn(sl), F32(0))
        return np.where(l > 0, l, F32(0)), f_up(np.sqrt(hi))


def idiv_cases(alo, ahi, blo, bhi):
    c1, c2 = alo >= 0, (~(alo >= 0)) & (ahi <= 0)
    with np.errstate(all="ignore"):
        ql = np.where(c1, alo / bhi, np.where(c2, alo / blo, alo / blo))
        qh = np.where(c1, ahi / blo, np.where(c2, ahi / bhi, ahi / blo))
    return f_dn(ql), f_up(qh)


def idiv_select(alo, ahi, blo, bhi):
    with np.errstate(all="ignore"):
        ql = alo / np.where(alo >= 0, bhi, blo)
        qh = ahi / np.where(ahi <= 0, bhi, blo)
    return f_dn(ql), f_up(qh)


def random_intervals(rng, n):
    """Valid intervals (lo <= hi, as outward rounding produces) with special
    endpoints: zeros, signed zeros, degenerate intervals, NaN."""
    a = (rng.normal(0, 1, n) * 10.0 ** rng.integers(-6, 6, n)).astype(F32)
    b = (rng.normal(0, 1, n) * 10.0 ** rng.integers(-6, 6, n)).astype(F32)
    k = rng.integers(0, 8, n)
    a = np.where(k == 0, F32(0), a)
    b = np.where(k == 1, F32(-0.0), b)
    b = np.where(k == 2, a, b)                        # degenerate
    a = np.where(k == 3, F32(np.nan), a)
    lo, hi = np.minimum(a, b), np.maximum(a, b)       # NaN propagates to both
    return lo, hi


def same(x, y):
    return np.array_equal(x.view(np.uint32), y.view(np.uint32)) or \
        np.all((x == y) | (np.isnan(x) & np.isnan(y)) | ((x == 0) & (y == 0)))


def test_select_forms_equal_the_case_forms():
    rng = np.random.default_rng(8)
    lo, hi = random_intervals(rng, 200_000)
    for f_case, f_sel in ((isqr_cases, isqr_select), (isqrt_cases, isqrt_select)):
        a, b = f_case(lo, hi), f_sel(lo, hi)
        assert same(a[0], b[0]) and same(a[1], b[1]), f_case.__name__
    blo = np.abs(rng.normal(0, 1, 200_000)).astype(F32) + F32(1e-3)
    bhi = blo + np.abs(rng.normal(0, 1, 200_000)).astype(F32)
    a, b = idiv_cases(lo, hi, blo, bhi), idiv_select(lo, hi, blo, bhi)
    assert same(a[0], b[0]) and same(a[1], b[1])
