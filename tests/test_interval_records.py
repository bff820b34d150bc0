"""The screened path's per-atom interval records (no GPU).

In lazy mode a candidate's position interval comes from a record of
outward-rounded FP32 bounds (x, v, tloc - T0) and the bounds of now - T0:
P = [x] + [v] * ([now - T0] - [tloc - T0]) in outward-rounded FP32.  The claim is
that P contains the FP64 position the exact path computes, x + v * fl(now - tloc).
This test replays the device's operation sequence (shadow_word, shadow_now,
atom_piv) with exact emulation of its directed roundings and checks the claim on
random states, including epochs T0 after an atom's local time.

Emulation is exact.  A product of two floats is exact in FP64.  A sum of two
floats is s + e in FP64 with Knuth's TwoSum error term e.  Rounding down or up
to FP32 takes the nearest float, steps one ulp where it lies on the wrong side
of s, and steps once more when it equals s and e points past it.
"""
import numpy as np

F32 = np.float32


def rd(x):
    f = x.astype(F32)
    return np.where(f.astype(np.float64) > x, np.nextafter(f, F32(-np.inf)), f)


def ru(x):
    f = x.astype(F32)
    return np.where(f.astype(np.float64) < x, np.nextafter(f, F32(np.inf)), f)


def f_dn(f):
    return np.nextafter(f, F32(-np.inf))


def f_up(f):
    return np.nextafter(f, F32(np.inf))


def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def add_rd(a, b):
    s, e = two_sum(a.astype(np.float64), b.astype(np.float64))
    f = rd(s)
    return np.where((f.astype(np.float64) == s) & (e < 0), np.nextafter(f, F32(-np.inf)), f)


def add_ru(a, b):
    s, e = two_sum(a.astype(np.float64), b.astype(np.float64))
    f = ru(s)
    return np.where((f.astype(np.float64) == s) & (e > 0), np.nextafter(f, F32(np.inf)), f)


def sub_rd(a, b):
    return add_rd(a, -b)


def sub_ru(a, b):
    return add_ru(a, -b)


def imul(alo, ahi, blo, bhi):
    p = [x.astype(np.float64) * y.astype(np.float64) for x in (alo, ahi) for y in (blo, bhi)]
    lo = np.minimum.reduce([rd(q) for q in p])
    hi = np.maximum.reduce([ru(q) for q in p])
    return lo, hi


def record_interval(x, v, tloc, T0, now):
    xl, xh = rd(x), ru(x)                                       # shadow_word, words 0-2
    vl, vh = rd(v), ru(v)
    d = tloc - T0                                               # shadow_word, word 3
    tl, th = f_dn(rd(d)), f_up(ru(d))
    dn = now - T0                                               # shadow_now
    nl, nh = f_dn(rd(dn)), f_up(ru(dn))
    dtl, dth = sub_rd(nl, th), sub_ru(nh, tl)                   # atom_piv: isub
    ml, mh = imul(vl, vh, dtl, dth)
    return add_rd(xl, ml), add_ru(xh, mh)                       # iadd


def test_records_contain_the_fp64_position():
    rng = np.random.default_rng(2026)
    n = 400_000
    for scale_t in (1e-3, 1.0, 1e2, 1e4):
        x = rng.uniform(-5.0, 450.0, n)
        v = rng.normal(0.0, 3.0, n)
        T0 = rng.uniform(0.0, scale_t, n)
        tloc = T0 + rng.uniform(-0.5, 0.5, n) * scale_t * 0.1   # before or after the epoch
        now = np.maximum(tloc, T0) + rng.exponential(0.05 * scale_t + 1e-6, n)
        exact = x + v * (now - tloc)                              # the FP64 path (round to nearest)
        lo, hi = record_interval(x, v, tloc, T0, now)
        inside = (lo.astype(np.float64) <= exact) & (exact <= hi.astype(np.float64))
        assert inside.all(), (scale_t, np.nonzero(~inside)[0][:5])
        # and the bounds stay tight: a few float ulps of the larger operand
        width = hi.astype(np.float64) - lo.astype(np.float64)
        assert np.median(width / (np.abs(x) + np.abs(v) * (now - np.minimum(tloc, T0)) + 1e-30)) < 1e-5


def test_emulated_sums_round_in_the_right_direction():
    rng = np.random.default_rng(3)
    a = (rng.normal(0, 1, 50_000) * 10.0 ** rng.integers(-8, 4, 50_000)).astype(F32)
    b = (rng.normal(0, 1, 50_000) * 10.0 ** rng.integers(-8, 4, 50_000)).astype(F32)
    from fractions import Fraction
    lo, hi = add_rd(a, b), add_ru(a, b)
    for k in range(0, 50_000, 97):   # exact rational check on a sample
        s = Fraction(float(a[k])) + Fraction(float(b[k]))
        assert Fraction(float(lo[k])) <= s <= Fraction(float(hi[k]))
        assert float(np.nextafter(lo[k], F32(np.inf))) > s or float(lo[k]) == s
        assert float(np.nextafter(hi[k], F32(-np.inf))) < s or float(hi[k]) == s


def test_emulated_directed_rounding_brackets_the_value():
    rng = np.random.default_rng(1)
    x = rng.normal(0, 100, 100_000) * 10.0 ** rng.integers(-6, 6, 100_000)
    lo, hi = rd(x), ru(x)
    assert (lo.astype(np.float64) <= x).all() and (x <= hi.astype(np.float64)).all()
    assert (hi.astype(np.float64) - lo.astype(np.float64) <= np.abs(x) * 2 ** -22).all()


def fma_ru(a, b, c):
    """fmaf(a, b, c) rounded up, for floats: a*b is exact in FP64, then the sum."""
    p = a.astype(np.float64) * b.astype(np.float64)
    s, e = two_sum(p, c.astype(np.float64))
    f = ru(s)
    return np.where((f.astype(np.float64) == s) & (e > 0), np.nextafter(f, F32(np.inf)), f)


def mul_ru(a, b):
    return ru(a.astype(np.float64) * b.astype(np.float64))


def eager_margin(m, xmax32, nhi, T0f, v_lo, v_hi):
    """The device's per-axis widening in eager mode (loop_body, atom_piv): with
    c = m 2^-51, mx = c max|x| + c (now - T0 + T0) |v|, all rounded up."""
    c = mul_ru(m.astype(F32), np.full_like(m, 2.0 ** -51, dtype=F32))
    mxa = mul_ru(c, np.full_like(c, xmax32))
    mxb = mul_ru(c, add_ru(nhi, T0f))
    vm = np.maximum(np.abs(v_lo), np.abs(v_hi))
    return fma_ru(mxb, vm, mxa)


def test_eager_records_contain_the_stepwise_position():
    """Eager mode: the record holds x(tr), v and tr - T0, where tr is the clock
    value of the pop that wrote it.  The reference then advances x += v dt_k at
    every pop and its clock t += dt_k, each step rounded.  The record's interval,
    widened by the rounding margin of the m pops since tr, must contain that
    step-by-step position."""
    rng = np.random.default_rng(77)
    n = 20_000
    box = 440.0
    xmax32 = ru(np.array([4.0 * box]))[0]
    for m_steps, dt_scale, t0_scale in ((1, 1e-3, 1.0), (40, 1e-4, 1e3), (400, 1e-5, 10.0), (2000, 1e-6, 1e4)):
        x = rng.uniform(-1.0, box + 1.0, n)
        v = rng.normal(0.0, 2.0, n) * 10.0 ** rng.integers(-3, 1, n)
        T0 = rng.uniform(0.0, t0_scale, n)
        t = T0 + rng.uniform(0.0, 1.0, n) * dt_scale * m_steps   # the clock when the record was written
        tr = t.copy()
        xs = x.copy()
        for _ in range(m_steps):                                 # UpdateData / the clock, step by step
            dt = rng.exponential(dt_scale, n)
            xs = xs + v * dt
            t = t + dt
        lo, hi = record_interval(x, v, tr, T0, t)                # tr plays tloc's part
        dn = t - T0
        nhi = f_up(ru(dn))
        T0f = ru(T0)
        vl, vh = rd(v), ru(v)
        mx = eager_margin(np.full(n, m_steps, np.float64), xmax32, nhi, T0f, vl, vh)
        lo, hi = sub_rd(lo, mx), add_ru(hi, mx)
        inside = (lo.astype(np.float64) <= xs) & (xs <= hi.astype(np.float64))
        assert inside.all(), (m_steps, np.nonzero(~inside)[0][:5])
        # the margin stays far below the float resolution of the position
        assert np.median(mx.astype(np.float64) / (np.abs(x) + 1.0)) < 1e-9 * max(m_steps, 1)
