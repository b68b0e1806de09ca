"""The double-float arithmetic of FP32CD's fast path, restated in numpy float32.

The fast FP32CD kernels (tristan-ff_gb300/csrc/ffe_physics.cuh: bmag64_df,
df_div and their one-cell forms) carry the B^2 denominators of the current
(src/algorithms/field_solver.F90:111) and of the cleaning (:298-328) as
double-float values hi + lo: the squares exact by the FMA, the sums by
Knuth's TwoSum, the quotient by one Newton step on the reciprocal of hi.
This checks the method itself on the CPU: every float32 operation below is
one correctly rounded numpy float32 operation, and an FMA is the exact
product in float64 (a float32 product has at most 48 significant bits) plus
one float32 rounding.  The GPU path is checked against the oracle by the
FP32CD cases of the GPU parity tests.
"""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    # a * b is exact in float64; its sum with c rounds (if at all) some 29
    # bits below float32's precision, so this is the FMA's result up to rare
    # double-rounding ties
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    t = f32(f32(a - f32(s - bb)) + f32(b - bb))
    return s, t


def bmag64_df(s8, s2a, s2b, t):
    """64 B^2 + t as (hi, lo) from the bare point sums (every term >= 0)."""
    u, w = f32(4 * s2a), f32(4 * s2b)
    p1, p2, p3 = f32(s8 * s8), f32(u * u), f32(w * w)
    e1, e2, e3 = fma(s8, s8, -p1), fma(u, u, -p2), fma(w, w, -p3)
    a, ta = two_sum(p1, p2)
    bm, tb = two_sum(a, p3)
    c, tc = two_sum(bm, t)
    lo = f32(f32(f32(ta + tb) + tc) + f32(f32(e1 + e2) + e3))
    hi = f32(c + lo)
    return hi, f32(lo - f32(hi - c))


def df_div(n, hi, lo):
    r = f32(1) / hi  # the kernels use the hardware estimate; one Newton step follows either way
    q = f32(n * r)
    res = fma(-q, lo, fma(-q, hi, n))
    return fma(res, r, q)


def _samples(rng, k):
    mag = 10.0 ** rng.uniform(-3, 3, size=(k, 3))
    sums = (rng.standard_normal((k, 3)) * mag).astype(np.float32)
    return sums


def test_denominator_carries_48_bits():
    rng = np.random.default_rng(7)
    worst = 0.0
    for s8, s2a, s2b in _samples(rng, 4000):
        t = f32(64e-7)
        hi, lo = bmag64_df(s8, s2a, s2b, t)
        exact = (float(s8) ** 2 + 16 * float(s2a) ** 2 + 16 * float(s2b) ** 2) + float(t)
        got = float(hi) + float(lo)
        worst = max(worst, abs(got - exact) / exact)
        # a float32 sum of the same terms is off by up to a few 2^-24
        assert abs(float(hi) - exact) <= 2.0 ** -22 * exact
    assert worst <= 2.0 ** -44, worst


def test_quotient_within_one_ulp():
    rng = np.random.default_rng(11)
    for s8, s2a, s2b in _samples(rng, 2000):
        n = f32(rng.standard_normal() * 10.0 ** rng.uniform(-2, 2))
        hi, lo = bmag64_df(s8, s2a, s2b, f32(64e-7))
        q = df_div(n, hi, lo)
        exact = float(n) / (float(hi) + float(lo))
        ulp = float(np.spacing(np.abs(f32(exact))))
        assert abs(float(q) - exact) <= ulp, (float(q), exact)


def test_zero_field_keeps_the_tiny_term():
    # B = 0: the current's denominator is 64 TINY alone, held exactly
    hi, lo = bmag64_df(f32(0), f32(0), f32(0), f32(64e-7))
    assert hi == f32(64e-7) and lo == 0
    assert df_div(f32(1), hi, lo) == f32(1) / f32(64e-7)
