"""CPU model of mul_round_f32 (csrc/xc_device.cuh): float(E * W) as
__double2float_rn(__dmul_rn((double)E, W)) gives it, formed in FP32 from
FMA-exact products with an FP64 fallback near rounding boundaries.  The
kernels use it for the per-window channel values float(E * (w - mean))
(CrossCorr.cc:123).  Every FP32 operation is restated with exact rationals
and round-to-nearest-even, and the result is held to the exact double-then-
float rounding, on random weights and means and on products placed next to
float rounding boundaries."""
import math
import random
import struct
from fractions import Fraction as Fr


def rn(x, p):
    """x rounded to p significant bits, nearest-even (normal range)."""
    if x == 0:
        return Fr(0)
    s = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while Fr(2) ** e > a:
        e -= 1
    while Fr(2) ** (e + 1) <= a:
        e += 1
    q = a / Fr(2) ** (e - p + 1)
    n = q.numerator // q.denominator
    rem = q - n
    if rem > Fr(1, 2) or (rem == Fr(1, 2) and n % 2 == 1):
        n += 1
    return s * n * Fr(2) ** (e - p + 1)


def f32(x):
    return rn(x, 24)


def f64(x):
    return rn(x, 53)


def exponent(a):
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while Fr(2) ** e > a:
        e -= 1
    while Fr(2) ** (e + 1) <= a:
        e += 1
    return e


def mul_round_f32(E, W):
    """Returns (value, took_fp64)."""
    h = f32(W)
    d = W - h
    l = f32(d)
    r = d - l
    assert f32(r) == r
    p1 = f32(E * h)
    if p1 == 0:
        return p1, False
    e1 = f32(E * h - p1)   # fma
    p2 = f32(E * l)
    e2 = f32(E * l - p2)
    p3 = f32(E * r)
    t = f32(f32(e1 + p2) + f32(e2 + p3))
    f = f32(p1 + t)
    res = f32((p1 - f) + t)
    e = exponent(abs(f))
    ulp = Fr(2) ** (e - 23)
    if abs(f) == Fr(2) ** e or abs(res) >= f32(ulp * f32(Fr(49998, 100000))):
        return f32(f64(E * W)), True
    return f, False


def as_f32(x):
    return Fr(struct.unpack("f", struct.pack("f", x))[0])


def test_random_weights_and_means():
    rng = random.Random(5)
    for it in range(6000):
        E = as_f32(rng.uniform(0, 2)) if it % 7 else as_f32(rng.choice([0.0, 1.0, 2.0, 1.5]))
        ln = rng.randint(1, 16384)
        cnt = rng.randint(0, 4 * ln)
        mean = f64(Fr(cnt, 4) / ln)   # __ddiv_rn((double)cnt * 0.25, len)
        for base in (0, 1):
            W = f64(base - mean)
            got, _ = mul_round_f32(E, W)
            assert got == f32(f64(E * W)), (E, W)


def test_products_next_to_rounding_boundaries():
    rng = random.Random(6)
    fallbacks = 0
    for it in range(3000):
        E = as_f32(rng.uniform(0.01, 2))
        f = as_f32(rng.uniform(0.01, 1.0))
        m = f + Fr(2) ** (exponent(f) - 24) * rng.choice([1, -1])   # a midpoint between floats
        W = f64(m / E + Fr(rng.randint(-50, 50), 2 ** 60))
        got, fb = mul_round_f32(E, W)
        assert got == f32(f64(E * W)), (E, W)
        fallbacks += fb
    assert fallbacks == 3000   # every one of them within the band takes FP64


def test_mean_terms_power_of_two_lengths():
    """mean_terms (xc_device.cuh): for a power-of-two length and a whole
    count, FP32 gives count / len and (len - count) / len with the bits of
    the FP64 division and subtractions, and split3 of those is (value, 0, 0)."""
    for k in range(0, 15):
        ln = 1 << k
        for count in sorted({0, 1, ln // 3, ln // 2, ln - 1, ln} | set(range(0, ln + 1, max(1, ln // 64)))):
            mean = f64(Fr(4 * count, 4) / ln)              # __ddiv_rn((double)cnt4 * 0.25, len)
            for base, fast in ((0, f32(Fr(0) - f32(Fr(count, ln)))), (1, f32(Fr(ln - count, ln)))):
                W = f64(base - mean)                          # __dsub_rn(base, mean)
                assert fast == W                              # FP32 result, exact
                h = f32(W)
                assert h == W and f64(W - h) == 0            # split3: (h, 0, 0)
