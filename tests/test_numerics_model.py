"""Host models of the device arithmetic behind the grouped scan's FP64 sums and row products
(rf_device.cuh), checked against exact rational arithmetic: the bounds the kernels' parity rests on.

* rf_df_split: a non-negative double -> two floats hi + lo with 0 <= v - (hi + lo) < 2^-46 v, for
  +0 and normal values in [2^-103, 2^91); everything else is refused.
* rf_df_add_same_sign: Knuth's two-sum and Dekker's renormalisation on binary32; sums of
  non-negative addends stay within a few 2^-46 of the exact sum, relative to it.
* rf_mul_1m / rf_mul_1p: fma(-x, y, x) and fma(x, y, x) agree with the twice-rounded x*(1-y),
  x*(1+y) to 2^-52 relative wherever the exponent band admits them.

numpy's float32 scalars round each operation to nearest-even, as the device's __fadd_rn does.
"""
import struct
from fractions import Fraction

import numpy as np

F32 = np.float32


def _words(v: float):
    b = struct.unpack("<Q", struct.pack("<d", v))[0]
    return (b >> 32) & 0xFFFFFFFF, b & 0xFFFFFFFF


def _f32(bits: int) -> np.float32:
    return np.frombuffer(struct.pack("<I", bits & 0xFFFFFFFF), dtype=np.float32)[0]


def df_split(v: float):
    """rf_df_split: (ok, hi, lo), the same integer steps as the device function."""
    h, l = _words(v)
    inrange = ((h - (920 << 20)) & 0xFFFFFFFF) < (194 << 20)
    hw = (h - (896 << 20)) & 0xFFFFFFFF
    hb = ((hw << 3) | (l >> 29)) & 0xFFFFFFFF  # __funnelshift_l(l, hw, 3)
    c = ((hb & 0x7F800000) - (23 << 23)) & 0xFFFFFFFF
    lf = F32(_f32(c + ((l & 0x1FFFFFFF) >> 6)) - _f32(c))
    hi = _f32(hb) if inrange else F32(0)
    lo = lf if inrange else F32(0)
    return inrange or (h | l) == 0, hi, lo


def df_add(ah, al, bh, bl):
    """rf_df_add_same_sign on binary32."""
    s = F32(ah + bh)
    bb = F32(s - ah)
    e = F32(F32(ah - F32(s - bb)) + F32(bh - bb))
    e = F32(e + F32(al + bl))
    nh = F32(s + e)
    nl = F32(e - F32(nh - s))
    return nh, nl


def test_split_bounds_and_range():
    rng = np.random.default_rng(1)
    vals = list(rng.uniform(1.0, 2.0, 4000) * 2.0 ** rng.integers(-103, 91, 4000))
    vals += [2.0 ** -103, np.nextafter(2.0 ** 91, 0), 1.0, np.nextafter(1.0, 2), 3.0, 0.1, 105000.0 - 1e-9]
    for v in vals:
        ok, hi, lo = df_split(float(v))
        assert ok, v
        err = Fraction(float(v)) - Fraction(float(hi)) - Fraction(float(lo))
        assert 0 <= err < Fraction(float(v)) * Fraction(1, 2 ** 46), v
        # hi keeps the leading 24 bits: lo is below hi's last place
        assert abs(float(lo)) < abs(float(hi)) * 2.0 ** -23
    ok, hi, lo = df_split(0.0)
    assert ok and hi == 0 and lo == 0
    for v in [-1.0, -0.0, 5e-324, 2.0 ** -104, 2.0 ** 91, float("inf"), float("nan"), -2.0 ** -103]:
        assert not df_split(v)[0], v


def test_double_float_sums_of_non_negative_addends():
    rng = np.random.default_rng(2)
    for spread, n in [(0, 2000), (7, 2000), (40, 500), (90, 300)]:
        vals = rng.uniform(1.0, 2.0, n) * 2.0 ** rng.integers(-spread // 2 - 1, spread // 2 + 1, n)
        vals[::17] = 0.0
        ah = al = F32(0)
        for v in vals:
            ok, bh, bl = df_split(float(v))
            assert ok
            ah, al = df_add(ah, al, bh, bl)
        exact = sum(Fraction(float(v)) for v in vals)
        got = Fraction(float(ah)) + Fraction(float(al))
        rel = abs(got - exact) / exact
        assert rel < Fraction(1, 10 ** 13), (spread, float(rel))
        # and the slot converts to the double nearest hi + lo within one rounding
        assert abs(Fraction(float(ah) + float(al)) - got) <= got * Fraction(1, 2 ** 53)


def fma_band(x: float, y: float) -> bool:
    hx = _words(x)[0] & 0x7FFFFFFF
    hy = _words(y)[0] & 0x7FFFFFFF
    return ((hx - (523 << 20)) & 0xFFFFFFFF) < (1000 << 20) and hy < (1523 << 20)


def _round(q: Fraction) -> float:
    return float(q)  # Fraction -> float rounds to nearest even


def test_fused_products_agree_inside_the_band():
    rng = np.random.default_rng(3)
    xs = list(rng.uniform(1.0, 2.0, 600) * 2.0 ** rng.integers(-499, 499, 600))
    ys = list(rng.uniform(-4.0, 4.0, 600) * 2.0 ** rng.integers(-60, 8, 600))
    ys += [1.0 - 2.0 ** -52, 1.0 + 2.0 ** -52, -1.0 + 2.0 ** -52, 0.5, 2.0, 1.0, -1.0, 0.0]
    xs += [2.0 ** -500, np.nextafter(2.0 ** 500, 0), 3.0, 7.5, 1e10, 2.0 ** 499, 1.0, 5.0]
    checked = 0
    for x in xs:
        for y in ys[::7]:
            x, y = float(x), float(y)
            if not fma_band(x, y):
                continue
            for sign in (-1, 1):
                fused = _round(Fraction(x) * Fraction(sign) * Fraction(y) + Fraction(x))
                plain = x * (1.0 + sign * y) if sign > 0 else x * (1.0 - y)
                if plain == 0.0 or fused == 0.0:
                    assert plain == 0.0 and fused == 0.0
                    continue
                assert abs(Fraction(fused) - Fraction(plain)) <= abs(Fraction(plain)) * Fraction(1, 2 ** 52), (x, y, sign)
                checked += 1
    assert checked > 5000
    # the band's edges
    assert fma_band(2.0 ** -500, 0.0) and not fma_band(np.nextafter(2.0 ** -500, 0), 0.0)
    assert fma_band(np.nextafter(2.0 ** 500, 0), 1.0) and not fma_band(2.0 ** 500, 1.0)
    assert fma_band(1.0, np.nextafter(2.0 ** 500, 0)) and not fma_band(1.0, 2.0 ** 500)
    for bad in [float("inf"), float("nan"), 5e-324]:
        assert not fma_band(bad, 0.5) and (bad == 5e-324 or not fma_band(1.0, bad))
