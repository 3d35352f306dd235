"""The float upper bound the step kernel uses to skip a cell's CFL speed sum
(key_below in samoa_gb300/csrc/swe_kernel.cuh), restated exactly on the CPU.

The cell update computes ds = RN(RN(z0(RN(leg s0)) + RN(hyp s1)) + RN(leg s2))
and the key RN(ds 2^k); a cell is skipped when a bound, evaluated in float with
every operand and operation rounded up and widened by 2^-20, is below the
warp's largest key. This test restates that bound with exact rational
arithmetic (the round-up of each float operation computed from the exact
result) and checks that it is never below the exact double key, over random
speeds spanning the bound's range, lengths of the mesh's depth tables, and
near-equal and zero speeds. The GPU tests check the kernel's dt against the
oracle; this one checks the mathematics the kernel relies on.
"""
import math
import struct
from fractions import Fraction

import numpy as np


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _f32_from_bits(b):
    return struct.unpack("<f", struct.pack("<I", b & 0xFFFFFFFF))[0]


def float_up(x):
    """float_up of the kernel: None when out of range, else a float32 value
    (as a Fraction) at least |x|, from the bit pattern."""
    a = _bits(x) & 0x7FFFFFFFFFFFFFFF
    if a == 0:
        return Fraction(0)
    e = (a >> 52) - 1023
    if e < -100 or e > 100:
        return None
    fb = (((e + 127) << 23) | ((a >> 29) & 0x7FFFFF)) + 1
    return Fraction(_f32_from_bits(fb))


def round_up_f32(x):
    """The smallest normal float32 >= x (x > 0, within float range), exactly."""
    if x == 0:
        return Fraction(0)
    assert x > 0
    e = math.floor(math.log2(x))
    # fix a possible off-by-one of the floating log2
    while Fraction(2) ** e > x:
        e -= 1
    while Fraction(2) ** (e + 1) <= x:
        e += 1
    ulp = Fraction(2) ** (e - 23)
    q = math.ceil(x / ulp)
    return q * ulp


def dbl_ru_to_f32(x):
    """__double2float_ru for positive normal doubles."""
    return round_up_f32(Fraction(x))


def bound_bits(leg, hyp, s, k):
    """The kernel's bound as the bit pattern of a double, or None (no skip)."""
    f = [float_up(v) for v in s]
    if any(v is None for v in f):
        return None
    lu, hu = dbl_ru_to_f32(leg), dbl_ru_to_f32(hyp)
    t = round_up_f32(lu * f[2])                 # __fmul_ru(up.x, f2)
    t = round_up_f32(hu * f[1] + t)             # __fmaf_ru(up.y, f1, .)
    u = round_up_f32(lu * f[0] + t)             # __fmaf_ru(up.x, f0, .)
    u = round_up_f32(u * (1 + Fraction(1, 2 ** 20)))
    if u == 0:
        return None
    if u >= Fraction(2) ** 128:  # float overflow: the kernel's ef == 255
        return None
    v = float(u * Fraction(2) ** k)  # exact: a float32 value times a power of two
    if math.isinf(v):
        return None
    return _bits(v)


def key_bits(leg, hyp, s, k):
    a = leg * s[0]
    a = 0.0 if a == 0.0 else a  # z0: -0 -> +0
    ds = (a + hyp * s[1]) + leg * s[2]
    return _bits(math.ldexp(ds, k))


def _check(leg, hyp, s, k):
    b = bound_bits(leg, hyp, s, k)
    if b is None:
        return False
    kb = key_bits(leg, hyp, s, k)
    assert kb <= b, (leg, hyp, s, k, kb, b)
    return True


def test_bound_never_below_key_random():
    rng = np.random.default_rng(2026)
    checked = 0
    for _ in range(20000):
        scaling = float(2.0 ** rng.uniform(-10, 30))
        d = int(rng.integers(0, 40))
        leg = scaling * math.sqrt(0.5) ** (d + 1)
        hyp = scaling * math.sqrt(0.5) ** d
        s = [float(2.0 ** rng.uniform(-99, 99)) if rng.random() > 0.1 else 0.0 for _ in range(3)]
        k = d + 1
        checked += _check(leg, hyp, s, k)
    assert checked > 15000


def test_bound_never_below_key_near_ties_and_signed_zeros():
    rng = np.random.default_rng(7)
    for _ in range(5000):
        base = float(rng.uniform(1.0, 300.0))
        s = [np.nextafter(base, np.inf) if rng.random() < 0.5 else base for _ in range(3)]
        s = [float(v) for v in s]
        if rng.random() < 0.2:
            s[int(rng.integers(0, 3))] = -0.0
        leg, hyp = 122.0703125 * 0.70710678118654757, 122.0703125
        assert _check(leg, hyp, s, 27)


def test_out_of_range_speeds_are_not_bounded():
    assert float_up(2.0 ** 101) is None
    assert float_up(2.0 ** -101) is None
    assert float_up(float("inf")) is None
    assert float_up(float("nan")) is None
    assert bound_bits(1.0, 1.0, [2.0 ** 101, 1.0, 1.0], 5) is None


def test_the_check_catches_a_bound_rounded_to_nearest():
    """The same comparison applied to a wrong bound (float round-to-nearest,
    no widening) finds keys above it: the check above has teeth."""
    rng = np.random.default_rng(5)
    bad = 0
    for _ in range(4000):
        base = float(rng.uniform(1.0, 300.0))
        s = [float(base * (1 + rng.uniform(-1e-7, 1e-7))) for _ in range(3)]
        leg, hyp = 0.70710678118654757 * 3.0, 3.0
        f = [Fraction(float(np.float32(v))) for v in s]
        lu, hu = Fraction(float(np.float32(leg))), Fraction(float(np.float32(hyp)))
        u = Fraction(float(np.float32(float(lu * f[0] + hu * f[1] + lu * f[2]))))
        b = _bits(float(u * 2 ** 10))
        bad += key_bits(leg, hyp, s, 10) > b
    assert bad > 0


def test_division_free_cfl_reduction_equals_the_per_cell_minimum():
    """The kernel's CFL reduction: with volume(d) = V 2^-(d+1) exactly (V =
    RN(scaling^2)), min over cells of RN(volume(d) / ds) equals
    RN(V / max over cells of ds 2^(d+1)), since RN(V / x) is monotone in x and
    the power-of-two scalings are exact (volumes and keys normal numbers)."""
    rng = np.random.default_rng(3)
    for _ in range(3000):
        scaling = float(2.0 ** rng.uniform(-5, 25))
        V = scaling * scaling
        n = int(rng.integers(1, 64))
        depths = rng.integers(0, 40, n)
        ds = [float(2.0 ** rng.uniform(-30, 30)) * (1 + float(rng.random())) for _ in range(n)]
        ref = min(math.ldexp(V, -(int(d) + 1)) / x for d, x in zip(depths, ds))
        keys = [math.ldexp(x, int(d) + 1) for d, x in zip(depths, ds)]
        assert V / max(keys) == ref
