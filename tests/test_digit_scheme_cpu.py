"""The arithmetic of the FP64-accurate digit products (gcge_gb300/csrc/
ozaki_tc.cu), restated with Python integers and checked exactly:

* the 55-bit fixed point X = |x| 2^(1077 - emax), truncated, formed as the
  kernel does (significand shifted left by 2, then right by
  min(emax - field, 63)), equals floor(|x| 2^(1077 - emax));
* its 7 digits (Y = X + 0x808080808080; d_0 = Y >> 48, d_i = byte 6 - i of Y
  less 128) rebuild X exactly, with d_0 in [0, 128] and d_i in [-128, 127];
* each digit's FP16 encoding (the pattern sign | 0x6400 | field, less
  +-1024 or +-(1024 + 128)) is the digit exactly;
* the level sums of 144 consecutive k stay below 2^24 (exact in FP32);
* the 128-bit integer to FP64 conversion rounds to nearest, ties to even.
"""
from fractions import Fraction
import math
import random
import struct

import numpy as np


def fields(x):
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    return b >> 63, (b >> 52) & 0x7FF, b & ((1 << 52) - 1)


def fixed55(x, emax):
    """The kernel's tc_fixed55 on Python integers: (Y, sign)."""
    s, ef, frac = fields(x)
    mant = frac | ((1 << 52) if ef > 0 else 0)
    r = min(emax - max(ef, 1), 63)
    X = ((mant << 2) & ((1 << 64) - 1)) >> r
    return X + 0x808080808080, s


def digits(Y):
    d = [Y >> 48]
    for i in range(1, 7):
        d.append(((Y >> (8 * (6 - i))) & 0xFF) - 128)
    return d


def test_fixed_point_and_digits_are_exact():
    rng = random.Random(5)
    for _ in range(20000):
        emax = rng.randint(1000, 1100)
        # values up to 2^(emax - 1023) in magnitude, down to far below it
        ef = rng.randint(max(1, emax - 80), emax)
        x = math.ldexp(1.0 + rng.random(), ef - 1023) * rng.choice((-1.0, 1.0))
        if fields(x)[1] > emax:
            continue
        Y, s = fixed55(x, emax)
        X = Y - 0x808080808080
        exact = math.floor(abs(Fraction(x)) * Fraction(2) ** (1077 - emax))
        assert X == exact
        assert 0 <= X < 2 ** 55
        d = digits(Y)
        assert 0 <= d[0] <= 128
        assert all(-128 <= v <= 127 for v in d[1:])
        assert sum(v << (8 * (6 - i)) for i, v in enumerate(d)) == X


def test_zero_subnormal_and_largest_value():
    for x, emax in ((0.0, 1023), (5e-324, 1), (2.5e-310, 1), (-1.7976931348623157e308, 2046),
                    (1.0, 1023), (np.nextafter(2.0, 0.0), 1023)):
        Y, _ = fixed55(x, emax)
        X = Y - 0x808080808080
        assert X == math.floor(abs(Fraction(x)) * Fraction(2) ** (1077 - emax))
        d = digits(Y)
        assert sum(v << (8 * (6 - i)) for i, v in enumerate(d)) == X


def fp16_digit(field, sign, digit0):
    """FP16 value of the kernel's packing: sign | 0x6400 | field, minus
    +-1024 (digit 0) or +-(1024 + 128) (the others)."""
    bits = (0x8000 if sign else 0) | 0x6400 | field
    v = np.frombuffer(np.uint16(bits).tobytes(), dtype=np.float16)[0]
    sub = np.float16(1024.0 if digit0 else 1152.0)
    return float(v - (-sub if sign else sub))


def test_fp16_encoding_is_exact():
    for field in range(0, 257):
        for sign in (0, 1):
            got0 = fp16_digit(field, sign, True)
            assert got0 == (-field if sign else field)
            if field <= 255:
                got = fp16_digit(field, sign, False)
                assert got == (-(field - 128) if sign else field - 128)


def test_level_sums_of_144_k_are_exact_in_fp32():
    # |d_i d'_j| <= 128^2 and at most 7 pairs per level
    worst = 144 * 7 * 128 * 128
    assert worst < 2 ** 24
    # paired levels of the drain stay in 32 bits
    l0, l1 = 144 * 128 * 128, 144 * 2 * 128 * 128
    l2, l3 = 144 * 3 * 128 * 128, 144 * 4 * 128 * 128
    assert l0 * 256 + l1 < 2 ** 31 and l2 * 256 + l3 < 2 ** 31


def i128_to_f64(vh, vl, e):
    """The kernel's tc_i128_f64 on Python integers (vh signed high word, vl
    unsigned low word), returning the double's bit pattern."""
    V = (vh << 64) + vl
    neg = V < 0
    M = -V if neg else V
    if M == 0:
        return 0
    lz = 128 - M.bit_length()
    T = M << lz  # top bit at 127
    th, tl = T >> 64, T & ((1 << 64) - 1)
    mant, rb = th >> 11, th & 0x7FF
    up = rb > 0x400 or (rb == 0x400 and (tl != 0 or (mant & 1)))
    field = 1023 + 127 - lz + e
    if field <= 0:
        bits = 0
    elif field >= 2047:
        bits = 0x7FF << 52
    else:
        bits = ((field - 1) << 52) + mant + (1 if up else 0)
        bits = min(bits, 0x7FF << 52)
    return bits | ((1 << 63) if neg else 0)


def test_int128_to_double_rounds_to_nearest_even():
    rng = random.Random(7)
    for _ in range(20000):
        nb = rng.randint(1, 100)
        V = rng.getrandbits(nb) * rng.choice((-1, 1))
        if rng.random() < 0.1:  # exact ties
            V = ((rng.getrandbits(53) | 1) << 20) + (1 << 19)
        e = rng.randint(-140, 40)
        vh, vl = V >> 64, V & ((1 << 64) - 1)
        got = struct.unpack("<d", struct.pack("<Q", i128_to_f64(vh, vl, e)))[0]
        want = float(Fraction(V) * Fraction(2) ** e)  # correctly rounded
        assert got == want, (V, e, got, want)
