"""CPU: the power-of-five table of the device's Eisel-Lemire conversion
(metada_gb300/csrc/mg_pow5.h) is the generator's exact output, its entries
bracket the powers they stand for, and the conversion steps of mg_io.cu's
eisel_lemire, restated here with Python integers, give float()'s correctly
rounded result on seeded cases (halfway points included)."""
import importlib.util
import struct
from fractions import Fraction
from pathlib import Path

import numpy as np

CSRC = Path(__file__).resolve().parent.parent / "metada_gb300" / "csrc"
_spec = importlib.util.spec_from_file_location("gen_pow5", CSRC / "gen_pow5.py")
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)
M64 = (1 << 64) - 1


def test_header_is_the_generator_output():
    assert (CSRC / "mg_pow5.h").read_text() == gen.render()


def test_entries_bracket_the_powers():
    for q in range(gen.QMIN, gen.QMAX + 1):
        t = gen.entry(q)
        assert (1 << 127) <= t < (1 << 128)
        if q >= 0:  # t = floor(5^q * 2^s) for the s that normalises it
            v = 5 ** q
            s = 128 - v.bit_length()
            x = Fraction(v) * Fraction(2) ** s
            assert t <= x < t + 1
        else:  # t = floor(2^(b + 127) / 5^-q) + 1 > the exact quotient
            v = 5 ** (-q)
            x = Fraction(1 << (v.bit_length() + 127), v)
            assert t - 1 <= x < t


def _el(w, q):
    """mg_io.cu's eisel_lemire in Python integers: bits, or None (host)."""
    if q < gen.QMIN or q > gen.QMAX:
        return None
    lz = 64 - w.bit_length()
    w = (w << lz) & M64
    t = gen.entry(q)
    th, tl = t >> 64, t & M64
    hi, lo = (w * th) >> 64, (w * th) & M64
    if (hi & 0x1FF) == 0x1FF:
        p2 = (w * tl) >> 64
        lo = (lo + p2) & M64
        if p2 > lo:
            hi += 1
    upper = hi >> 63
    shift = upper + 9
    mant = hi >> shift
    power2 = (((217706 * q) >> 16) + 63) + upper - lz + 1023
    if power2 <= 0:
        return None
    if lo <= 1 and -4 <= q <= 23 and (mant & 3) == 1 and ((mant << shift) & M64) == hi:
        mant &= ~1
    mant += mant & 1
    mant >>= 1
    if mant >= (2 << 52):
        mant, power2 = 1 << 52, power2 + 1
    mant &= ~(1 << 52)
    if power2 >= 0x7FF:
        return None
    return (power2 << 52) | mant


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def test_conversion_steps_match_float():
    rng = np.random.default_rng(3)
    checked = 0
    for _ in range(40_000):
        nd = int(rng.integers(1, 20))
        w = int(rng.integers(1, 10 ** min(nd, 18))) * (10 if nd == 19 else 1) + int(rng.integers(0, 10))
        q = int(rng.integers(-330, 300))
        r = _el(w, q)
        if r is not None:
            assert r == _bits(float(f"{w}e{q}")), (w, q)
            checked += 1
    for _ in range(5_000):  # exact midpoints between neighbouring doubles
        e = int(rng.integers(-40, 40))
        m = int(rng.integers(1 << 52, 1 << 53))
        v = Fraction(2 * m + 1) * Fraction(2) ** (e - 1)
        k = v.denominator.bit_length() - 1
        n, q = v.numerator * 5 ** k, -k
        while n % 10 == 0:
            n, q = n // 10, q + 1
        if n < 10 ** 19:
            r = _el(n, q)
            assert r == _bits(float(f"{n}e{q}")), (n, q)
            checked += 1
    assert checked > 35_000
