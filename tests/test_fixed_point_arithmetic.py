"""CPU restatement of the fixed-point arithmetic of the FP64 constant-coefficient
stage kernels (hpc-reading-course_gb300/csrc/wave2d_fixed.cuh), checked with exact
rational arithmetic.

fx_from: a double v with biased exponent e <= emax becomes the integer
trunc(v / 2^(emax - 1075)); fx_to: an integer s becomes s * 2^(emax - 1075)
truncated to a double (towards zero). The interior stencil times its
denominator is an integer combination of the converted values, so the only
roundings are the conversions. The checks: round trips are exact at emax, each
conversion errs by less than one unit, and a stencil evaluated this way stays
within the bound those conversions allow, at the reference's FP64 accuracy.
"""
import struct
from fractions import Fraction

import numpy as np
import pytest

DEN = {2: 2, 4: 12, 6: 60}
WEIGHTS = {2: (1,), 4: (8, -1), 6: (45, -9, 1)}  # on (v_k - v_-k), k = 1..R
COEF = {2: [Fraction(-1, 2), 0, Fraction(1, 2)],
        4: [Fraction(1, 12), Fraction(-2, 3), 0, Fraction(2, 3), Fraction(-1, 12)],
        6: [Fraction(-1, 60), Fraction(3, 20), Fraction(-3, 4), 0, Fraction(3, 4), Fraction(-3, 20),
            Fraction(1, 60)]}


def bits(v: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def from_bits(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b & 0xFFFFFFFFFFFFFFFF))[0]


def dexp(v: float) -> int:
    return (bits(v) >> 52) & 0x7FF


def fx_from(v: float, emax: int) -> int:
    b = bits(v)
    e = (b >> 52) & 0x7FF
    m = (b & ((1 << 52) - 1)) | (1 << 52)
    sh = 64 if e == 0 else emax - e
    mag = 0 if sh >= 64 else m >> sh
    return -mag if b >> 63 else mag


def fx_to(s: int, emax: int) -> float:
    """The kernel's bit assembly: eb = emax + 11, exponent eb - lz, 52 fraction bits
    below the leading one, truncated. Valid for emax in [64, 2030] (the tile guard)."""
    assert 64 <= emax <= 2030
    a = -s if s < 0 else s
    if a == 0:
        return 0.0
    lz = 64 - a.bit_length()
    n = (a << lz) & ((1 << 64) - 1)
    mh, ml = n >> 43, (n >> 11) & 0xFFFFFFFF
    hw = ((((emax + 11) - lz - 1) << 20) + mh) & 0xFFFFFFFF
    if s < 0:
        hw |= 0x80000000
    return from_bits((hw << 32) | ml)


def test_round_trip_is_exact_at_the_box_maximum():
    rng = np.random.default_rng(0)
    for v in np.concatenate([rng.standard_normal(2000), rng.standard_normal(200) * 1e-200, [1.0, -1.0, 2.0 ** -958]]):
        v = float(v)
        e = dexp(v)  # >= 64 for all of these: the range the tile guard lets through
        assert fx_to(fx_from(v, e), e) == v


def test_fx_from_truncates_within_one_unit():
    rng = np.random.default_rng(1)
    for _ in range(3000):
        v = float(rng.standard_normal() * 10.0 ** rng.integers(-6, 6))
        emax = dexp(v) + int(rng.integers(0, 70))
        unit = Fraction(2) ** (emax - 1075)
        q = fx_from(v, emax)
        assert abs(Fraction(v) - q * unit) < unit
        assert abs(q * unit) <= abs(Fraction(v))
        assert abs(q) < 2 ** 53


def test_fx_to_truncates_to_the_double_below():
    rng = np.random.default_rng(2)
    for _ in range(3000):
        s = int(rng.integers(-(2 ** 62), 2 ** 62)) >> int(rng.integers(0, 62))
        emax = int(rng.integers(64, 2000))
        exact = Fraction(s) * Fraction(2) ** (emax - 1075)
        got = fx_to(s, emax)
        if s == 0:
            assert got == 0.0
            continue
        assert abs(Fraction(got)) <= abs(exact)
        nxt = np.nextafter(got, np.inf if got > 0 else -np.inf)
        assert abs(Fraction(float(nxt))) > abs(exact)  # the next double away from zero overshoots


def test_special_values():
    assert fx_from(0.0, 1023) == 0 and fx_from(-0.0, 1023) == 0
    assert fx_from(5e-324, 1023) == 0  # subnormals flush
    assert fx_from(1.0, 1023 + 80) == 0  # far below the box maximum
    assert fx_from(-3.0, dexp(-3.0)) == -(3 << 51)


@pytest.mark.parametrize("order", [2, 4, 6])
def test_integer_stencil_matches_exact_sum(order):
    """den * sum c_s v_s evaluated on the converted values and scaled back: its error
    against the exact sum stays within the conversions' truncations (each value to
    under one unit of 2^(emax-1075), the result to under one ulp), for smooth and
    rough lines and for values spanning many binades."""
    R = order // 2
    rng = np.random.default_rng(order)
    for trial in range(1500):
        kind = trial % 3
        x = np.linspace(-1, 1, 2 * R + 1) * rng.uniform(1e-4, 1e-2) + rng.uniform(-1, 1)
        if kind == 0:
            line = np.exp(-x ** 2 / 0.05 ** 2)  # smooth: the sum cancels
        elif kind == 1:
            line = rng.standard_normal(2 * R + 1)  # rough
        else:
            line = rng.standard_normal(2 * R + 1) * 10.0 ** rng.integers(-30, 5, size=2 * R + 1)
        emax = max(dexp(float(v)) for v in line)
        V = [fx_from(float(v), emax) for v in line]
        S = sum(w * (V[R + k + 1] - V[R - k - 1]) for k, w in enumerate(WEIGHTS[order]))
        exact = sum(COEF[order][s] * Fraction(float(line[s])) for s in range(2 * R + 1)) * DEN[order]
        unit = Fraction(2) ** (emax - 1075)
        if emax < 64:  # the tile guard: such boxes convert to zeros
            continue
        got = fx_to(S, emax)  # = den * sum, in true units
        # each converted value errs by under one unit (2 * sum|w| values' worth), the
        # conversion back by under one ulp (2^-52 relative)
        bound = 2 * sum(abs(w) for w in WEIGHTS[order]) * unit + abs(Fraction(got)) * Fraction(1, 2 ** 52)
        assert abs(Fraction(got) - exact) <= bound
        # the sum itself (got / den) within a few ulps of the largest value: the accuracy
        # of the reference's FP64 evaluation, whose partial sums round at 2^-53 of theirs
        vmax = max(abs(Fraction(float(v))) for v in line)
        assert abs(Fraction(got) - exact) / DEN[order] <= 8 * Fraction(2) ** -52 * vmax
