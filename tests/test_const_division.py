"""Division by a constant with a precomputed reciprocal (``div_by`` and ``rn_reciprocal`` in
svierosion_gb300/csrc/common.cuh), checked in exact rational arithmetic.

The device routine computes q = RN(x rd), r = RN(x - d q) (exact in one fused multiply-add) and
RN(q + r rd) with rd = RN(1/d); the reinitialisation sweeps use it for every x / h.  Each step
is restated here with round-to-nearest-even on exact rationals, and the result must equal the
correctly rounded quotient RN(x / d) that IEEE division gives.
"""

import random
from fractions import Fraction as F

import numpy as np


def rn32(v: F) -> F:
    """Round an exact rational to the nearest float32 (ties to even); normal range only."""
    if v == 0:
        return F(0)
    sign = -1 if v < 0 else 1
    a = abs(v)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if F(2) ** e > a:
        e -= 1
    if F(2) ** (e + 1) <= a:
        e += 1
    m = a / F(2) ** (e - 23)
    mi = m.numerator // m.denominator
    rem = m - mi
    if rem > F(1, 2) or (rem == F(1, 2) and mi % 2 == 1):
        mi += 1
    return sign * F(mi) * F(2) ** (e - 23)


def rn_reciprocal(d: float) -> F:
    """Host routine: float(1/d) corrected to the neighbour with d*r closest to 1."""
    d32 = np.float32(d)
    r = np.float32(1.0 / float(d32))
    cands = [r, np.nextafter(r, np.float32(0)), np.nextafter(r, np.float32(np.inf))]
    errs = [abs(1.0 - float(d32) * float(c)) for c in cands]
    return F(float(cands[int(np.argmin(errs))]))


def f32(v) -> F:
    return F(float(np.float32(v)))


def test_reciprocal_is_correctly_rounded():
    rng = random.Random(3)
    for _ in range(400):
        d = f32(10 ** rng.uniform(-5, 2))
        assert rn_reciprocal(float(d)) == rn32(1 / d)


def test_div_by_equals_ieee_division():
    rng = random.Random(7)
    divisors = [f32(2.078 / 400), f32(1 / 64), f32(0.05), f32(0.1), f32(1 / 3), f32(2.078 / 256)]
    divisors += [f32(rng.uniform(1e-4, 1.0)) for _ in range(10)]
    divisors.append(F((1 << 24) - 1, 1 << 30))  # all-ones significand
    for d in divisors:
        rd = rn_reciprocal(float(d))
        xs = [f32(rng.choice((-1, 1)) * 10 ** rng.uniform(-8, 1)) for _ in range(800)]
        xs += [F(rng.getrandbits(23) | (1 << 23), 1 << 23) * rng.choice((-1, 1)) for _ in range(200)]
        for x in xs:
            q = rn32(x * rd)
            r = rn32(x - q * d)
            assert rn32(q + r * rd) == rn32(x / d), (x, d)
