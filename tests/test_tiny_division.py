"""CPU check of the rounding argument behind the reference-mode division of
tiny numerators (rz_device.cuh: unscale_quotient, DivDH::checked,
div_rn_tiny_scaled).

A numerator a below 2^-96 is divided at 2^64 times its size: qs = RN(a*2^64/b)
and the remainder rs = a*2^64 - qs*b are exact (float32), and the quotient is
taken back as RN(qs*2^-64), except where qs*2^-64 lies exactly halfway between
two subnormals, where the sign of rs picks the side.  Here every float32
operation is evaluated exactly in rational arithmetic and rounded once to
float32 (ties to even, subnormals included), and the result is compared with
the correctly rounded quotient RN(a/b).  The GPU self-test
(test_tiny_numerator_divisions_match_ieee) checks the CUDA code itself against
IEEE division.
"""
from fractions import Fraction as F

import numpy as np

TWO64, TWOM64, TWOM86 = F(2) ** 64, F(1, 2 ** 64), F(1, 2 ** 86)


def rn32(x: F) -> F:
    """x rounded to the nearest float32 (ties to even, with subnormals)."""
    if x == 0:
        return F(0)
    s = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if F(2) ** e > a:
        e -= 1
    q = F(2) ** (max(e, -126) - 23)  # spacing of the binade, or of the subnormals
    n = a / q
    m = n.numerator // n.denominator
    rem = n - m
    if rem > F(1, 2) or (rem == F(1, 2) and m % 2 == 1):
        m += 1
    return s * m * q


def fl(v: float) -> F:
    return F(float(np.float32(v)))


def unscale(qs: F, rs: F) -> F:
    q = rn32(qs * TWOM64)
    mid = abs(rn32(q * TWO64 - qs)) == TWOM86
    qm = rn32(rn32(qs + (TWOM86 if rs > 0 else -TWOM86)) * TWOM64)
    return qm if (mid and rs != 0) else q


def scaled_quotient(a: F, b: F) -> F:
    """The tiny-numerator path: qs correctly rounded at 2^64 scale (as
    Markstein's division by DH gives it after the exhaustive check, and IEEE
    division by lhs), its exact remainder, then unscale."""
    as_ = rn32(a * TWO64)
    assert as_ == a * TWO64  # scaling by 2^64 is exact
    qs = rn32(as_ / b)
    rs = rn32(-qs * b + as_)
    assert rs == as_ - qs * b  # the remainder of a correctly rounded quotient is exact
    return unscale(qs, rs)


def tiny_numerators(rng, n):
    out = []
    for _ in range(n):
        if rng.random() < 0.5:  # subnormal bit pattern
            bits = int(rng.integers(1, 1 << 23))
        else:  # normal, exponent -126 .. -97
            bits = (int(rng.integers(1, 31)) << 23) | int(rng.integers(0, 1 << 23))
        v = np.array([bits], np.uint32).view(np.float32)[0]
        out.append(F(float(-v if rng.random() < 0.5 else v)))
    return out


def test_scaled_division_by_dh_is_correctly_rounded():
    rng = np.random.default_rng(7)
    for dh in (10.0, 12.5, 7.3, 5.0):
        b = fl(dh)
        for a in tiny_numerators(rng, 400):
            assert scaled_quotient(a, b) == rn32(a / b), (dh, a)


def test_scaled_division_by_general_divisors_is_correctly_rounded():
    rng = np.random.default_rng(8)
    for a in tiny_numerators(rng, 1200):
        b = fl(2.0 ** rng.uniform(-29.9, 10.0))
        assert scaled_quotient(a, b) == rn32(a / b), (a, b)


def test_quotients_at_subnormal_midpoints():
    """Numerators whose quotient lies within a hair of a midpoint between two
    subnormals (where rounding qs*2^-64 a second time can go the wrong way),
    including exact midpoints (ties to even)."""
    rng = np.random.default_rng(9)
    hits = 0
    for _ in range(1500):
        b = fl(2.0 ** rng.uniform(-20.0, 6.0))
        k = int(rng.integers(0, 1 << 22))
        m = (2 * k + 1) * F(1, 2 ** 150)  # a midpoint of the subnormal grid
        a = rn32(m * b)  # numerator whose quotient is next to m
        if a == 0 or abs(a) >= F(1, 2 ** 96):
            continue
        want = rn32(a / b)
        got = scaled_quotient(a, b)
        assert got == want, (a, b)
        qs = rn32(a * TWO64 / b)
        if abs(rn32(rn32(qs * TWOM64) * TWO64 - qs)) == TWOM86:
            hits += 1  # qs*2^-64 itself sat on the midpoint
    assert hits > 100
