"""The staged-reciprocal division of the solves (div_staged in csrc/lu.cuh), restated
on the host with exact fused multiply-adds: for divisors whose significand is at most
2 - 2^-48 and exponents within +-900, t = RN(x*yl), q0 = RN(x*yh + t), r = x - d*q0,
q = RN(q0 + r*yh) equals IEEE x / d, including quotients within 2^-50 ulp of a rounding
midpoint.  (The GPU tests run the same cases through the device code.)"""
from fractions import Fraction

import numpy as np


def _fma(a: float, b: float, c: float) -> float:
    return float(Fraction(a) * Fraction(b) + Fraction(c))  # exact, then correctly rounded


def _staged(x: float, d: float) -> float:
    yh = 1.0 / d
    yl = _fma(-d, yh, 1.0) * yh
    q0 = _fma(x, yh, x * yl)
    r = _fma(-d, q0, x)
    return _fma(r, yh, q0)


def _in_range(x: float, d: float) -> bool:
    bx = int(np.float64(x).view(np.uint64))
    bd = int(np.float64(d).view(np.uint64))
    ex, ed = ((bx >> 52) & 0x7FF) - 1023, ((bd >> 52) & 0x7FF) - 1023
    return (-900 <= ex <= 900 and -900 <= ed <= 900 and -900 <= ex - ed <= 900
            and (bd & 0xFFFFFFFFFFFFF) <= 0xFFFFFFFFFFFF0)


def _near_midpoint(rng, count):
    """b/d = M/2^54 - eps/(D*2^54) with M/2^54 halfway between two doubles."""
    out = []
    while len(out) < count:
        D = int(rng.integers(2 ** 52, 2 ** 53)) | 1
        eps = int(rng.choice([-7, -5, -3, -1, 1, 3, 5, 7]))
        M = (eps * pow(D, -1, 2 ** 54)) % 2 ** 54
        B, rem = divmod(M * D - eps, 2 ** 54)
        if rem or not (2 ** 53 <= M < 2 ** 54 and 2 ** 52 <= B < 2 ** 53):
            continue
        e1, e2 = (int(v) for v in rng.integers(-300, 300, 2))
        out.append((float(np.ldexp(float(B), e1)) * (1 if rng.random() < 0.5 else -1), float(np.ldexp(float(D), e2))))
    return out


def test_staged_division_equals_ieee_division():
    rng = np.random.default_rng(5)
    cases = _near_midpoint(rng, 10000)
    cases += [(float(a), float(b)) for a, b in rng.standard_normal((3000, 2))]
    # divisors just below the excluded top significands, and large/small exponents in range
    cases += [(float(rng.standard_normal()), float(np.ldexp(2.0 - k * 2.0 ** -52, int(e))))
              for k, e in zip(range(16, 400), rng.integers(-800, 800, 384))]
    checked = 0
    for x, d in cases:
        if x == 0.0 or not _in_range(x, d):
            continue
        assert _staged(x, d) == x / d, (x.hex(), d.hex())
        checked += 1
    assert checked > 13000
