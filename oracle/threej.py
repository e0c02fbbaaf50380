"""ORACLE (test infrastructure only): exact Wigner 3j symbols.

Restates the quantity TroveFortran/fort_func.f90:7-104 (three_j) computes, but evaluates
the Racah formula in exact rational arithmetic and rounds the final square root once,
correctly, to the nearest double.  The reference evaluates the same formula through
log-factorials in floating point, so its values differ from these by a few ulps at most.

Table layout: GpuManager::InitializeAndTransferConstants (BaseClasses/GpuManager.cpp:166-181)
    T[jI + kI (jmax+1) + (jF-jI+1)(jmax+1)^2 + (kF-kI+1) 3 (jmax+1)^2] = 3j(jI 1 jF; kI, kF-kI, -kF)
for |jF-jI| <= 1, 0 <= kI <= jI, max(kI-1,0) <= kF <= min(kI+1, jF); zero elsewhere.

Nothing outside tests/, the smoke check and bench.py's CPU baseline may import this.
"""
from __future__ import annotations

from fractions import Fraction
from math import factorial, isqrt
import numpy as np


def _sqrt_rational_rounded(p: int, q: int) -> float:
    """Nearest double to sqrt(p/q), p >= 0, q > 0 (exact integer decision)."""
    if p == 0:
        return 0.0
    if p >= q << 100:
        raise ValueError("argument out of the range this helper handles")
    # k >= 0 with 2^52 <= floor(sqrt(p/q) 2^k) < 2^53
    k = max(0, (106 - (p.bit_length() - q.bit_length())) // 2)
    while True:
        m0 = isqrt((p << (2 * k)) // q)
        if m0 < (1 << 52):
            k += 1
        elif m0 >= (1 << 53):
            k -= 1
        else:
            break
    # nearest of m0, m0+1: compare p 4^k / q with (m0 + 1/2)^2 (no ties: sqrt of a rational
    # that is not a perfect square is irrational, and a perfect square gives m0 exactly)
    m = m0 + 1 if 4 * (p << (2 * k)) > (2 * m0 + 1) ** 2 * q else m0
    return float(np.ldexp(float(m), -k))


def three_j_exact(j1: int, j2: int, j3: int, m1: int, m2: int, m3: int) -> float:
    """Correctly rounded (j1 j2 j3; m1 m2 m3) for integer arguments."""
    if m1 + m2 + m3 != 0:
        return 0.0
    if j3 > j1 + j2 or j3 < abs(j1 - j2) or min(j1, j2, j3) < 0:
        return 0.0
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    f = factorial
    delta = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))
    pref2 = delta * (f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3))
    s = Fraction(0)
    tmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    tmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    for t in range(tmin, tmax + 1):
        den = (f(t) * f(j3 - j2 + t + m1) * f(j3 - j1 + t - m2) * f(j1 + j2 - j3 - t)
               * f(j1 - t - m1) * f(j2 - t + m2))
        s += Fraction((-1) ** t, den)
    if s == 0:
        return 0.0
    sign = (-1) ** ((j1 - j2 - m3) % 2) * (1 if s > 0 else -1)
    v2 = pref2 * s * s
    return sign * _sqrt_rational_rounded(v2.numerator, v2.denominator)


def threej_table(jmax: int) -> np.ndarray:
    n = jmax + 1
    t = np.zeros(n * n * 9, np.float64)
    for jI in range(0, jmax + 1):
        for jF in range(max(jI - 1, 0), min(jI + 1, jmax) + 1):
            for kI in range(0, jI + 1):
                for kF in range(max(kI - 1, 0), min(kI + 1, jF) + 1):
                    t[jI + kI * n + (jF - jI + 1) * n * n + (kF - kI + 1) * n * n * 3] = \
                        three_j_exact(jI, 1, jF, kI, kF - kI, -kF)
    return t
