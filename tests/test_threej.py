"""Wigner 3j: known-answer tests of the exact oracle evaluator, and the product's C++ table
(gain_threej_table) against it bit for bit."""
import itertools
import math
from fractions import Fraction

import numpy as np
import pytest


def test_closed_forms_j2_equal_1():
    """Edmonds' closed forms for (j 1 j'; m, m2, -m-m2), checked in exact arithmetic."""
    import threej
    for j in range(0, 12):
        for m in range(-j, j + 1):
            # (j 1 j; m 0 -m) = (-1)^(j-m+1) m / sqrt(j (j+1) (2j+1))
            if j > 0:
                ex = (-1) ** (j - m + 1) * m / math.sqrt(j * (j + 1) * (2 * j + 1))
                assert threej.three_j_exact(j, 1, j, m, 0, -m) == pytest.approx(ex, rel=1e-15, abs=1e-300)
            # (j 1 j+1; m 0 -m) = (-1)^(j-m+1) sqrt((j+m+1)(j-m+1) / ((2j+1)(j+1)(2j+3)))
            ex = (-1) ** (j - m + 1) * math.sqrt((j + m + 1) * (j - m + 1) / ((2 * j + 1) * (j + 1) * (2 * j + 3)))
            assert threej.three_j_exact(j, 1, j + 1, m, 0, -m) == pytest.approx(ex, rel=1e-15)


def test_orthogonality_sum_rule():
    """sum_{m1,m2} (2 j3 + 1) (j1 j2 j3; m1 m2 m3)^2 = 1 for every allowed j3, m3."""
    import threej
    for j1 in range(0, 9):
        for j3 in range(max(j1 - 1, 0), j1 + 2):
            if j1 + j3 < 1:
                continue
            for m3 in range(-j3, j3 + 1):
                s = sum((2 * j3 + 1) * threej.three_j_exact(j1, 1, j3, m1, m2, m3) ** 2
                        for m1 in range(-j1, j1 + 1) for m2 in (-1, 0, 1))
                assert s == pytest.approx(1.0, abs=4e-15)


def test_correct_rounding():
    """|3j| is the double nearest the exact value: with x^2 the exact rational square
    (closed form of (j 1 j+1; m 0 -m)), (|v| - ulp/2)^2 < x^2 < (|v| + ulp/2)^2."""
    import threej
    for j in (0, 1, 4, 10, 17, 30):
        for m in range(-j, j + 1, max(1, j // 3)):
            v = abs(threej.three_j_exact(j, 1, j + 1, m, 0, -m))
            x2 = Fraction((j + m + 1) * (j - m + 1), (2 * j + 1) * (j + 1) * (2 * j + 3))
            half = Fraction(float(np.spacing(v))) / 2
            assert (Fraction(v) - half) ** 2 < x2 < (Fraction(v) + half) ** 2


def test_table_layout_and_zeroes():
    import threej
    jmax = 6
    t = threej.threej_table(jmax)
    n = jmax + 1
    for jI, jF, kI, kF in itertools.product(range(n), range(n), range(n), range(n)):
        if abs(jF - jI) > 1 or kI > jI or kF > jF or abs(kF - kI) > 1:
            continue
        idx = jI + kI * n + (jF - jI + 1) * n * n + (kF - kI + 1) * n * n * 3
        assert t[idx] == threej.three_j_exact(jI, 1, jF, kI, kF - kI, -kF)
    # (j 1 j; 0 0 0) vanishes exactly (odd j1 + j2 + j3)
    for j in range(1, n):
        assert t[j + 0 + 1 * n * n + 1 * n * n * 3] == 0.0


def test_library_table_bit_exact(built_lib):
    import gainls
    import threej
    for jmax in (0, 1, 2, 11, 31):
        assert np.array_equal(gainls.threej_table(jmax), threej.threej_table(jmax))
