"""CPU checks of the FP64-accurate block product's integer arithmetic (tests/oz_model.py): the
digit split, the bounds that keep the kernel's FP32 accumulators exact and its float-to-integer
conversions in range, and the error bound of an output against the exact dot product."""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from tests import oz_model as M


def test_digits_reconstruct_and_stay_in_range():
    rng = np.random.default_rng(3)
    cases = [0, 1, -1, 2 ** 55, -(2 ** 55), 2 ** 55 - 1, 2 ** 54, -(2 ** 54), 0x7F7F7F7F7F7F, -0x808080808080]
    cases += [int(v) for v in rng.integers(-(2 ** 55), 2 ** 55, size=3000, dtype=np.int64)]
    for X in cases:
        d = M.digits(X)
        assert sum(v * 256 ** (6 - s) for s, v in enumerate(d)) == X
        assert -128 <= d[0] <= 128 and all(-128 <= v <= 127 for v in d[1:])
        if abs(X) <= 2 ** 54:
            assert -64 <= d[0] <= 64


def test_level_bounds_keep_accumulators_exact():
    """With |a_0| <= 128, |b_0| <= 64 and every other digit in [-128, 127], over K = 64 terms:
    |I_L| < 2^22 for L <= 3 (magic-number conversion), < 2^23 for L = 4 (exact in FP32), and the
    level 5..6 part scaled by 2^36 stays below 2^22."""
    amax = [128] + [128] * 6
    bmax = [64] + [128] * 6
    bound = [64 * sum(amax[s] * bmax[L - s] for s in range(7) if 0 <= L - s < 7) for L in range(13)]
    assert all(bound[L] < 2 ** 22 for L in range(4))
    assert bound[4] < 2 ** 23
    assert bound[5] / 16 + bound[6] / 4096 < 2 ** 22
    # the dropped levels cost at most this many units of R
    dropped = sum(Fraction(bound[L], 2 ** (8 * L - 36)) for L in range(7, 13))
    assert dropped < 6.1


def _bound_units(xs, us):
    X, EE = M.encode_column(xs)
    Y, F = M.encode_output_column(us)
    unit = Fraction(2) ** (EE + F - 1071)
    return X, Y, EE, F, unit


def test_outputs_within_documented_error_bound():
    rng = np.random.default_rng(11)
    q, _ = np.linalg.qr(rng.normal(size=(64, 64)))
    worst = 0.0
    for trial in range(60):
        xs = rng.normal(size=64) * 10.0 ** rng.uniform(-20, 0, size=64)
        if trial % 5 == 0:
            xs[rng.integers(64, size=8)] = 0.0
        if trial % 7 == 0:
            xs = np.where(rng.random(64) < 0.5, -1.0, 0.5)  # powers of two: top digits at the limit
        us = q[trial % 64] * (2.0 ** -30 if trial % 11 == 0 else 1.0)
        got = M.output(xs, us)
        exact = M.exact_dot(xs, us)
        X, Y, EE, F, unit = _bound_units(xs, us)
        half_ulp = Fraction(math.ulp(float(exact))) / 2 if exact != 0 else Fraction(0)
        bound = (half_ulp + sum(Fraction(abs(float(u))) for u in us) * Fraction(2) ** (EE - 1078)
                 + sum(Fraction(abs(float(x))) for x in xs) * Fraction(2) ** (F - 55) + 7 * unit)
        err = abs(Fraction(got) - exact)
        assert err <= bound, (trial, float(err), float(bound))
        worst = max(worst, float(err / bound))
    assert worst > 0.0


def test_zero_column_and_zero_coefficients():
    assert M.output([0.0] * 64, list(np.linspace(-1, 1, 64))) == 0.0
    assert M.output(list(np.linspace(-1, 1, 64)), [0.0] * 64) == 0.0
