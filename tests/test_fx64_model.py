"""CPU checks of the fixed-point (QS_ARITH_FX64) algorithm through its integer model.

The model (tests/fx64_model.py) follows the kernel step for step; here it is held to the error
bound the kernel documents, |S - exact| <= ulp(S)/2 + 2^-54 * max|c| * max|v| per output, against
exact rational dot products, on amplitudes spanning many orders of magnitude, zeros, subnormals and
real and complex gates. The GPU tests then require the kernel to equal the model bit for bit.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from tests.fx64_model import apply_dense1, exact_dot, rows_of


def _states(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    scale = 10.0 ** rng.uniform(-30, 0, size=v.size)  # magnitudes over 30 decades
    w = v * scale
    w[0] = 0.0
    w[1] = 5e-320 - 3e-321j  # subnormal doubles
    w[2] = -0.0
    return [v, w]


def _gates(rng):
    out = []
    for _ in range(6):
        z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
        out.append(np.linalg.qr(z)[0])
    th = rng.uniform(0, 2 * math.pi)
    out.append(np.array([[math.cos(th / 2), -math.sin(th / 2)], [math.sin(th / 2), math.cos(th / 2)]]))  # RY
    out.append(np.array([[1, 1], [1, -1]]) / math.sqrt(2))                                                 # H
    out.append(np.array([[1e-9, 1], [1, -1e-9]], dtype=complex))                                           # unbalanced
    return out


def test_model_meets_the_error_bound_against_exact_products():
    rng = np.random.default_rng(7)
    n = 5
    worst = 0.0
    for st in _states(rng, n):
        for u in _gates(rng):
            for target in (0, 2, n - 1):
                got = apply_dense1(st, u, target)
                idx = np.arange(1 << n)
                for i0 in idx[(idx >> target) & 1 == 0]:
                    i1 = i0 | (1 << target)
                    v = [st[i0].real, st[i0].imag, st[i1].real, st[i1].imag]
                    outs = [got[i0].real, got[i0].imag, got[i1].real, got[i1].imag]
                    for o, row in enumerate(rows_of(u)):
                        ex = exact_dot(row, v)
                        bound = Fraction(math.ulp(float(ex))) / 2 + Fraction(2) ** -54 * \
                            Fraction(max(abs(c) for c in row)) * Fraction(max(abs(x) for x in v))
                        err = abs(Fraction(outs[o]) - ex)
                        assert err <= bound, (target, o, float(err), float(bound))
                        if bound:
                            worst = max(worst, float(err / bound))
    assert worst > 0.0


def test_model_is_at_least_as_accurate_as_fp64_fma_on_random_gates():
    """Summed over many outputs, the fixed-point error is below the FMA chain's (both exact-checked)."""
    rng = np.random.default_rng(11)
    n = 6
    err_fx = err_fma = Fraction(0)
    st = _states(rng, n)[0]
    for u in _gates(rng)[:6]:
        got = apply_dense1(st, u, 1)
        idx = np.arange(1 << n)
        for i0 in idx[(idx >> 1) & 1 == 0]:
            i1 = i0 | 2
            v = [st[i0].real, st[i0].imag, st[i1].real, st[i1].imag]
            outs = [got[i0].real, got[i0].imag, got[i1].real, got[i1].imag]
            for o, row in enumerate(rows_of(u)):
                ex = exact_dot(row, v)
                acc = row[3] * v[3]
                for t in (2, 1, 0):  # fma(c_t, v_t, acc), correctly rounded
                    acc = float(Fraction(row[t]) * Fraction(v[t]) + Fraction(acc))
                err_fx += abs(Fraction(outs[o]) - ex)
                err_fma += abs(Fraction(acc) - ex)
    assert err_fx < err_fma
