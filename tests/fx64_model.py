"""Integer model of the fixed-point (QS_ARITH_FX64) dense 1-qubit gate, for tests.

It follows the kernel's steps with numpy int64 arithmetic: tuple exponent E (the largest
exponent field, at least 1), the truncated 60-bit integers V = sign(v) trunc(|v| 2^(1082 - E)) in
sign-carrying limbs Vh = sign (|V| >> 30), Vl = sign (|V| & (2^30 - 1)), host coefficients
C = RN(c 2^(60 - ec)) in balanced 30-bit
limbs, A = sum Vh*Ch, B = sum (Vh*Cl + Vl*Ch), R = A + (B >> 30), and
S = RN(R) * 2^(E + ec - 1082). Every step is integer work or one correctly rounded conversion,
so the GPU must reproduce these doubles bit for bit. exact_dot() gives the exact value of a
dot product of doubles (Python integers) for checking the error bound.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

MASK30 = (1 << 30) - 1


def _split30(x: np.ndarray):
    lo = ((x & MASK30) ^ (1 << 29)) - (1 << 29)  # low 30 bits as a value in [-2^29, 2^29)
    return (x - lo) >> 30, lo


def coeff_row(c) -> tuple[np.ndarray, np.ndarray, int]:
    """Limbs of C_t = RN(c_t * 2^(60 - ec)) and k0 = ec - 1082 for one output row."""
    c = [float(x) for x in c]
    cmax = max(abs(x) for x in c)
    ec = math.frexp(cmax)[1] if cmax > 0 else 0
    C = np.array([int(round(Fraction(math.ldexp(x, 60 - ec)))) for x in c], dtype=np.int64)
    h, lo = _split30(C)
    return h, lo, ec - 1082


def _efield(bits: np.ndarray) -> np.ndarray:
    return ((bits >> 52) & 0x7FF).astype(np.int64)


def encode(v: np.ndarray, E: np.ndarray):
    """Sign-carrying limbs of V = sign(v) trunc(|v| 2^(1082 - E)) (E per element, >= 1)."""
    bits = v.view(np.uint64)
    e = _efield(bits)
    ee = np.maximum(e, 1)
    m = (bits & np.uint64((1 << 52) - 1)).astype(np.int64) | np.where(e != 0, 1 << 52, 0).astype(np.int64)
    m = m << 7
    d = E - ee
    m = np.where(d < 64, m >> np.minimum(d, 63), 0)
    sgn = np.where((bits >> 63) == 1, -1, 1)
    return sgn * (m >> 30), sgn * (m & MASK30)


def to_double(R: np.ndarray, k: np.ndarray) -> np.ndarray:
    d = R.astype(np.float64)  # int64 -> double rounds to nearest even
    return np.ldexp(d, k.astype(np.int32))


def rows_of(u: np.ndarray):
    """The four coefficient rows (y0.re, y0.im, y1.re, y1.im) over (x0.re, x0.im, x1.re, x1.im)."""
    rows = []
    for r in range(2):
        a, b = complex(u[r, 0]), complex(u[r, 1])
        rows.append([a.real, -a.imag, b.real, -b.imag])
        rows.append([a.imag, a.real, b.imag, b.real])
    return rows


def apply_dense1(state: np.ndarray, u: np.ndarray, target: int) -> np.ndarray:
    """The fixed-point kernel's result for a dense 2x2 gate u on `target` (new array)."""
    n = int(state.size).bit_length() - 1
    st = np.ascontiguousarray(state, dtype=np.complex128)
    idx = np.arange(1 << n, dtype=np.int64)
    i0 = idx[(idx >> target) & 1 == 0]
    i1 = i0 | (1 << target)
    v = [st[i0].real.copy(), st[i0].imag.copy(), st[i1].real.copy(), st[i1].imag.copy()]
    E = np.maximum.reduce([np.maximum(_efield(x.view(np.uint64)), 1) for x in v])
    if np.any(E >= 0x7FF):
        raise ValueError("non-finite amplitudes take the FP64 path")
    lim = [encode(x, E) for x in v]
    real = bool(np.all(np.asarray(u).imag == 0))
    out = []
    for o, row in enumerate(rows_of(u)):
        ch, cl, k0 = coeff_row(row)
        terms = [o & 1, 2 + (o & 1)] if real else range(4)
        A = np.zeros_like(E)
        B = np.zeros_like(E)
        for t in terms:
            vh, vl = lim[t]
            A = A + vh * ch[t]
            B = B + vh * cl[t] + vl * ch[t]
        out.append(to_double(A + (B >> 30), E + k0))
    res = st.copy()
    res[i0] = out[0] + 1j * out[1]
    res[i1] = out[2] + 1j * out[3]
    return res


def exact_dot(c, v) -> Fraction:
    """sum c_t v_t exactly."""
    return sum((Fraction(float(a)) * Fraction(float(b)) for a, b in zip(c, v)), Fraction(0))


def ulp(x: float) -> float:
    return math.ulp(x) if x != 0 else math.ulp(0.0)
