"""Integer model of the FP64-accurate block product (k_tile_oz), for tests.

It restates the kernel's arithmetic with Python integers: a column x (64 doubles) is scaled by the
power of two of its largest exponent field EE and rounded to X = round(x 2^(1077 - EE)) (|X| < 2^55,
ties away from zero); an output column u of the block's real form by F = frexp exponent of its
largest magnitude, Y = round(u 2^(54 - F)) (|Y| <= 2^54); both are cut into 7 balanced base-256
digits (X + 0x808080808080: digits 1..6 are bytes - 128, digit 0 the top part); level sums
I_L = sum_k sum_{s+t=L} a_s b_t for L <= 6 (levels 0..4 held exactly by the kernel's FP32
accumulators, 5..6 summed in one accumulator that the model keeps exact); R = round(2^36 sum_L
I_L 2^-8L) and the output R 2^(EE + F - 1071). The kernel differs from the model only in the
rounding of its level 5..6 accumulator (FP32) and in the output's final rounding (the same
correctly rounded conversion).
"""
from __future__ import annotations

import math
import struct
from fractions import Fraction

BIAS = 0x808080808080
SLICES = 7


def efield(x: float) -> int:
    return (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def encode_column(xs) -> tuple[list[int], int]:
    """X_k for the column's components and EE = max(largest exponent field, 1)."""
    EE = max(1, max(efield(float(x)) for x in xs))
    out = []
    for x in xs:
        x = float(x)
        if x == 0.0:
            out.append(0)
            continue
        # |x| 2^(1077 - EE) exactly, rounded to nearest, ties away from zero
        v = Fraction(abs(x)) * Fraction(2) ** (1077 - EE)
        r = math.floor(v + Fraction(1, 2))
        out.append(r if x > 0 else -r)
    return out, EE


def encode_output_column(us) -> tuple[list[int], int]:
    """Y_k (ties to even, as the host's llrint) and F."""
    mx = max(abs(float(u)) for u in us)
    F = math.frexp(mx)[1] if mx > 0 else 0
    return [int(round(Fraction(float(u)) * Fraction(2) ** (54 - F))) for u in us], F


def digits(X: int) -> list[int]:
    """Balanced base-256 digits, most significant first: X = sum_s d_s 256^(6-s)."""
    Xb = X + BIAS
    d = [0] * SLICES
    for i in range(6):
        d[6 - i] = ((Xb >> (8 * i)) & 255) - 128
    d[0] = Xb >> 48
    return d


def level_sums(X: list[int], Y: list[int]) -> list[int]:
    """I_L for L = 0..12 (the kernel keeps 0..6)."""
    da = [digits(x) for x in X]
    db = [digits(y) for y in Y]
    out = [0] * (2 * SLICES - 1)
    for a, b in zip(da, db):
        for s in range(SLICES):
            for t in range(SLICES):
                out[s + t] += a[s] * b[t]
    return out


def product_R(X: list[int], Y: list[int]) -> tuple[int, list[int]]:
    """R = round(2^36 sum_{L<=6} I_L 2^-8L) as the kernel assembles it (levels 0..4 exact, the level
    5..6 part rounded once at 2^-36), and the level sums."""
    I = level_sums(X, Y)
    R = (I[0] << 36) + (I[1] << 28) + (I[2] << 20) + (I[3] << 12) + (I[4] << 4)
    tail = Fraction(I[5], 1 << 4) + Fraction(I[6], 1 << 12)
    R += math.floor(tail + Fraction(1, 2)) if tail >= 0 else -math.floor(-tail + Fraction(1, 2))
    return R, I


def output(xs, us) -> float:
    """The modelled output sum_k u_k x_k for one column and one output component."""
    X, EE = encode_column(xs)
    Y, F = encode_output_column(us)
    R, _ = product_R(X, Y)
    return math.ldexp(float(R), EE + F - 1071) if R != 0 else 0.0


def exact_dot(xs, us) -> Fraction:
    return sum((Fraction(float(a)) * Fraction(float(b)) for a, b in zip(xs, us)), Fraction(0))
