"""QS_ARITH_FX64 on the GPU: the fixed-point dense 1-qubit kernel.

Bar: (1) the kernel equals the integer model (tests/fx64_model.py) bit for bit, zeros compared by
value, on states whose magnitudes span 30 decades, with zeros and subnormals, for complex and real
gates on low, middle and high targets; (2) on the 12-qubit, 200-gate parity circuit and on the
layered Haar + CNOT family at 16 qubits and 40 layers, its largest deviation from the oracle (the
reference's FP64 operation order) is no larger than the FP64 FMA form's, and both stay within
the 1e-12 floored-relative bound; (3) non-finite amplitudes take the FP64 path.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.fixtures import floored_rel_err, value_equal
from tests.fx64_model import apply_dense1

pytestmark = pytest.mark.gpu

FX64, FMA = 3, 1


@pytest.fixture(scope="module")
def q():
    import quaru_gb300

    return quaru_gb300


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle

    return oracle


def _states(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    w = v * 10.0 ** rng.uniform(-30, 0, size=v.size)
    w[3] = 0.0
    w[5] = 4e-318 + 1e-320j
    w[6] = -0.0 + 2e-300j
    return [v, w]


def _gates(rng):
    from quaru_gb300.operation import Operation

    out = []
    for _ in range(3):
        z = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
        out.append(np.linalg.qr(z)[0])
    th = rng.uniform(0, 2 * math.pi)
    out.append(np.array([[math.cos(th / 2), -math.sin(th / 2)], [math.sin(th / 2), math.cos(th / 2)]],
                        dtype=complex))
    out.append(np.array([[1, 1], [1, -1]], dtype=complex) / math.sqrt(2))
    out.append(np.array([[3e-9, 1], [1, -3e-9]], dtype=complex))
    return out, Operation


@pytest.mark.parametrize("n", [1, 5, 12])
def test_fx64_equals_integer_model_bit_for_bit(q, n):
    rng = np.random.default_rng(900 + n)
    gates, Operation = _gates(rng)
    if n >= 3:
        states = _states(rng, n)
    else:
        v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        states = [v / np.linalg.norm(v)]
    for st in states:
        for u in gates:
            for t in sorted({0, n // 2, n - 1}):
                g = q.Register.from_int(n, 0)
                g.set_arith(FX64)
                g.state = st
                g.try_apply_fast(Operation(u, [t]))
                want = apply_dense1(st, u, t)
                assert value_equal(g.state, want), (n, t)


def _max_err(q, orc, n, ops, arith):
    o = orc.OracleRegister.from_int(n, 0)
    g = q.Register.from_int(n, 0)
    g.set_arith(arith)
    for op in ops:
        o.try_apply_fast(op.matrix, op.targets)
        g.try_apply_fast(op)
    ref, got = o.state, g.state
    return floored_rel_err(got, ref), float(np.sum(np.abs(got - ref)))


def test_fx64_is_at_least_as_close_to_the_oracle_as_fp64_fma(q, orc):
    from quaru_gb300.workloads import flatten, layered_circuit, parity_circuit

    cases = [(12, parity_circuit().gates), (16, flatten(layered_circuit(16, 40, 4242)))]
    for n, ops in cases:
        fx_max, fx_sum = _max_err(q, orc, n, ops, FX64)
        fma_max, fma_sum = _max_err(q, orc, n, ops, FMA)
        assert fx_max <= 1e-12 and fma_max <= 1e-12, (n, fx_max, fma_max)
        assert fx_max <= fma_max and fx_sum <= fma_sum, (n, fx_max, fma_max, fx_sum, fma_sum)


def test_fx64_non_finite_amplitudes_take_the_fp64_path(q):
    from quaru_gb300.operation import Operation

    n = 4
    rng = np.random.default_rng(5)
    st = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    st[2] = complex(np.inf, 0.0)
    u = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0]
    res = {}
    for arith in (FX64, FMA):
        g = q.Register.from_int(n, 0)
        g.set_arith(arith)
        g.state = st
        g.try_apply_fast(Operation(u, [1]))
        res[arith] = g.state
    bad = ~np.isfinite(res[FMA])
    assert np.array_equal(bad, ~np.isfinite(res[FX64])) and bad.any()
    assert value_equal(res[FX64][bad], res[FMA][bad])
    assert np.all(np.abs(res[FX64][~bad] - res[FMA][~bad]) <= 1e-15 * np.abs(res[FMA][~bad]) + 1e-300)
