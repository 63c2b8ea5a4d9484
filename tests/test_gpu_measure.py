"""Measurement on the GPU against the oracle: try_measure, measure_sequence (measure_circuit) and
the live-subspace bookkeeping.

Bar: complex128 registers in QS_ARITH_EXACT up to 20 qubits reproduce the reference's probability
sums, outcomes and collapsed amplitudes bit for bit (+0 == -0); the parallel forms (FMA arithmetic,
larger registers) give identical outcomes for the same draws and states within 1e-14 floored;
complex64 within 1e-6. Gates between measurements release exactly the qubits they act on.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.fixtures import floored_rel_err, value_equal

pytestmark = pytest.mark.gpu


def _state(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def _pair(n, st, arith, precision=0):
    import quaru_gb300 as q
    from oracle import oracle

    o = oracle.OracleRegister.from_int(n, 0)
    o.state = np.ascontiguousarray(st)
    g = q.Register.from_int(n, 0, precision=precision)
    g.set_arith(arith)
    g.state = st
    return o, g


@pytest.mark.parametrize("n", [1, 5, 12, 20])
def test_exact_sequence_is_bit_identical(n):
    rng = np.random.default_rng(40 + n)
    st = _state(rng, n)
    targets = [int(x) for x in rng.integers(0, n, size=min(2 * n, 14))] + [0, 0]  # repeats included
    draws = [float(x) for x in rng.uniform(size=len(targets))]
    o, g = _pair(n, st, 0)
    want = [bool(o.measure(t, d)) for t, d in zip(targets, draws)]
    got = g.measure_sequence(targets, draws)
    assert got == want
    assert value_equal(g.state, o.state)
    # one call per measurement gives the same
    o2, g2 = _pair(n, st, 0)
    for t, d in zip(targets, draws):
        r = g2.measure(t, d)
        assert r == bool(o2.measure(t, d))
        assert g2.last_probs == o2.last_probs  # the reference's sequential sums, exactly
    assert value_equal(g2.state, o2.state)


@pytest.mark.parametrize("arith,precision,tol", [(1, 0, 1e-14), (2, 0, 1e-14), (1, 1, 1e-6)])
def test_parallel_forms_measure_like_the_oracle(arith, precision, tol):
    n = 16
    rng = np.random.default_rng(7 + arith + 10 * precision)
    st = _state(rng, n)
    targets = list(range(n))
    draws = [float(x) for x in rng.uniform(size=n)]
    o, g = _pair(n, st, arith, precision)
    want = [bool(o.measure(t, d)) for t, d in zip(targets, draws)]
    assert g.measure_sequence(targets, draws) == want
    assert floored_rel_err(g.state, o.state) <= tol


def test_gates_between_measurements_release_their_qubits():
    """Measure, apply gates on measured and unmeasured qubits, measure again: the engine's live
    subspace must follow, checked against the oracle for the exact (bit-identical) and FMA forms."""
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation

    n = 10
    rng = np.random.default_rng(99)
    st = _state(rng, n)
    u = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0]
    program = [("m", 2), ("m", 5), ("g", Operation(u, [7])), ("m", 7), ("g", O.hadamard(2)), ("m", 2),
               ("g", O.cnot(5, 0)), ("m", 0), ("m", 5), ("g", O.swap(1, 3)), ("m", 3), ("m", 9)]
    for arith in (0, 1):
        o, g = _pair(n, st, arith)
        draw_rng = np.random.default_rng(5)
        for kind, x in program:
            if kind == "m":
                d = float(draw_rng.uniform())
                assert g.measure(x, d) == bool(o.measure(x, d))
            else:
                g.try_apply_fast(x)
                o.try_apply_fast(x.matrix, x.targets)
        if arith == 0:
            assert value_equal(g.state, o.state)
        else:
            assert floored_rel_err(g.state, o.state) <= 1e-13


def test_measure_all_at_24_qubits_sequence_equals_single_calls():
    import quaru_gb300 as q

    n = 24
    rng = np.random.default_rng(3)
    st = _state(rng, n)
    draws = [float(x) for x in rng.uniform(size=n)]
    a = q.Register.from_int(n, 0)
    a.set_arith(q.QS_ARITH_FMA)
    a.state = st
    b = a.clone()
    seq = a.measure_sequence(list(range(n)), draws)
    one = [b.measure(t, d) for t, d in enumerate(draws)]
    assert seq == one
    sa, sb = a.state, b.state
    nz = np.flatnonzero(sb)
    assert np.array_equal(np.flatnonzero(sa), nz) and nz.size == 1
    assert math.isclose(abs(sa[nz[0]]), 1.0, rel_tol=1e-14)


def test_sequence_rejects_bad_targets_before_any_work():
    import quaru_gb300 as q

    g = q.Register.from_int(4, 5)
    st = g.state
    with pytest.raises(RuntimeError):
        g.measure_sequence([0, 4], [0.5, 0.5])
    assert value_equal(g.state, st)


@pytest.mark.parametrize("n,arith,precision", [(17, 1, 0), (17, 2, 0), (17, 1, 1), (21, 0, 0)])
def test_compact_sequence_bit_identical_to_in_place(monkeypatch, n, arith, precision):
    """Sequences of three or more distinct targets on a register with no measurement recorded run on
    a compact copy of the live subspace; QS_MEASURE_COMPACT=off keeps them in place. Both forms visit
    the same pairs in the same order and divide the same way (the correctly rounded quotient for the
    exact arithmetic, here above the 20 qubits of the reference-order sums), so outcomes, probability
    sums and every amplitude of the final state (zeros included, by sign) agree bit for bit. Targets
    in random order, low and high."""
    import quaru_gb300 as q

    rng = np.random.default_rng(500 + n + arith + 10 * precision)
    st = _state(rng, n)
    targets = [int(x) for x in rng.permutation(n)[:9]]
    draws = [float(x) for x in rng.uniform(size=len(targets))]
    runs = []
    for mode in ("on", "off"):
        monkeypatch.setenv("QS_MEASURE_COMPACT", mode)
        g = q.Register.from_int(n, 0, precision=precision)
        g.set_arith(arith)
        g.state = st
        out = g.measure_sequence(targets, draws)
        runs.append((out, g.last_sequence_probs, g.state))
    (oa, pa, sa), (ob, pb, sb) = runs
    assert oa == ob
    assert pa == pb
    assert np.array_equal(sa.view(np.uint64), sb.view(np.uint64))  # read back as complex128
    # the live amplitudes survive: 2^(n - 9) of them, each |a|^2 summing to 1
    assert np.count_nonzero(sa) == 1 << (n - len(targets))
    assert math.isclose(float(np.sum(np.abs(sa) ** 2)), 1.0, rel_tol=1e-6 if precision else 1e-13)
