"""GPU engine vs the CPU oracle on seeded inputs.

Bar: under QS_ARITH_EXACT every amplitude is bit-identical to the oracle
(+0 == -0), for every gate class; under QS_ARITH_FMA generic gates agree
within 1e-12 (floored relative, see tests/fixtures.floored_rel_err);
complex64 registers agree within 1e-4; permutation gates are bit-identical in
every mode. Measurement outcomes are identical for the same draws.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.fixtures import floored_rel_err, value_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def q():
    import quaru_gb300

    return quaru_gb300


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle

    return oracle


def rand_state(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def rand_unitary(rng, k):
    d = 1 << k
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / math.sqrt(2)
    qm, r = np.linalg.qr(z)
    return qm * (np.diag(r) / np.abs(np.diag(r)))


def run_pair(q, orc, n, ops, arith=0, state=None, precision=0):
    o = orc.OracleRegister.from_int(n, 0)
    g = q.Register.from_int(n, 0, precision=precision)
    g.set_arith(arith)
    if state is not None:
        o.state = np.ascontiguousarray(state.astype(np.complex128))
        g.state = state
    for op in ops:
        o.try_apply_fast(op.matrix, op.targets)
        g.try_apply_fast(op)
    return o.state, g.state


def one_qubit_gates(rng, t):
    from quaru_gb300 import operation as O

    th, ph, la = rng.uniform(0, 2 * math.pi, size=3)
    return [O.hadamard(t), O.not_(t), O.pauli_y(t), O.pauli_z(t), O.phase(t), O.identity(t),
            O.phase_theta(th, t), O.ry(th, t), O.rz(ph, t), O.u(th, ph, la, t),
            O.Operation(rand_unitary(rng, 1), [t])]


@pytest.mark.parametrize("n", [1, 2, 3, 6, 11])
def test_single_qubit_gates_every_target_bit_exact(q, orc, n):
    rng = np.random.default_rng(100 + n)
    ops = [g for t in range(n) for g in one_qubit_gates(rng, t)]
    o, g = run_pair(q, orc, n, ops, state=rand_state(rng, n))
    assert value_equal(g, o)


@pytest.mark.parametrize("k", [2, 3, 4, 5, 6, 7])
def test_dense_k_qubit_bit_exact(q, orc, k):
    from quaru_gb300.operation import Operation

    rng = np.random.default_rng(200 + k)
    n = k + 3
    ops = []
    for _ in range(3):
        targets = list(rng.permutation(n)[:k])
        ops.append(Operation(rand_unitary(rng, k), targets))
        ops.append(Operation(rand_unitary(rng, k).real.astype(complex), targets[::-1]))  # real, non-unitary
    st = rand_state(rng, n)
    o, g = run_pair(q, orc, n, ops, state=st)
    assert value_equal(g, o)
    o2, g2 = run_pair(q, orc, n, ops, arith=1, state=st)
    assert floored_rel_err(g2, o2) <= 1e-12


def test_controlled_and_anticontrolled_dense_bit_exact(q, orc):
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation

    rng = np.random.default_rng(300)
    n = 9
    ops = []
    for k in range(1, 5):
        base = Operation(rand_unitary(rng, k), list(rng.permutation(n)[:k]))
        free = [x for x in range(n) if x not in base.targets]
        c1 = int(rng.choice(free))
        ops.append(O.to_controlled(base, c1))
        # a 0-controlled gate: U on the control = 0 half, identity on the other
        m = np.eye(1 << (k + 1), dtype=complex)
        m[: 1 << k, : 1 << k] = base.matrix
        ops.append(Operation(m, base.targets + [c1]))
        # doubly controlled
        free2 = [x for x in free if x != c1]
        ops.append(O.to_controlled(O.to_controlled(base, c1), int(rng.choice(free2))))
    o, g = run_pair(q, orc, n, ops, state=rand_state(rng, n))
    assert value_equal(g, o)


def test_permutation_gates_bit_exact_all_modes(q, orc):
    from quaru_gb300 import operation as O

    rng = np.random.default_rng(400)
    n = 10
    ops = []
    for _ in range(30):
        a, b, c, d, e, f = (int(x) for x in rng.permutation(n)[:6])
        ops += [O.cnot(a, b), O.swap(c, d), O.cnx([a, b], c), O.cnx([a, b, c, d], e), O.cnz([a, b], c),
                O.not_(f), O.pauli_y(e), O.phase(d), O.cnx([a, b, c, d, e], f)]
    ops.append(O.to_quantum_gate(lambda x: (x * 7) % 16, [1, 3, 5, 7]))   # permutation
    ops.append(O.to_quantum_gate(lambda x: (x * 6) % 16, [0, 2, 4, 6]))   # not injective
    st = rand_state(rng, n)
    for arith in (0, 1):
        o, g = run_pair(q, orc, n, ops, arith=arith, state=st)
        assert value_equal(g, o)
    o, g = run_pair(q, orc, n, ops, precision=1, state=st)
    assert floored_rel_err(g, o) <= 1e-6


def test_monomial_with_phases_and_wide_gates(q, orc):
    from quaru_gb300.operation import Operation

    rng = np.random.default_rng(500)
    n = 9
    ops = []
    for k in (0, 1, 2, 3, 5, 6, 8):
        d = 1 << k
        p = rng.permutation(d)
        m = np.zeros((d, d), dtype=complex)
        m[np.arange(d), p] = np.exp(1j * rng.uniform(0, 2 * np.pi, size=d))
        ops.append(Operation(m, list(rng.permutation(n)[:k])))
        diag = np.diag(np.exp(1j * rng.uniform(0, 2 * np.pi, size=d)))
        ops.append(Operation(diag, list(rng.permutation(n)[:k])))
    ops.append(Operation(np.zeros((2, 2), dtype=complex), [3]))  # the zero matrix
    ops.append(Operation(np.array([[2.5 - 1j]]), []))  # k = 0: scalar
    o, g = run_pair(q, orc, n, ops, state=rand_state(rng, n))
    assert value_equal(g, o)


def test_large_dense_and_hadamard_transform(q, orc):
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation

    rng = np.random.default_rng(600)
    n = 9
    ops = [O.hadamard_transform([0, 3, 5, 6, 8, 1]), Operation(rand_unitary(rng, 6), [2, 4, 0, 7, 8, 5]),
           Operation(rand_unitary(rng, 8), list(rng.permutation(n)[:8]))]
    st = rand_state(rng, n)
    o, g = run_pair(q, orc, n, ops, state=st)
    assert value_equal(g, o)
    o, g = run_pair(q, orc, n, ops, arith=1, state=st)
    assert floored_rel_err(g, o) <= 1e-12


def test_random_circuit_c64_within_tolerance(q, orc):
    from quaru_gb300.workloads import parity_circuit

    c = parity_circuit(n=10, m=300, seed=77)
    o, g = run_pair(q, orc, c.n, c.gates, precision=1)
    assert floored_rel_err(g, o) <= 1e-4


def test_measure_matches_oracle(q, orc):
    rng = np.random.default_rng(700)
    n = 11
    for trial in range(4):
        st = rand_state(rng, n)
        o = orc.OracleRegister.from_int(n, 0)
        o.state = st.copy()
        g = q.Register.from_int(n, 0)
        g.state = st
        for t in rng.permutation(n):
            x = float(rng.random())
            ro = o.measure(int(t), x)
            rg = g.measure(int(t), x)
            assert ro == rg
            assert abs(o.last_probs[0] - g.last_probs[0]) <= 1e-14
            assert abs(o.last_probs[1] - g.last_probs[1]) <= 1e-14
            assert floored_rel_err(g.state, o.state) <= 1e-13


def test_c64_collapse_rounding(q):
    """complex64 collapse: x * RN(1/sqrt(total)) in FP64, rounded to float (nearest even) on the
    integer pipe: bit-identical to numpy's float64 product cast to float32."""
    rng = np.random.default_rng(702)
    n = 12
    st = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)).astype(np.complex64)
    st /= np.float32(np.linalg.norm(st.astype(np.complex128)))
    g = q.Register.from_int(n, 0, precision=1)
    g.state = st
    target = 3
    out = g.measure(target, 0.4)
    p0, p1 = g.last_probs
    rinv = 1.0 / math.sqrt(p1 if out else p0)
    exp = np.zeros_like(st)
    keep = ((np.arange(1 << n) >> target) & 1) == int(out)
    exp.real[keep] = (st.real[keep].astype(np.float64) * rinv).astype(np.float32)
    exp.imag[keep] = (st.imag[keep].astype(np.float64) * rinv).astype(np.float32)
    assert np.array_equal(g.state, exp.astype(np.complex128))  # float values read back exactly


def test_measure_outcome_rule_and_collapse_exact(q, orc):
    # draw == prob_0 exactly gives false (x > prob_0 is false), src/register.rs:321
    g = q.Register.new([False, False]).apply(__import__("quaru_gb300").operation.hadamard(0))
    st = g.state
    p0 = float(np.sum(np.abs(st[::2]) ** 2))
    assert g.measure(0, p0) is False
    # collapse divides by sqrt(total) exactly as IEEE division does
    rng = np.random.default_rng(701)
    n = 12
    st = rand_state(rng, n)
    o = orc.OracleRegister.from_int(n, 0)
    o.state = st.copy()
    g = q.Register.from_int(n, 0)
    g.state = st
    o.measure(5, 0.3)
    g.measure(5, 0.3)
    if o.last_probs == g.last_probs:  # same divisor: quotients must be identical
        assert value_equal(g.state, o.state)


def test_state_roundtrip_probabilities_clone_eq(q, orc):
    from quaru_gb300 import operation as O

    rng = np.random.default_rng(800)
    n = 8
    st = rand_state(rng, n)
    g = q.Register.from_int(n, 0)
    g.state = st
    assert value_equal(g.state, st)
    o = orc.OracleRegister.from_int(n, 0)
    o.state = st.copy()
    assert np.array_equal(g.probabilities(), o.probabilities())
    h = g.clone()
    assert h == g
    h.apply(O.not_(3))
    assert not (h == g)
    g64 = q.Register.from_int(n, 0, precision=1)
    g64.state = st
    assert np.max(np.abs(g64.state - st)) < 1e-7
    assert g.size() == n and g64.precision == 1


@pytest.mark.parametrize("n", [10, 20])
def test_from_qubits_product_state_bit_exact(q, orc, n):
    """n = 20 also covers the doubling levels above the first 16 qubits."""
    rng = np.random.default_rng(900 + n)
    qs = []
    for _ in range(n):
        v = rng.normal(size=2) + 1j * rng.normal(size=2)
        qs.append(v / np.linalg.norm(v))
    o = orc.OracleRegister.try_from_qubits(qs)
    g = q.Register.try_from_qubits(qs)
    assert value_equal(g.state, o.state)


def test_apply_circuit_matches_single_calls(q):
    from quaru_gb300.workloads import parity_circuit

    c = parity_circuit(n=11, m=250, seed=5)
    a = q.Register.from_int(c.n, 0)
    for gte in c.gates:
        a.apply(gte)
    b = q.Register.from_int(c.n, 0)
    b.apply_gates(c.gates)
    assert value_equal(a.state, b.state)


def test_error_codes(q):
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation

    g = q.Register.new([False] * 4)
    with pytest.raises(q.OperationError) as e:
        g.try_apply_fast(Operation(np.eye(8, dtype=complex), [0, 4, 4]))
    assert e.value.kind == "InvalidTarget" and e.value.payload == (4,)  # duplicate before range
    with pytest.raises(q.OperationError) as e:
        g.try_apply_fast(Operation(np.eye(4, dtype=complex), [7, 5]))
    assert e.value.payload == (7,)  # first out-of-range target in list order
    with pytest.raises(q.OperationError) as e:
        g.try_apply_fast(Operation(np.eye(3, dtype=complex), [0, 1]))
    assert e.value.kind == "InvalidDimensions" and e.value.payload == (3, 3)
    with pytest.raises(q.OperationError) as e:
        g.try_measure(4, 0.5)
    assert e.value.kind == "InvalidTarget" and e.value.payload == (4,)
    with pytest.raises(q.OperationError) as e:
        g.try_apply_all(O.cnot(0, 1))
    assert e.value.kind == "InvalidArity" and e.value.payload == (2,)
    with pytest.raises(q.OperationError) as e:
        g.apply_gates([O.hadamard(0), O.cnot(0, 9)])
    assert e.value.payload == (9,)
    assert np.array_equal(g.state, q.Register.new([False] * 4).state)  # nothing applied


@pytest.mark.parametrize("n", [1, 2, 7, 12])
def test_df64_random_circuits_within_tolerance(q, orc, n):
    from quaru_gb300.workloads import parity_circuit

    c = parity_circuit(n=max(n, 3), m=400, seed=300 + n) if n >= 3 else None
    rng = np.random.default_rng(310 + n)
    if c is None:
        from quaru_gb300.operation import Operation

        ops = [Operation(rand_unitary(rng, 1), [int(rng.integers(n))]) for _ in range(200)]
        nn = n
    else:
        ops, nn = c.gates, c.n
    o, g = run_pair(q, orc, nn, ops, arith=2, state=rand_state(rng, nn))
    assert floored_rel_err(g, o) <= 1e-12


def test_df64_dense_multi_qubit_gates(q, orc):
    """DF64: dense 2- and 3-qubit gates (double-float kernel), their controlled forms, and 4-qubit
    gates (FP64 kernel), 60 gates deep, within the 1e-12 floored bound of the FP64 oracle."""
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation

    rng = np.random.default_rng(320)
    n = 12
    ops = []
    for i in range(60):
        k = (2, 3, 2, 3, 4)[i % 5]
        tg = [int(x) for x in rng.permutation(n)[:k + 1]]
        g = Operation(rand_unitary(rng, k), tg[:k])
        ops.append(O.to_controlled(g, tg[k]) if i % 7 == 3 else g)
    o, g = run_pair(q, orc, n, ops, arith=2, state=rand_state(rng, n))
    assert floored_rel_err(g, o) <= 1e-12


def test_df64_deep_layered_circuit(q, orc):
    from quaru_gb300.workloads import flatten, layered_circuit

    n = 14
    ops = flatten(layered_circuit(n, 30, 99))
    o, g = run_pair(q, orc, n, ops, arith=2)
    assert floored_rel_err(g, o) <= 1e-12
    # tiny amplitudes (down to 1e-30) stay within the floored bound too
    rng = np.random.default_rng(12)
    st = rand_state(rng, 10) * np.logspace(0, -30, 1 << 10)
    st /= np.linalg.norm(st)
    o, g = run_pair(q, orc, 10, flatten(layered_circuit(10, 5, 7)), arith=2, state=st)
    assert floored_rel_err(g, o) <= 1e-12


@pytest.fixture(scope="module")
def layered18(orc):
    """The benchmarks' layered family (Haar 1q on every qubit + CNOTs on a random matching) at its
    full 40-layer depth on 18 qubits (1080 gates, the 28-qubit configuration's seed), on the oracle."""
    from quaru_gb300.workloads import flatten, layered_circuit, workload_seed

    n = 18
    ops = flatten(layered_circuit(n, 40, workload_seed("layered_28q")))
    o = orc.OracleRegister.from_int(n, 0)
    for op in ops:
        o.try_apply_fast(op.matrix, op.targets)
    return n, ops, o.state


@pytest.mark.parametrize("arith,fuse", [(1, 0), (2, 0), (3, 0), (1, 1), (2, 1), (3, 1), (1, 2), (2, 2), (3, 2)])
def test_layered_family_full_depth_every_form(q, layered18, arith, fuse):
    """FP64 FMA, double-float and fixed-point arithmetic; one sweep per gate, cache-blocked stages and
    dense blocks: all within the 1e-12 floored bound of the oracle after 1080 gates."""
    n, ops, ref = layered18
    g = q.Register.from_int(n, 0)
    g.set_arith(arith)
    g.apply_gates(ops, fuse=fuse)
    assert floored_rel_err(g.state, ref) <= 1e-12
