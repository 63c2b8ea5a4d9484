"""Batched persistent forward + adjoint (qs_batch_*) against per-circuit qs_adjoint_gradient."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def per_circuit(circuits, params, precision):
    import quaru_gb300 as q

    es, gs = [], []
    off = 0
    for n, gates, npar, terms in circuits:
        reg = q.Register.from_int(n, 0, precision=precision)
        reg.set_arith(q.QS_ARITH_FMA)  # FP64 reference for the complex128 forms
        e, g = reg.adjoint_gradient(gates, params[off:off + npar], terms)
        es.append(e)
        gs.append(g)
        off += npar
    return np.array(es), np.concatenate(gs)


@pytest.mark.parametrize("precision,arith,tol", [(0, 1, 1e-10), (0, 2, 1e-10), (1, 1, 2e-4)])
def test_batch_matches_single_circuit_path(precision, arith, tol):
    """Circuits of 3..13 qubits (one tile up to 11 qubits, several above); items of one tile (cl = 8)
    and autotuned; arith = 2: complex128 stages in double-float tiles."""
    from quaru_gb300.batch import Batch
    from quaru_gb300.workloads import ansatz_batch

    circuits, params = ansatz_batch(count=24, qmin=3, qmax=13, lmin=1, lmax=4, seed=99)
    params = np.array(params)
    for cl in (0, 8):
        b = Batch(circuits, precision=precision, chunk_log2=cl, ctas_per_sm=2 if cl else 0, arith=arith)
        e, g = b.run(params)
        e2, g2 = b.run(params)  # graph replay gives the same numbers
        assert np.array_equal(e, e2) and np.array_equal(g, g2)
        re, rg = per_circuit(circuits, params, precision)
        assert np.max(np.abs(e - re)) < tol
        assert np.max(np.abs(g - rg)) < tol
    # new parameters through the same graph
    p2 = params + 0.1
    e3, g3 = b.run(p2)
    re3, rg3 = per_circuit(circuits, p2, precision)
    assert np.max(np.abs(g3 - rg3)) < tol


@pytest.mark.parametrize("precision,arith,tol", [(0, 1, 1e-10), (0, 2, 1e-10), (1, 1, 2e-4)])
def test_batch_larger_circuits_fixed_gates(precision, arith, tol):
    """12..16 qubits with fixed 1-qubit gates mixed in (their stages stay FP64 under DF64): items of
    1, 4 and 16 tiles."""
    from quaru_gb300 import ParamGate
    from quaru_gb300 import operation as O
    from quaru_gb300.batch import Batch
    from quaru_gb300.workloads import ansatz_batch

    circuits, params = ansatz_batch(count=6, qmin=12, qmax=16, lmin=2, lmax=3, seed=7)
    mixed = []
    for i, (n, gates, npar, terms) in enumerate(circuits):
        g = list(gates)
        if i % 2:
            g.insert(len(g) // 2, ParamGate.fixed(O.hadamard(n - 1)))
            g.insert(len(g) // 3, ParamGate.fixed(O.Operation(np.array([[0, 1j], [1j, 0]]), [0])))
        mixed.append((n, g, npar, terms))
    params = np.array(params)
    re, rg = per_circuit(mixed, params, precision)
    for cl in (10, 12, 14):
        b = Batch(mixed, precision=precision, chunk_log2=cl, ctas_per_sm=1, arith=arith)
        e, g = b.run(params)
        assert np.max(np.abs(e - re)) < tol
        assert np.max(np.abs(g - rg)) < tol


@pytest.mark.parametrize("precision,arith", [(0, 1), (0, 2), (1, 1)])
def test_batch_tiny_and_mixed_sizes(precision, arith):
    """1- and 2-qubit circuits (a tile is the whole 2- or 4-amplitude state) next to a 12-qubit one."""
    from quaru_gb300 import ParamGate
    from quaru_gb300 import operation as O
    from quaru_gb300.batch import Batch

    circuits = [
        (1, [ParamGate.ry(0, 0), ParamGate.rz(0, 1), ParamGate.rx(0, 0)], 2, [(0.7, 0, 1), (0.4, 1, 0)]),
        (2, [ParamGate.ry(0, 0), ParamGate.ry(1, 1), ParamGate.fixed(O.cnot(0, 1)), ParamGate.rz(1, 2),
             ParamGate.fixed(O.hadamard(0))], 3, [(1.1, 0, 3), (-0.3, 2, 0), (0.5, 3, 3)]),
        (12, [ParamGate.ry(q, q) for q in range(12)] + [ParamGate.fixed(O.cnot(q, q + 1)) for q in range(11)]
         + [ParamGate.rz(q, 12 + q) for q in range(12)], 24, [(0.9, 0, 0b11), (0.6, 1 << 11, 0)]),
    ]
    params = np.random.default_rng(5).uniform(0, 2 * np.pi, size=2 + 3 + 24)
    tol = 1e-10 if precision == 0 else 2e-4
    re, rg = per_circuit(circuits, params, precision)
    b = Batch(circuits, precision=precision, arith=arith)
    e, g = b.run(params)
    assert np.max(np.abs(e - re)) < tol
    assert np.max(np.abs(g - rg)) < tol


def test_batch_rejects_unsupported_gates():
    import quaru_gb300 as q
    from quaru_gb300 import ParamGate
    from quaru_gb300 import operation as O
    from quaru_gb300.batch import Batch

    with pytest.raises(q.EngineError):
        Batch([(3, [ParamGate.fixed(O.swap(0, 1))], 0, [(1.0, 0, 1)])])
    with pytest.raises(q.EngineError):
        Batch([(3, [ParamGate.ry(0, 2)], 1, [(1.0, 0, 1)])])


def _energy(n, gates, params, terms, precision=0):
    import quaru_gb300 as q

    reg = q.Register.from_int(n, 0, precision=precision)
    reg.set_arith(q.QS_ARITH_FMA)
    reg.apply_gates([g.operation(params) for g in gates])
    return reg.expval_pauli(terms)


def test_batch_at_the_benchmark_size():
    """The benchmark's batch itself: 256 circuits of 10..22 qubits with 4..12 layers (the defaults of ansatz_batch).
    FP64 (autotuned chunking, as the benchmark runs it), complex128 double-float and complex64 batches
    against the loop of FP64 single-circuit gradients; central finite differences (h = 1e-6) on
    parameters of the three largest circuits within 1e-6."""
    from quaru_gb300.batch import Batch
    from quaru_gb300.workloads import ansatz_batch

    circuits, params = ansatz_batch()
    params = np.array(params)
    re, rg = per_circuit(circuits, params, 0)
    for precision, arith, tol, cl, ct in [(0, 1, 1e-10, 0, 0), (0, 2, 1e-10, 12, 2), (1, 1, 2e-4, 12, 2)]:
        b = Batch(circuits, precision=precision, arith=arith, chunk_log2=cl, ctas_per_sm=ct)
        e, g = b.run(params)
        assert np.max(np.abs(e - re)) < tol, (precision, arith)
        assert np.max(np.abs(g - rg)) < tol, (precision, arith)
        del b
    offs = np.cumsum([0] + [c[2] for c in circuits])
    largest = sorted(range(len(circuits)), key=lambda i: -circuits[i][0])[:3]
    h = 1e-6
    for i in largest:
        n, gates, npar, terms = circuits[i]
        p = params[offs[i]:offs[i] + npar].copy()
        for j in (0, npar // 2, npar - 1):
            pp, pm = p.copy(), p.copy()
            pp[j] += h
            pm[j] -= h
            fd = (_energy(n, gates, pp, terms) - _energy(n, gates, pm, terms)) / (2 * h)
            assert abs(fd - rg[offs[i] + j]) < 1e-6, (i, j, fd, rg[offs[i] + j])
