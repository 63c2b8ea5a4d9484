"""Cache-blocked stages (fuse=1) against gate-by-gate application and the oracle.

Under QS_ARITH_EXACT a fused run must be bit-identical to the unfused run (the
tile kernel applies each gate with the same arithmetic); FMA and DF64 stay
within 1e-12 of the FP64 oracle, complex64 within 1e-4.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.fixtures import floored_rel_err, value_equal

pytestmark = pytest.mark.gpu


def rand_unitary(rng, k):
    d = 1 << k
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / math.sqrt(2)
    qm, r = np.linalg.qr(z)
    return qm * (np.diag(r) / np.abs(np.diag(r)))


def mixed_circuit(rng, n, m):
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation
    from quaru_gb300.workloads import SplitMix64, random_gate

    sm = SplitMix64(int(rng.integers(1 << 30)))
    ops = [random_gate(sm, n) for _ in range(m)]
    # extra structure: controlled dense gates, 0-controls, a wide gate and a dense 2-qubit gate
    for _ in range(6):
        a, b, c = (int(x) for x in rng.permutation(n)[:3])
        ops.insert(int(rng.integers(len(ops))), O.to_controlled(Operation(rand_unitary(rng, 1), [a]), b))
        ops.insert(int(rng.integers(len(ops))), O.cnx([b, c], a))
    ops.insert(len(ops) // 2, Operation(rand_unitary(rng, 2), [int(x) for x in rng.permutation(n)[:2]]))
    if n >= 7:
        ops.insert(len(ops) // 3, Operation(rand_unitary(rng, 6), [int(x) for x in rng.permutation(n)[:6]]))
    return ops


@pytest.mark.parametrize("n", [4, 11, 12, 15, 20])
def test_fused_exact_bit_identical(n):
    import quaru_gb300 as q

    rng = np.random.default_rng(1000 + n)
    ops = mixed_circuit(rng, n, 300)
    a = q.Register.from_int(n, 0)
    a.apply_gates(ops, fuse=0)
    b = q.Register.from_int(n, 0)
    b.apply_gates(ops, fuse=1)
    assert value_equal(a.state, b.state)
    if n >= 12:
        c = q.Register.from_int(n, 0)
        c.apply_gates(ops, fuse=1, tile_qubits=8)
        assert value_equal(a.state, c.state)


@pytest.mark.parametrize("arith", [1, 2])
def test_fused_fma_df64_within_tolerance(arith):
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister
    from quaru_gb300.workloads import flatten, layered_circuit

    n = 16
    ops = flatten(layered_circuit(n, 12, 4242)) + mixed_circuit(np.random.default_rng(5), n, 100)
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    g = q.Register.from_int(n, 0)
    g.set_arith(arith)
    g.apply_gates(ops, fuse=1)
    assert floored_rel_err(g.state, o.state) <= 1e-12


def test_fused_c64_within_tolerance():
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister
    from quaru_gb300.workloads import flatten, layered_circuit

    n = 15
    ops = flatten(layered_circuit(n, 10, 77))
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    g = q.Register.from_int(n, 0, precision=1)
    g.apply_gates(ops, fuse=1)
    assert floored_rel_err(g.state, o.state) <= 1e-4
    h = q.Register.from_int(n, 0, precision=1)
    h.apply_gates(ops, fuse=0)
    assert floored_rel_err(g.state, h.state) <= 1e-5


@pytest.mark.parametrize("n,tile", [(12, 12), (15, 9), (15, 12), (18, 13), (20, 12)])
def test_fused_c64_register_passes_full_gate_set(n, tile):
    """complex64 stages over the whole gate mix (Haar, H, X, Y, Z, phase, CNOT, SWAP, Toffoli,
    controlled-U, 0-controls, dense 2-qubit, a 6-qubit gate): register passes in the copy-warp kernel
    (common variants; 4096- and 8192-amplitude tiles) and in the general tile kernel (the rest)."""
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister
    from quaru_gb300 import operation as O
    from quaru_gb300.workloads import flatten, layered_circuit

    rng = np.random.default_rng(300 + n + tile)
    ops = flatten(layered_circuit(n, 3, 900 + n)) + mixed_circuit(rng, n, 250)
    ops += [O.hadamard(i) for i in range(n)] + [O.rz(0.1 * i + 0.05, i) for i in range(n)]
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    g = q.Register.from_int(n, 0, precision=1)
    g.apply_gates(ops, fuse=1, tile_qubits=tile)
    assert floored_rel_err(g.state, o.state) <= 1e-4
    h = q.Register.from_int(n, 0, precision=1)
    h.apply_gates(ops, fuse=0)
    assert floored_rel_err(g.state, h.state) <= 2e-5


@pytest.mark.parametrize("n,precision", [(9, 0), (11, 0), (12, 1), (11, 1)])
def test_fused_deep_circuit_on_a_single_tile(n, precision):
    """A circuit whose every gate fits one tile (n <= T): stages are capped in length, so the op
    tables stay within shared memory; results equal the gate-by-gate run."""
    import quaru_gb300 as q
    from quaru_gb300.workloads import flatten, layered_circuit

    ops = flatten(layered_circuit(n, 30, 31 + n))  # 30 layers: > 600 gates
    a = q.Register.from_int(n, 0, precision=precision)
    a.apply_gates(ops, fuse=0)
    b = q.Register.from_int(n, 0, precision=precision)
    b.apply_gates(ops, fuse=1)
    if precision == 0:
        assert value_equal(a.state, b.state)
    else:
        assert floored_rel_err(b.state, a.state) <= 5e-5


def test_fused_large_state_permutation_round_trip_bit_exact():
    """24 qubits: a permutation-and-phase circuit followed by its inverse restores the state exactly."""
    import quaru_gb300 as q
    from quaru_gb300 import operation as O

    n = 24
    rng = np.random.default_rng(9)
    ops = []
    for _ in range(200):
        a, b, c = (int(x) for x in rng.permutation(n)[:3])
        ops += [O.cnot(a, b), O.swap(b, c), O.cnx([a, c], b), O.pauli_y(c), O.not_(a)]
    inv = []
    for g in reversed(ops):
        inv.append(O.Operation(np.ascontiguousarray(np.asarray(g.matrix).conj().T), g.targets))
    reg = q.Register.from_int(n, 0)
    reg.apply_gates([O.hadamard(i) for i in range(n)] + [O.rz(0.3 * i, i) for i in range(n)], fuse=1)
    before = reg.state
    reg.apply_gates(ops + inv, fuse=1)
    assert value_equal(reg.state, before)


@pytest.mark.parametrize("n", [12, 14, 17])
def test_dense_block_fusion_tensor_cores_c64(n):
    """fuse=2 on complex64: 5-qubit blocks as 3xTF32 tensor-core GEMMs, FP32 accumulation."""
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister
    from quaru_gb300.workloads import flatten, layered_circuit

    ops = flatten(layered_circuit(n, 8, 500 + n)) + mixed_circuit(np.random.default_rng(n), n, 60)
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    for w in (5, 3):
        g = q.Register.from_int(n, 0, precision=1)
        g.apply_gates(ops, fuse=2, max_width=w)
        st = g.state
        assert floored_rel_err(st, o.state) <= 2e-5, w
        f = abs(np.vdot(st, o.state)) ** 2 / (np.vdot(st, st).real * np.vdot(o.state, o.state).real)
        assert 1 - f <= 1e-9, w


def test_dense_block_fusion_c128_and_small_registers():
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister

    for n, prec, tol in ((13, 0, 1e-12), (7, 1, 2e-5), (5, 0, 1e-12)):
        ops = mixed_circuit(np.random.default_rng(n + 7), n, 150)
        o = OracleRegister.from_int(n, 0)
        o.apply_sequence([(g.matrix, g.targets) for g in ops])
        g = q.Register.from_int(n, 0, precision=prec)
        g.set_arith(1)
        g.apply_gates(ops, fuse=2)
        assert floored_rel_err(g.state, o.state) <= tol, (n, prec)


@pytest.mark.parametrize("n", [12, 15])
def test_dense_block_fusion_c128_double_float(n):
    """fuse=2 on complex128 with double-float arithmetic: blocks of width 2 and 3 (the automatic width)
    through the double-float dense kernels, 4 through FP64; all within 1e-12 of the oracle."""
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister
    from quaru_gb300.workloads import flatten, layered_circuit

    ops = flatten(layered_circuit(n, 6, 600 + n)) + mixed_circuit(np.random.default_rng(n + 9), n, 80)
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    for w in (0, 2, 3, 4):
        g = q.Register.from_int(n, 0)
        g.set_arith(2)
        g.apply_gates(ops, fuse=2, max_width=w)
        assert floored_rel_err(g.state, o.state) <= 1e-12, w


def _floored_err_chunked(got: np.ndarray, ref: np.ndarray, chunk: int = 1 << 24) -> float:
    """floored_rel_err over large states, a chunk at a time (no state-sized temporaries)."""
    n = int(np.log2(ref.size))
    floor = 2.0 ** (-n / 2.0)
    worst = 0.0
    for i in range(0, ref.size, chunk):
        r = ref[i:i + chunk]
        worst = max(worst, float(np.max(np.abs(got[i:i + chunk] - r) / np.maximum(np.abs(r), floor))))
    return worst


def test_fusion_widths_at_28_qubits_match_unfused_fp64():
    """The benchmark's 28-qubit fusion-width configuration (40 layers for stages and 2- and 3-qubit
    blocks, 10 layers for 4- and 5-qubit blocks, double-float arithmetic as timed) against one FP64
    FMA sweep per gate on the same gates, within the 1e-12 floored bound."""
    import quaru_gb300 as q
    from quaru_gb300.workloads import flatten, layered_circuit, workload_seed

    n = 28
    refs = {}
    for layers in (40, 10):
        ops = flatten(layered_circuit(n, layers, workload_seed("layered_28q")))
        r = q.Register.from_int(n, 0)
        r.set_arith(q.QS_ARITH_FMA)
        r.apply_gates(ops, fuse=0)
        refs[layers] = (ops, r.state)
        del r
    for fuse, width, layers in [(1, 5, 40), (2, 2, 40), (2, 3, 40), (2, 4, 10), (2, 5, 10)]:
        ops, ref = refs[layers]
        g = q.Register.from_int(n, 0)
        g.set_arith(q.QS_ARITH_DF64)
        g.apply_gates(ops, fuse=fuse, max_width=width)
        err = _floored_err_chunked(g.state, ref)
        del g
        assert err <= 1e-12, (fuse, width, layers, err)
