"""FP64-accurate fused blocks on complex128 registers: fuse=2 under QS_ARITH_FX64 runs every block
of up to 5 qubits as a split-integer product on the BF16 tensor cores (k_tile_oz).

Bar: (1) on the layered Haar + CNOT family plus a mixed circuit at 12..17 qubits, at the automatic
width and at widths 3 and 5, the result stays within the 1e-12 floored-relative bound of the oracle
(the reference's FP64 operation order) and its largest deviation from the oracle is at most 4x that
of the unfused FP64 FMA form on the same gates; (2) states whose magnitudes span 30 decades, with
zeros and subnormal amplitudes; (3) non-finite amplitudes take the FP64 path (the same non-finite
positions as the FMA form, finite values close); (4) gates wider than a block (a 6-qubit
controlled permutation, a 6-qubit dense gate) run on their own between tensor-core stages.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.fixtures import floored_rel_err

pytestmark = pytest.mark.gpu

FX64, FMA = 3, 1


def _unitary(rng, k):
    d = 1 << k
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / math.sqrt(2)
    qm, r = np.linalg.qr(z)
    return qm * (np.diag(r) / np.abs(np.diag(r)))


def _circuit(n, seed, layers=8):
    from tests.test_gpu_fusion import mixed_circuit
    from quaru_gb300.workloads import flatten, layered_circuit

    return flatten(layered_circuit(n, layers, 700 + seed)) + mixed_circuit(np.random.default_rng(seed), n, 60)


@pytest.mark.parametrize("n", [12, 14, 17])
def test_oz_blocks_match_oracle_within_fma_error(n):
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister

    ops = _circuit(n, n)
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    f = q.Register.from_int(n, 0)
    f.set_arith(FMA)
    f.apply_gates(ops, fuse=0)
    fma_err = float(np.max(np.abs(f.state - o.state)))
    for w in (0, 3, 5):
        g = q.Register.from_int(n, 0)
        g.set_arith(FX64)
        g.apply_gates(ops, fuse=2, max_width=w)
        st = g.state
        assert floored_rel_err(st, o.state) <= 1e-12, w
        err = float(np.max(np.abs(st - o.state)))
        assert err <= max(4.0 * fma_err, 1e-15), (w, err, fma_err)


def test_oz_blocks_wide_dynamic_range_zeros_subnormals():
    """A state whose amplitudes span 30 decades (with exact zeros and subnormals) through one fused
    5-qubit block, against the FP64 FMA form of the same block, component by component: within
    2^-50 of the column's largest magnitude times the row's 1-norm."""
    import quaru_gb300 as q
    from quaru_gb300.operation import Operation

    n = 13
    rng = np.random.default_rng(41)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v *= 10.0 ** rng.uniform(-30, 0, size=v.size)
    u = _unitary(rng, 5)
    tq = [0, 3, 6, 9, 12]
    ops = [Operation(u, tq)]
    # column of each amplitude: its bits outside the block (the 2^8 assignments of the other qubits)
    other = [i for i in range(n) if i not in tq]
    idx = np.arange(1 << n)
    col = np.zeros(1 << n, dtype=np.int64)
    for k, bit in enumerate(other):
        col |= ((idx >> bit) & 1) << k
    v[7] = 0.0
    v[100] = 4e-318 + 1e-320j
    v[2049] = -0.0 + 2e-300j
    v[col == 5] = 0.0  # one all-zero column
    v[col == 9] *= 1e-300  # one column of tiny amplitudes, some subnormal
    g = q.Register.from_int(n, 0)
    g.set_arith(FX64)
    g.state = v
    g.apply_gates(ops, fuse=2)
    f = q.Register.from_int(n, 0)
    f.set_arith(FMA)
    f.state = v
    f.apply_gates(ops, fuse=0)
    a, b = g.state, f.state
    # per column of the block: bound by the column's largest component
    vmax = np.zeros(1 << len(other))
    np.maximum.at(vmax, col, np.maximum(np.abs(v.real), np.abs(v.imag)))
    bound = 2.0 ** -50 * vmax[col] * 2 * np.max(np.sum(np.abs(u), axis=1)) + 1e-320
    assert np.all(np.abs(a.real - b.real) <= bound)
    assert np.all(np.abs(a.imag - b.imag) <= bound)
    assert np.all(a[col == 5] == 0)  # the all-zero column stays exactly zero


def test_oz_blocks_nonfinite_take_fp64_path():
    import quaru_gb300 as q
    from quaru_gb300.operation import Operation

    n = 12
    rng = np.random.default_rng(5)
    v = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) / 64
    v[17] = np.inf
    v[1000] = complex(np.nan, 0.0)
    u = _unitary(rng, 5)
    ops = [Operation(u, [1, 2, 4, 8, 11])]
    g = q.Register.from_int(n, 0)
    g.set_arith(FX64)
    g.state = v
    g.apply_gates(ops, fuse=2)
    f = q.Register.from_int(n, 0)
    f.set_arith(FMA)
    f.state = v
    f.apply_gates(ops, fuse=0)
    a, b = g.state, f.state
    assert np.array_equal(np.isfinite(a), np.isfinite(b))
    fin = np.isfinite(b)
    assert np.max(np.abs(a[fin] - b[fin])) <= 1e-14


def test_oz_wide_gates_run_between_tensor_stages():
    import quaru_gb300 as q
    from oracle.oracle import OracleRegister
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation

    n = 13
    rng = np.random.default_rng(77)
    ops = []
    for i in range(n):
        ops.append(Operation(_unitary(rng, 1), [i]))
    ops.append(O.cnx([0, 2, 4, 6, 8], 12))  # 6-qubit controlled permutation
    for i in range(0, n, 2):
        ops.append(Operation(_unitary(rng, 1), [i]))
    ops.append(Operation(_unitary(rng, 6), [1, 3, 5, 7, 9, 11]))  # 6-qubit dense gate
    ops.append(O.cnx([1, 3, 5, 7, 9], 0))
    for i in range(n):
        ops.append(Operation(_unitary(rng, 1), [i]))
    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.matrix, g.targets) for g in ops])
    for prec, arith, tol in ((0, FX64, 1e-12), (1, FMA, 2e-5)):
        g = q.Register.from_int(n, 0, precision=prec)
        g.set_arith(arith)
        g.apply_gates(ops, fuse=2)
        assert floored_rel_err(g.state, o.state) <= tol, prec


def test_oz_blocks_28_qubits_match_unfused_fp64():
    """The benchmark's 28-qubit width configuration (10 layers of the layered family) as FP64-accurate
    5-qubit tensor-core blocks against one FP64 FMA sweep per gate, within the 1e-12 floored bound."""
    import quaru_gb300 as q
    from quaru_gb300.workloads import flatten, layered_circuit, workload_seed
    from tests.test_gpu_fusion import _floored_err_chunked

    n = 28
    ops = flatten(layered_circuit(n, 10, workload_seed("layered_28q")))
    r = q.Register.from_int(n, 0)
    r.set_arith(FMA)
    r.apply_gates(ops, fuse=0)
    ref = r.state
    del r
    g = q.Register.from_int(n, 0)
    g.set_arith(FX64)
    g.apply_gates(ops, fuse=2, max_width=5)
    err = _floored_err_chunked(g.state, ref)
    assert err <= 1e-12, err
