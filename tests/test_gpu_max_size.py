"""Registers past 2^31 and 2^32 amplitudes: the largest states one GB300 holds.

No CPU oracle can follow states of 32 and 33 qubits, so these tests check properties that do not
depend on the size: single-qubit marginals of basis states are exactly 0 or 1; H on the top qubit
splits it evenly; measuring collapses the other qubits back to exact 0/1 marginals; a circuit
followed by its inverse returns to the basis state it started from (fused forward, unfused or
differently fused inverse, so the two paths check each other: register passes, 3xTF32 and
FP64-accurate tensor-core blocks, FMA and double-float tiles, single sweeps); a product state's
marginals are |b_q|^2. Every amplitude index above bit 31 goes through the kernels' 64-bit index
arithmetic.
Each test skips when the GPU has less free memory than its state needs.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def q():
    import quaru_gb300

    return quaru_gb300


def need_bytes(nbytes: int) -> None:
    import torch

    free, _ = torch.cuda.mem_get_info()
    if free < nbytes + (8 << 30):
        pytest.skip(f"needs {nbytes / 2**30:.0f} GiB of free device memory, {free / 2**30:.0f} GiB free")


def marginals(q, reg, norms: list | None = None) -> np.ndarray:
    """p1 / (p0 + p1) of every qubit from try_measure's two probability sums
    (qs_measure_probabilities, one reduction sweep per qubit); p0 + p1 appended to `norms`."""
    lib = q._lib.load()
    out = np.zeros(reg.size())
    p0, p1 = ctypes.c_double(0), ctypes.c_double(0)
    for t in range(reg.size()):
        rc = lib.qs_measure_probabilities(reg.handle, t, ctypes.byref(p0), ctypes.byref(p1), None)
        assert rc == 0
        out[t] = p1.value / (p0.value + p1.value)
        if norms is not None:
            norms.append(p0.value + p1.value)
    return out


def bits_of(k: int, n: int) -> np.ndarray:
    return np.array([(k >> i) & 1 for i in range(n)], dtype=float)


def inverse(ops):
    from quaru_gb300.operation import Operation

    return [Operation(np.conj(np.asarray(o.matrix)).T.copy(), list(o.targets)) for o in reversed(ops)]


def test_basis_measure_collapse_33_qubits_c64(q):
    """complex64, 33 qubits (64 GiB): amplitude indices use bit 32."""
    from quaru_gb300 import operation as O

    n = 33
    need_bytes(8 << n)
    k = (1 << 32) | (1 << 31) | (1 << 17) | 5
    r = q.Register.from_int(n, k, precision=q.QS_PREC_C64)
    assert np.array_equal(marginals(q, r), bits_of(k, n))
    r.try_apply_fast(O.hadamard(32))
    r.try_apply_fast(O.cnot(32, 0))  # qubit 0 follows qubit 32: (|..1> + |..0>) pairs
    m = marginals(q, r)
    # H halves |a|^2 exactly: both branches hold the same float magnitudes
    assert m[32] == 0.5 and m[0] == 0.5
    rest = [i for i in range(n) if i not in (0, 32)]
    assert np.array_equal(m[rest], bits_of(k, n)[rest])
    # draw above p0 -> outcome 1 (src/register.rs:321); the collapse zeroes the qubit-32 = 0 half,
    # where qubit 0 is 1
    assert r.measure(32, 0.9) is True
    m = marginals(q, r)
    assert m[32] == 1.0 and m[0] == 0.0
    assert np.array_equal(m[rest], bits_of(k, n)[rest])


@pytest.mark.parametrize("fwd_fuse,inv_fuse", [(1, 0), (2, 1)])
def test_circuit_and_inverse_33_qubits_c64(q, fwd_fuse, inv_fuse):
    """complex64, 33 qubits: a layered circuit (Haar on every qubit + CNOT matching) and its
    inverse, in register passes, 3xTF32 blocks and single sweeps."""
    from quaru_gb300.workloads import flatten, layered_circuit

    n = 33
    need_bytes(8 << n)
    k = (1 << 32) | 0x2A5A5
    ops = flatten(layered_circuit(n, 2, 4100 + fwd_fuse))
    r = q.Register.from_int(n, k, precision=q.QS_PREC_C64)
    r.apply_gates(ops, fuse=fwd_fuse)
    m = marginals(q, r)
    assert np.all((m > 1e-4) & (m < 1 - 1e-4))  # the circuit entangles every qubit
    r.apply_gates(inverse(ops), fuse=inv_fuse)
    assert np.max(np.abs(marginals(q, r) - bits_of(k, n))) < 2e-5


@pytest.mark.parametrize("arith", [1, 2])
def test_circuit_and_inverse_32_qubits_c128(q, arith):
    """complex128, 32 qubits (64 GiB): forward fused (FMA tiles or DF64 tiles), inverse as
    single sweeps; FP64-level agreement."""
    from quaru_gb300.workloads import flatten, layered_circuit

    n = 32
    need_bytes(16 << n)
    k = (1 << 31) | (1 << 30) | 0x1234
    ops = flatten(layered_circuit(n, 2, 4200 + arith))
    r = q.Register.from_int(n, k)
    r.set_arith(arith)
    r.apply_gates(ops, fuse=1)
    m = marginals(q, r)
    assert np.all((m > 1e-4) & (m < 1 - 1e-4))
    r.apply_gates(inverse(ops), fuse=0)
    norms: list = []
    assert np.max(np.abs(marginals(q, r, norms) - bits_of(k, n))) < 1e-11
    assert max(abs(x - 1.0) for x in norms) < 1e-12


def test_fixed_point_blocks_and_inverse_32_qubits_c128(q):
    """complex128, 32 qubits: the FP64-accurate tensor-core blocks (fixed-point arithmetic, fuse = 2:
    one 5-qubit block per 12-qubit tile stage, tile indices past bit 19, amplitude indices past bit
    31), inverse as fixed-point single sweeps; FP64-level agreement."""
    from quaru_gb300.workloads import flatten, layered_circuit

    n = 32
    need_bytes(16 << n)
    k = (1 << 31) | (1 << 29) | 0x4321
    ops = flatten(layered_circuit(n, 2, 4300))
    r = q.Register.from_int(n, k)
    r.set_arith(q.QS_ARITH_FX64)
    r.apply_gates(ops, fuse=2, max_width=5)
    m = marginals(q, r)
    assert np.all((m > 1e-4) & (m < 1 - 1e-4))
    r.apply_gates(inverse(ops), fuse=0)
    norms: list = []
    assert np.max(np.abs(marginals(q, r, norms) - bits_of(k, n))) < 1e-11
    assert max(abs(x - 1.0) for x in norms) < 1e-12


def test_product_state_32_qubits_c128(q):
    """try_from_qubits at 32 qubits: marginals are |b_q|^2 of each qubit's (a_q, b_q)."""
    n = 32
    need_bytes(16 << n)
    rng = np.random.default_rng(32)
    qubits, p1 = [], []
    for _ in range(n):
        v = rng.normal(size=2) + 1j * rng.normal(size=2)
        v /= np.linalg.norm(v)
        qubits.append(v.reshape(2, 1))
        p1.append(abs(v[1]) ** 2)
    r = q.Register.try_from_qubits(qubits)
    norms: list = []
    assert np.max(np.abs(marginals(q, r, norms) - np.array(p1))) < 1e-12
    assert max(abs(x - 1.0) for x in norms) < 1e-12
