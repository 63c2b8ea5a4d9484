"""QuantumCircuit / apply_circuit and the OpenQASM front end.

Parse errors are raised before any device work, so those checks run on the
CPU; running programs needs the GPU.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

BELL = """OPENQASM 2.0;
// a Hadamard built from U, then CX
gate hh a { U(pi / 2, 0, pi) a; }
qreg q[3];
creg c[3];
hh q[0];
CX q[0], q[1];
"""


def test_parse_errors_are_reported_before_device_work():
    from quaru_gb300.openqasm import OpenQASMError, run_openqasm_source

    bad = {
        "OPENQASM 2.0;\nqreg q[2];\nfoo q[0];\n": "unknown gate",
        "OPENQASM 2.0;\nqreg q[2];\nU(0,0) q[0];\n": "U takes",
        "OPENQASM 2.0;\nqreg q[2];\nCX q[0] q[1];\n": "expected ';'",
        "OPENQASM 3.0;\n": "only OpenQASM 2",
        "OPENQASM 2.0;\nqreg q[2];\nmeasure q[0] -> c[0];\n": "unknown classical register",
        "OPENQASM 2.0;\nqreg q[2];\nU(0,0,0) q[5];\n": "out of range",
        "OPENQASM 2.0;\nqreg q[2];\ngate g(a) x { U(a, b, 0) x; }\ng(1) q[0];\n": "unknown parameter",
    }
    for src, needle in bad.items():
        with pytest.raises(OpenQASMError) as e:
            run_openqasm_source(src)
        assert e.value.kind == "OpenQASMParseError" and needle in str(e.value), (src, str(e.value))


def test_circuit_builder_rules():
    from quaru_gb300 import operation as O
    from quaru_gb300.circuit import QuantumCircuit

    c = QuantumCircuit()
    c.add_operation(O.hadamard(0))
    c.add_measurement(0)
    with pytest.raises(RuntimeError):
        c.add_operation(O.not_(0))
    with pytest.raises(RuntimeError):
        c.add_measurement(0)
    with pytest.raises(RuntimeError):
        c.add_conditional_operation(O.not_(1), [(2, True)])
    c.add_conditional_operation(O.not_(1), [(0, True)])
    with pytest.raises(RuntimeError):
        c.add_operation(O.not_(2))


def test_reduction_passes_match_reference_behaviour():  # src/operation.rs:600-651
    from quaru_gb300 import operation as O
    from quaru_gb300.circuit import QuantumCircuit

    c = QuantumCircuit()
    for op in (O.hadamard(0), O.cnot(0, 1), O.cnot(0, 1), O.hadamard(0)):
        c.add_operation(op)
    assert len(c.reduce_circuit_cancel_gates().get_operations()) == 0
    c = QuantumCircuit()
    c.add_operation(O.hadamard(0))
    c.add_operation(O.not_(0))
    assert len(c.reduce_circuit_gates_with_same_targets().get_operations()) == 1
    c = QuantumCircuit()
    c.add_operation(O.hadamard(0))
    c.add_operation(O.hadamard(0))
    assert len(c.reduce_circuit_cancel_gates().get_operations()) == 0


def test_combining_overlapping_gates():  # src/operation.rs:114-178
    from quaru_gb300 import operation as O
    from quaru_gb300.circuit import QuantumCircuit

    # a 1-qubit gate followed by an overlapping 2-qubit gate: one 4x4 operation on the larger
    # gate's targets, equal to applying the two in circuit order
    c = QuantumCircuit()
    c.add_operation(O.hadamard(0))
    c.add_operation(O.cnot(0, 1))
    ops = c.reduce_gates_with_one_off_size(2).get_operations()
    assert len(ops) == 1 and list(ops[0].targets) == [1, 0]
    h = np.array(O.hadamard(0).matrix)
    want = np.array(O.cnot(0, 1).matrix) @ np.kron(h, np.eye(2))
    assert np.allclose(ops[0].matrix, want, atol=0)
    # overlapping gates of equal arity cannot be combined: the reference's combine_ops multiplies a
    # 4x4 by an 8x8 matrix and ndarray panics; here it raises
    for second in (O.cnot(1, 2), O.swap(0, 1)):
        c = QuantumCircuit()
        c.add_operation(O.cnot(0, 1))
        c.add_operation(second)
        with pytest.raises(RuntimeError, match="equal arity"):
            c.reduce_gates_with_one_off_size(2)


@pytest.mark.gpu
def test_bell_program_and_broadcast():
    from quaru_gb300.openqasm import run_openqasm_source

    r = run_openqasm_source(BELL)
    p = r.qregs["q"].probabilities()
    # angles pass through f32 as in the reference (src/openqasm.rs:98), so pi/2 is off by ~4e-8
    assert abs(p[0] - 0.5) < 1e-7 and abs(p[3] - 0.5) < 1e-7 and abs(p.sum() - 1) < 1e-12
    assert r.cregs["c"] == [False, False, False]
    # qelib1 gates, broadcasting over a register, measurement into a register
    src = 'OPENQASM 2.0;\ninclude "qelib1.inc";\nqreg a[4];\ncreg m[4];\nx a;\nmeasure a -> m;\n'
    r = run_openqasm_source(src)
    assert r.cregs["m"] == [True] * 4


@pytest.mark.gpu
def test_teleportation_program_with_conditionals():
    """Teleports U(theta, phi, 0)|0> from q[0] to q[2] with if(...) corrections, for many seeds."""
    from quaru_gb300.openqasm import run_openqasm_source

    th, ph = 1.1, 0.4
    src = f"""OPENQASM 2.0;
include "qelib1.inc";
qreg q[3];
creg c0[1];
creg c1[1];
U({th}, {ph}, 0) q[0];
h q[1];
cx q[1], q[2];
cx q[0], q[1];
h q[0];
measure q[0] -> c0[0];
measure q[1] -> c1[0];
if(c1 == 1) x q[2];
if(c0 == 1) z q[2];
"""
    thf, phf = float(np.float32(th)), float(np.float32(ph))
    want = np.array([math.cos(thf / 2), complex(math.cos(phf), math.sin(phf)) * math.sin(thf / 2)])
    for seed in range(12):
        r = run_openqasm_source(src, seed=seed)
        st = r.qregs["q"].state
        b = (1 if r.cregs["c0"][0] else 0) | (2 if r.cregs["c1"][0] else 0)
        amp = np.array([st[b], st[b | 4]])
        assert abs(abs(np.vdot(amp, want)) - 1) < 1e-9


@pytest.mark.gpu
def test_run_errors_and_reset():
    from quaru_gb300.openqasm import OpenQASMError, run_openqasm_source

    with pytest.raises(OpenQASMError) as e:
        run_openqasm_source("OPENQASM 2.0;\nqreg a[1];\nqreg b[1];\nCX a[0], b[0];\n")
    assert e.value.kind == "OpenQASMRunError"
    r = run_openqasm_source('OPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\ncreg c[2];\nx q;\n'
                            'measure q -> c;\nreset q;\nreset c;\n')
    assert r.cregs["c"] == [False, False]
    assert abs(r.qregs["q"].state[0] - 1) < 1e-15


@pytest.mark.gpu
def test_apply_circuit_teleportation_circuit():  # examples/quantum_teleportation.rs:100-119
    import quaru_gb300 as q
    from quaru_gb300 import operation as O
    from quaru_gb300.circuit import QuantumCircuit

    rng = np.random.default_rng(3)
    for fuse in (0, 1):
        for _ in range(10):
            theta, phi = rng.uniform(0, math.pi), rng.uniform(0, 2 * math.pi)
            q0 = np.array([math.cos(theta / 2), math.sin(theta / 2) * complex(math.cos(phi), math.sin(phi))])
            reg = q.Register.new([False] * 3, rng=rng.random)
            reg.state = np.kron(np.kron([1, 0], [1, 0]), q0)
            circ = QuantumCircuit()
            for op in (O.hadamard(2), O.cnot(2, 1), O.cnot(0, 1), O.hadamard(0)):
                circ.add_operation(op)
            circ.add_measurement(1)
            circ.add_measurement(0)
            circ.add_conditional_operation(O.not_(2), [(1, True)])
            circ.add_conditional_operation(O.pauli_z(2), [(0, True)])
            circ.reduce_circuit_cancel_gates()
            circ.reduce_circuit_gates_with_same_targets()
            res = reg.apply_circuit(circ, fuse=fuse)
            assert [t for t, _ in res] == [1, 0]
            st = reg.state
            a = sum(s for i, s in enumerate(st) if not (i >> 2) & 1)
            b = sum(s for i, s in enumerate(st) if (i >> 2) & 1)
            norm = math.sqrt(abs(a) ** 2 + abs(b) ** 2)
            assert np.all(np.abs(np.array([a, b]) / norm - q0) < 1e-8)
