"""Observables and adjoint gradients on the GPU.

Checks: <a|b> and <psi|H|psi> against numpy; adjoint gradients against
central finite differences (h = 1e-6, FP64) and the parameter-shift rule
(E(theta + pi/2) - E(theta - pi/2)) / 2, to 1e-6; complex64 (mixed) gradients
against FP64 gradients; the register's state is unchanged by a gradient call.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rand_state(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def pauli_apply(psi, x, z):
    """numpy reference: (P psi)_i = i^{|x&z|} (-1)^{|z & (i^x)|} psi_{i^x}."""
    idx = np.arange(psi.size)
    j = idx ^ x
    sign = np.array([(-1) ** bin(z & int(v)).count("1") for v in j])
    return (1j ** bin(x & z).count("1")) * sign * psi[j]


def energy_np(psi, terms):
    return float(np.real(sum(c * np.vdot(psi, pauli_apply(psi, x, z)) for c, x, z in terms)))


def test_inner_product_and_fidelity():
    import quaru_gb300 as q

    rng = np.random.default_rng(1)
    n = 12
    a, b = rand_state(rng, n), rand_state(rng, n)
    ra, rb = q.Register.from_int(n, 0), q.Register.from_int(n, 0)
    ra.state, rb.state = a, b
    assert abs(ra.inner_product(rb) - np.vdot(a, b)) < 1e-13
    r64 = q.Register.from_int(n, 0, precision=1)
    r64.state = a
    f = abs(r64.inner_product(ra)) ** 2 / (r64.inner_product(r64).real * ra.inner_product(ra).real)
    assert abs(1 - f) < 1e-12


def test_expval_pauli_matches_numpy():
    import quaru_gb300 as q

    rng = np.random.default_rng(2)
    n = 10
    psi = rand_state(rng, n)
    terms = [(float(rng.normal()), int(rng.integers(1 << n)), int(rng.integers(1 << n))) for _ in range(12)]
    terms += [(0.7, 0, 0b11), (-1.3, 0b100, 0), (0.25, 0b1000, 0b1000)]
    reg = q.Register.from_int(n, 0)
    reg.state = psi
    assert abs(reg.expval_pauli(terms) - energy_np(psi, terms)) < 1e-12


def test_expval_pauli_complex64_matches_numpy():
    """complex64 state: H|psi> summed on the FP32 pipe in compensated float pairs and rounded once to
    float, so <psi|H|psi> is within a few float roundings of lambda of the FP64 value."""
    import quaru_gb300 as q

    rng = np.random.default_rng(3)
    n = 11
    psi = rand_state(rng, n).astype(np.complex64).astype(np.complex128)
    terms = [(float(rng.normal()), int(rng.integers(1 << n)), int(rng.integers(1 << n))) for _ in range(40)]
    terms += [(0.7, 0, 0b11), (-1.3, 0b100, 0), (0.25, 0b1000, 0b1000), (1e-3, 0b110, 0b011)]
    reg = q.Register.from_int(n, 0, precision=1)
    reg.state = psi
    bound = 4 * 2.0 ** -24 * sum(abs(c) for c, _, _ in terms)
    assert abs(reg.expval_pauli(terms) - energy_np(psi, terms)) < bound


def energy_gpu(q, n, gates, params, terms, precision=0):
    reg = q.Register.from_int(n, 0, precision=precision)
    reg.set_arith(1)
    reg.apply_gates([g.operation(params) for g in gates])
    return reg.expval_pauli(terms)


@pytest.mark.parametrize("n,layers", [(5, 3), (8, 2)])
def test_adjoint_matches_finite_differences_and_shift(n, layers):
    import quaru_gb300 as q
    from quaru_gb300.workloads import ansatz, chain_hamiltonian, SplitMix64

    rng = SplitMix64(77 + n)
    gates, npar = ansatz(n, layers)
    params = np.array([2 * math.pi * rng.uniform() for _ in range(npar)])
    terms = chain_hamiltonian(n, rng) + [(0.4, 0b11, 0b01)]  # a Y X term as well
    reg = q.Register.from_int(n, 0)
    before = reg.state
    e, grad = reg.adjoint_gradient(gates, params, terms)
    assert np.array_equal(reg.state, before)
    # energy against the oracle's forward run
    from oracle.oracle import OracleRegister

    o = OracleRegister.from_int(n, 0)
    o.apply_sequence([(g.operation(params).matrix, g.operation(params).targets) for g in gates])
    assert abs(e - energy_np(o.state, terms)) < 1e-11
    h = 1e-6
    for p in range(npar):
        pp, pm = params.copy(), params.copy()
        pp[p] += h
        pm[p] -= h
        fd = (energy_gpu(q, n, gates, pp, terms) - energy_gpu(q, n, gates, pm, terms)) / (2 * h)
        pp[p] = params[p] + math.pi / 2
        pm[p] = params[p] - math.pi / 2
        ps = (energy_gpu(q, n, gates, pp, terms) - energy_gpu(q, n, gates, pm, terms)) / 2
        assert abs(grad[p] - fd) < 1e-6, (p, grad[p], fd)
        assert abs(grad[p] - ps) < 1e-9, (p, grad[p], ps)


@pytest.mark.parametrize("n,precision,arith", [(7, 0, 1), (8, 1, 1), (9, 0, 2), (11, 0, 1), (13, 0, 1), (12, 1, 1),
                                               (12, 0, 2), (14, 0, 2), (17, 1, 1), (18, 0, 2)])
def test_adjoint_tiled_mixed_gates(n, precision, arith):
    """n >= 6: forward as fused stages and the reverse sweep as tiled stages (one tile holding the whole
    state up to 8 qubits, 8-qubit tiles at 11-15, 10 at 17; at 18 qubits the double-float forward
    runs as 3-qubit dense blocks). RX/RY/RZ mixed with
    fixed gates of every kind the tiles hold (H, S, CZ, CNOT, Toffoli, controlled rotation) and one
    they do not (a dense 2-qubit unitary: its own sweeps), one parameter shared by three rotations;
    every parameter against central differences, and against parameter shift where that is exact.
    arith = 2 (DF64) runs the stages whose fixed gates are pure moves in double-float tiles."""
    import quaru_gb300 as q
    from quaru_gb300 import operation as O
    from quaru_gb300.register import ParamGate
    from quaru_gb300.workloads import SplitMix64, chain_hamiltonian

    rng = SplitMix64(500 + n)
    nrng = np.random.default_rng(n)
    gates, npar = [], 0
    for layer in range(3):
        for qb in range(n):
            k = (qb + layer) % 3
            mk = (ParamGate.rx, ParamGate.ry, ParamGate.rz)[k]
            gates.append(mk(qb, npar))
            npar += 1
        a, b, c = (int(x) for x in nrng.permutation(n)[:3])
        gates += [ParamGate.fixed(O.hadamard(a)), ParamGate.fixed(O.phase(b)), ParamGate.fixed(O.cnz([a], b)),
                  ParamGate.fixed(O.cnot(b, c)), ParamGate.fixed(O.cnx([a, b], c)),
                  ParamGate.fixed(O.to_controlled(O.Operation(np.array([[0.6, 0.8j], [0.8j, 0.6]]), [c]), a))]
        z = nrng.normal(size=(4, 4)) + 1j * nrng.normal(size=(4, 4))
        gates.append(ParamGate.fixed(O.Operation(np.linalg.qr(z)[0], [a, c])))
    shared = npar  # one parameter used by three rotations: its gradient is their sum
    gates += [ParamGate.ry(0, shared), ParamGate.rx(n // 2, shared), ParamGate.rz(n - 1, shared)]
    npar += 1
    params = np.array([2 * math.pi * rng.uniform() for _ in range(npar)])
    terms = chain_hamiltonian(n, rng) + [(0.3, 0b101, 0b100)]
    reg = q.Register.from_int(n, 0, precision=precision)
    reg.set_arith(arith)
    before = reg.state
    e, grad = reg.adjoint_gradient(gates, params, terms)
    assert np.array_equal(reg.state, before)
    tol_ps, tol_fd = (1e-9, 1e-6) if precision == 0 else (2e-4, 2e-4)
    for p in range(npar):
        pp, pm = params.copy(), params.copy()
        if p != shared:  # the shift rule is exact for a parameter of a single rotation
            pp[p] += math.pi / 2
            pm[p] -= math.pi / 2
            ps = (energy_gpu(q, n, gates, pp, terms) - energy_gpu(q, n, gates, pm, terms)) / 2
            assert abs(grad[p] - ps) < tol_ps, (p, grad[p], ps)
        pp[p], pm[p] = params[p] + 1e-6, params[p] - 1e-6
        fd = (energy_gpu(q, n, gates, pp, terms) - energy_gpu(q, n, gates, pm, terms)) / 2e-6
        assert abs(grad[p] - fd) < tol_fd, (p, grad[p], fd)


def test_param_circuit_and_pauli_sum_match_plain_lists():
    """ParamCircuit / PauliSum (records converted once) give the same energy and gradient as lists."""
    import quaru_gb300 as q
    from quaru_gb300.workloads import ansatz_problem

    gates, params, terms = ansatz_problem(n=12, layers=3)
    for precision in (0, 1):
        reg = q.Register.from_int(12, 0, precision=precision)
        e1, g1 = reg.adjoint_gradient(gates, params, terms)
        e2, g2 = reg.adjoint_gradient(q.ParamCircuit(gates), params, q.PauliSum(terms))
        assert e1 == e2 and np.array_equal(g1, g2)


def test_adjoint_20_qubit_ansatz_fp64_and_mixed():
    """20 qubits, 10 layers, 400 parameters: spot-check 6 parameters by parameter shift and central
    differences; the complex64 (mixed) gradient agrees with FP64 to 1e-4 and its state has 1 - F <= 1e-6."""
    import quaru_gb300 as q
    from quaru_gb300.workloads import ansatz_problem

    gates, params, terms = ansatz_problem()
    params = np.array(params)
    n = 20
    reg = q.Register.from_int(n, 0)
    e, grad = reg.adjoint_gradient(gates, params, terms)
    r64 = q.Register.from_int(n, 0, precision=1)
    e64, grad64 = r64.adjoint_gradient(gates, params, terms)
    assert np.max(np.abs(grad64 - grad)) < 1e-4
    assert abs(e64 - e) < 1e-4
    for p in (0, 57, 133, 200, 321, 399):
        pp, pm = params.copy(), params.copy()
        pp[p] += math.pi / 2
        pm[p] -= math.pi / 2
        ps = (energy_gpu(q, n, gates, pp, terms) - energy_gpu(q, n, gates, pm, terms)) / 2
        assert abs(grad[p] - ps) < 1e-9
        pp[p], pm[p] = params[p] + 1e-6, params[p] - 1e-6
        fd = (energy_gpu(q, n, gates, pp, terms) - energy_gpu(q, n, gates, pm, terms)) / 2e-6
        assert abs(grad[p] - fd) < 1e-6
    # fidelity of the mixed forward state
    a = q.Register.from_int(n, 0)
    a.set_arith(1)
    a.apply_gates([g.operation(params) for g in gates])
    b = q.Register.from_int(n, 0, precision=1)
    b.apply_gates([g.operation(params) for g in gates])
    f = abs(b.inner_product(a)) ** 2 / (a.inner_product(a).real * b.inner_product(b).real)
    assert 1 - f <= 1e-6


def test_adjoint_rejects_bad_gates():
    import quaru_gb300 as q
    from quaru_gb300 import ParamGate

    reg = q.Register.from_int(3, 0)
    with pytest.raises(q.OperationError) as e:
        reg.adjoint_gradient([ParamGate.ry(5, 0)], [0.1], [(1.0, 0, 1)])
    assert e.value.kind == "InvalidTarget" and e.value.payload == (5,)
    with pytest.raises(q.EngineError):
        reg.adjoint_gradient([ParamGate.ry(0, 3)], [0.1], [(1.0, 0, 1)])
    with pytest.raises(q.EngineError):  # a Pauli term on qubit 3 of a 3-qubit register
        reg.adjoint_gradient([ParamGate.ry(0, 0)], [0.1], [(1.0, 0b1000, 0)])
    with pytest.raises(q.EngineError):
        reg.expval_pauli([(1.0, 0, 0b10000)])
