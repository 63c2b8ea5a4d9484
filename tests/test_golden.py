"""The committed golden fixture of the 12-qubit parity circuit, replayed on the oracle (CPU) and on the GPU engine."""
from __future__ import annotations

import numpy as np
import pytest

from tests.fixtures import floored_rel_err, golden_state, load_parity_golden, sha, value_equal


def test_oracle_reproduces_golden(oracle_mod):
    doc, gates, draws = load_parity_golden()
    reg = oracle_mod.OracleRegister.from_int(doc["n"], 0)
    reg.apply_sequence([(g.matrix, g.targets) for g in gates])
    assert sha(reg.state) == doc["sha256_after_gates"]
    assert value_equal(reg.state, golden_state())
    bits = [int(reg.measure(q, draws[q])) for q in range(doc["n"])]
    assert bits == doc["bitstring"]
    assert sha(reg.state) == doc["sha256_after_measure"]


@pytest.mark.gpu
def test_gpu_matches_golden_bit_exact():
    import quaru_gb300 as q

    doc, gates, draws = load_parity_golden()
    reg = q.Register.from_int(doc["n"], 0)
    for g in gates:  # one try_apply_fast call per gate, the reference's path
        reg.try_apply_fast(g)
    st = reg.state
    assert value_equal(st, golden_state())
    assert sha(st) == doc["sha256_after_gates"]
    bits = []
    for qb in range(doc["n"]):
        bits.append(int(reg.measure(qb, draws[qb])))
        p0, p1 = reg.last_probs
        r0, r1 = (float.fromhex(x) for x in doc["measure_probs"][qb])
        assert p0 == r0 and p1 == r1  # sequential sums in the reference's order
    assert bits == doc["bitstring"]
    assert sha(reg.state) == doc["sha256_after_measure"]  # the collapsed state, bit for bit


@pytest.mark.gpu
def test_gpu_measure_sequence_matches_golden_bit_exact():
    import quaru_gb300 as q

    doc, gates, draws = load_parity_golden()
    reg = q.Register.from_int(doc["n"], 0)
    reg.apply_gates(gates)
    bits = reg.measure_sequence(list(range(doc["n"])), draws)
    assert [int(b) for b in bits] == doc["bitstring"]
    assert sha(reg.state) == doc["sha256_after_measure"]


@pytest.mark.gpu
@pytest.mark.parametrize("fuse", [0, 1])
def test_gpu_circuit_call_matches_golden(fuse):
    import quaru_gb300 as q

    doc, gates, _ = load_parity_golden()
    reg = q.Register.from_int(doc["n"], 0)
    reg.apply_gates(gates, fuse=fuse)
    assert value_equal(reg.state, golden_state())


@pytest.mark.gpu
def test_gpu_fma_and_c64_within_tolerance():
    import quaru_gb300 as q

    doc, gates, _ = load_parity_golden()
    ref = golden_state()
    reg = q.Register.from_int(doc["n"], 0)
    reg.set_arith(q.QS_ARITH_FMA)
    reg.apply_gates(gates)
    assert floored_rel_err(reg.state, ref) <= 1e-12
    rdf = q.Register.from_int(doc["n"], 0)
    rdf.set_arith(q.QS_ARITH_DF64)
    rdf.apply_gates(gates)
    assert floored_rel_err(rdf.state, ref) <= 1e-12
    r64 = q.Register.from_int(doc["n"], 0, precision=q.QS_PREC_C64)
    r64.apply_gates(gates)
    assert floored_rel_err(r64.state, ref) <= 1e-4
