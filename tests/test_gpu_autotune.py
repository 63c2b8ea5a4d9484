"""The fusion autotuner (qs_circuit_autotune) and qs_apply_circuit with autotuned options.

Bar: the tuner times every candidate of its mode and keeps the fastest; a second query returns the
cached choice; circuits run with the tuned options give the oracle's result (bit for bit under
QS_ARITH_EXACT for single sweeps and stages, within 1e-12 floored for dense blocks and the other
forms); QS_AUTOTUNE=off takes the fixed rules.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from tests.fixtures import floored_rel_err, value_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,arith", [(0, 0), (0, 1), (0, 2), (0, 3), (1, 1)])
def test_tuner_times_every_candidate_and_keeps_the_fastest(prec, arith):
    import quaru_gb300 as q

    n = 13
    rep = q.circuit_autotune(n, prec, arith, 3, retune=True)
    c = rep["candidates"]
    kinds = {x["fuse"] for x in c}
    assert kinds == {0, 1, 2} and len(c) >= 6
    best = min(c, key=lambda x: x["ms"])
    assert (rep["fuse"], rep["max_width"], rep["tile_qubits"]) == (best["fuse"], best["max_width"], best["tile_qubits"])
    again = q.circuit_autotune(n, prec, arith, 3)
    assert again["from_cache"] and again["candidates"] == []
    assert (again["fuse"], again["max_width"], again["tile_qubits"]) == (rep["fuse"], rep["max_width"], rep["tile_qubits"])
    for mode, kind in ((1, {1}), (2, {2})):
        r = q.circuit_autotune(n, prec, arith, mode, retune=True)
        assert {x["fuse"] for x in r["candidates"]} == kind and r["fuse"] in kind


@pytest.mark.parametrize("arith", [0, 1, 2, 3])
def test_autotuned_circuits_match_the_oracle(arith):
    import quaru_gb300 as q
    from oracle import oracle
    from quaru_gb300.workloads import flatten, layered_circuit, parity_circuit

    for n, ops in ((12, parity_circuit().gates), (14, flatten(layered_circuit(14, 6, 77)))):
        o = oracle.OracleRegister.from_int(n, 0)
        for op in ops:
            o.try_apply_fast(op.matrix, op.targets)
        for fuse in (1, 2, 3):
            g = q.Register.from_int(n, 0)
            g.set_arith(arith)
            g.apply_gates(ops, fuse=fuse)
            choice = q.circuit_autotune(n, 0, arith, fuse)
            if arith == 0 and choice["fuse"] in (0, 1):
                assert value_equal(g.state, o.state), (n, fuse, choice)
            else:
                assert floored_rel_err(g.state, o.state) <= 1e-12, (n, fuse, choice)


def test_autotune_off_uses_the_fixed_rules():
    import quaru_gb300 as q
    from oracle import oracle
    from quaru_gb300.workloads import parity_circuit

    c = parity_circuit()
    o = oracle.OracleRegister.from_int(c.n, 0)
    for op in c.gates:
        o.try_apply_fast(op.matrix, op.targets)
    os.environ["QS_AUTOTUNE"] = "off"
    try:
        g = q.Register.from_int(c.n, 0)
        g.apply_gates(c.gates, fuse=3)  # stages at the automatic tile size: bit-exact under EXACT
        assert value_equal(g.state, o.state)
    finally:
        del os.environ["QS_AUTOTUNE"]


def test_autotune_rejects_bad_arguments():
    import quaru_gb300 as q

    for args in ((0, 0, 1, 3), (12, 5, 1, 3), (12, 0, 9, 3), (12, 0, 1, 0), (12, 0, 1, 4)):
        with pytest.raises(q.EngineError):
            q.circuit_autotune(*args)
