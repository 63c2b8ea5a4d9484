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
        reg.set_arith(q.QS_ARITH_FMA)
        e, g = reg.adjoint_gradient(gates, params[off:off + npar], terms)
        es.append(e)
        gs.append(g)
        off += npar
    return np.array(es), np.concatenate(gs)


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 2e-4)])
def test_batch_matches_single_circuit_path(precision, tol):
    from quaru_gb300.batch import Batch
    from quaru_gb300.workloads import config5

    circuits, params = config5(count=24, qmin=3, qmax=13, lmin=1, lmax=4, seed=99)
    params = np.array(params)
    for cl in (0, 8):
        b = Batch(circuits, precision=precision, chunk_log2=cl, ctas_per_sm=2 if cl else 0)
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


def test_batch_rejects_unsupported_gates():
    import quaru_gb300 as q
    from quaru_gb300 import ParamGate
    from quaru_gb300 import operation as O
    from quaru_gb300.batch import Batch

    with pytest.raises(q.EngineError):
        Batch([(3, [ParamGate.fixed(O.swap(0, 1))], 0, [(1.0, 0, 1)])])
    with pytest.raises(q.EngineError):
        Batch([(3, [ParamGate.ry(0, 2)], 1, [(1.0, 0, 1)])])
