"""Two implementations of Quaru's Register API for the shared test suite.

"oracle": the CPU restatement of the reference algorithm in oracle/.
"gpu":    quaru_gb300.Register (the product), on the GB300.
Both expose new/from_int/try_from_qubits/apply/try_apply_fast/apply_all/
try_apply_all/measure(target, draw)/state/size/clone; errors carry .code and
.payload like OperationError.
"""
from __future__ import annotations

import numpy as np

OPERATION_ERRORS = {1: "InvalidTarget", 2: "InvalidDimensions", 3: "InvalidArity", 4: "InvalidQubit"}


class OracleReg:
    def __init__(self, r):
        self.r = r

    @property
    def state(self) -> np.ndarray:
        return self.r.state.copy()

    @state.setter
    def state(self, v):
        self.r.state = np.ascontiguousarray(np.asarray(v, dtype=np.complex128).ravel())

    def size(self) -> int:
        return self.r.n

    def clone(self):
        return OracleReg(self.r.clone())

    def try_apply_fast(self, op):
        self.r.try_apply_fast(op.matrix, op.targets)
        return self

    try_apply = try_apply_fast

    def apply(self, op):
        try:
            return self.try_apply_fast(op)
        except Exception as e:
            raise RuntimeError("Could not apply operation") from e

    def try_apply_all(self, op):
        self.r.try_apply_all(op.matrix, op.arity())
        return self

    def apply_all(self, op):
        try:
            return self.try_apply_all(op)
        except Exception as e:
            raise RuntimeError("Could not apply operation") from e

    def apply_gates(self, ops, **_):
        self.r.apply_sequence([(op.matrix, op.targets) for op in ops])
        return self

    def measure(self, target: int, draw: float) -> bool:
        return self.r.measure(target, draw)

    try_measure = measure

    def probabilities(self):
        return self.r.probabilities()

    def __eq__(self, other):
        return bool(np.all(np.abs(self.state - other.state) < 1e-8))


class Backend:
    def __init__(self, name: str):
        self.name = name
        if name == "oracle":
            from oracle import oracle

            self._o = oracle
        else:
            import quaru_gb300

            self._q = quaru_gb300

    def new(self, bits):
        if self.name == "oracle":
            return OracleReg(self._o.OracleRegister.new(bits))
        return self._q.Register.new(bits)

    def from_int(self, n, k):
        if self.name == "oracle":
            return OracleReg(self._o.OracleRegister.from_int(n, k))
        return self._q.Register.from_int(n, k)

    def try_from_qubits(self, qubits):
        if self.name == "oracle":
            return OracleReg(self._o.OracleRegister.try_from_qubits(qubits))
        return self._q.Register.try_from_qubits(qubits)


def equal_qubits(a, b) -> bool:
    """math::equal_qubits (src/math.rs:21-29): every |a_i - b_i| < 1e-8."""
    return bool(np.all(np.abs(np.asarray(a) - np.asarray(b)) < 1e-8))
