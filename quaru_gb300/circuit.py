"""QuantumCircuit (src/operation.rs:79-322): gates, measurements and conditional gates.

The reduction passes are restated from the reference for API parity; note that
reduce_circuit_cancel_gates drops any two equal consecutive real gates, which is
only correct for involutions (as in the reference, src/operation.rs:201-202).
For exact fusion use Register.apply_circuit(..., fuse=1) or fuse=2 instead.
"""
from __future__ import annotations

import numpy as np

from .operation import Operation


class QuantumCircuit:
    def __init__(self):
        self.operations: list[Operation] = []
        self.measurement_targets: list[int] = []
        self.conditional_operations: list[tuple[Operation, list[tuple[int, bool]]]] = []

    @classmethod
    def new(cls) -> "QuantumCircuit":
        return cls()

    def reset_register(self) -> "QuantumCircuit":  # :95-100
        self.operations.clear()
        self.measurement_targets.clear()
        self.conditional_operations.clear()
        return self

    def get_operations(self):
        return self.operations

    def get_measurement_targets(self):
        return self.measurement_targets

    def get_conditional_operations(self):
        return self.conditional_operations

    def clear_operations(self) -> None:
        self.operations.clear()

    def add_operation(self, op: Operation) -> None:  # :276-288
        if any(t in self.measurement_targets for t in op.targets):
            raise RuntimeError("Cannot add operation after measurement")
        if self.conditional_operations:
            raise RuntimeError("Cannot add operation after conditional operation (yet...)")
        self.operations.append(op)

    def add_measurement(self, target: int) -> None:  # :292-297
        if target in self.measurement_targets:
            raise RuntimeError("Cannot add measurement after measurement")
        self.measurement_targets.append(target)

    def add_conditional_operation(self, op: Operation, condition) -> None:  # :302-321
        if any(t in self.measurement_targets for t in op.targets):
            raise RuntimeError("Cannot add operation after measurement")
        if not all(c[0] in self.measurement_targets for c in condition):
            raise RuntimeError("Condition must be a measurement")
        self.conditional_operations.append((op, list(condition)))

    # ---- reduction passes (restated)
    def reduce_circuit_gates_with_same_targets(self) -> "QuantumCircuit":  # :218-240
        out, i, ops = [], 0, self.operations
        while i < len(ops):
            m, t = ops[i].matrix, list(ops[i].targets)
            j = i + 1
            while j < len(ops) and list(ops[j].targets) == t:
                m = ops[j].matrix @ m
                j += 1
            out.append(Operation(np.ascontiguousarray(m), t))
            i = j
        self.operations = out
        return self

    def reduce_non_overlapping_gates(self) -> "QuantumCircuit":  # :243-269
        out, i, ops = [], 0, self.operations
        while i < len(ops):
            m, t = ops[i].matrix, list(ops[i].targets)
            j = i + 1
            while j < len(ops) and not any(x in ops[j].targets for x in t):
                m = np.kron(ops[j].matrix, m)
                t += list(ops[j].targets)
                j += 1
            out.append(Operation(np.ascontiguousarray(m), t))
            i = j
        self.operations = out
        return self

    def reduce_gates_with_one_off_size(self, max_size: int) -> "QuantumCircuit":  # :114-178
        self.reduce_circuit_gates_with_same_targets()
        ops, out, i = self.operations, [], 0
        while i < len(ops):
            if i == len(ops) - 1:
                out.append(ops[i])
                break
            a, b = ops[i], ops[i + 1]
            if len(a.targets) > max_size or len(b.targets) > max_size:
                out.append(a)
                i += 1
                continue
            if any(t in b.targets for t in a.targets):
                out.append(self._combine(a, b))
                i += 2
            else:
                out.append(a)
                i += 1
        self.operations = out
        return self

    @staticmethod
    def _combine(a: Operation, b: Operation) -> Operation:  # :147-178
        if len(a.targets) > 2 or len(b.targets) > 2:
            raise RuntimeError("Cannot combine operations with more than 2 targets")
        diff = len(a.targets) - len(b.targets)
        eye = np.eye(2, dtype=complex)
        if diff < 0:
            targets = list(b.targets)
            ext = np.kron(eye, a.matrix) if a.targets[0] == b.targets[0] else np.kron(a.matrix, eye)
            m = b.matrix @ ext
        else:
            if len(a.targets) == len(b.targets):
                # The reference multiplies op1 (2^k x 2^k) by kron(eye(2), op2) (2^(k+1) square) here
                # too, and ndarray's dot panics on the shape mismatch (src/operation.rs:166-174): two
                # overlapping operations of equal arity cannot be combined.
                raise RuntimeError(f"Cannot combine operations of equal arity {len(a.targets)} on targets "
                                   f"{list(a.targets)} and {list(b.targets)}: shapes do not match")
            targets = list(a.targets)
            ext = np.kron(eye, b.matrix) if b.targets[0] == a.targets[0] else np.kron(b.matrix, eye)
            m = a.matrix @ ext
        return Operation.new(m, targets)

    def reduce_circuit_cancel_gates(self) -> "QuantumCircuit":  # :189-216
        ops = list(self.operations)
        out, i = [], 0
        while i < len(ops):
            if i == len(ops) - 1:
                out.append(ops[i])
                break
            a, b = ops[i], ops[i + 1]
            if np.all(np.asarray(a.matrix).imag == 0) and list(a.targets) == list(b.targets) and \
                    np.array_equal(a.matrix, b.matrix):
                i += 1
            else:
                out.append(a)
            i += 1
        self.operations = out
        if len(out) == len(ops) or len(out) <= 1:
            return self
        return self.reduce_circuit_cancel_gates()
