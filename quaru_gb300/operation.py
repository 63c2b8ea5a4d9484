"""Quaru's Operation and gate constructors (src/operation.rs), host side.

An Operation is a dense complex matrix plus an ordered target list; local
matrix index bit j corresponds to targets[j] (src/register.rs:163-176). The
constructors build the same matrices as the reference, entry for entry.
"""
from __future__ import annotations

import cmath
import math
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

FRAC_1_SQRT_2 = 0.7071067811865476  # std::f64::consts::FRAC_1_SQRT_2


@dataclass
class Operation:
    """src/operation.rs:49-52."""

    matrix: np.ndarray
    targets: list[int]

    @staticmethod
    def new(matrix, targets: Sequence[int]) -> "Operation | None":
        """Operation::new (src/operation.rs:60-70): None unless the matrix is 2^k x 2^k."""
        m = np.asarray(matrix, dtype=np.complex128)
        k = len(targets)
        if m.ndim != 2 or m.shape[0] != 2 ** k or m.shape[1] != 2 ** k:
            return None
        return Operation(np.ascontiguousarray(m), list(int(t) for t in targets))

    def arity(self) -> int:
        return len(self.targets)


def _real(rows) -> np.ndarray:
    return np.ascontiguousarray(np.array(rows, dtype=np.float64).astype(np.complex128))


def identity(target: int) -> Operation:  # src/operation.rs:340-345
    return Operation(_real([[1.0, 0.0], [0.0, 1.0]]), [target])


def hadamard(target: int) -> Operation:  # src/operation.rs:350-355
    return Operation(_real(FRAC_1_SQRT_2 * np.array([[1.0, 1.0], [1.0, -1.0]])), [target])


def hadamard_transform(targets: Sequence[int]) -> Operation:  # src/operation.rs:358-366
    m = hadamard(targets[0]).matrix
    for t in list(targets)[1:]:
        m = np.kron(hadamard(t).matrix, m)
    return Operation(np.ascontiguousarray(m), list(targets))


def cnot(control: int, target: int) -> Operation:  # src/operation.rs:372-382
    return Operation(_real([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]]), [target, control])


def to_quantum_gate(f: Callable[[int], int], targets: Sequence[int]) -> Operation:  # src/operation.rs:386-401
    n = 1 << len(targets)
    m = np.zeros((n, n), dtype=np.complex128)
    for c in range(n):
        m[f(c), c] = 1.0
    return Operation(m, list(targets))


def to_controlled(op: Operation, control: int) -> Operation:  # src/operation.rs:406-422
    old = 1 << op.arity()
    m = np.zeros((2 * old, 2 * old), dtype=np.complex128)
    for i in range(old):
        m[i, i] = 1.0
    m[old:, old:] = op.matrix
    return Operation(m, list(op.targets) + [control])


def swap(t1: int, t2: int) -> Operation:  # src/operation.rs:427-437
    return Operation(_real([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]]), [t1, t2])


def phase(target: int) -> Operation:  # src/operation.rs:443-451 (the S gate)
    return Operation(np.array([[1, 0], [0, 1j]], dtype=np.complex128), [target])


def not_(target: int) -> Operation:  # src/operation.rs:458-463
    return Operation(_real([[0.0, 1.0], [1.0, 0.0]]), [target])


def pauli_y(target: int) -> Operation:  # src/operation.rs:468-476
    return Operation(np.array([[0, -1j], [1j, 0]], dtype=np.complex128), [target])


def pauli_z(target: int) -> Operation:  # src/operation.rs:481-486
    return Operation(_real([[1.0, 0.0], [0.0, -1.0]]), [target])


def cnx(controls: Sequence[int], target: int) -> Operation:  # src/operation.rs:491-513
    targets = [target] + list(controls)
    n = 2 ** len(targets)
    m = np.zeros((n, n))
    for i in range(n - 2):
        m[i, i] = 1.0
    m[n - 1, n - 2] = 1.0
    m[n - 2, n - 1] = 1.0
    return Operation(_real(m), targets)


def cnz(controls: Sequence[int], target: int) -> Operation:  # src/operation.rs:520-536
    targets = [target] + list(controls)
    n = 2 ** len(targets)
    m = np.zeros((n, n))
    for i in range(n - 1):
        m[i, i] = 1.0
    m[n - 1, n - 1] = -1.0
    return Operation(_real(m), targets)


def _cexp(z: complex) -> complex:
    # num-complex exp: from_polar(exp(re), im)
    r = math.exp(z.real)
    return complex(r * math.cos(z.imag), r * math.sin(z.imag))


def u(theta: float, phi: float, lam: float, target: int) -> Operation | None:
    """openqasm::u (src/openqasm.rs:145-163), the OpenQASM U(theta, phi, lambda) gate."""
    c = math.cos(theta / 2.0)
    s = math.sin(theta / 2.0)
    m = np.array([
        [_cexp(complex(0.0, -(phi + lam) / 2.0)) * c, -_cexp(complex(0.0, -(phi - lam) / 2.0)) * s],
        [_cexp(complex(0.0, (phi - lam) / 2.0)) * s, _cexp(complex(0.0, (phi + lam) / 2.0)) * c],
    ], dtype=np.complex128)
    return Operation.new(m, [target])


def phase_theta(theta: float, target: int) -> Operation:
    """diag(1, e^{i theta}), built through Operation::new as examples/shors.rs:322-330 does."""
    return Operation(np.array([[1, 0], [0, cmath.exp(1j * theta)]], dtype=np.complex128), [target])


def ry(theta: float, target: int) -> Operation:
    """RY(theta) = exp(-i theta Y / 2) = [[cos, -sin], [sin, cos]] of theta/2 (a real matrix)."""
    c, s = math.cos(theta / 2.0), math.sin(theta / 2.0)
    return Operation(_real([[c, -s], [s, c]]), [target])


def rz(theta: float, target: int) -> Operation:
    """RZ(theta) = exp(-i theta Z / 2) = diag(e^{-i theta/2}, e^{i theta/2})."""
    return Operation(np.array([[cmath.exp(-0.5j * theta), 0], [0, cmath.exp(0.5j * theta)]],
                              dtype=np.complex128), [target])


def kron_targets(ops: Sequence[Operation]) -> Operation:
    """Tensor product of operations on disjoint targets (later ops on higher local bits)."""
    m = np.array([[1.0 + 0j]])
    targets: list[int] = []
    for op in ops:
        m = np.kron(op.matrix, m)
        targets += op.targets
    return Operation(np.ascontiguousarray(m), targets)
