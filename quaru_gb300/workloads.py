"""Seeded synthetic workloads: the 12-qubit parity circuit, the layered random-circuit family, and
hardware-efficient ansatz circuits (single and batched) for the gradient benchmarks.

All randomness comes from SplitMix64 (Steele, Lea, Flood: "Fast splittable
pseudorandom number generators", OOPSLA 2014) so that the GPU runs, the CPU
oracle and the fixtures see identical gates. Haar-random 2x2 unitaries follow
Mezzadri, "How to generate random matrices from the classical compact
groups" (Notices AMS 54, 2007): QR of a complex Gaussian matrix with the
phases of R's diagonal moved into Q.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import operation as O
from .operation import Operation

MASK = (1 << 64) - 1
BASE_SEED = 0x5EED0000


class SplitMix64:
    def __init__(self, seed: int):
        self.s = seed & MASK

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        """Uniform in [0, 1) with 53 random bits."""
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def randint(self, n: int) -> int:
        return self.next_u64() % n

    def normal(self) -> float:
        """Standard normal by Box-Muller."""
        u1 = 1.0 - self.uniform()
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)

    def distinct(self, n: int, k: int) -> list[int]:
        """k distinct values of range(n): a Fisher-Yates prefix."""
        p = list(range(n))
        for i in range(k):
            j = i + self.randint(n - i)
            p[i], p[j] = p[j], p[i]
        return p[:k]

    def haar2(self) -> np.ndarray:
        z = np.array([[complex(self.normal(), self.normal()) for _ in range(2)] for _ in range(2)]) / math.sqrt(2.0)
        # Gram-Schmidt QR
        a0, a1 = z[:, 0], z[:, 1]
        r00 = np.linalg.norm(a0)
        q0 = a0 / r00
        r01 = np.vdot(q0, a1)
        v = a1 - r01 * q0
        r11 = np.linalg.norm(v)
        q1 = v / r11
        # phases of R's diagonal: r00, r11 are real positive here, so Q is already Haar
        return np.ascontiguousarray(np.stack([q0, q1], axis=1))


# Base seed of each named workload (BASE_SEED + a fixed offset per workload).
WORKLOAD_SEEDS = {
    "parity_12q": BASE_SEED + 1,    # the 12-qubit, 200-gate parity circuit
    "layered_28q": BASE_SEED + 2,   # the layered family at 28 qubits (and its smaller test instances)
    "layered_30q": BASE_SEED + 3,   # the layered family of the 30-qubit gate-sweep benchmark (and its host samples)
    "ansatz_20q": BASE_SEED + 4,    # the 20-qubit, 400-parameter ansatz and its observable
    "ansatz_batch": BASE_SEED + 5,  # the batch of 256 ansatz circuits
}


def workload_seed(name: str) -> int:
    return WORKLOAD_SEEDS[name]


# ---------------------------------------------------------------- the parity circuit
PARITY_GATE_SET = ("H", "X", "Y", "Z", "PHASE", "CNOT", "SWAP", "TOFFOLI", "HAAR")


def random_gate(rng: SplitMix64, n: int, kind: str | None = None) -> Operation:
    kind = kind or PARITY_GATE_SET[rng.randint(len(PARITY_GATE_SET))]
    if kind == "H":
        return O.hadamard(rng.randint(n))
    if kind == "X":
        return O.not_(rng.randint(n))
    if kind == "Y":
        return O.pauli_y(rng.randint(n))
    if kind == "Z":
        return O.pauli_z(rng.randint(n))
    if kind == "PHASE":
        return O.phase_theta(2.0 * math.pi * rng.uniform(), rng.randint(n))
    if kind == "CNOT":
        c, t = rng.distinct(n, 2)
        return O.cnot(c, t)
    if kind == "SWAP":
        a, b = rng.distinct(n, 2)
        return O.swap(a, b)
    if kind == "TOFFOLI":
        c1, c2, t = rng.distinct(n, 3)
        return O.cnx([c1, c2], t)
    if kind == "HAAR":
        return Operation(rng.haar2(), [rng.randint(n)])
    raise ValueError(kind)


@dataclass
class ParityCircuit:
    n: int
    gates: list[Operation]
    draws: list[float]


def parity_circuit(n: int = 12, m: int = 200, seed: int | None = None) -> ParityCircuit:
    """n-qubit |0..0>, m gates uniform over PARITY_GATE_SET, then one draw per qubit for measuring q0..q(n-1)."""
    rng = SplitMix64(workload_seed("parity_12q") if seed is None else seed)
    gates = [random_gate(rng, n) for _ in range(m)]
    draws = [rng.uniform() for _ in range(n)]
    return ParityCircuit(n, gates, draws)


# ---------------------------------------------------------------- the layered random-circuit family
def layered_circuit(n: int, depth: int, seed: int) -> list[list[Operation]]:
    """Per layer: a Haar-random 1-qubit unitary on every qubit (0..n-1), then CNOTs on a
    random perfect matching (control, target) = (p[2i], p[2i+1]) of a shuffled qubit list."""
    rng = SplitMix64(seed)
    layers = []
    for _ in range(depth):
        layer = [Operation(rng.haar2(), [q]) for q in range(n)]
        p = rng.distinct(n, n)
        for i in range(n // 2):
            layer.append(O.cnot(p[2 * i], p[2 * i + 1]))
        layers.append(layer)
    return layers


def flatten(layers: list[list[Operation]]) -> list[Operation]:
    return [g for layer in layers for g in layer]


# ---------------------------------------------------------------- hardware-efficient ansatz circuits
def ansatz(n: int, layers: int):
    """Hardware-efficient ansatz: per layer RY(theta) then RZ(theta) on every qubit, then a CNOT
    ladder i -> i+1 for i = 0..n-2. Returns (ParamGate list, number of parameters)."""
    from .register import ParamGate

    gates = []
    p = 0
    for _ in range(layers):
        for q in range(n):
            gates.append(ParamGate.ry(q, p))
            p += 1
        for q in range(n):
            gates.append(ParamGate.rz(q, p))
            p += 1
        for q in range(n - 1):
            gates.append(ParamGate.fixed(O.cnot(q, q + 1)))
    return gates, p


def chain_hamiltonian(n: int, rng: SplitMix64):
    """sum_{i<n-1} a_i Z_i Z_{i+1} + sum_i b_i X_i with a, b ~ N(0, 1): (coeff, x_mask, z_mask) terms."""
    terms = [(rng.normal(), 0, (1 << i) | (1 << (i + 1))) for i in range(n - 1)]
    terms += [(rng.normal(), 1 << i, 0) for i in range(n)]
    return terms


def ansatz_problem(n: int = 20, layers: int = 10, seed: int | None = None):
    rng = SplitMix64(workload_seed("ansatz_20q") if seed is None else seed)
    gates, npar = ansatz(n, layers)
    params = [2.0 * math.pi * rng.uniform() for _ in range(npar)]
    return gates, params, chain_hamiltonian(n, rng)


def ansatz_batch(count: int = 256, qmin: int = 10, qmax: int = 22, lmin: int = 4, lmax: int = 12,
                 seed: int | None = None):
    """Batch of ansatz circuits: qubits ~ U{qmin..qmax}, layers ~ U{lmin..lmax}, parameters ~ U[0, 2pi),
    random Z / ZZ / X observables with N(0, 1) coefficients. Returns (circuits, params) where each circuit
    is (n, gates, nparams, terms) and params is the concatenation."""
    rng = SplitMix64(workload_seed("ansatz_batch") if seed is None else seed)
    circuits, params = [], []
    for _ in range(count):
        n = qmin + rng.randint(qmax - qmin + 1)
        layers = lmin + rng.randint(lmax - lmin + 1)
        gates, npar = ansatz(n, layers)
        terms = []
        for _ in range(n):
            kind = rng.randint(3)
            a = rng.randint(n)
            if kind == 0:
                terms.append((rng.normal(), 0, 1 << a))
            elif kind == 1:
                b = (a + 1 + rng.randint(n - 1)) % n
                terms.append((rng.normal(), 0, (1 << a) | (1 << b)))
            else:
                terms.append((rng.normal(), 1 << a, 0))
        circuits.append((n, gates, npar, terms))
        params += [2.0 * math.pi * rng.uniform() for _ in range(npar)]
    return circuits, params
