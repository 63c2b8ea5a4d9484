"""Quaru's Register (src/register.rs) backed by a GB300 state vector.

Same names, argument meaning and error behaviour as the reference: the
try_* methods raise OperationError (the Rust Result's Err), the plain methods
are the panicking forms. measure() takes the uniform draw from a
caller-supplied generator because the reference's thread_rng
(src/register.rs:317-318) cannot be seeded; by default numpy's generator is
used.
"""
from __future__ import annotations

import ctypes
from typing import Callable, Iterable, Sequence

import numpy as np

from . import _lib
from .operation import Operation


class OperationError(Exception):
    """src/register.rs:10-20. kind is one of InvalidTarget, InvalidDimensions, InvalidArity, InvalidQubit."""

    KINDS = {_lib.QS_INVALID_TARGET: "InvalidTarget", _lib.QS_INVALID_DIMENSIONS: "InvalidDimensions",
             _lib.QS_INVALID_ARITY: "InvalidArity", _lib.QS_INVALID_QUBIT: "InvalidQubit"}

    def __init__(self, code: int, payload: tuple, message: str = ""):
        self.code = code
        self.kind = self.KINDS.get(code, "Other")
        self.payload = payload
        super().__init__(f"{self.kind}{payload} {message}".strip())

    def __eq__(self, other) -> bool:
        return isinstance(other, OperationError) and (self.code, self.payload) == (other.code, other.payload)

    def __hash__(self):
        return hash((self.code, self.payload))


class EngineError(RuntimeError):
    """A device-side failure (CUDA error, out of memory, timeout) or a bad argument."""


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _sp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t))


def _check(rc: int, err: np.ndarray | None = None) -> None:
    if rc == _lib.QS_OK:
        return
    msg = _lib.last_error()
    if rc in OperationError.KINDS:
        if rc == _lib.QS_INVALID_DIMENSIONS:
            payload = (int(err[0]), int(err[1]))
        else:
            payload = (int(err[0]),) if err is not None else ()
        raise OperationError(rc, payload, msg)
    raise EngineError(f"quaru_gb300 error {rc}: {msg}")


def _matrix(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, dtype=np.complex128))


class Register:
    """A quantum register of n qubits whose state lives in GPU memory (src/register.rs:22-37)."""

    def __init__(self, handle: int, rng: Callable[[], float] | None = None):
        self._h = ctypes.c_void_p(handle)
        self._rng = rng or np.random.default_rng().random

    # ---- construction (src/register.rs:41-102)
    @classmethod
    def new(cls, input_bits: Sequence[bool], precision: int = _lib.QS_PREC_C128, rng=None) -> "Register":
        lib = _lib.load()
        b = np.ascontiguousarray(np.array([1 if x else 0 for x in input_bits], dtype=np.uint8))
        h = ctypes.c_void_p()
        _check(lib.qs_register_new(b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(b), precision,
                                   ctypes.byref(h)))
        return cls(h.value, rng)

    @classmethod
    def from_int(cls, n: int, k: int, precision: int = _lib.QS_PREC_C128, rng=None) -> "Register":
        lib = _lib.load()
        h = ctypes.c_void_p()
        _check(lib.qs_register_from_int(n, k, precision, ctypes.byref(h)))
        return cls(h.value, rng)

    @classmethod
    def try_from_qubits(cls, qubits, precision: int = _lib.QS_PREC_C128, rng=None) -> "Register":
        lib = _lib.load()
        q = np.ascontiguousarray(np.array([np.asarray(x, dtype=np.complex128).ravel() for x in qubits]))
        if q.size and q.shape[1] != 2:
            raise OperationError(_lib.QS_INVALID_QUBIT, (0,), "each qubit needs 2 amplitudes")
        err = np.zeros(3, dtype=np.uintp)
        h = ctypes.c_void_p()
        _check(lib.qs_register_try_from_qubits(_dp(q.view(np.float64)), q.shape[0], precision, ctypes.byref(h),
                                               _sp(err)), err)
        return cls(h.value, rng)

    @classmethod
    def from_qubits(cls, qubits, precision: int = _lib.QS_PREC_C128, rng=None) -> "Register":
        try:
            return cls.try_from_qubits(qubits, precision, rng)
        except OperationError as e:
            raise RuntimeError("Incorrect input qubits") from e

    def clone(self) -> "Register":
        h = ctypes.c_void_p()
        _check(_lib.load().qs_register_clone(self._h, ctypes.byref(h)))
        return Register(h.value, self._rng)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.qs_register_free(h)
            self._h = ctypes.c_void_p()

    # ---- properties
    def size(self) -> int:
        return int(_lib.load().qs_register_size(self._h))

    @property
    def precision(self) -> int:
        return int(_lib.load().qs_register_precision(self._h))

    def set_arith(self, arith: int) -> None:
        _check(_lib.load().qs_register_set_arith(self._h, arith))

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @property
    def stream(self) -> int:
        return int(_lib.load().qs_register_stream(self._h) or 0)

    # ---- gate application (src/register.rs:134-191, 259-281)
    def try_apply_fast(self, op: Operation) -> "Register":
        m = _matrix(op.matrix)
        t = np.ascontiguousarray(np.array(list(op.targets), dtype=np.uintp))
        err = np.zeros(3, dtype=np.uintp)
        rows = m.shape[0]
        cols = m.shape[1] if m.ndim == 2 else 1
        _check(_lib.load().qs_try_apply_fast(self._h, _dp(m.view(np.float64)), rows, cols, _sp(t), len(t),
                                             _sp(err)), err)
        return self

    try_apply = try_apply_fast

    def apply(self, op: Operation) -> "Register":
        try:
            return self.try_apply_fast(op)
        except OperationError as e:
            raise RuntimeError("Could not apply operation") from e

    def try_apply_all(self, op: Operation) -> "Register":
        m = _matrix(op.matrix)
        err = np.zeros(3, dtype=np.uintp)
        _check(_lib.load().qs_try_apply_all(self._h, _dp(m.view(np.float64)), m.shape[0], m.shape[1],
                                            op.arity(), _sp(err)), err)
        return self

    def apply_all(self, op: Operation) -> "Register":
        try:
            return self.try_apply_all(op)
        except OperationError as e:
            raise RuntimeError("Could not apply operation") from e

    def apply_gates(self, ops: Iterable[Operation], fuse: int = 0, max_width: int = 0, tile_qubits: int = 0):
        """The operations loop of apply_circuit (src/register.rs:346-350) in one library call."""
        ops = list(ops)
        table, keep = gate_table(ops)
        opts = _lib.QsCircuitOptions(fuse, max_width, tile_qubits, 0)
        err = np.zeros(3, dtype=np.uintp)
        rc = _lib.load().qs_apply_circuit(self._h, table.ctypes.data_as(ctypes.POINTER(_lib.QsGate)), len(ops),
                                          ctypes.byref(opts), _sp(err))
        del keep
        _check(rc, err)
        return self

    def apply_circuit(self, circuit, fuse: int = 0) -> list:
        """Register::apply_circuit (src/register.rs:345-369): the gates (one library call), then the
        measurements in order, then each conditional gate whose (target, value) conditions all hold."""
        if circuit.get_operations():
            self.apply_gates(circuit.get_operations(), fuse=fuse)
        measures = self.measure_circuit(circuit) if circuit.get_measurement_targets() else []
        for op, cond in circuit.get_conditional_operations():
            if all((t, v) in measures for t, v in cond):
                self.apply(op)
        return measures

    def measure_circuit(self, circuit) -> list:
        """Register::measure_circuit (src/register.rs:371-377): one qs_measure_sequence call."""
        targets = list(circuit.get_measurement_targets())
        return list(zip(targets, self.measure_sequence(targets)))

    def measure_sequence(self, targets, draws=None) -> list:
        """Measure targets in order (qs_measure_sequence) with the given draws (default: this
        register's generator, one draw per target); returns the outcomes."""
        targets = [int(t) for t in targets]
        if draws is None:
            draws = [self._rng() for _ in targets]
        tg = np.array(targets, dtype=np.uintp)
        dr = np.array(draws, dtype=np.float64)
        if dr.size != tg.size:
            raise ValueError("one draw per target")
        out = np.zeros(tg.size, dtype=np.int32)
        p0 = np.zeros(tg.size, dtype=np.float64)
        p1 = np.zeros(tg.size, dtype=np.float64)
        err = np.zeros(3, dtype=np.uintp)
        try:
            _check(_lib.load().qs_measure_sequence(self._h, _sp(tg), tg.size, _dp(dr),
                                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(p0),
                                                   _dp(p1), _sp(err)), err)
        except OperationError as e:
            raise RuntimeError("Could not measure bit") from e
        self.last_sequence_probs = list(zip(p0.tolist(), p1.tolist()))
        return [bool(x) for x in out]

    # ---- measurement (src/register.rs:291-342)
    def try_measure(self, target: int, draw: float | None = None) -> bool:
        x = self._rng() if draw is None else float(draw)
        out = ctypes.c_int(0)
        p0, p1 = ctypes.c_double(0), ctypes.c_double(0)
        err = np.zeros(3, dtype=np.uintp)
        _check(_lib.load().qs_try_measure(self._h, target, x, ctypes.byref(out), ctypes.byref(p0), ctypes.byref(p1),
                                          _sp(err)), err)
        self.last_probs = (p0.value, p1.value)
        return bool(out.value)

    def measure(self, target: int, draw: float | None = None) -> bool:
        try:
            return self.try_measure(target, draw)
        except OperationError as e:
            raise RuntimeError("Could not measure bit") from e

    # ---- host views (src/register.rs:35, 379-413)
    @property
    def state(self) -> np.ndarray:
        st = np.zeros(1 << self.size(), dtype=np.complex128)
        _check(_lib.load().qs_get_state(self._h, _dp(st.view(np.float64))))
        return st

    @state.setter
    def state(self, value) -> None:
        v = np.ascontiguousarray(np.asarray(value, dtype=np.complex128).ravel())
        if v.size != 1 << self.size():
            raise ValueError("state has the wrong length")
        _check(_lib.load().qs_set_state(self._h, _dp(v.view(np.float64))))

    def probabilities(self) -> np.ndarray:
        p = np.zeros(1 << self.size(), dtype=np.float64)
        _check(_lib.load().qs_probabilities(self._h, _dp(p)))
        return p

    def print_probabilities(self) -> None:
        n = self.size()
        for i, p in enumerate(self.probabilities()):
            print(f"{i:0{n}b}: {p * 100.0}%")

    def print_nonzero_probabilities(self) -> None:
        n = self.size()
        for i, p in enumerate(self.probabilities()):
            if p > 0.0:
                print(f"{i:0{n}b}: {p * 100.0}%")

    def print_state(self) -> None:
        n = self.size()
        for i, s in enumerate(self.state):
            print(f"{i:0{n}b}: {s}")

    def eq(self, other: "Register", tol: float = 1e-8) -> bool:
        e = ctypes.c_int(0)
        _check(_lib.load().qs_register_eq(self._h, other._h, tol, ctypes.byref(e)))
        return bool(e.value)

    def __eq__(self, other) -> bool:  # PartialEq, src/register.rs:409-413
        return isinstance(other, Register) and self.eq(other, 1e-8)

    __hash__ = None

    def synchronize(self) -> None:
        _check(_lib.load().qs_synchronize(self._h))

    # ---- observables and gradients
    def inner_product(self, other: "Register") -> complex:
        """<self|other> accumulated in FP64 on the GPU."""
        re, im = ctypes.c_double(0), ctypes.c_double(0)
        _check(_lib.load().qs_inner_product(self._h, other._h, ctypes.byref(re), ctypes.byref(im)))
        return complex(re.value, im.value)

    def expval_pauli(self, terms) -> float:
        """<psi|H|psi> for H = sum of (coeff, x_mask, z_mask) Pauli terms."""
        arr = _pauli_array(terms)
        v = ctypes.c_double(0)
        _check(_lib.load().qs_expval_pauli(self._h, arr, len(terms), ctypes.byref(v)))
        return v.value

    def adjoint_gradient(self, gates, params, terms):
        """Energy and gradient of the parameterised circuit `gates` (a list of ParamGate, or a
        ParamCircuit built once from one) for observable `terms` (a list of (coeff, x_mask, z_mask),
        or a PauliSum)."""
        if isinstance(gates, ParamCircuit):
            table, keep = gates.table, None
        else:
            table, keep = param_gate_table(gates)
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64))
        arr = terms.array if isinstance(terms, PauliSum) else _pauli_array(terms)
        grad = np.zeros(max(1, p.size), dtype=np.float64)
        e = ctypes.c_double(0)
        err = np.zeros(3, dtype=np.uintp)
        _check(_lib.load().qs_adjoint_gradient(self._h, table.ctypes.data_as(ctypes.POINTER(_lib.QsParamGate)),
                                               len(gates), _dp(p), p.size, arr, len(terms), ctypes.byref(e),
                                               _dp(grad), _sp(err)), err)
        del keep
        return e.value, grad[: p.size]


_GATE_DTYPE = np.dtype([("k", "<u8"), ("targets", "<u8"), ("matrix", "<u8")])  # qs_gate (include/quaru_gpu.h)


def gate_table(ops):
    """qs_gate records for `ops` as one numpy array, targets and matrices in two shared buffers
    addressed by offset (a few array operations per call instead of ctypes objects per gate).
    Raises InvalidDimensions(rows, cols) for a matrix that is not 2^k x 2^k, which the engine could
    not detect from the record. Returns (table, buffers to keep alive while the table is in use)."""
    import itertools

    n = len(ops)
    tl = [op.targets for op in ops]
    ks = np.fromiter((len(t) for t in tl), dtype=np.uint64, count=n)
    flat = np.fromiter(itertools.chain.from_iterable(tl), dtype=np.uintp, count=int(ks.sum()) if n else 0)
    if flat.size == 0:
        flat = np.zeros(1, dtype=np.uintp)
    mats = [np.asarray(op.matrix, dtype=np.complex128) for op in ops]
    for m, k in zip(mats, ks.tolist()):
        d = 1 << k
        if m.shape != (d, d):
            rows = m.shape[0] if m.ndim >= 1 else 0
            raise OperationError(_lib.QS_INVALID_DIMENSIONS, (rows, m.shape[1] if m.ndim == 2 else 1),
                                 f"for {k} targets")
    mflat = np.concatenate([m.reshape(-1) for m in mats]) if mats else np.zeros(1, dtype=np.complex128)
    table = np.zeros(max(1, n), dtype=_GATE_DTYPE)
    if n:
        sizes = np.left_shift(np.uint64(1), 2 * ks)
        table["k"][:n] = ks
        table["targets"][:n] = flat.ctypes.data + 8 * (np.cumsum(ks) - ks)
        table["matrix"][:n] = mflat.ctypes.data + 16 * (np.cumsum(sizes) - sizes)
    return table, (flat, mflat)


_PARAM_GATE_DTYPE = np.dtype([("kind", "<i4"), ("param", "<i4"), ("k", "<u8"), ("targets", "<u8"),
                              ("matrix", "<u8")])  # the layout of qs_param_gate (include/quaru_gpu.h)


def param_gate_table(gates):
    """qs_param_gate records for `gates` as one numpy array (targets and matrices in two shared
    buffers, addressed by offset): a few array operations per call instead of one ctypes object
    per gate. Returns (table, buffers to keep alive while the table is in use)."""
    import itertools

    n = len(gates)
    fixed = _lib.QS_GATE_FIXED
    tl = [g.op.targets if g.kind == fixed else (g.target,) for g in gates]
    ks = np.fromiter((len(t) for t in tl), dtype=np.uint64, count=n)
    flat = np.fromiter(itertools.chain.from_iterable(tl), dtype=np.uintp, count=int(ks.sum()) if n else 0)
    if flat.size == 0:
        flat = np.zeros(1, dtype=np.uintp)
    table = np.zeros(max(1, n), dtype=_PARAM_GATE_DTYPE)
    if n:
        table["kind"][:n] = np.fromiter((g.kind for g in gates), dtype=np.int32, count=n)
        table["param"][:n] = np.fromiter((g.param for g in gates), dtype=np.int32, count=n)
        table["k"][:n] = ks
        table["targets"][:n] = flat.ctypes.data + 8 * (np.cumsum(ks) - ks)
    fidx = [i for i in range(n) if gates[i].kind == fixed]
    mats = [np.ascontiguousarray(np.asarray(gates[i].op.matrix, dtype=np.complex128)).ravel() for i in fidx]
    mflat = np.concatenate(mats) if mats else np.zeros(1, dtype=np.complex128)
    if fidx:
        sizes = np.fromiter((m.size for m in mats), dtype=np.uint64, count=len(mats))
        table["matrix"][fidx] = mflat.ctypes.data + 16 * (np.cumsum(sizes) - sizes)
    return table, (flat, mflat)


class ParamCircuit:
    """A parameterised circuit converted once into the engine's gate records, for repeated gradient
    calls with new parameters (an optimiser loop): the per-call cost is the engine's alone."""

    def __init__(self, gates):
        self.gates = list(gates)
        self.table, self._keep = param_gate_table(self.gates)

    def __len__(self) -> int:
        return len(self.gates)


class PauliSum:
    """An observable (list of (coeff, x_mask, z_mask)) converted once into the engine's term records."""

    def __init__(self, terms):
        self.terms = list(terms)
        self.array = _pauli_array(self.terms)

    def __len__(self) -> int:
        return len(self.terms)


class ParamGate:
    """A gate of a parameterised circuit: a rotation R_A(params[param]) on `target`, or a fixed Operation."""

    def __init__(self, kind: int, target: int = 0, param: int = -1, op: Operation | None = None):
        self.kind, self.target, self.param, self.op = kind, target, param, op

    @classmethod
    def rx(cls, target: int, param: int) -> "ParamGate":
        return cls(_lib.QS_GATE_RX, target, param)

    @classmethod
    def ry(cls, target: int, param: int) -> "ParamGate":
        return cls(_lib.QS_GATE_RY, target, param)

    @classmethod
    def rz(cls, target: int, param: int) -> "ParamGate":
        return cls(_lib.QS_GATE_RZ, target, param)

    @classmethod
    def fixed(cls, op: Operation) -> "ParamGate":
        return cls(_lib.QS_GATE_FIXED, op=op)

    def operation(self, params) -> Operation:
        """The gate as a plain Operation at the given parameters."""
        from . import operation as O

        if self.kind == _lib.QS_GATE_FIXED:
            return self.op
        th = float(params[self.param])
        if self.kind == _lib.QS_GATE_RY:
            return O.ry(th, self.target)
        if self.kind == _lib.QS_GATE_RZ:
            return O.rz(th, self.target)
        c, s = np.cos(th / 2.0), np.sin(th / 2.0)
        return Operation(np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128), [self.target])


def _pauli_array(terms):
    arr = (_lib.QsPauliTerm * max(1, len(terms)))()
    for i, (c, x, z) in enumerate(terms):
        arr[i].coeff = float(c)
        arr[i].x_mask = int(x)
        arr[i].z_mask = int(z)
    return arr


def circuit_autotune(n: int, precision: int = _lib.QS_PREC_C128, arith: int = _lib.QS_ARITH_FMA, fuse: int = 3,
                     retune: bool = False) -> dict:
    """qs_circuit_autotune: the fusion form qs_apply_circuit uses for this size, precision and arithmetic
    (fuse 1: tile size, 2: block width, 3: any form), with each candidate's measured time when the
    candidates were timed by this call."""
    rep = _lib.QsAutotuneReport()
    _check(_lib.load().qs_circuit_autotune(n, precision, arith, fuse, int(retune), ctypes.byref(rep)))
    cands = [{"fuse": rep.cand_fuse[i], "max_width": rep.cand_width[i], "tile_qubits": rep.cand_tile[i],
              "ms": rep.cand_ms[i]} for i in range(rep.count)]
    return {"fuse": rep.fuse, "max_width": rep.max_width, "tile_qubits": rep.tile_qubits,
            "from_cache": bool(rep.from_cache), "candidates": cands}
