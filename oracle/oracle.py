"""ctypes bindings of the CPU oracle (quaru_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use this module, as the oracle the GPU results are compared with.
The product (quaru_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11", "-Wall"]

ORC_OK, ORC_INVALID_TARGET, ORC_INVALID_DIMENSIONS, ORC_INVALID_ARITY, ORC_INVALID_QUBIT = range(5)


def build() -> Path:
    """Compile quaru_oracle.c with gcc (no FMA contraction)."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "quaru_oracle.c"
    hdr = HERE / "quaru_oracle.h"
    if LIB.exists() and LIB.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    subprocess.run([os.environ.get("CC", "gcc"), *CFLAGS, str(src), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.POINTER
        dp, sp, u8p = P(ctypes.c_double), P(ctypes.c_size_t), P(ctypes.c_uint8)
        sz = ctypes.c_size_t
        L.orc_register_new.argtypes = [u8p, sz, dp]
        L.orc_register_from_int.argtypes = [sz, sz, dp]
        L.orc_register_try_from_qubits.argtypes = [dp, sz, dp, sp]
        L.orc_register_try_from_qubits.restype = ctypes.c_int
        L.orc_try_apply_fast.argtypes = [dp, sz, dp, sz, sz, sp, sz, sp]
        L.orc_try_apply_fast.restype = ctypes.c_int
        L.orc_try_apply_all.argtypes = [dp, sz, dp, sz, sz, sz, sp]
        L.orc_try_apply_all.restype = ctypes.c_int
        L.orc_try_measure.argtypes = [dp, sz, sz, ctypes.c_double, P(ctypes.c_int), dp, dp, sp]
        L.orc_try_measure.restype = ctypes.c_int
        L.orc_probabilities.argtypes = [dp, sz, dp]
        L.orc_apply_sequence.argtypes = [dp, sz, sz, sp, sp, sp, sp, dp, sp]
        L.orc_apply_sequence.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _sp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t))


class OracleError(Exception):
    def __init__(self, code: int, payload: tuple):
        super().__init__(f"oracle error {code} {payload}")
        self.code = code
        self.payload = payload


class OracleRegister:
    """CPU restatement of Quaru's Register (src/register.rs) as a numpy complex128 vector."""

    def __init__(self, state: np.ndarray, n: int):
        self.state = np.ascontiguousarray(state, dtype=np.complex128)
        self.n = n

    @classmethod
    def new(cls, bits) -> "OracleRegister":
        n = len(bits)
        st = np.zeros(1 << n, dtype=np.complex128)
        b = np.ascontiguousarray(np.array(bits, dtype=np.uint8))
        lib().orc_register_new(b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), n, _dp(st.view(np.float64)))
        return cls(st, n)

    @classmethod
    def from_int(cls, n: int, k: int) -> "OracleRegister":
        st = np.zeros(1 << n, dtype=np.complex128)
        lib().orc_register_from_int(n, k, _dp(st.view(np.float64)))
        return cls(st, n)

    @classmethod
    def try_from_qubits(cls, qubits) -> "OracleRegister":
        q = np.ascontiguousarray(np.array(qubits, dtype=np.complex128).reshape(-1, 2))
        n = q.shape[0]
        st = np.zeros(1 << n, dtype=np.complex128)
        err = np.zeros(3, dtype=np.uintp)
        rc = lib().orc_register_try_from_qubits(_dp(q.view(np.float64)), n, _dp(st.view(np.float64)), _sp(err))
        if rc:
            raise OracleError(rc, (int(err[0]),))
        return cls(st, n)

    def clone(self) -> "OracleRegister":
        return OracleRegister(self.state.copy(), self.n)

    def try_apply_fast(self, matrix, targets) -> None:
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex128))
        t = np.ascontiguousarray(np.array(list(targets), dtype=np.uintp))
        err = np.zeros(3, dtype=np.uintp)
        rc = lib().orc_try_apply_fast(_dp(self.state.view(np.float64)), self.n, _dp(m.view(np.float64)),
                                      m.shape[0], m.shape[1] if m.ndim == 2 else 1, _sp(t), len(t), _sp(err))
        if rc:
            raise OracleError(rc, (int(err[0]), int(err[1])) if rc == ORC_INVALID_DIMENSIONS else (int(err[0]),))

    def apply(self, op) -> "OracleRegister":
        self.try_apply_fast(op.matrix, op.targets)
        return self

    def try_apply_all(self, matrix, k: int = 1) -> None:
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex128))
        err = np.zeros(3, dtype=np.uintp)
        rc = lib().orc_try_apply_all(_dp(self.state.view(np.float64)), self.n, _dp(m.view(np.float64)),
                                     m.shape[0], m.shape[1], k, _sp(err))
        if rc:
            raise OracleError(rc, (int(err[0]),))

    def measure(self, target: int, draw: float) -> bool:
        out = ctypes.c_int(0)
        p0, p1 = ctypes.c_double(0), ctypes.c_double(0)
        err = np.zeros(3, dtype=np.uintp)
        rc = lib().orc_try_measure(_dp(self.state.view(np.float64)), self.n, target, draw, ctypes.byref(out),
                                   ctypes.byref(p0), ctypes.byref(p1), _sp(err))
        if rc:
            raise OracleError(rc, (int(err[0]),))
        self.last_probs = (p0.value, p1.value)
        return bool(out.value)

    def probabilities(self) -> np.ndarray:
        p = np.zeros(1 << self.n, dtype=np.float64)
        lib().orc_probabilities(_dp(self.state.view(np.float64)), self.n, _dp(p))
        return p

    def apply_sequence(self, gates) -> None:
        """gates: iterable of (matrix, targets)."""
        gates = list(gates)
        ks = np.array([len(t) for _, t in gates], dtype=np.uintp)
        toff = np.zeros(len(gates), dtype=np.uintp)
        moff = np.zeros(len(gates), dtype=np.uintp)
        tl, ml = [], []
        to = mo = 0
        for g, (m, t) in enumerate(gates):
            toff[g], moff[g] = to, mo
            tl.extend(int(x) for x in t)
            mm = np.ascontiguousarray(np.asarray(m, dtype=np.complex128)).view(np.float64).ravel()
            ml.append(mm)
            to += len(t)
            mo += mm.size
        targets = np.ascontiguousarray(np.array(tl if tl else [0], dtype=np.uintp))
        mats = np.ascontiguousarray(np.concatenate(ml) if ml else np.zeros(1))
        err = np.zeros(3, dtype=np.uintp)
        rc = lib().orc_apply_sequence(_dp(self.state.view(np.float64)), self.n, len(gates), _sp(ks), _sp(toff),
                                      _sp(targets), _sp(moff), _dp(mats), _sp(err))
        if rc:
            raise OracleError(rc, (int(err[0]), int(err[2])))
