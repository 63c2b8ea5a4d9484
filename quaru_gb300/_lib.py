"""ctypes binding of libquaru_gb300.so (the C ABI in include/quaru_gpu.h).

The library is built in-tree by quaru_gb300/build.py. There is no CPU
fallback: if the shared library is missing or cannot be loaded, importing the
engine raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libquaru_gb300.so"

QS_OK = 0
QS_INVALID_TARGET = 1
QS_INVALID_DIMENSIONS = 2
QS_INVALID_ARITY = 3
QS_INVALID_QUBIT = 4
QS_INVALID_ARGUMENT = 5
QS_CUDA_ERROR = 6
QS_OUT_OF_MEMORY = 7
QS_TIMEOUT = 8
QS_QASM_PARSE_ERROR = 9
QS_QASM_RUN_ERROR = 10

QS_PREC_C128 = 0
QS_PREC_C64 = 1

QS_ARITH_EXACT = 0
QS_ARITH_FMA = 1
QS_ARITH_DF64 = 2
QS_ARITH_FX64 = 3

# Every symbol include/quaru_gpu.h declares, with (restype, argtypes).
_P = ctypes.POINTER
_dp = _P(ctypes.c_double)
_sp = _P(ctypes.c_size_t)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_i = ctypes.c_int


class QsGate(ctypes.Structure):
    _fields_ = [("k", ctypes.c_size_t), ("targets", _sp), ("matrix", _dp)]


class QsCircuitOptions(ctypes.Structure):
    _fields_ = [("fuse", ctypes.c_int), ("max_width", ctypes.c_int), ("tile_qubits", ctypes.c_int),
                ("reserved", ctypes.c_int)]


class QsPauliTerm(ctypes.Structure):
    _fields_ = [("coeff", ctypes.c_double), ("x_mask", ctypes.c_uint64), ("z_mask", ctypes.c_uint64)]


class QsParamGate(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("param", ctypes.c_int), ("k", ctypes.c_size_t), ("targets", _sp),
                ("matrix", _dp)]


QS_GATE_FIXED, QS_GATE_RX, QS_GATE_RY, QS_GATE_RZ = 0, 1, 2, 3


class QsBatchCircuit(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("gates", ctypes.POINTER(QsParamGate)), ("m", ctypes.c_size_t),
                ("nparams", ctypes.c_size_t), ("terms", ctypes.POINTER(QsPauliTerm)), ("nterms", ctypes.c_size_t)]


class QsBatchOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("chunk_log2", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("arith", ctypes.c_int)]

AUTOTUNE_MAX = 16


class QsAutotuneReport(ctypes.Structure):
    _fields_ = [("fuse", ctypes.c_int), ("max_width", ctypes.c_int), ("tile_qubits", ctypes.c_int),
                ("from_cache", ctypes.c_int), ("count", ctypes.c_int),
                ("cand_fuse", ctypes.c_int * AUTOTUNE_MAX), ("cand_width", ctypes.c_int * AUTOTUNE_MAX),
                ("cand_tile", ctypes.c_int * AUTOTUNE_MAX), ("cand_ms", ctypes.c_double * AUTOTUNE_MAX)]


SIGNATURES = {
    "qs_register_new": (_i, [_P(ctypes.c_uint8), _sz, _i, _P(_vp)]),
    "qs_register_from_int": (_i, [_sz, _sz, _i, _P(_vp)]),
    "qs_register_try_from_qubits": (_i, [_dp, _sz, _i, _P(_vp), _sp]),
    "qs_register_clone": (_i, [_vp, _P(_vp)]),
    "qs_register_free": (None, [_vp]),
    "qs_register_size": (_sz, [_vp]),
    "qs_register_precision": (_i, [_vp]),
    "qs_register_set_arith": (_i, [_vp, _i]),
    "qs_try_apply_fast": (_i, [_vp, _dp, _sz, _sz, _sp, _sz, _sp]),
    "qs_try_apply_all": (_i, [_vp, _dp, _sz, _sz, _sz, _sp]),
    "qs_apply_circuit": (_i, [_vp, _P(QsGate), _sz, _P(QsCircuitOptions), _sp]),
    "qs_try_measure": (_i, [_vp, _sz, ctypes.c_double, _P(_i), _dp, _dp, _sp]),
    "qs_measure_probabilities": (_i, [_vp, _sz, _dp, _dp, _sp]),
    "qs_measure_sequence": (_i, [_vp, _sp, _sz, _dp, _P(_i), _dp, _dp, _sp]),
    "qs_circuit_autotune": (_i, [_sz, _i, _i, _i, _i, _P(QsAutotuneReport)]),
    "qs_measure_probabilities_noalloc": (_i, [_vp, _sz, _i, _sz, _vp, _vp, _sp]),
    "qs_inner_product": (_i, [_vp, _vp, _dp, _dp]),
    "qs_expval_pauli": (_i, [_vp, _P(QsPauliTerm), _sz, _dp]),
    "qs_adjoint_gradient": (_i, [_vp, _P(QsParamGate), _sz, _dp, _sz, _P(QsPauliTerm), _sz, _dp, _dp, _sp]),
    "qs_batch_create": (_i, [_P(QsBatchCircuit), _sz, _P(QsBatchOptions), _P(_vp), _sp]),
    "qs_batch_run": (_i, [_vp, _dp, _dp, _dp]),
    "qs_batch_config": (_i, [_vp, _P(_i), _P(_i)]),
    "qs_batch_free": (None, [_vp]),
    "qs_qasm_run": (_i, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint64, _i, _P(_vp)]),
    "qs_qasm_run_file": (_i, [ctypes.c_char_p, ctypes.c_uint64, _i, _P(_vp)]),
    "qs_qasm_qreg_count": (_sz, [_vp]),
    "qs_qasm_qreg_name": (ctypes.c_char_p, [_vp, _sz]),
    "qs_qasm_qreg": (_vp, [_vp, _sz]),
    "qs_qasm_creg_count": (_sz, [_vp]),
    "qs_qasm_creg_name": (ctypes.c_char_p, [_vp, _sz]),
    "qs_qasm_creg_size": (_sz, [_vp, _sz]),
    "qs_qasm_creg_bits": (_i, [_vp, _sz, _P(ctypes.c_uint8)]),
    "qs_qasm_free": (None, [_vp]),
    "qs_get_state": (_i, [_vp, _dp]),
    "qs_set_state": (_i, [_vp, _dp]),
    "qs_probabilities": (_i, [_vp, _dp]),
    "qs_register_eq": (_i, [_vp, _vp, ctypes.c_double, _P(_i)]),
    "qs_synchronize": (_i, [_vp]),
    "qs_register_stream": (_vp, [_vp]),
    "qs_last_error": (ctypes.c_char_p, []),
    "qs_launch_count": (ctypes.c_uint64, []),
    "qs_version": (ctypes.c_char_p, []),
    "qs_selftest_bounded_waits": (_i, [_P(_i), _P(_i)]),
}

_lib: ctypes.CDLL | None = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load the engine library (building it first if it is missing) and bind every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        from . import build as _build

        _build.build()
    if not p.exists():
        raise RuntimeError(f"quaru_gb300: {p} is missing; run quaru_gb300/build.py (needs nvcc)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError here means the library lacks a declared symbol
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().qs_last_error().decode(errors="replace")
