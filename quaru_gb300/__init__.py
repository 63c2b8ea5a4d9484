"""quaru_gb300 — a GB300 (sm_103a) state-vector engine behind Quaru's Register API.

The compute path is libquaru_gb300.so (CUDA kernels + the C ABI in
include/quaru_gpu.h); this package is the host-side mirror of the reference's
Rust API (Register, Operation, the gate constructors) over that ABI.
"""
from . import _lib
from ._lib import (QS_ARITH_DF64, QS_ARITH_EXACT, QS_ARITH_FMA, QS_ARITH_FX64, QS_PREC_C64, QS_PREC_C128)
from .operation import Operation
from .register import EngineError, OperationError, ParamCircuit, ParamGate, PauliSum, Register, circuit_autotune

__all__ = ["Register", "ParamGate", "ParamCircuit", "PauliSum", "Operation", "OperationError", "EngineError", "QS_PREC_C128", "QS_PREC_C64",
           "QS_ARITH_EXACT", "QS_ARITH_FMA", "QS_ARITH_DF64", "QS_ARITH_FX64", "circuit_autotune"]


def version() -> str:
    return _lib.load().qs_version().decode()
