"""OpenQASM 2.0 front end (src/openqasm.rs), running on the GB300 engine.

run_openqasm(path) returns an OpenQASMResult with one Register per qreg and a
list of bits per creg; OpenQASMError carries the parse or run error, as the
reference's OpenQASMError::{OpenQASMParseError, OpenQASMRunError}. The parser
is the library's own (the reference's openqasm-parser crate is external).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .operation import u  # noqa: F401  (openqasm::u lives in operation.py)
from .register import Register, _check


class OpenQASMError(Exception):
    def __init__(self, code: int, message: str):
        self.code = code
        self.kind = {_lib.QS_QASM_PARSE_ERROR: "OpenQASMParseError",
                     _lib.QS_QASM_RUN_ERROR: "OpenQASMRunError"}.get(code, "Other")
        super().__init__(f"{self.kind}: {message}")


@dataclass
class OpenQASMResult:
    qregs: dict = field(default_factory=dict)
    cregs: dict = field(default_factory=dict)


def _collect(res) -> OpenQASMResult:
    lib = _lib.load()
    out = OpenQASMResult()
    try:
        for i in range(lib.qs_qasm_qreg_count(res)):
            name = lib.qs_qasm_qreg_name(res, i).decode()
            h = ctypes.c_void_p()
            _check(lib.qs_register_clone(ctypes.c_void_p(lib.qs_qasm_qreg(res, i)), ctypes.byref(h)))
            out.qregs[name] = Register(h.value)
        for i in range(lib.qs_qasm_creg_count(res)):
            name = lib.qs_qasm_creg_name(res, i).decode()
            bits = np.zeros(lib.qs_qasm_creg_size(res, i), dtype=np.uint8)
            lib.qs_qasm_creg_bits(res, i, bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
            out.cregs[name] = [bool(b) for b in bits]
    finally:
        lib.qs_qasm_free(res)
    return out


def run_openqasm_source(source: str, seed: int = 0, precision: int = _lib.QS_PREC_C128,
                        base_dir: str | None = None) -> OpenQASMResult:
    lib = _lib.load()
    res = ctypes.c_void_p()
    rc = lib.qs_qasm_run(source.encode(), base_dir.encode() if base_dir else None, seed, precision,
                         ctypes.byref(res))
    if rc in (_lib.QS_QASM_PARSE_ERROR, _lib.QS_QASM_RUN_ERROR):
        raise OpenQASMError(rc, _lib.last_error())
    _check(rc)
    return _collect(res)


def run_openqasm(path: str | os.PathLike, seed: int = 0, precision: int = _lib.QS_PREC_C128) -> OpenQASMResult:
    """openqasm::run_openqasm (src/openqasm.rs:52-142)."""
    lib = _lib.load()
    res = ctypes.c_void_p()
    rc = lib.qs_qasm_run_file(os.fspath(path).encode(), seed, precision, ctypes.byref(res))
    if rc in (_lib.QS_QASM_PARSE_ERROR, _lib.QS_QASM_RUN_ERROR):
        raise OpenQASMError(rc, _lib.last_error())
    _check(rc)
    return _collect(res)
