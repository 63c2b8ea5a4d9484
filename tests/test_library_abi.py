"""CPU checks of the C ABI: the in-tree library loads and exports every symbol include/quaru_gpu.h declares."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols() -> list[str]:
    text = (ROOT / "include" / "quaru_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qs_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from quaru_gb300 import _lib

    return _lib.load()


def test_header_declares_the_reference_surface():
    syms = declared_symbols()
    for s in ("qs_register_new", "qs_register_from_int", "qs_register_try_from_qubits", "qs_try_apply_fast",
              "qs_try_apply_all", "qs_try_measure", "qs_get_state", "qs_set_state", "qs_probabilities",
              "qs_register_eq", "qs_register_clone", "qs_apply_circuit"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_every_symbol():
    from quaru_gb300 import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_version_and_error_without_gpu(lib):
    assert lib.qs_version().startswith(b"quaru-gb300")
    assert isinstance(lib.qs_last_error(), bytes)


def test_null_arguments_are_rejected_before_any_device_work(lib):
    h = ctypes.c_void_p()
    assert lib.qs_register_new(None, 3, 0, ctypes.byref(h)) == 5  # QS_INVALID_ARGUMENT
    assert lib.qs_register_from_int(3, 0, 7, ctypes.byref(h)) == 5  # unknown precision
    assert lib.qs_register_from_int(3, 8, 0, ctypes.byref(h)) == 5  # basis index out of range
    assert lib.qs_try_apply_fast(None, None, 2, 2, None, 1, None) == 5
    assert lib.qs_get_state(None, None) == 5


def test_no_cpu_fallback_without_gpu(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.qs_register_from_int(4, 0, 0, ctypes.byref(h))
    assert rc in (6, 7)  # QS_CUDA_ERROR / QS_OUT_OF_MEMORY: the engine refuses to run without a GPU
    assert not h.value


def test_gate_table_records_point_at_each_gate():
    """The qs_gate records Register.apply_gates builds (one numpy array, shared target and matrix
    buffers) hold each gate's arity, targets and row-major matrix; a matrix of the wrong shape is
    InvalidDimensions before anything reaches the engine."""
    import numpy as np

    from quaru_gb300 import _lib
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation
    from quaru_gb300.register import OperationError, gate_table

    assert ctypes.sizeof(_lib.QsGate) == 24
    rng = np.random.default_rng(4)
    ops = [O.hadamard(3), O.cnot(0, 5), O.cnx([1, 2], 4),
           Operation(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)), [7, 1, 6])]
    table, keep = gate_table(ops)
    for rec, op in zip(table, ops):
        k = int(rec["k"])
        t = np.frombuffer((ctypes.c_size_t * k).from_address(int(rec["targets"])), dtype=np.uintp)
        m = np.frombuffer((ctypes.c_double * (2 * 4 ** k)).from_address(int(rec["matrix"])), dtype=np.float64)
        assert list(t) == list(op.targets)
        assert np.array_equal(m.view(np.complex128).reshape(1 << k, 1 << k), np.asarray(op.matrix))
    with pytest.raises(OperationError) as e:
        gate_table([O.hadamard(0), Operation(np.eye(2), [0, 1])])
    assert e.value.kind == "InvalidDimensions" and e.value.payload == (2, 2)


def test_param_gate_table_records_point_at_each_gate():
    """qs_param_gate records (ParamCircuit, Register.adjoint_gradient): kind, parameter index, arity,
    targets, and the fixed gates' matrices; rotations carry no matrix."""
    import numpy as np

    from quaru_gb300 import _lib
    from quaru_gb300 import operation as O
    from quaru_gb300.register import ParamCircuit, ParamGate

    assert ctypes.sizeof(_lib.QsParamGate) == 32
    gates = [ParamGate.ry(2, 0), ParamGate.fixed(O.cnot(2, 5)), ParamGate.rz(5, 1),
             ParamGate.fixed(O.cnx([0, 1], 3)), ParamGate.rx(4, 0)]
    pc = ParamCircuit(gates)
    assert len(pc) == len(gates)
    for rec, g in zip(pc.table, gates):
        assert int(rec["kind"]) == g.kind
        k = int(rec["k"])
        t = np.frombuffer((ctypes.c_size_t * k).from_address(int(rec["targets"])), dtype=np.uintp)
        if g.kind == _lib.QS_GATE_FIXED:
            assert list(t) == list(g.op.targets)
            m = np.frombuffer((ctypes.c_double * (2 * 4 ** k)).from_address(int(rec["matrix"])), dtype=np.float64)
            assert np.array_equal(m.view(np.complex128).reshape(1 << k, 1 << k), np.asarray(g.op.matrix))
        else:
            assert k == 1 and list(t) == [g.target] and int(rec["param"]) == g.param
            assert int(rec["matrix"]) == 0
