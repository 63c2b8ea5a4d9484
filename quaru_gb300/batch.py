"""Batched forward + adjoint gradients for many circuits (one persistent launch in a CUDA graph)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .register import EngineError, OperationError, ParamGate, _check, _dp, _pauli_array, _sp, param_gate_table


class Batch:
    """Circuits (ParamGate lists, parameter counts, Pauli observables) prepared once; run() replays the graph."""

    def __init__(self, circuits, precision: int = _lib.QS_PREC_C128, chunk_log2: int = 0, ctas_per_sm: int = 0,
                 arith: int = _lib.QS_ARITH_FMA):
        lib = _lib.load()
        self._keep = []
        arr = (_lib.QsBatchCircuit * max(1, len(circuits)))()
        self.nparams = []
        for i, (n, gates, nparams, terms) in enumerate(circuits):
            table, bufs = param_gate_table(gates)
            cg = table.ctypes.data_as(ctypes.POINTER(_lib.QsParamGate))
            pt = _pauli_array(terms)
            self._keep += [table, bufs, pt]
            arr[i].n, arr[i].gates, arr[i].m = n, cg, len(gates)
            arr[i].nparams, arr[i].terms, arr[i].nterms = nparams, pt, len(terms)
            self.nparams.append(nparams)
        opts = _lib.QsBatchOptions(precision, chunk_log2, ctas_per_sm, arith)
        h = ctypes.c_void_p()
        err = np.zeros(3, dtype=np.uintp)
        _check(lib.qs_batch_create(arr, len(circuits), ctypes.byref(opts), ctypes.byref(h), _sp(err)), err)
        self._h = h
        self.count = len(circuits)

    def run(self, params):
        """params: concatenated per circuit. Returns (energies[count], grads concatenated)."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float64))
        e = np.zeros(self.count)
        g = np.zeros(max(1, sum(self.nparams)))
        _check(_lib.load().qs_batch_run(self._h, _dp(p), _dp(e), _dp(g)))
        return e, g[: sum(self.nparams)]

    def config(self):
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        _lib.load().qs_batch_config(self._h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.qs_batch_free(h)
            self._h = ctypes.c_void_p()
