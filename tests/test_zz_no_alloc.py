"""qs_measure_probabilities_noalloc: measurement probabilities without any device allocation.

This entry point serves callers that cannot call cudaMalloc (a framework that
owns all device memory through its own allocator, a fixed memory budget, a
path where allocation and its implicit synchronisation are not allowed). They
pass a state vector they allocated themselves and a device output; the
library's partial sums live in a static device array. Here the test itself
allocates the caller-side buffers with torch (the entry point allocates
nothing) and checks that two calls in a row give exactly the sums the register
path (qs_measure_probabilities) gives: both use the same grid and the same
reduction order and read complex64 amplitudes exactly (subnormal floats
included), so the doubles must be identical. n = 24 needs 4096 partial blocks,
the most the static array holds. This file is named so that pytest collects it
last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    # a few amplitudes far below the float normal range (2^-126): subnormal in complex64
    v[1 % v.size] = 3e-40 + 2e-41j
    return v


def _register_probs(lib, reg, target):
    p0, p1 = ctypes.c_double(0), ctypes.c_double(0)
    assert lib.qs_measure_probabilities(reg.handle, target, ctypes.byref(p0), ctypes.byref(p1), None) == 0
    return p0.value, p1.value


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_register_path_on_consecutive_calls(precision):
    import torch

    import quaru_gb300 as q
    from quaru_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(4242 + precision)
    np_dtype = np.complex128 if precision == 0 else np.complex64
    for n in (1, 6, 13, 19, 24):
        st = _state(rng, n).astype(np_dtype)
        reg = q.Register.from_int(n, 0, precision=precision)
        reg.state = st.astype(np.complex128)
        buf = torch.from_numpy(st).to("cuda")          # the caller's own state buffer
        out = torch.empty(2, dtype=torch.float64, device="cuda")  # the caller's own output
        stream = torch.cuda.current_stream()
        torch.cuda.synchronize()
        err = np.zeros(3, dtype=np.uintp)
        for target in sorted({0, n // 2, n - 1}):
            want = _register_probs(lib, reg, target)
            for _call in range(2):
                out.fill_(-1.0)
                rc = lib.qs_measure_probabilities_noalloc(
                    ctypes.c_void_p(buf.data_ptr()), n, precision, target, ctypes.c_void_p(out.data_ptr()),
                    ctypes.c_void_p(stream.cuda_stream), err.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)))
                assert rc == 0, _lib.last_error()
                stream.synchronize()
                got = out.cpu().numpy()
                assert got[0] == want[0] and got[1] == want[1], (n, target, got, want)


def test_noalloc_rejects_invalid_requests():
    import torch

    from quaru_gb300 import _lib

    lib = _lib.load()
    buf = torch.zeros(16, dtype=torch.complex128, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    err = np.zeros(3, dtype=np.uintp)
    errp = err.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t))
    b, o = ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(out.data_ptr())
    assert lib.qs_measure_probabilities_noalloc(b, 4, 0, 4, o, None, errp) == 1  # InvalidTarget(4)
    assert int(err[0]) == 4
    assert lib.qs_measure_probabilities_noalloc(None, 4, 0, 0, o, None, errp) == 5
    assert lib.qs_measure_probabilities_noalloc(b, 4, 0, 0, None, None, errp) == 5
    assert lib.qs_measure_probabilities_noalloc(b, 0, 0, 0, o, None, errp) == 5
    assert lib.qs_measure_probabilities_noalloc(b, 41, 0, 0, o, None, errp) == 5
    assert lib.qs_measure_probabilities_noalloc(b, 4, 3, 0, o, None, errp) == 5
    assert "n must be" in _lib.last_error() or "precision" in _lib.last_error()
    # misaligned state (8 bytes into a complex128 buffer) and misaligned out are refused on the host
    b8 = ctypes.c_void_p(buf.data_ptr() + 8)
    assert lib.qs_measure_probabilities_noalloc(b8, 3, 0, 0, o, None, errp) == 5
    assert "aligned" in _lib.last_error()
    o4 = ctypes.c_void_p(out.data_ptr() + 4)
    assert lib.qs_measure_probabilities_noalloc(b, 3, 0, 0, o4, None, errp) == 5
