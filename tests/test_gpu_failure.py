"""Failure detection on the GPU without a fault: the engine's bounded device waits (the tile and pass
kernels' mbarrier wait, the batched kernel's completion-counter wait) run on conditions nothing
satisfies, give up after their limit, report it, and leave the context usable."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_waits_give_up_and_the_context_stays_usable():
    import quaru_gb300 as q
    from quaru_gb300 import operation as O

    lib = q._lib.load()
    mbar, counter = ctypes.c_int(-1), ctypes.c_int(-1)
    assert lib.qs_selftest_bounded_waits(ctypes.byref(mbar), ctypes.byref(counter)) == 0
    assert mbar.value == 1 and counter.value == 1
    # the context still runs work: H on qubit 0 of |000>
    r = q.Register.from_int(3, 0)
    r.try_apply_fast(O.hadamard(0))
    st = r.state
    assert st[0] == O.FRAC_1_SQRT_2 and st[1] == O.FRAC_1_SQRT_2 and np.count_nonzero(st) == 2
