"""CPU checks of the tile planner (quaru_gb300/csrc/qs_plan.cpp) with an emulated tile kernel.

tests/cpp/tile_emulator.cpp links the engine's own planner and classifier
and replays the planned stages tile by tile on the CPU; the result must equal
the oracle's gate-by-gate amplitudes (value-exact: the emulator applies each
gate with the oracle's arithmetic for k <= 2).
"""
from __future__ import annotations

import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "tile_emulator.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "tile_emulator"


@pytest.fixture(scope="module")
def emulator():
    EXE.parent.mkdir(exist_ok=True)
    srcs = [SRC, ROOT / "quaru_gb300/csrc/qs_plan.cpp", ROOT / "quaru_gb300/csrc/qs_classify.cpp"]
    if not EXE.exists() or EXE.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        import shutil

        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        cuda_inc = Path(nvcc).resolve().parent.parent / "include"
        subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "include"),
                        "-I", str(cuda_inc), *map(str, srcs), "-o", str(EXE)], check=True)
    return EXE


def run_emulator(exe, n, T, L, ops, state, mode="exact", max_ops=None, widest=False):
    buf = bytearray(struct.pack("<4i", n, T, L, len(ops)))
    for op in ops:
        t = list(op.targets)
        buf += struct.pack("<i", len(t)) + struct.pack(f"<{len(t)}i", *t)
        buf += np.ascontiguousarray(np.asarray(op.matrix, dtype=np.complex128)).tobytes()
    buf += np.ascontiguousarray(state, dtype=np.complex128).tobytes()
    argv = [str(exe), mode] + ([str(max_ops)] if max_ops else [])
    r = subprocess.run(argv, input=bytes(buf), capture_output=True, check=True)
    out = np.frombuffer(r.stdout[: 16 << n], dtype=np.complex128)
    stages, passes, most = struct.unpack("<3i", r.stdout[16 << n:])
    if widest:
        return out, stages, most
    return (out, stages, passes) if mode == "pass" else (out, stages)


def cases():
    from quaru_gb300 import operation as O
    from quaru_gb300.operation import Operation
    from quaru_gb300.workloads import SplitMix64, flatten, layered_circuit, parity_circuit, random_gate

    c = parity_circuit()
    yield "parity12", c.n, c.gates
    yield "layered14", 14, flatten(layered_circuit(14, 6, 3))
    rng = np.random.default_rng(3)
    sm = SplitMix64(11)
    ops = [random_gate(sm, 13) for _ in range(250)]
    for _ in range(10):
        a, b, cc, d, e = (int(x) for x in rng.permutation(13)[:5])
        ops.insert(int(rng.integers(len(ops))), O.to_controlled(Operation(np.array([[0.6, 0.8], [0.8, -0.6]]), [a]), b))
        ops.insert(int(rng.integers(len(ops))), O.cnz([b, cc, d], a))
        ops.insert(int(rng.integers(len(ops))), O.cnx([a, b, cc, d], e))
    yield "controls", 13, ops


@pytest.mark.parametrize("T,L", [(11, 5), (8, 3), (6, 6), (12, 5)])
def test_planned_tiles_match_oracle(emulator, oracle_mod, T, L):
    for name, n, ops in cases():
        rng = np.random.default_rng(len(ops))
        st = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        st /= np.linalg.norm(st)
        o = oracle_mod.OracleRegister.from_int(n, 0)
        o.state = st.copy()
        o.apply_sequence([(g.matrix, g.targets) for g in ops])
        got, stages = run_emulator(emulator, n, min(T, n), min(L, n), ops, st)
        assert stages < len(ops), name
        bad = np.nonzero(~((got.view(np.float64) == o.state.view(np.float64))))[0]
        assert bad.size == 0, f"{name}: {bad.size} values differ, first at {bad[:4]}"


@pytest.mark.parametrize("T,L", [(12, 5), (9, 5), (10, 3), (13, 5)])
def test_register_passes_match_oracle(emulator, oracle_mod, T, L):
    """The complex64 stage program: gates scheduled into 16-register passes (lane-bit gates
    through partner tuples), commuting gates reordered; equal to the oracle up to rounding."""
    for name, n, ops in cases():
        rng = np.random.default_rng(len(ops) + 7)
        st = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        st /= np.linalg.norm(st)
        o = oracle_mod.OracleRegister.from_int(n, 0)
        o.state = st.copy()
        o.apply_sequence([(g.matrix, g.targets) for g in ops])
        got, stages, passes = run_emulator(emulator, n, min(T, n), min(L, n), ops, st, mode="pass")
        assert stages < len(ops), name
        if min(T, n) >= 9:
            assert passes > 0, name
        err = np.max(np.abs(got - o.state) / np.maximum(np.abs(o.state), 2.0 ** (-n / 2)))
        assert err < 1e-12, f"{name}: relative error {err}"


FUSE_SRC = ROOT / "tests" / "cpp" / "fuse_check.cpp"
FUSE_EXE = ROOT / "tests" / "cpp" / "_build" / "fuse_check"


@pytest.fixture(scope="module")
def fuser():
    FUSE_EXE.parent.mkdir(exist_ok=True)
    srcs = [FUSE_SRC, ROOT / "quaru_gb300/csrc/qs_fuse.cpp"]
    if not FUSE_EXE.exists() or FUSE_EXE.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(ROOT / "include"), *map(str, srcs), "-o",
                        str(FUSE_EXE)], check=True)
    return FUSE_EXE


@pytest.mark.parametrize("W", [2, 3, 5])
def test_fused_blocks_reproduce_gate_by_gate(fuser, oracle_mod, W):
    from quaru_gb300.operation import Operation

    for name, n, ops in cases():
        if name == "controls":  # include a gate wider than W
            ops = ops + [Operation(np.eye(64, dtype=complex)[np.random.default_rng(1).permutation(64)],
                                   [0, 2, 4, 6, 8, 10])]
        rng = np.random.default_rng(len(ops) + W)
        st = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        st /= np.linalg.norm(st)
        buf = bytearray(struct.pack("<3i", n, W, len(ops)))
        for op in ops:
            t = list(op.targets)
            buf += struct.pack("<i", len(t)) + struct.pack(f"<{len(t)}i", *t)
            buf += np.ascontiguousarray(np.asarray(op.matrix, dtype=np.complex128)).tobytes()
        buf += np.ascontiguousarray(st, dtype=np.complex128).tobytes()
        r = subprocess.run([str(fuser)], input=bytes(buf), capture_output=True, check=True)
        got = np.frombuffer(r.stdout[: 16 << n], dtype=np.complex128)
        nblocks = struct.unpack("<i", r.stdout[16 << n:])[0]
        o = oracle_mod.OracleRegister.from_int(n, 0)
        o.state = st.copy()
        o.apply_sequence([(g.matrix, g.targets) for g in ops])
        assert nblocks < len(ops)
        assert np.max(np.abs(got - o.state)) < 1e-12, name


@pytest.mark.parametrize("max_ops", [4, 32])
def test_stage_gate_cap(emulator, oracle_mod, max_ops):
    """plan_tiles with a cap on the gates per stage (the adjoint's reverse sweep plans with 32): no
    stage exceeds it, and the capped plan still gives the oracle's amplitudes exactly."""
    for name, n, ops in cases():
        rng = np.random.default_rng(len(ops) + 11)
        st = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        st /= np.linalg.norm(st)
        o = oracle_mod.OracleRegister.from_int(n, 0)
        o.state = st.copy()
        o.apply_sequence([(g.matrix, g.targets) for g in ops])
        got, stages, most = run_emulator(emulator, n, min(11, n), min(5, n), ops, st, max_ops=max_ops, widest=True)
        assert 0 < most <= max_ops, (name, most)
        _, uncapped = run_emulator(emulator, n, min(11, n), min(5, n), ops, st)
        assert stages >= uncapped, name
        bad = np.nonzero(~((got.view(np.float64) == o.state.view(np.float64))))[0]
        assert bad.size == 0, f"{name}: {bad.size} values differ"
