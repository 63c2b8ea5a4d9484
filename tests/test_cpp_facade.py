"""The C++ facade include/quaru/quaru.hpp: compiled on the CPU, run on the GPU."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "facade_test.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "facade_test"


@pytest.fixture(scope="module")
def facade_exe():
    from quaru_gb300 import _lib

    _lib.load()  # builds the library if needed
    EXE.parent.mkdir(exist_ok=True)
    lib_dir = ROOT / "quaru_gb300"
    deps = [SRC, ROOT / "include" / "quaru" / "quaru.hpp", ROOT / "include" / "quaru_gpu.h", lib_dir / "libquaru_gb300.so"]
    if not EXE.exists() or EXE.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        subprocess.run(["g++", "-O1", "-std=c++17", "-Wall", "-I", str(ROOT / "include"), str(SRC), "-o", str(EXE),
                        "-L", str(lib_dir), "-lquaru_gb300", f"-Wl,-rpath,{lib_dir}"], check=True)
    return EXE


def test_facade_compiles_and_links(facade_exe):
    assert facade_exe.exists()


@pytest.mark.gpu
def test_facade_reference_tests_pass(facade_exe, tmp_path):
    r = subprocess.run([str(facade_exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all passed" in r.stdout
