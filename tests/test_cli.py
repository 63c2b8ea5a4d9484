"""The command shell (quaru_gb300.cli), the counterpart of the reference's interactive CLI
(src/bin/cli.rs): classical-register commands and error handling on the CPU, a Bell-pair session
on the GPU."""
from __future__ import annotations

import io

import pytest


def _run(script: str, *argv: str) -> str:
    from quaru_gb300.cli import main

    out = io.StringIO()
    assert main(list(argv), stdin=io.StringIO(script), out=out) == 0
    return out.getvalue()


def test_classical_registers_and_errors_without_a_gpu():
    text = _run("create c bits 3\nshow bits\nfrobnicate\napply nowhere hadamard 0\nhelp\nexit\nshow bits\n")
    assert "Classical register of size: 3" in text and "[false, false, false]" in text
    assert "error: unknown command frobnicate" in text
    assert "error: no quantum register nowhere" in text
    assert "create q|c NAME SIZE" in text
    assert text.count("Classical register") == 1  # nothing runs after exit


@pytest.mark.gpu
def test_bell_pair_session():
    script = """create q r 2
create c c 2
apply r hadamard 0
apply r cnot 0 1
show r
measure r 0 c 0
measure r 1 c 1
show c
circuit r
apply r swap 0 0
"""
    text = _run(script, "--seed", "7")
    assert "00: +0.707107+0.000000i" in text and "11: +0.707107+0.000000i" in text
    outs = [line.split()[-1] for line in text.splitlines() if line.startswith("Qubit at measured")]
    assert len(outs) == 2 and outs[0] == outs[1]
    assert f"[{outs[0]}, {outs[1]}]" in text
    assert "|q0>-H-O-M---" in text and "|q1>---X---M-" in text
    assert "error: swap takes two distinct targets" in text
