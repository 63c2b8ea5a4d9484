"""CPU check of bench.py's reference arm: one JSON line with the contract's keys, on a small sample."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3", "--cpu-qubits", "14"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT, check=True).stdout
    lines = [line for line in out.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["higher_is_better"] is True
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "config", "cpu_baseline",
                "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["sample_qubits"] == 14


def test_cpu_sweep_stops_at_the_limit():
    """The host sweep runs n = 12, 14, ... and stops at the first size past the limit."""
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--cpu-sweep", "--cpu-limit", "0.5"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT, check=True).stdout
    d = json.loads([line for line in out.splitlines() if line.startswith("{")][-1])
    runs = d["cpu_sweep"]["runs"]
    assert runs[0]["qubits"] == 12 and all(r["completed"] for r in runs[:-1]) and not runs[-1]["completed"]
    assert d["cpu_sweep"]["largest_completed_qubits"] == (runs[-2]["qubits"] if len(runs) > 1 else None)
    assert d["parity_12q"]["gates"] == 200 and len(d["parity_12q"]["bitstring"]) == 12
