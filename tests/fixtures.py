"""Loading the committed golden fixtures and comparing amplitudes."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

from quaru_gb300.operation import Operation

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_parity_golden():
    doc = json.loads((GOLDEN / "parity12.json").read_text())
    gates = []
    for g in doc["gates"]:
        k = len(g["targets"])
        vals = np.array([complex(float.fromhex(re), float.fromhex(im)) for re, im in g["matrix"]])
        gates.append(Operation(vals.reshape(1 << k, 1 << k), g["targets"]))
    draws = [float.fromhex(x) for x in doc["draws"]]
    return doc, gates, draws


def golden_state() -> np.ndarray:
    return np.fromfile(GOLDEN / "parity12_state.bin", dtype="<f8").view(np.complex128)


def sha(a: np.ndarray) -> str:
    b = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64).copy()
    b[b == 0.0] = 0.0
    return hashlib.sha256(b.astype("<f8").tobytes()).hexdigest()


def value_equal(a: np.ndarray, b: np.ndarray) -> bool:
    """Bit-identical IEEE values, with +0 == -0 (and NaN == NaN at the same place)."""
    a = np.asarray(a, dtype=np.complex128).view(np.float64)
    b = np.asarray(b, dtype=np.complex128).view(np.float64)
    return bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def floored_rel_err(got: np.ndarray, ref: np.ndarray) -> float:
    """max_i |got_i - ref_i| / max(|ref_i|, 2^(-n/2)): the per-amplitude criterion for generic gates."""
    n = int(np.log2(ref.size))
    floor = 2.0 ** (-n / 2.0)
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor)))
