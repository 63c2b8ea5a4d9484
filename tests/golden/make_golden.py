"""Generate the committed golden fixtures from the CPU oracle.

parity12.json: the seeded 12-qubit, 200-gate parity circuit (gates as hex
floats, so replaying it needs no libm), the 12 measurement draws, the SHA-256
of the oracle's amplitudes after the gates and after measuring q0..q11, and
the measured bitstring. parity12_state.bin: the post-gate amplitudes
(interleaved little-endian float64).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.oracle import OracleRegister  # noqa: E402
from quaru_gb300.workloads import parity_circuit  # noqa: E402

HERE = Path(__file__).resolve().parent


def sha(a: np.ndarray) -> str:
    b = np.ascontiguousarray(a, dtype=np.complex128).view(np.float64).copy()
    b[b == 0.0] = 0.0  # +0 and -0 hash alike
    return hashlib.sha256(b.astype("<f8").tobytes()).hexdigest()


def main() -> None:
    c = parity_circuit()
    reg = OracleRegister.from_int(c.n, 0)
    reg.apply_sequence([(g.matrix, g.targets) for g in c.gates])
    post_gates = reg.state.copy()
    bits, probs = [], []
    for q in range(c.n):
        bits.append(int(reg.measure(q, c.draws[q])))
        probs.append([p.hex() for p in reg.last_probs])
    doc = {
        "description": "12-qubit |0..0>, 200 seeded gates over {H,X,Y,Z,phase(theta),CNOT,SWAP,Toffoli,Haar}, "
                       "then measure q0..q11 with the listed draws; amplitudes from the CPU oracle",
        "n": c.n,
        "gates": [{"targets": list(map(int, g.targets)),
                   "matrix": [[float(v.real).hex(), float(v.imag).hex()] for v in np.asarray(g.matrix).ravel()]}
                  for g in c.gates],
        "draws": [float(x).hex() for x in c.draws],
        "sha256_after_gates": sha(post_gates),
        "sha256_after_measure": sha(reg.state),
        "bitstring": bits,
        "measure_probs": probs,
    }
    (HERE / "parity12.json").write_text(json.dumps(doc, indent=1))
    post_gates.astype(np.complex128).view(np.float64).astype("<f8").tofile(HERE / "parity12_state.bin")
    print("wrote", HERE / "parity12.json", "bits", "".join(map(str, bits)))


if __name__ == "__main__":
    main()
