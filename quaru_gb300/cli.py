"""A command shell over the engine: the counterpart of Quaru's interactive CLI (src/bin/cli.rs).

The reference's shell offers, from a menu, to create quantum and classical registers, apply a
unary gate (identity, Hadamard, phase, NOT, Pauli Y, Pauli Z) or a binary one (CNOT, swap), measure
a qubit (optionally into a classical bit), show a register, draw a register's circuit and run an
OpenQASM file (src/bin/cli.rs:239-284, src/cli_utils/types.rs). This shell offers the same actions
as line commands, so it can be driven interactively or by a script on standard input:

    create q|c NAME SIZE           apply QREG GATE TARGET [TARGET]     measure QREG QUBIT [CREG BIT]
    show REG                       circuit QREG                        qasm PATH
    help                           exit

Run with `python -m quaru_gb300.cli [--size N] [--seed S]`; --size creates "qreg0" like the
reference's flag. Measurement draws come from a SplitMix64 generator seeded with --seed. Gate
application and measurement run on the GPU through the C ABI.
"""
from __future__ import annotations

import argparse
import shlex
import sys
from typing import TextIO

from . import operation as O
from .register import Register
from .workloads import SplitMix64

UNARY = {"identity": (O.identity, "I"), "hadamard": (O.hadamard, "H"), "phase": (O.phase, "P"),
         "not": (O.not_, "X"), "pauli_y": (O.pauli_y, "Y"), "pauli_z": (O.pauli_z, "Z")}
BINARY = {"cnot": (O.cnot, "cnot"), "swap": (O.swap, "swap")}


class Shell:
    """The simulator state: named quantum registers with their gate history, named classical ones."""

    def __init__(self, seed: int = 0, out: TextIO = sys.stdout):
        self.qregs: dict[str, Register] = {}
        self.history: dict[str, list[tuple[str, list[int]]]] = {}
        self.cregs: dict[str, list[bool]] = {}
        self.rng = SplitMix64(seed)
        self.out = out

    def say(self, text: str) -> None:
        print(text, file=self.out)

    # ---- commands
    def create(self, kind: str, name: str, size: str) -> None:
        n = int(size)
        if n < 1:
            raise ValueError("size must be at least 1")
        if name in self.qregs or name in self.cregs:
            raise ValueError(f"register {name} exists")
        if kind == "q":
            self.qregs[name] = Register.new([False] * n, rng=self.rng.uniform)
            self.history[name] = []
        elif kind == "c":
            self.cregs[name] = [False] * n
        else:
            raise ValueError("register kind is q or c")

    def _qreg(self, name: str) -> Register:
        if name not in self.qregs:
            raise ValueError(f"no quantum register {name}")
        return self.qregs[name]

    def apply(self, reg: str, gate: str, *targets: str) -> None:
        r = self._qreg(reg)
        t = [int(x) for x in targets]
        for q in t:
            if not 0 <= q < r.size():
                raise ValueError(f"qubit {q} out of range")
        if gate in UNARY:
            if len(t) != 1:
                raise ValueError(f"{gate} takes one target")
            r.apply(UNARY[gate][0](t[0]))
        elif gate in BINARY:
            if len(t) != 2 or t[0] == t[1]:
                raise ValueError(f"{gate} takes two distinct targets")
            r.apply(BINARY[gate][0](t[0], t[1]))  # cnot: control, target
        else:
            raise ValueError(f"unknown gate {gate}")
        self.history[reg].append((gate, t))

    def measure(self, reg: str, qubit: str, creg: str | None = None, bit: str | None = None) -> None:
        r = self._qreg(reg)
        q = int(qubit)
        if not 0 <= q < r.size():
            raise ValueError(f"qubit {q} out of range")
        if creg is not None and (creg not in self.cregs or bit is None or not 0 <= int(bit) < len(self.cregs[creg])):
            raise ValueError("no such classical bit")
        res = r.measure(q)
        if creg is not None:
            self.cregs[creg][int(bit)] = res
        self.history[reg].append(("measure", [q]))
        self.say(f"Qubit at measured {str(res).lower()}")

    def show(self, name: str) -> None:
        if name in self.cregs:
            bits = self.cregs[name]
            self.say(f"Classical register of size: {len(bits)}")
            self.say("[" + ", ".join(str(b).lower() for b in bits) + "]")
            return
        r = self._qreg(name)
        n = r.size()
        self.say(f"Quantum register of size: {n}")
        for i, s in enumerate(r.state):
            self.say(f"{i:0{n}b}: {s.real:+.6f}{s.imag:+.6f}i")

    def circuit(self, name: str) -> None:
        """One text line per qubit and a column per operation; CNOT draws its control as O."""
        n = self._qreg(name).size()
        rows = [[f"|q{q}>"] for q in range(n)]
        for gate, t in self.history[name]:
            col = ["-"] * n
            if gate == "cnot":
                col[t[0]], col[t[1]] = "O", "X"
            elif gate == "swap":
                col[t[0]] = col[t[1]] = "x"
            elif gate == "measure":
                col[t[0]] = "M"
            elif gate == "qasm":
                col = ["#"] * n
            else:
                col[t[0]] = UNARY[gate][1]
            if len(t) == 2:
                lo, hi = sorted(t)
                for q in range(lo + 1, hi):
                    col[q] = "|"
            for q in range(n):
                rows[q].append(col[q])
        for row in rows:
            self.say(row[0] + "-" + "-".join(row[1:]) + ("-" if len(row) > 1 else ""))

    def qasm(self, path: str) -> None:
        from .openqasm import run_openqasm

        res = run_openqasm(path, seed=self.rng.next_u64())
        for name, reg in res.qregs.items():
            self.qregs[name] = reg
            self.history[name] = [("qasm", [])]
        self.cregs.update(res.cregs)
        self.say(f"ran {path}: quantum {sorted(res.qregs)} classical {sorted(res.cregs)}")

    # ---- dispatch
    def run_line(self, line: str) -> bool:
        """Execute one command line; False once the shell should exit."""
        words = shlex.split(line)
        if not words or words[0].startswith("#"):
            return True
        cmd, args = words[0], words[1:]
        if cmd in ("exit", "quit"):
            return False
        if cmd == "help":
            self.say(__doc__.split("\n\n")[2])
            return True
        handler = {"create": self.create, "apply": self.apply, "measure": self.measure, "show": self.show,
                   "circuit": self.circuit, "qasm": self.qasm}.get(cmd)
        try:
            if handler is None:
                raise ValueError(f"unknown command {cmd} (try help)")
            handler(*args)
        except (ValueError, TypeError, RuntimeError) as e:
            self.say(f"error: {e}")
        return True


def main(argv: list[str] | None = None, stdin: TextIO = sys.stdin, out: TextIO = sys.stdout) -> int:
    ap = argparse.ArgumentParser(description="Quaru shell on the GB300 engine")
    ap.add_argument("--size", type=int, help="create quantum register qreg0 with this many qubits")
    ap.add_argument("--seed", type=int, default=0, help="seed of the measurement draws")
    args = ap.parse_args(argv)
    sh = Shell(args.seed, out)
    if args.size:
        sh.create("q", "qreg0", str(args.size))
    interactive = stdin.isatty()
    while True:
        if interactive:
            print("quaru> ", end="", file=out, flush=True)
        line = stdin.readline()
        if not line or not sh.run_line(line):
            return 0


if __name__ == "__main__":
    sys.exit(main())
