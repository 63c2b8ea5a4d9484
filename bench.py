#!/usr/bin/env python
"""Gate-sweep benchmark of the GB300 state-vector engine.

Workload: the 30-qubit layered random circuit family — per layer a
Haar-random 1-qubit unitary on every qubit, then CNOTs on a random perfect
matching (15 CNOTs) — on a complex128 state (16 GiB, far larger than the
129 MB L2, so no flush is needed between steps). One step = one layer
(45 gates), applied through the reference-facing call (qs_try_apply_fast, one
call per gate, matrices from host memory). Synthetic seeded gates (SplitMix64).
The headline arithmetic is plain FP64 (fused multiply-add, `--arith fma`); the
other arithmetic forms of the dense 1-qubit sweep are timed beside it under
their own names (`dense1_forms`).

metric: HBM GB/s per gate sweep = sum over gates of the algorithmic bytes
(one read + one write of every amplitude a gate changes: 2*N*16 for a dense
1-qubit gate, N*16 for a CNOT) / time.

`--impl reference` times the reference algorithm on the host (the C
restatement of Register::try_apply_fast in oracle/, single-threaded like the
reference) on the same metric, with the same sample the GPU arm's
`cpu_baseline` uses (whole layers of the family at CPU_QUBITS qubits).
`--cpu-sweep` runs the family (40 layers) on the host at n = 12, 14, ... until
a size exceeds `--cpu-limit` seconds.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30-qubit gate-sweep HBM GB/s"
UNIT = "GB/s"
FALLBACK_HBM_GBS = 6800.0
FP64_PEAK_TFLOPS_MEASURED = 1.194  # FP64 FMA rate measured on a GB300 (8 independent chains/thread)


def gate_bytes(op, n: int, amp_bytes: int) -> float:
    """Algorithmic HBM bytes of one gate sweep (read + write of each amplitude the gate changes)."""
    m = np.asarray(op.matrix)
    N = float(1 << n)
    k = len(op.targets)
    if k == 1 and not (m[0, 1] == 0 and m[1, 0] == 0 and m[0, 0] == 1):  # dense or anti-diagonal 1q
        return 2.0 * N * amp_bytes
    if k == 2 and np.array_equal(m, np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])):
        return 2.0 * (N / 2) * amp_bytes  # CNOT: the control = 1 half
    return 2.0 * N * amp_bytes


def is_haar(op) -> bool:
    return len(op.targets) == 1


def read_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def read_traffic(precision: str, arith: str) -> float | None:
    """DRAM bytes per launch of the dense 1-qubit kernel at 30 qubits, from the committed ncu summary."""
    p = ROOT / "profiles" / "roofline_traffic.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())[f"dense1_{precision}_{arith}_30q_bytes_per_launch"])
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- CPU (reference algorithm) timing
CPU_QUBITS = 22   # host sample size: a 64 MiB state (plus the reference's per-gate clone), beyond the host caches
CPU_SWEEP_LAYERS = 40


def cpu_layers_gbps(n: int, layers, budget_s: float | None = None, limit_s: float | None = None) -> dict:
    """Time the oracle's restatement of Register::try_apply_fast (clone + per-tuple gather, mat-vec,
    scatter; 1 thread like the reference) over whole layers of the family, one gate after another.
    budget_s: stop after the first layer that ends past it. limit_s: abandon the run once it passes
    it (the run then counts as not completed)."""
    from oracle.oracle import OracleRegister

    reg = OracleRegister.from_int(n, 0)
    done_layers, gates, nbytes = 0, 0, 0.0
    t0 = time.perf_counter()
    completed = True
    for layer in layers:
        for g in layer:
            reg.try_apply_fast(g.matrix, g.targets)
            gates += 1
            nbytes += gate_bytes(g, n, 16)
            if limit_s is not None and time.perf_counter() - t0 > limit_s:
                completed = False
                break
        if not completed:
            break
        done_layers += 1
        if budget_s is not None and time.perf_counter() - t0 >= budget_s:
            break
    el = time.perf_counter() - t0
    return {"qubits": n, "layers": done_layers, "gates": gates, "seconds": el, "gates_per_s": gates / el,
            "gbps": nbytes / el / 1e9, "completed": completed}


def cpu_parity_circuit_seconds() -> dict:
    """The 12-qubit, 200-gate parity configuration on the oracle, measuring every qubit."""
    from oracle.oracle import OracleRegister
    from quaru_gb300.workloads import parity_circuit

    c = parity_circuit()
    t0 = time.perf_counter()
    reg = OracleRegister.from_int(c.n, 0)
    for g in c.gates:
        reg.try_apply_fast(g.matrix, g.targets)
    bits = [int(reg.measure(t, c.draws[t])) for t in range(c.n)]
    return {"seconds": time.perf_counter() - t0, "gates": len(c.gates), "bitstring": "".join(map(str, bits))}


def cpu_sweep(limit_s: float, start: int = 12, stop: int = 30) -> dict:
    """The family at n = start, start+2, ... (40 layers each) until a size runs past limit_s."""
    from quaru_gb300.workloads import layered_circuit, workload_seed

    runs = []
    largest = None
    for n in range(start, stop + 1, 2):
        r = cpu_layers_gbps(n, layered_circuit(n, CPU_SWEEP_LAYERS, workload_seed("layered_28q")), limit_s=limit_s)
        runs.append(r)
        if not r["completed"]:
            break
        largest = r
    return {"limit_s": limit_s, "layers": CPU_SWEEP_LAYERS, "runs": runs,
            "largest_completed_qubits": largest["qubits"] if largest else None,
            "largest_completed_gbps": largest["gbps"] if largest else None,
            "largest_completed_gates_per_s": largest["gates_per_s"] if largest else None}


def cpu_sample_text(n: int, r: dict) -> str:
    return (f"{n}-qubit instance of the layered family ({r['layers']} whole layers, {r['gates']} gates, "
            f"{r['seconds']:.1f} s): the oracle's C restatement of Register::try_apply_fast (clone + per-tuple "
            f"gather/mat-vec/scatter), 1 thread as in the reference; GB/s per sweep does not depend on the "
            f"size once the state exceeds the host caches, and the 30-qubit state plus its per-gate clone "
            f"would need 32 GiB of host memory")


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from quaru_gb300.workloads import layered_circuit, workload_seed

    n = args.cpu_qubits
    layers = layered_circuit(n, args.warmup + args.steps, workload_seed("layered_30q"))
    cpu_layers_gbps(n, layers[: args.warmup])  # warm-up layers, untimed
    r = cpu_layers_gbps(n, layers[args.warmup:])
    value = r["gbps"]
    nw = args.qubits
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{nw}-qubit layered random circuit (per layer: Haar 1q on all {nw} qubits + "
                               f"{nw // 2} CNOTs on a random perfect matching), one layer per step",
                   "qubits": nw, "precision": "c128", "sample_qubits": n, "parallelism": "single (host)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": cpu_sample_text(n, r) + "; one layer per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_cpu_sweep(args) -> None:
    out = {"cpu_sweep": cpu_sweep(args.cpu_limit), "parity_12q": cpu_parity_circuit_seconds(), "cores": 1,
           "host_cpus": os.cpu_count(), "machine": os.uname().machine}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- GPU arm
def ARITH_CODES(q) -> dict:
    return {"exact": q.QS_ARITH_EXACT, "fma": q.QS_ARITH_FMA, "df64": q.QS_ARITH_DF64, "fx64": q.QS_ARITH_FX64}


# what each arithmetic form of a complex128 dense gate computes in
ARITH_DTYPE = {"exact": "f64", "fma": "f64", "df64": "f32x2 (double-float)",
               "fx64": "int64 fixed point, rounded once to f64 (FP64-accurate)"}


def dense1_forms(q, torch, reg, layers, n: int, peak: float, count: int = 8) -> dict:
    """The dense 1-qubit sweep (k_dense1) in every arithmetic form on the same register: CUDA events
    around each of `count` Haar gates after 2 warm-up gates; GB/s = 2 * 2^n * 16 / average time."""
    haar = [g for layer in layers for g in layer if is_haar(g)][: count + 2]
    stream = torch.cuda.ExternalStream(reg.stream)
    out = {}
    for name, code in ARITH_CODES(q).items():
        reg.set_arith(code)
        for g in haar[:2]:
            reg.try_apply_fast(g)
        evs = []
        for g in haar[2:]:
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            reg.try_apply_fast(g)
            b.record(stream)
            evs.append((a, b))
        reg.synchronize()
        ms = statistics.mean(a.elapsed_time(b) for a, b in evs)
        gbs = 2.0 * (1 << n) * 16 / (ms / 1e3) / 1e9
        out[name] = {"ms": ms, "gbs": gbs, "frac_of_measured_hbm": gbs / peak, "arith": ARITH_DTYPE[name]}
    return out


def slowest_rank_seconds(dist, seconds: list, device: str) -> list:
    """Each timing's maximum over all ranks (one all-reduce): a job of replicas takes as long as its
    slowest rank. `dist` is None on a single process."""
    import torch

    t = torch.tensor(seconds, dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def job_gbs(rank_bytes: float, world: int, seconds: float) -> float:
    """Whole-job GB/s of `world` replicas that each moved `rank_bytes` over the timed steps, in
    `seconds` (the slowest rank's time for those steps)."""
    return rank_bytes * world / seconds / 1e9


def run_ours(args) -> None:
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    import quaru_gb300 as q
    from quaru_gb300 import _lib
    from quaru_gb300.workloads import layered_circuit, workload_seed

    lib = _lib.load()
    n = args.qubits
    arith = ARITH_CODES(q)[args.arith]
    prec = q.QS_PREC_C64 if args.precision == "c64" else q.QS_PREC_C128
    amp = 8 if prec == q.QS_PREC_C64 else 16
    nlayers = max(args.warmup + args.steps, 1)
    layers = layered_circuit(n, min(nlayers, 40), workload_seed("layered_30q"))
    reg = q.Register.from_int(n, 0, precision=prec)
    reg.set_arith(arith)
    stream = torch.cuda.ExternalStream(reg.stream)

    def layer(i):
        return layers[i % len(layers)]

    def barrier():
        reg.synchronize()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # ---- device-timed loop: inputs resident, no host read-back
    for i in range(args.warmup):
        for g in layer(i):
            reg.try_apply_fast(g)
    barrier()
    haar_events = []
    step_bytes = 0.0
    launches0 = lib.qs_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for i in range(args.warmup, args.warmup + args.steps):
            for g in layer(i):
                if is_haar(g) and len(haar_events) < 64:
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    reg.try_apply_fast(g)
                    b.record(stream)
                    haar_events.append((a, b))
                else:
                    reg.try_apply_fast(g)
                step_bytes += gate_bytes(g, n, amp)
        ev1.record(stream)
        barrier()
        launches = lib.qs_launch_count() - launches0
        dev_s = ev0.elapsed_time(ev1) / 1e3

        # ---- end-to-end loop: host gate data in, a host read-back of a result every step
        for i in range(args.warmup):
            for g in layer(i):
                reg.try_apply_fast(g)
            reg_p = reg  # noqa: F841
        barrier()
        h2d = 0
        t0 = time.perf_counter()
        for i in range(args.warmup, args.warmup + args.steps):
            for g in layer(i):
                reg.try_apply_fast(g)
                h2d += np.asarray(g.matrix).nbytes + 8 * len(g.targets)
            p0 = _measure_probs(lib, reg, 0)
        barrier()
        e2e_s = time.perf_counter() - t0
    clk = clocks.summary()

    fused = None
    if not args.no_fused:
        # The same layers through qs_apply_circuit with cache-blocked stages.
        fl = [g for i in range(args.warmup, args.warmup + args.steps) for g in layer(i)]
        reg.apply_gates([g for i in range(args.warmup) for g in layer(i)], fuse=1)
        barrier()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        l0 = lib.qs_launch_count()
        f0.record(stream)
        reg.apply_gates(fl, fuse=1)
        f1.record(stream)
        barrier()
        fs = f0.elapsed_time(f1) / 1e3
        fused = {"gates_per_s": len(fl) / fs, "ms_per_step": 1e3 * fs / args.steps,
                 "speedup_vs_unfused": dev_s / fs, "launches": int(lib.qs_launch_count() - l0),
                 "tile_qubits": q.circuit_autotune(n, prec, arith, 1)["tile_qubits"]}
        # fuse = 3: the autotuned form
        reg.apply_gates([g for i in range(args.warmup) for g in layer(i)], fuse=3)
        barrier()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        l0 = lib.qs_launch_count()
        a0.record(stream)
        reg.apply_gates(fl, fuse=3)
        a1.record(stream)
        barrier()
        ats = a0.elapsed_time(a1) / 1e3
        fused["autotuned"] = {"choice": q.circuit_autotune(n, prec, arith, 3), "gates_per_s": len(fl) / ats,
                              "ms_per_step": 1e3 * ats / args.steps, "speedup_vs_unfused": dev_s / ats,
                              "launches": int(lib.qs_launch_count() - l0)}
        if prec == q.QS_PREC_C128:
            # dense fused blocks at the automatic width (double-float arithmetic: 3-qubit blocks)
            b0 = torch.cuda.Event(enable_timing=True)
            b1 = torch.cuda.Event(enable_timing=True)
            reg.apply_gates([g for i in range(args.warmup) for g in layer(i)], fuse=2)
            barrier()
            l0 = lib.qs_launch_count()
            b0.record(stream)
            reg.apply_gates(fl, fuse=2)
            b1.record(stream)
            barrier()
            bs = b0.elapsed_time(b1) / 1e3
            fused["blocks"] = {"gates_per_s": len(fl) / bs, "ms_per_step": 1e3 * bs / args.steps,
                               "speedup_vs_unfused": dev_s / bs, "launches": int(lib.qs_launch_count() - l0),
                               "max_width": q.circuit_autotune(n, prec, arith, 2)["max_width"]}
            # the same layers as FP64-accurate 5-qubit blocks: split-integer products on the BF16 tensor
            # cores (k_tile_oz), one stage per block; time per stage from CUDA events around each launch
            reg.set_arith(q.QS_ARITH_FX64)
            reg.apply_gates([g for i in range(args.warmup) for g in layer(i)], fuse=2, max_width=5)
            barrier()
            o0 = torch.cuda.Event(enable_timing=True)
            o1 = torch.cuda.Event(enable_timing=True)
            l0 = lib.qs_launch_count()
            o0.record(stream)
            reg.apply_gates(fl, fuse=2, max_width=5)
            o1.record(stream)
            barrier()
            os_ = o0.elapsed_time(o1) / 1e3
            stages = int(lib.qs_launch_count() - l0)
            reg.set_arith(arith)
            fused["blocks_fx64_tensor"] = {
                "gates_per_s": len(fl) / os_, "ms_per_step": 1e3 * os_ / args.steps, "speedup_vs_unfused": dev_s / os_,
                "launches": stages, "ms_per_stage": 1e3 * os_ / stages,
                "hbm_frac_per_stage": 2.0 * (1 << n) * 16 / (os_ / stages) / 1e9 / read_peaks()[0],
                "arith": "FP64-accurate split-integer products on the BF16 tensor cores (tcgen05 kind::f16)"}
        if prec == q.QS_PREC_C64:
            # dense 5-qubit blocks as 3xTF32 tensor-core GEMMs
            b0 = torch.cuda.Event(enable_timing=True)
            b1 = torch.cuda.Event(enable_timing=True)
            reg.apply_gates([g for i in range(args.warmup) for g in layer(i)], fuse=2)
            barrier()
            l0 = lib.qs_launch_count()
            b0.record(stream)
            reg.apply_gates(fl, fuse=2)
            b1.record(stream)
            barrier()
            bs = b0.elapsed_time(b1) / 1e3
            fused["blocks_tf32x3"] = {"gates_per_s": len(fl) / bs, "ms_per_step": 1e3 * bs / args.steps,
                                      "speedup_vs_unfused": dev_s / bs, "launches": int(lib.qs_launch_count() - l0)}

    peak, peak_kind = read_peaks()
    forms = None
    fx_layer = None
    if prec == q.QS_PREC_C128 and not args.no_forms:
        forms = dense1_forms(q, torch, reg, layers, n, peak)
        # the same timed layers in the FP64-accurate fixed-point form (CNOTs stay index moves)
        reg.set_arith(q.QS_ARITH_FX64)
        for i in range(args.warmup):
            for g in layer(i):
                reg.try_apply_fast(g)
        barrier()
        x0 = torch.cuda.Event(enable_timing=True)
        x1 = torch.cuda.Event(enable_timing=True)
        x0.record(stream)
        for i in range(args.warmup, args.warmup + args.steps):
            for g in layer(i):
                reg.try_apply_fast(g)
        x1.record(stream)
        barrier()
        xs = x0.elapsed_time(x1) / 1e3
        fx_ms = forms["fx64"]["ms"]
        fx_layer = {"value": step_bytes / xs / 1e9, "unit": UNIT, "ms_per_step": 1e3 * xs / args.steps,
                    "gates_per_s": len(layer(0)) * args.steps / xs, "arith": ARITH_DTYPE["fx64"],
                    "roofline": {"kernel": "k_dense1_fx (dense 1-qubit gate sweep, c128, fixed-point arithmetic)",
                                 "bound": "hbm", "achieved": forms["fx64"]["gbs"], "peak": peak, "unit": "GB/s",
                                 "frac": forms["fx64"]["gbs"] / peak, "traffic": read_traffic("c128", "fx64"),
                                 "peak_source": peak_kind, "bytes_per_launch": 2.0 * (1 << n) * 16,
                                 "ms_per_launch": fx_ms}}
        reg.set_arith(arith)
    del reg
    torch.cuda.synchronize()
    tuned = None if args.no_fused else autotune_section(q, args)
    meas = None if args.no_measure else measure_section(q, torch, args)
    widths = None if args.no_widths else width_section(q, torch, args)
    precision = None if args.no_precision else precision_section(q, torch, args)
    adjoint = None if args.no_adjoint else adjoint_section(q, torch, args)
    batch = None if args.no_batch else batch_section(q, args)

    dev_s, e2e_s = slowest_rank_seconds(dist, [dev_s, e2e_s], "cuda")
    value = job_gbs(step_bytes, world, dev_s)
    e2e = job_gbs(step_bytes, world, e2e_s)

    haar_ms = [a.elapsed_time(b) for a, b in haar_events]
    avg_haar_s = statistics.mean(haar_ms) / 1e3 if haar_ms else float("nan")
    per_launch_bytes = 2.0 * (1 << n) * amp
    achieved = per_launch_bytes / avg_haar_s / 1e9
    flops_per_launch = (1 << n) * 8 * 2.0  # 8 FMAs per amplitude for a dense complex 2x2
    gates_per_step = len(layer(0))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    cpu = None
    if world == 1 and not args.no_cpu:
        # the same sample as `--impl reference`: whole layers at CPU_QUBITS qubits, same seed
        n_cpu = args.cpu_qubits
        r = cpu_layers_gbps(n_cpu, layered_circuit(n_cpu, 40, workload_seed("layered_30q")), budget_s=args.cpu_budget)
        cpu = {"value": r["gbps"], "unit": UNIT, "cores": 1, "kind": "port", "sample": cpu_sample_text(n_cpu, r),
               "gates_per_s": r["gates_per_s"], "host_cpus": os.cpu_count(),
               "sweep": cpu_sweep(args.cpu_limit, stop=n_cpu), "parity_12q": cpu_parity_circuit_seconds()}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == q.QS_PREC_C64 else ARITH_DTYPE[args.arith],
        "data": "synthetic (seeded Haar 1q + CNOT matchings, SplitMix64)",
        "config": {"workload": f"{n}-qubit layered random circuit (per layer: Haar 1q on all {n} qubits + "
                               f"{n // 2} CNOTs on a random perfect matching), one layer per step",
                   "qubits": n, "precision": args.precision, "arith": args.arith, "fuse": 0,
                   "gates_per_step": gates_per_step, "parallelism": "replicas" if world > 1 else "single",
                   "l2": f"state {(1 << n) * amp / 2**30:.0f} GiB >> 129 MB L2: inputs larger than L2, no flush"},
        "gates_per_s": gates_per_step * args.steps * world / dev_s,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": 16},
        "gpu_launches": int(launches),
        "roofline": {"kernel": f"k_dense1 (dense 1-qubit gate sweep, {args.precision}, {args.arith} arithmetic)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": read_traffic(args.precision, args.arith), "peak_source": peak_kind,
                     "bytes_per_launch": per_launch_bytes,
                     "fp64_equivalent_tflops": flops_per_launch / avg_haar_s / 1e12,
                     "fp64_pipe_peak_tflops_measured": FP64_PEAK_TFLOPS_MEASURED},
        "kernel_ms": {"dense1_avg": avg_haar_s * 1e3, "samples": len(haar_ms)},
        "dense1_forms": forms,
        "fp64_accurate_fx64": fx_layer,
        "autotune": tuned,
        "measure": meas,
        "clocks": clk,
        "fused": fused,
        "fusion_widths": widths,
        "precision_form": precision,
        "adjoint": adjoint,
        "batch": batch,
        "cpu_baseline": cpu,
        "probe": {"p0_qubit0": p0},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def autotune_section(q, args) -> dict:
    """The fusion autotuner at the bench's size: for each precision / arithmetic, the form it picks for
    qs_apply_circuit (fuse = 3: single sweeps, stages with their tile size, or dense blocks with their
    width) and the stand-in workload's time under every candidate (re-timed here)."""
    out = {}
    for name, prec, arith in (("c128_fma", q.QS_PREC_C128, q.QS_ARITH_FMA), ("c128_fx64", q.QS_PREC_C128, q.QS_ARITH_FX64),
                              ("c128_df64", q.QS_PREC_C128, q.QS_ARITH_DF64), ("c64", q.QS_PREC_C64, q.QS_ARITH_FMA)):
        out[name] = q.circuit_autotune(args.qubits, prec, arith, 3, retune=True)
    return out


def measure_section(q, torch, args) -> dict:
    """Measurement: the 12-qubit, 200-gate parity configuration end to end on the GPU (gates one call
    each, then every qubit measured in one qs_measure_sequence call, complex128 exact arithmetic:
    reference-order sums), and measuring all qubits of a dense 30-qubit complex128 state as one
    sequence (each pass reads only the live subspace and fuses the next qubit's sums) against one
    qs_try_measure call per qubit."""
    from quaru_gb300.workloads import flatten, layered_circuit, parity_circuit, workload_seed

    c = parity_circuit()
    reps = []
    for _ in range(5):
        t0 = time.perf_counter()
        r = q.Register.from_int(c.n, 0)
        for g in c.gates:
            r.try_apply_fast(g)
        bits = r.measure_sequence(list(range(c.n)), c.draws)
        reps.append(time.perf_counter() - t0)
        del r
    out = {"parity_12q": {"workload": "12 qubits, 200 gates, measure all 12 (seeded draws)", "ms": 1e3 * min(reps),
                          "bitstring": "".join(str(int(b)) for b in bits)}}
    n = args.qubits
    a = q.Register.from_int(n, 0)
    a.set_arith(q.QS_ARITH_FMA)
    a.apply_gates(flatten(layered_circuit(n, 1, workload_seed("layered_30q"))))
    b = a.clone()
    draws = [float(x) for x in np.random.default_rng(30).uniform(size=n)]
    a.synchronize()
    b.synchronize()
    t0 = time.perf_counter()
    seq = a.measure_sequence(list(range(n)), draws)
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    one = [b.measure(t, d) for t, d in enumerate(draws)]
    t_one = time.perf_counter() - t0
    out[f"measure_all_{n}q"] = {"sequence_ms": 1e3 * t_seq, "per_qubit_calls_ms": 1e3 * t_one,
                                "speedup": t_one / t_seq, "same_outcomes": seq == one,
                                "first_pass_bytes": 3.0 * (1 << n) * 16}
    del a, b
    return out


def width_section(q, torch, args) -> dict:
    """The plain form at scale: a 28-qubit complex128 layered circuit (Haar on every qubit + a CNOT
    matching per layer) with fusion off (one sweep per gate), cache-blocked stages, and dense fused
    blocks of width 2..5 (each block one sweep or one tensor-core stage). Per variant: ms, gates/s,
    sweeps, and the HBM GB/s those sweeps move (each gate's own bytes unfused, 2 * 2^n * 16 bytes per
    fused sweep). Arithmetic per variant: plain FP64 (fused multiply-add; its blocks are FP64 dense
    sweeps), the FP64-accurate fixed-point form (`fx64`: single sweeps on the integer pipes, blocks as
    split-integer products on the BF16 tensor cores; every width pads its blocks to 5 qubits), and
    double-float (`df64`, narrower than FP64: 24 + 24 significand bits) for comparison. Layers: 40,
    except 10 for the FP64 blocks of 3..5 qubits, whose FP64 dense sweeps are slow."""
    from quaru_gb300.workloads import flatten, layered_circuit, workload_seed

    n = 28
    lib = q._lib.load()
    reg = q.Register.from_int(n, 0)
    stream = torch.cuda.ExternalStream(reg.stream)
    sweep_bytes = 2.0 * (1 << n) * 16
    out = {"workload": f"{n}-qubit layered random circuit (per layer: Haar 1q on every qubit + {n // 2} CNOTs on "
                       f"a random perfect matching), complex128", "qubits": n}
    A = {"fma": q.QS_ARITH_FMA, "fx64": q.QS_ARITH_FX64, "df64": q.QS_ARITH_DF64}
    variants = [("fma_unfused", "fma", 0, 5, 40), ("fma_stages", "fma", 1, 5, 40), ("fma_blocks_w2", "fma", 2, 2, 40),
                ("fma_blocks_w3", "fma", 2, 3, 10), ("fma_blocks_w4", "fma", 2, 4, 10), ("fma_blocks_w5", "fma", 2, 5, 10),
                ("fx64_unfused", "fx64", 0, 5, 40), ("fx64_blocks_w2", "fx64", 2, 2, 40),
                ("fx64_blocks_w3", "fx64", 2, 3, 40), ("fx64_blocks_w4", "fx64", 2, 4, 40),
                ("fx64_blocks_w5", "fx64", 2, 5, 40),
                ("df64_unfused", "df64", 0, 5, 40), ("df64_blocks_w3", "df64", 2, 3, 40)]
    for name, ar, fuse, width, layers in variants:
        reg.set_arith(A[ar])
        ops = flatten(layered_circuit(n, layers, workload_seed("layered_28q")))
        reg.apply_gates(ops[: 3 * (n + n // 2)], fuse=fuse, max_width=width)  # warm-up: 3 layers
        reg.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        l0 = lib.qs_launch_count()
        a.record(stream)
        reg.apply_gates(ops, fuse=fuse, max_width=width)
        b.record(stream)
        reg.synchronize()
        s = a.elapsed_time(b) / 1e3
        sweeps = int(lib.qs_launch_count() - l0)
        # bytes the sweeps move: per gate (a CNOT touches half the state) unfused, whole states otherwise
        moved = sum(gate_bytes(g, n, 16) for g in ops) if fuse == 0 else sweeps * sweep_bytes
        out[name] = {"arith": ar, "fuse": fuse, "max_width": width if fuse == 2 else None, "layers": layers,
                     "gates": len(ops), "ms": 1e3 * s, "gates_per_s": len(ops) / s, "sweeps": sweeps,
                     "hbm_gbs": moved / s / 1e9}
    out["fx64_blocks_w5_vs_fma_unfused"] = out["fx64_blocks_w5"]["gates_per_s"] / out["fma_unfused"]["gates_per_s"]
    out["fx64_blocks_w5_vs_fx64_unfused"] = out["fx64_blocks_w5"]["gates_per_s"] / out["fx64_unfused"]["gates_per_s"]
    return out


def precision_section(q, torch, args) -> dict:
    """The layered family at the bench's size for 40 layers: complex128 gate by gate in FP64 FMA
    arithmetic (the plain FP64 form) against complex128 double-float sweeps and complex64 fused stages
    (register passes, and 5-qubit dense blocks as 3xTF32 tensor-core GEMMs), with
    1 - F = 1 - |<x|fp64>|^2 / (<x|x><fp64|fp64>) accumulated in FP64 on the GPU after every 10
    layers, and the gates/s of each form."""
    from quaru_gb300.workloads import flatten, layered_circuit, workload_seed

    n = args.qubits
    layers = layered_circuit(n, 40, workload_seed("layered_30q"))
    torch.cuda.synchronize()
    regs = {"fp64_plain": q.Register.from_int(n, 0),
            "c128_fx64": q.Register.from_int(n, 0),
            "c128_fx64_blocks": q.Register.from_int(n, 0),
            "c128_df64": q.Register.from_int(n, 0),
            "c64_passes": q.Register.from_int(n, 0, precision=q.QS_PREC_C64),
            "c64_blocks_tf32x3": q.Register.from_int(n, 0, precision=q.QS_PREC_C64)}
    regs["fp64_plain"].set_arith(q.QS_ARITH_FMA)  # the plain FP64 form: FP64 fused multiply-add
    regs["c128_fx64"].set_arith(q.QS_ARITH_FX64)  # FP64-accurate fixed point, one sweep per gate
    regs["c128_fx64_blocks"].set_arith(q.QS_ARITH_FX64)  # FP64-accurate 5-qubit blocks on the tensor cores
    regs["c128_df64"].set_arith(q.QS_ARITH_DF64)
    fuse = {"fp64_plain": 0, "c128_fx64": 0, "c128_fx64_blocks": 2, "c128_df64": 0, "c64_passes": 1,
            "c64_blocks_tf32x3": 2}
    secs = {k: 0.0 for k in regs}
    gates = 0
    checkpoints = []
    for k in range(4):
        chunk = flatten(layers[10 * k:10 * k + 10])
        gates += len(chunk)
        for name, r in regs.items():
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            st = torch.cuda.ExternalStream(r.stream)
            ev0.record(st)
            r.apply_gates(chunk, fuse=fuse[name])
            ev1.record(st)
            ev1.synchronize()
            secs[name] += ev0.elapsed_time(ev1) / 1e3
        ref = regs["fp64_plain"]
        nref = ref.inner_product(ref).real
        cp = {"layers": 10 * (k + 1)}
        for name in ("c128_fx64", "c128_fx64_blocks", "c128_df64", "c64_passes", "c64_blocks_tf32x3"):
            r = regs[name]
            f = abs(r.inner_product(ref)) ** 2 / (nref * r.inner_product(r).real)
            cp[f"one_minus_fidelity_{name}"] = 1.0 - f
        checkpoints.append(cp)
    out = {"workload": f"{n}-qubit layered family, 40 layers ({gates} gates), same seed as the main run",
           "checkpoints": checkpoints,
           "gates_per_s": {k: gates / v for k, v in secs.items()}}
    out["mixed_vs_fp64_gates_per_s"] = {k: secs["fp64_plain"] / secs[k]
                                        for k in ("c128_df64", "c64_passes", "c64_blocks_tf32x3")}
    out["fp64_accurate_vs_fp64_gates_per_s"] = {k: secs["fp64_plain"] / secs[k] for k in ("c128_fx64", "c128_fx64_blocks")}
    out["fp64_plain_arith"] = "FP64 fused multiply-add, one sweep per gate"
    del regs
    return out


def adjoint_section(q, torch, args) -> dict:
    """Gradient throughput on the 20-qubit, 10-layer ansatz (400 parameters, ZZ + X chain observable):
    FP64 (complex128, FP64 FMA arithmetic), complex128 with double-float arithmetic, and mixed (complex64
    state, FP64 accumulations), with the mixed run's 1 - F."""
    from quaru_gb300.workloads import ansatz_problem

    gates, params, terms = ansatz_problem()
    circuit, observable = q.ParamCircuit(gates), q.PauliSum(terms)  # converted once, as an optimiser loop would
    n = 20
    out = {"workload": "20-qubit hardware-efficient ansatz, 10 layers (RY, RZ on every qubit + CNOT ladder), "
                       "400 parameters, H = sum a_i Z_i Z_i+1 + sum b_i X_i"}
    grads = {}
    for name, prec, arith in (("fp64", q.QS_PREC_C128, q.QS_ARITH_FMA), ("c128_df64", q.QS_PREC_C128, q.QS_ARITH_DF64),
                              ("mixed", q.QS_PREC_C64, q.QS_ARITH_FMA)):
        reg = q.Register.from_int(n, 0, precision=prec)
        reg.set_arith(arith)
        for _ in range(3):
            e, g = reg.adjoint_gradient(circuit, params, observable)
        reps = 5
        t0 = time.perf_counter()
        for _ in range(reps):
            e, g = reg.adjoint_gradient(circuit, params, observable)
        dt = (time.perf_counter() - t0) / reps
        grads[name] = g
        out[name] = {"ms_per_gradient": 1e3 * dt, "grads_per_s": len(params) / dt, "energy": e}
    out["mixed_vs_fp64_speedup"] = out["fp64"]["ms_per_gradient"] / out["mixed"]["ms_per_gradient"]
    out["max_grad_diff_df64_vs_fp64"] = float(np.max(np.abs(grads["c128_df64"] - grads["fp64"])))
    out["max_grad_diff_mixed_vs_fp64"] = float(np.max(np.abs(grads["mixed"] - grads["fp64"])))
    a = q.Register.from_int(n, 0)
    a.set_arith(q.QS_ARITH_FMA)
    b = q.Register.from_int(n, 0, precision=q.QS_PREC_C64)
    ops = [gt.operation(params) for gt in gates]
    a.apply_gates(ops)
    b.apply_gates(ops)
    f = abs(b.inner_product(a)) ** 2 / (a.inner_product(a).real * b.inner_product(b).real)
    out["mixed_one_minus_fidelity"] = 1.0 - f
    return out


def batch_section(q, args) -> dict:
    """256 ansatz circuits (10..22 qubits, 4..12 layers): one persistent graph replay per run (FP64,
    complex128 with double-float tiles, complex64) vs a loop of single-circuit adjoint calls (FP64)."""
    from quaru_gb300.batch import Batch
    from quaru_gb300.workloads import ansatz_batch

    circuits, params = ansatz_batch()
    params = np.array(params)
    ngrads = len(params)
    out = {"workload": "256 ansatz circuits, qubits ~ U{10..22}, layers ~ U{4..12}, random Z/ZZ/X observables",
           "circuits": len(circuits), "parameters": ngrads}
    for name, prec, arith in (("fp64", q.QS_PREC_C128, q.QS_ARITH_FMA), ("c128_df64", q.QS_PREC_C128, q.QS_ARITH_DF64),
                              ("mixed", q.QS_PREC_C64, q.QS_ARITH_FMA)):
        t0 = time.perf_counter()
        b = Batch(circuits, precision=prec, arith=arith)
        setup = time.perf_counter() - t0
        b.run(params)
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            e, g = b.run(params)
        dt = (time.perf_counter() - t0) / reps
        cl, ct = b.config()
        out[name] = {"s_per_batch": dt, "circuits_per_s": len(circuits) / dt, "grads_per_s": ngrads / dt,
                     "setup_s_incl_autotune": setup, "chunk_log2": cl, "ctas_per_sm": ct}
        del b
    # the plain loop: one qs_adjoint_gradient call per circuit (FP64)
    t0 = time.perf_counter()
    off = 0
    for n, gates, npar, terms in circuits:
        reg = q.Register.from_int(n, 0)
        reg.set_arith(q.QS_ARITH_FMA)
        reg.adjoint_gradient(gates, params[off:off + npar], terms)
        off += npar
    loop = time.perf_counter() - t0
    out["loop_fp64"] = {"s_per_batch": loop, "circuits_per_s": len(circuits) / loop, "grads_per_s": ngrads / loop}
    out["batch_vs_loop_fp64"] = loop / out["fp64"]["s_per_batch"]
    return out


def _measure_probs(lib, reg, target: int) -> float:
    import ctypes

    p0, p1 = ctypes.c_double(0), ctypes.c_double(0)
    rc = lib.qs_measure_probabilities(reg.handle, target, ctypes.byref(p0), ctypes.byref(p1), None)
    if rc:
        raise RuntimeError(f"qs_measure_probabilities failed: {rc}")
    return p0.value


def run_kernels(args) -> None:
    """A small workload that launches every kernel family once per repetition (for ncu captures):
    init (basis and product state), dense 1-qubit (exact, FMA, DF64, fixed point; complex64),
    CNOT/permutation, dense 3-qubit, 6-qubit permutation and dense gates, probability reduction,
    read-back and collapse (both precisions), measurement sequences (fused collapse + next sums;
    the compact live subspace; reference-order sums), stages (complex128 FMA tiles, complex128 FP64-accurate tensor-core blocks,
    complex64 register passes, complex64 3xTF32 tensor-core blocks), adjoint (FP64 and mixed), batch
    (FP64 and mixed)."""
    import quaru_gb300 as q
    from quaru_gb300 import operation as O
    from quaru_gb300.batch import Batch
    from quaru_gb300.workloads import ansatz_batch, ansatz_problem, flatten, layered_circuit

    n = args.qubits
    rng = np.random.default_rng(1)
    layers = flatten(layered_circuit(n, 2, 7))
    haar = [g for g in layers if len(g.targets) == 1][:3]
    u3 = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0]
    for rep in range(args.steps):
        for arith in (q.QS_ARITH_EXACT, q.QS_ARITH_FMA, q.QS_ARITH_DF64, q.QS_ARITH_FX64):
            r = q.Register.from_int(n, 0)
            r.set_arith(arith)
            for g in haar:
                r.try_apply_fast(g)
        r.try_apply_fast(O.cnot(3, n - 2))
        r.try_apply_fast(O.cnx([1, 2], n - 1))
        r.try_apply_fast(O.Operation(u3, [0, n // 2, n - 3]))
        r.measure(n - 1, 0.5)
        r.measure_sequence([0, 1, n // 2], [0.3, 0.6, 0.4])  # fused collapse + next sums, live subspace
        fresh = q.Register.from_int(n, 0)  # no measurement recorded: a sequence on the compact live subspace
        fresh.set_arith(q.QS_ARITH_FMA)
        fresh.apply_gates(layers[: n + n // 2])
        fresh.measure_sequence([0, 3, n // 2, n - 1], [0.3, 0.6, 0.4, 0.7])
        del fresh
        small = q.Register.from_int(12, 0)  # exact arithmetic: the reference's summation order
        small.apply_gates(layers[:12] if n == 12 else flatten(layered_circuit(12, 1, 7)))
        small.measure_sequence(list(range(12)), [0.5] * 12)
        r.apply_gates(layers, fuse=1)
        r.apply_gates(layers, fuse=2, max_width=5)  # fixed point: FP64-accurate tensor-core blocks
        # wide gates (out-of-place kernels), a product-state register, the probability read-back
        perm = np.eye(64)[np.random.default_rng(2).permutation(64)]
        r.try_apply_fast(O.Operation(perm, [0, 3, 7, 11, n - 5, n - 2]))
        r.try_apply_fast(O.Operation(np.linalg.qr(rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64)))[0],
                                     [1, 4, 6, 9, n - 4, n - 1]))
        pq = [np.array([[np.cos(0.1 * i)], [np.sin(0.1 * i)]], dtype=complex) for i in range(n)]
        p_reg = q.Register.try_from_qubits(pq)
        p_reg.probabilities()
        c = q.Register.from_int(n, 0, precision=q.QS_PREC_C64)
        c.apply_gates(layers[:len(layers) // 2], fuse=0)
        c.apply_gates(layers, fuse=1)
        c.apply_gates(layers, fuse=2)
        c.measure(n - 1, 0.5)
        del r, c, p_reg
    gates, params, terms = ansatz_problem()
    for prec in (q.QS_PREC_C128, q.QS_PREC_C64):  # FP64 and mixed (complex64) adjoint gradients
        reg = q.Register.from_int(20, 0, precision=prec)
        reg.set_arith(q.QS_ARITH_FMA)
        reg.adjoint_gradient(gates, params, terms)
    circuits, bp = ansatz_batch(count=16, qmin=10, qmax=18, lmin=2, lmax=4, seed=3)
    for prec in (q.QS_PREC_C128, q.QS_PREC_C64):
        b = Batch(circuits, precision=prec, chunk_log2=11, ctas_per_sm=2)
        b.run(bp)
    print(json.dumps({"kernels": "done", "qubits": n, "launches": int(q._lib.load().qs_launch_count())}))


def run_case(args) -> None:
    """Small profiling workloads (for ncu captures of one kernel family, --qubits 26 by default):
    dense-<arith>: four dense 1-qubit Haar sweeps on a dense complex128 register in that arithmetic;
    blocks-c64: two layers of the family as 5-qubit 3xTF32 blocks on a complex64 register;
    blocks-fx64: the same layers as FP64-accurate 5-qubit blocks on a complex128 register (split
    integer products on the tensor cores); stages-c64: the same layers as register passes;
    measure-all: every qubit of a dense complex128 register measured in one sequence."""
    import quaru_gb300 as q
    from quaru_gb300.workloads import flatten, layered_circuit, workload_seed

    n = args.qubits
    if args.case.startswith("dense-"):
        arith = ARITH_CODES(q)[args.case.split("-", 1)[1]]
        layer = layered_circuit(n, 1, workload_seed("layered_30q"))[0]
        r = q.Register.from_int(n, 0)
        r.set_arith(q.QS_ARITH_DF64)
        r.apply_gates(layer)  # a dense state
        r.set_arith(arith)
        for g in [g for g in layer if is_haar(g)][:4]:
            r.try_apply_fast(g)
    elif args.case in ("blocks-c64", "stages-c64"):
        r = q.Register.from_int(n, 0, precision=q.QS_PREC_C64)
        ops = flatten(layered_circuit(n, 2, workload_seed("layered_30q")))
        if args.case == "blocks-c64":
            r.apply_gates(ops, fuse=2, max_width=5)
        else:
            r.apply_gates(ops, fuse=1, tile_qubits=12)
    elif args.case == "blocks-fx64":
        r = q.Register.from_int(n, 0)
        r.set_arith(q.QS_ARITH_FX64)
        r.apply_gates(flatten(layered_circuit(n, 2, workload_seed("layered_30q"))), fuse=2, max_width=5)
    elif args.case == "measure-all":
        r = q.Register.from_int(n, 0)
        r.set_arith(q.QS_ARITH_FMA)
        r.apply_gates(flatten(layered_circuit(n, 1, workload_seed("layered_30q"))))
        r.measure_sequence(list(range(n)), [0.5] * n)
    else:
        raise SystemExit(f"unknown case {args.case}")
    r.synchronize()
    print(json.dumps({"case": args.case, "qubits": n, "launches": int(q._lib.load().qs_launch_count())}))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--precision", choices=["c128", "c64"], default="c128")
    ap.add_argument("--arith", choices=["exact", "fma", "df64", "fx64"], default="fma",
                    help="arithmetic of the headline sweep (default: plain FP64, fused multiply-add)")
    ap.add_argument("--cpu-qubits", type=int, default=CPU_QUBITS,
                    help="size of the host sample (cpu_baseline and --impl reference)")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of the host sample (whole layers)")
    ap.add_argument("--cpu-limit", type=float, default=20.0,
                    help="per-size time limit of the host sweep over n = 12, 14, ... (--cpu-sweep: default 600)")
    ap.add_argument("--cpu-sweep", action="store_true", help="run only the host sweep and print its JSON")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the per-arithmetic dense 1-qubit timing")
    ap.add_argument("--no-measure", action="store_true", help="skip the measurement section")
    ap.add_argument("--no-fused", action="store_true", help="skip the fused (tiled) circuit timing")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-gradient section")
    ap.add_argument("--no-precision", action="store_true", help="skip the 40-layer precision-form section")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-gradient section")
    ap.add_argument("--no-widths", action="store_true", help="skip the 28-qubit fusion-width section")
    ap.add_argument("--kernels", action="store_true", help="run the per-kernel profiling workload instead")
    ap.add_argument("--case", help="run one small profiling workload instead (see run_case)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps are required")
    if args.cpu_sweep:
        if "--cpu-limit" not in sys.argv:
            args.cpu_limit = 600.0
        run_cpu_sweep(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.kernels:
        run_kernels(args)
    elif args.case:
        run_case(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
