#!/usr/bin/env python3
"""Benchmark: 30-qubit complex128 brickwork + QFT circuit, gate application on one GB300.

Workload (the metric's configuration): 20 brickwork layers of Rz(a) Ry(b) Rz(c) on every wire plus
alternating CNot(i -> i+1) pairs, then a 30-qubit QFT (H + CRk(k) in quantr's examples/qft.rs
pattern, then wire swaps): 2 570 gates on a 16 GiB complex128 state, seeded synthetic angles.

A step = one `Circuit::simulate` of that circuit from |0...0> on a device-resident register
(set_zero + qgpu_apply_program), timed with CUDA events on the library's stream. The 16 GiB state
is larger than L2 (129 MB), so no flush is needed between steps.

Units (GB/s):
  value       gate-apply bytes per second: each gate counts 2 * 16 B * T_gate, where T_gate is the
              amplitudes it may change (2^n for H/X/Y/rotations/Phase/Custom, 2^(n-1) for
              S/T/Z/CNot/CY/Swap, 2^(n-2) for CZ/CR/CRk/Toffoli) - the bytes a gate-by-gate
              simulator such as quantr moves. Gate fusion moves fewer bytes than this, so value
              can exceed the HBM peak.
  pct_peak    bytes the engine's passes actually move (2 * 16 B * amplitudes each pass may
              change) per second, over the measured HBM peak.
  roofline    the dominant kernel: its per-launch algorithmic bytes / its average CUDA-event
              duration, against the measured HBM peak (MEASURED_PEAKS.json). For the float-pair
              pair-block kernels, which the FP32 pipe bounds, roofline.compute adds their lane
              operations per second against the nominal FP32 lane rate.
  e2e         the same gate-apply GB/s through the public API (Circuit.simulate + measure_all of
              10^6 shots + norm), program upload and histogram download inside the timed region.

--impl reference times the restated reference (the oracle's HashMap engine, a port of
src/circuit/simulation.rs: the Rust crate itself cannot be built without a Rust toolchain) on the
host cores, on a bounded sample of the same family, in the same unit.
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

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "30q c128 gate-apply HBM GB/s (% peak); adjoint grads/s vs plain at 1e-7"
UNIT = "GB/s"
FULL = {"H", "X", "Y", "Rx", "Ry", "Rz", "Phase", "X90", "Y90", "MX90", "MY90", "Custom"}
HALF = {"Z", "S", "Sdag", "T", "Tdag", "CNot", "CY", "Swap"}
QUARTER = {"CZ", "CR", "CRk", "Toffoli"}


def gate_bytes(prog, amp_bytes: int = 16) -> float:
    from quantr_gb300._native import KINDS

    dim = float(1 << prog.n)
    total = 0.0
    for k in prog.ops["kind"]:
        name = KINDS[int(k)]
        frac = 1.0 if name in FULL else 0.5 if name in HALF else 0.25 if name in QUARTER else 0.0
        total += 2.0 * amp_bytes * dim * frac
    return total


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None
        self._summary = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        """Parses (once) and removes the sample file; later calls return the same summary."""
        if self._summary is None:
            self._summary = self._parse()
        return self._summary

    def _parse(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i in range(4) if r[i].lower() == "active"})
        load = [r[0] for r in rows]
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def host_cpu() -> dict:
    """CPU model and core count of the host the CPU baseline runs on."""
    model = None
    try:
        for line in open("/proc/cpuinfo"):
            key = line.split(":")[0].strip().lower()
            if key in ("model name", "cpu model", "hardware"):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if model is None:
        try:  # Arm hosts: lscpu names the core type
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.strip().lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    import platform

    return {"model": model or platform.processor() or "unknown", "arch": platform.machine(),
            "nproc": os.cpu_count()}


class PinnedToOneCore:
    """Pins the calling thread to one core (by default the last allowed one) for a
    single-threaded timing, as `taskset -c <core>` would, and restores the previous affinity
    afterwards."""

    def __init__(self, core: int | None = None):
        self.want = core

    def __enter__(self):
        self.saved = None
        self.core = None
        if hasattr(os, "sched_getaffinity"):
            self.saved = os.sched_getaffinity(0)
            self.core = max(self.saved) if self.want is None else self.want
            os.sched_setaffinity(0, {self.core})
        return self

    def __exit__(self, *exc):
        if self.saved is not None:
            os.sched_setaffinity(0, self.saved)


def cpu_reference_sample(n: int, budget_s: float, seed: int = 2, layers: int = 20) -> dict:
    """The restated reference (oracle HashMap engine, single thread pinned to one core) on the
    first gates of the same brickwork + QFT family at n qubits, run until budget_s elapses (all
    of the circuit when budget_s is None)."""
    from oracle import oracle as orc
    from quantr_gb300 import workloads as W
    from quantr_gb300.program import Program

    prog = W.brickwork_qft(n=n, layers=layers, seed=seed)
    state = np.zeros(1 << n, dtype=np.complex128)
    state[0] = 1.0
    orc.lib()  # build/load outside the timed region
    done_bytes = 0.0
    gates = 0
    chunk = 16
    with PinnedToOneCore() as pin:
        t0 = time.perf_counter()
        while gates < len(prog.ops) and (budget_s is None or time.perf_counter() - t0 < budget_s):
            sub = Program(n, prog.ops[gates:gates + chunk], prog.mats, prog.none)
            state = orc.simulate(sub, state, engine=orc.HASHMAP)
            done_bytes += gate_bytes(sub)
            gates += len(sub.ops)
        dt = time.perf_counter() - t0
    cpu = host_cpu()
    return {"value": done_bytes / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"first {gates} of {len(prog.ops)} gates of the same brickwork+QFT family at "
                      f"{n} qubits (restated reference HashMap engine, 1 thread pinned to core "
                      f"{pin.core}, {dt:.1f} s)",
            "seconds": dt, "gates": gates, "total_gates": int(len(prog.ops)),
            "seconds_per_gate": dt / max(1, gates), "cpu": cpu, "pinned_core": pin.core,
            "state": state if gates == len(prog.ops) else None}


def adjoint_leg(reps: int = 5, shift: bool = True) -> dict:
    """Differentiation config: 20-qubit ansatz, 10 layers of Ry Rz + CNot ring (400 angles),
    H = sum a_i Z_i Z_i+1 + sum b_i X_i. Adjoint gradient vs parameter shift (+-pi/2, 800 plain
    simulations + energies) on the same GPU; host wall clock around the blocking calls."""
    from quantr_gb300 import _native as nat
    from quantr_gb300 import gradients as GR
    from quantr_gb300 import workloads as W

    an = W.ansatz(n=20, layers=10, seed=4)
    prog = an.program()
    h = nat.Handle(20)
    e, g = GR.energy_and_gradient(h, prog, an.a, an.b)  # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        e, g = GR.energy_and_gradient(h, prog, an.a, an.b)
    t_adj = (time.perf_counter() - t0) / reps
    nparam = int(np.isin(prog.ops["kind"], list(GR.ROTATIONS)).sum())
    out = {"workload": "20q ansatz, 10 layers Ry Rz + CNot ring, ZZ+X observable, c128",
           "params": nparam, "energy": e, "adjoint_ms": 1e3 * t_adj,
           "grads_per_s": nparam / t_adj, "timer": "host wall clock around blocking calls"}
    if shift:
        GR.energy(h, prog, an.a, an.b)
        t0 = time.perf_counter()
        ps = GR.parameter_shift(h, prog, an.a, an.b)
        t_ps = time.perf_counter() - t0
        out.update({"param_shift_ms": 1e3 * t_ps, "speedup_vs_param_shift": t_ps / t_adj,
                    "max_abs_diff_vs_param_shift": float(np.max(np.abs(g - ps)))})
    h.close()
    return out


def run_precision(args) -> None:
    """Precision configuration (a secondary line, not the headline): the brickwork family on
    complex64 at 33 qubits and complex128 at 32 qubits (64 GiB each), register-tile passes and
    6-qubit dense blocks of up to 12 gates; and the 26-qubit cross-check of identical circuits
    against the complex128 tile path (max |delta a|, 1 - fidelity, norm drift)."""
    from quantr_gb300 import _native as nat
    from quantr_gb300 import workloads as W

    out = {"impl": "ours", "config": "precision", "cross_check_26q": {}, "full": {}}
    prog26 = W.brickwork_qft(n=26, layers=20, seed=3)

    def run26(precision, blocks):
        h = nat.Handle(26, precision)
        if blocks:
            h.set_fusion(6, 12)
        h.apply(prog26.ops, prog26.mats, prog26.none)
        a = h.download()
        nrm = h.norm()
        h.close()
        return a, nrm

    ref, _ = run26(nat.QGPU_C128, 0)
    for name, prec, blocks in [("c64_blocks", nat.QGPU_C64, 1), ("c64_tiles", nat.QGPU_C64, 0),
                               ("c128_blocks", nat.QGPU_C128, 1)]:
        a, nrm = run26(prec, blocks)
        fid = abs(np.vdot(ref, a)) ** 2 / (np.vdot(a, a).real * np.vdot(ref, ref).real)
        out["cross_check_26q"][name] = {"max_abs_err": float(np.max(np.abs(a - ref))),
                                        "one_minus_fidelity": float(1.0 - fid),
                                        "norm_drift": float(nrm - 1.0)}
    if args.precision_cross_only:  # the 26-qubit cross-check alone (a small case for ncu)
        print(json.dumps(out), flush=True)
        return
    peak = measured_peaks()["hbm_gbs"]
    for n, prec, pname, block_layers in [(33, nat.QGPU_C64, "c64", args.precision_layers),
                                         (32, nat.QGPU_C128, "c128", 1)]:
        res = {}
        for label, blocks, layers in [("tiles", 0, args.precision_layers), ("blocks", 1, block_layers)]:
            prog = W.brickwork_qft(n=n, layers=layers, seed=3, qft=False)
            h = nat.Handle(n, prec)
            if blocks:
                h.set_fusion(6, 12)
            h.set_profiling(True)
            h.profile(reset=True)
            t0 = time.perf_counter()
            h.apply(prog.ops, prog.mats, prog.none)
            h.synchronize()
            wall = time.perf_counter() - t0
            prof = h.profile(reset=True)
            nrm = h.norm()
            h.close()
            res[label] = {"layers": layers, "gates": int(len(prog.ops)), "wall_s": wall,
                          "norm_drift": nrm - 1.0,
                          "kernels": {k: {"launches": v[0], "ms_per_launch": v[1] / v[0],
                                          "GBps": v[2] / (v[1] / 1e3) / 1e9,
                                          "frac": v[2] / (v[1] / 1e3) / 1e9 / peak}
                                      for k, v in prof.items()}}
        out["full"][f"{n}q_{pname}"] = res
    print(json.dumps(out), flush=True)


def run_batch_leg(args) -> None:
    """Batching configuration (a secondary line): independent ansatz circuits of 10..24 qubits,
    4 layers each, own angles and observables; energies + adjoint gradients for every circuit in
    one qgpu_batch_run call per rank. Under torchrun the circuits shard across ranks by cost
    (batch.shard) and the results come back with one all-reduce of flat arrays; the time is the
    slowest rank's, between barriers. Reports circuits/s and, per size, the fusion budget and
    adjoint sweep form the autotuner picked."""
    import torch

    from quantr_gb300 import _native as nat
    from quantr_gb300 import batch as B
    from quantr_gb300 import gradients as GR

    world, rank, local = dist_setup()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cs = B.batch_config(count=args.batch_count)
    sizes = {}
    for c in cs:
        sizes[c.n] = sizes.get(c.n, 0) + 1
    out = {"impl": "ours", "config": "batch", "circuits": len(cs), "n_gpus": world,
           "qubits_histogram": sizes, "results": {}}

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for pname, prec in (("c128", nat.QGPU_C128), ("c64", nat.QGPU_C64)):
        B.run_batch(cs[:8], precision=prec)  # warm-up (module load, graph path)
        tuned = {}

        def runner(part, prec=prec):
            e, g, t = B.run_batch(part, precision=prec)
            tuned.update(t)
            return e, g

        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e, g = B.run_distributed(cs, runner=runner)
        torch.cuda.synchronize()
        dt = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device=dev)
        if world > 1:
            torch.distributed.all_reduce(dt, op=torch.distributed.ReduceOp.MAX)
        dt = float(dt.item())
        out["results"][pname] = {"seconds": dt, "circuits_per_s": len(cs) / dt,
                                 "tuned_per_qubits": tuned,
                                 "small_circuits_in_shared_memory": sum(
                                     1 for c in cs if c.n <= (12 if pname == "c128" else 13))}
        if pname == "c128" and rank == 0:
            rng = np.random.default_rng(0)
            worst = 0.0
            for i in rng.choice(len(cs), size=8, replace=False):
                h = nat.Handle(cs[i].n)
                ei, gi = GR.energy_and_gradient(h, cs[i].program, cs[i].a, cs[i].b)
                h.close()
                worst = max(worst, abs(ei - e[i]), float(np.max(np.abs(gi - g[i]))))
            out["results"][pname]["max_abs_diff_vs_single_circuit_adjoint"] = worst
    if rank == 0:
        print(json.dumps(out), flush=True)


def _sweep_worker(job):
    """One CPU-sweep entry in its own spawned process, pinned to one core: the restated
    reference (HashMap engine, single-threaded) on a whole circuit."""
    kind, n, core = job
    from oracle import oracle as orc
    from quantr_gb300 import workloads as W

    with PinnedToOneCore(core):
        if kind == "random_columns":
            prog = W.random_columns(n=n, columns=40, seed=1)
        else:
            prog = W.brickwork_qft(n=n, layers=20, seed=2)
        orc.lib()
        t0 = time.perf_counter()
        state = orc.simulate(prog, engine=orc.HASHMAP)
        dt = time.perf_counter() - t0
        out = {"workload": kind, "qubits": n, "gates": int(len(prog.ops)), "seconds": dt,
               "seconds_per_gate": dt / len(prog.ops),
               "amplitude_updates_per_s": gate_bytes(prog) / 32.0 / dt,
               "gate_apply_gbs": gate_bytes(prog) / dt / 1e9, "core": core}
        if kind == "random_columns":  # measure_all(1000): 1000 linear scans of the register
            u = np.random.default_rng(1).random(1000)
            t0 = time.perf_counter()
            for x in u:
                orc.measure_linear(state, float(x))
            out["measure_all_1000_seconds"] = time.perf_counter() - t0
    return out


def run_cpu_sweep(args) -> None:
    """CPU baseline sweep: the restated reference, single-threaded and pinned, on the 12-qubit
    random-columns circuit in full (plus measure_all(1000)) and on the whole brickwork + QFT
    circuit at n = 10, 12, ..., args.sweep_max qubits. Each circuit runs in its own process on its
    own core, all at once (the largest n bounds the wall time). With a GPU present, the GPU's
    fast and exact modes on the same circuits are timed beside them."""
    import multiprocessing as mp

    cores = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else \
        list(range(os.cpu_count() or 1))
    jobs = [("random_columns", 12)] + [("brickwork_qft", n)
                                       for n in range(10, args.sweep_max + 1, 2)]
    jobs = [(k, n, cores[(len(cores) - 1 - i) % len(cores)]) for i, (k, n) in enumerate(jobs)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(len(jobs)) as pool:
        pending = pool.map_async(_sweep_worker, jobs)
        gpu = sweep_gpu_points(args, jobs) if args.sweep_gpu else None
        res = pending.get()
    out = {"impl": "reference", "config": "cpu-sweep", "cpu": host_cpu(),
           "threads_per_circuit": 1, "concurrent_circuits": len(jobs),
           "wall_s": time.perf_counter() - t0, "results": res, "gpu": gpu}
    print(json.dumps(out), flush=True)


def sweep_gpu_points(args, jobs) -> list:
    import torch

    from quantr_gb300 import _native as nat
    from quantr_gb300 import workloads as W

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    pts = []
    for kind, n, _ in jobs:
        prog = (W.random_columns(n=n, columns=40, seed=1) if kind == "random_columns"
                else W.brickwork_qft(n=n, layers=20, seed=2))
        pt = {"workload": kind, "qubits": n}
        for name, mode in (("fast", nat.QGPU_MODE_FAST), ("exact", nat.QGPU_MODE_EXACT)):
            h, ms, _ = timed_simulation(nat, n, prog, nat.QGPU_C128, mode, 3, 20, dev)
            h.close()
            pt[f"{name}_ms_per_circuit"] = ms
            pt[f"{name}_gate_apply_gbs"] = gate_bytes(prog) / (ms / 1e3) / 1e9
        pts.append(pt)
    return pts


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _reference_worker(job):
    """One host core's share of a reference-arm step (a spawned process): the restated
    reference on the whole circuit, pinned to `core`."""
    n, budget, core = job
    with PinnedToOneCore(core):
        r = cpu_reference_sample(n, budget_s=budget)
    return {k: r[k] for k in ("value", "seconds", "gates", "total_gates")}


def run_reference(args) -> None:
    """The reference arm: quantr's simulate path (the restated reference, single-threaded as the
    crate is) on every host core at once, one independent simulation of the same family at
    args.ref_n qubits per core, each pinned to its core; value = the bytes all cores' gates move
    (the same gate-equivalent GB/s) over the step's wall time."""
    import multiprocessing as mp

    world, rank, _ = dist_setup()
    if rank != 0:
        return
    n = args.ref_n
    cores = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else \
        list(range(os.cpu_count() or 1))
    ctx = mp.get_context("spawn")
    vals, walls, per_core = [], [], []
    with ctx.Pool(len(cores)) as pool:
        for _ in range(args.warmup):
            pool.map(_reference_worker, [(n, 0.5, c) for c in cores])
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_reference_worker, [(n, args.ref_budget, c) for c in cores])
            wall = time.perf_counter() - t0
            vals.append(sum(r["value"] * r["seconds"] for r in res) / wall)
            walls.append(wall)
            per_core.append(statistics.median(r["value"] for r in res))
    v = statistics.median(vals)
    cpu = host_cpu()
    sample = (f"{len(cores)} independent single-threaded simulations of the brickwork+QFT family "
              f"at {n} qubits ({res[0]['gates']} of {res[0]['total_gates']} gates each), one per "
              f"host core, pinned; restated reference HashMap engine")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(walls), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"brickwork+QFT {args.n}q c128 family, bounded sample at {n} qubits",
                   "qubits": n, "layers": 20, "seed": 2},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": len(cores), "kind": "port",
                         "sample": sample, "cpu": cpu,
                         "single_core_value": statistics.median(per_core)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def timed_simulation(nat, n, prog, precision, mode, warmup, steps, dev):
    """Simulates `prog` from |0...0> on a fresh handle: `warmup` untimed runs, then `steps` runs
    timed with CUDA events on the handle's stream, with per-pass profiling. Returns the handle
    (holding the last result), ms per step and the per-kernel profile."""
    import torch

    h = nat.Handle(n, precision, mode)
    stream = torch.cuda.ExternalStream(h.stream(), device=dev)
    for _ in range(warmup):
        h.set_zero()
        h.apply(prog.ops, prog.mats, prog.none)
    h.set_profiling(True)
    h.profile(reset=True)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        h.set_zero()
        h.apply(prog.ops, prog.mats, prog.none)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    return h, ev0.elapsed_time(ev1) / steps, h.profile(reset=True)


def mode_summary(prof, ms, steps, gbytes, peak) -> dict:
    pass_bytes = sum(v[2] for v in prof.values()) / steps
    dom_name, (dl, dms, db) = max(prof.items(), key=lambda kv: kv[1][1])
    dom_gbs = (db / dl) / (dms / dl / 1e3) / 1e9
    return {"ms_per_step": ms, "value": gbytes / (ms / 1e3) / 1e9,
            "pct_peak": (pass_bytes / (ms / 1e3) / 1e9) / peak,
            "dominant_kernel": {"name": dom_name, "launches_per_step": dl / steps,
                                "share_of_step": dms / steps / ms, "achieved_gbs": dom_gbs,
                                "frac": dom_gbs / peak}}


def reference_precision_leg(args, nat, prog, fast_handle, gbytes, peak, dev) -> dict:
    """The same circuit in QGPU_MODE_F64 (native f64 FMA, the fast mode's plan) and in
    QGPU_MODE_EXACT (one pass per gate, f64 products and sums in the reference's order: equal to
    the oracle value for value), each timed, then compared on the device with the fast-mode
    result: max |a_fast - a_exact|, max |a_f64 - a_exact|, 1 - fidelity and norm drift, without
    downloading the 16 GiB registers."""
    out = {}
    hx, ms_x, prof_x = timed_simulation(nat, args.n, prog, nat.QGPU_C128, nat.QGPU_MODE_EXACT,
                                        0, 1, dev)
    if not prof_x:  # exact mode: one k_group pass per non-identity gate over the whole register
        ng = int((prog.ops["kind"] != 0).sum())
        prof_x = {"k_group": [ng, ms_x, ng * 32.0 * (1 << args.n)]}
    out["exact"] = mode_summary(prof_x, ms_x, 1, gbytes, peak)
    out["exact"].update({"steps": 1, "warmup": 0, "norm_drift": hx.norm() - 1.0})
    hf, ms_f, prof_f = timed_simulation(nat, args.n, prog, nat.QGPU_C128, nat.QGPU_MODE_F64,
                                        1, args.f64_steps, dev)
    out["f64"] = mode_summary(prof_f, ms_f, args.f64_steps, gbytes, peak)
    out["f64"].update({"steps": args.f64_steps, "warmup": 1, "norm_drift": hf.norm() - 1.0})
    nx = hx.norm()
    for name, h in (("fast", fast_handle), ("f64", hf)):
        mx, inner = h.compare(hx)
        nh = h.norm()
        out.setdefault(name, {})
        out[name]["vs_exact"] = {"max_abs_diff": mx,
                                 "one_minus_fidelity": 1.0 - abs(inner) ** 2 / (nh * nx),
                                 "tolerance": 1e-12, "within_tolerance": bool(mx <= 1e-12)}
    hf.close()
    hx.close()
    return out


def same_n_leg(args, nat, W, dev, sample) -> dict:
    """The GPU arm on the CPU baseline's own size (the same family at args.ref_n qubits), so the
    two numbers compare equal configurations; when the CPU sample ran the whole circuit, the
    GPU's amplitudes are also compared with the restated reference's."""
    n = args.ref_n
    prog = W.brickwork_qft(n=n, layers=args.layers, seed=2)
    gbytes = gate_bytes(prog)
    out = {"qubits": n, "gates": int(len(prog.ops)), "cpu_value": sample["value"],
           "cpu_gates_timed": sample["gates"], "unit": UNIT}
    for name, mode in (("fast", nat.QGPU_MODE_FAST), ("exact", nat.QGPU_MODE_EXACT)):
        h, ms, _ = timed_simulation(nat, n, prog, nat.QGPU_C128, mode, 3, 20, dev)
        out[f"gpu_{name}"] = {"value": gbytes / (ms / 1e3) / 1e9, "ms_per_step": ms}
        if sample.get("state") is not None:
            a = h.download()
            out[f"gpu_{name}"]["max_abs_diff_vs_cpu_reference"] = float(
                np.max(np.abs(a - sample["state"])))
            out[f"gpu_{name}"]["equal_to_cpu_reference"] = bool(np.array_equal(a, sample["state"]))
        h.close()
    out["note"] = ("CUDA events around 20 steps of set_zero + apply; the state (256 KiB) is "
                   "L2-resident at this size")
    return out


def run_ours(args) -> None:
    import torch

    from quantr_gb300 import _native as nat
    from quantr_gb300 import workloads as W

    world, rank, local = dist_setup()
    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    precision = nat.QGPU_C64 if args.precision == "c64" else nat.QGPU_C128
    amp_bytes = 8 if precision == nat.QGPU_C64 else 16
    mode = {"fast": nat.QGPU_MODE_FAST, "f64": nat.QGPU_MODE_F64, "exact": nat.QGPU_MODE_EXACT}[args.mode]
    prog = W.brickwork_qft(n=args.n, layers=args.layers, seed=2)
    gbytes = gate_bytes(prog, amp_bytes)

    h = nat.Handle(args.n, precision, mode)
    stream = torch.cuda.ExternalStream(h.stream(), device=dev)
    for _ in range(args.warmup):
        h.set_zero()
        h.apply(prog.ops, prog.mats, prog.none)
    h.set_profiling(True)
    h.profile(reset=True)
    launches0 = h.launch_count()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for _ in range(args.steps):
            h.set_zero()
            h.apply(prog.ops, prog.mats, prog.none)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier()
    launches = h.launch_count() - launches0
    ms = ev0.elapsed_time(ev1) / args.steps
    prof = h.profile(reset=True)
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    value = gbytes * world / (ms_max / 1e3) / 1e9
    pass_bytes = sum(v[2] for v in prof.values()) / args.steps
    norm = h.norm()
    checksum = h.checksum()
    peaks = measured_peaks()
    precision_leg = None
    if (not args.no_parity and world == 1 and precision == nat.QGPU_C128
            and args.mode == "fast"):
        precision_leg = reference_precision_leg(args, nat, prog, h, gbytes, peaks["hbm_gbs"], dev)
        precision_leg["fast"].update(mode_summary(prof, ms_max, args.steps, gbytes,
                                                  peaks["hbm_gbs"]))
    h.close()

    dom = max(prof.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms, dom_bytes) = dom
    achieved = (dom_bytes / dom_launches) / (dom_ms / dom_launches / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        tj = json.loads(tf.read_text())
        kt = tj.get(f"{args.precision}:{dom_name}")
        if kt:
            traffic = kt["dram_bytes_per_amplitude"] * (1 << args.n)
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "peak_source": peaks["source"], "launches_per_step": dom_launches / args.steps,
                "share_of_step": dom_ms / args.steps / ms}
    # The float-pair pair-block kernels are bound by the FP32 pipe rather than HBM: one 4x4
    # complex block costs 91 packed f32x2 instructions (182 lane operations) per amplitude, and a
    # k_pair2 launch applies two blocks. Their compute roofline is against the nominal FP32 lane
    # rate at the sampled SM clock (152 SMs x 128 lanes).
    blocks_per_launch = {"k_pair<ffr>": 1, "k_pair<ff>": 1, "k_pair2<ffr>": 2, "k_pair2<ff>": 2}
    if dom_name in blocks_per_launch:
        csum = clocks.summary()
        mhz = csum.get("sm_mhz") or 2070.0
        lane_ops = 182.0 * (1 << args.n) * blocks_per_launch[dom_name]
        tops = lane_ops / (dom_ms / dom_launches / 1e3) / 1e12
        peak_tops = 152 * 128 * mhz * 1e6 / 1e12
        roofline["compute"] = {
            "pipe": "FP32 (float-pair Dot2 in packed f32x2)", "achieved": tops, "peak": peak_tops,
            "unit": "T lane-op/s", "frac": tops / peak_tops,
            "ops_per_amplitude_per_block": 182, "blocks_per_launch": blocks_per_launch[dom_name],
            "peak_source": f"nominal: 152 SMs x 128 FP32 lanes x {mhz:.0f} MHz (sampled SM clock)"}
    kernels = {k: {"launches_per_step": v[0] / args.steps, "ms_per_step": v[1] / args.steps,
                   "GBps": (v[2] / (v[1] / 1e3) / 1e9) if v[1] > 0 else None}
               for k, v in prof.items()}

    # ---- end to end through the public API -------------------------------------------------
    e2e = None
    if not args.no_e2e:
        qc = W.brickwork_qft_circuit(args.n, layers=args.layers, seed=2)
        qc.set_backend(precision=args.precision, mode=args.mode)
        sim = qc.clone_and_simulate()
        sim.print_warnings(True)
        sim.measure_all(args.shots)
        del sim
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        io = [0, 0]
        for _ in range(args.e2e_steps):
            sim = qc.clone_and_simulate()
            sim.print_warnings(True)
            bins = sim.measure_all(args.shots).take()
            nrm = sim.handle.norm()
            a, b = sim.handle.io_bytes()
            io[0] += a
            io[1] += b
            sim.handle.close()
            del sim
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.e2e_steps
        t = torch.tensor([e2e_ms], dtype=torch.float64, device=dev)
        if world > 1:
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
        e2e = {"value": gbytes * world / (e2e_ms / 1e3) / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": io[0] // args.e2e_steps,
               "d2h_bytes_per_step": io[1] // args.e2e_steps,
               "ms_per_step": e2e_ms, "shots": args.shots, "timer": "host wall clock",
               "distinct_outcomes": len(bins), "norm": nrm}

    if rank != 0:
        return
    cpu = None
    same_n = None
    if world == 1 and not args.no_cpu_baseline:
        sample = cpu_reference_sample(args.ref_n, budget_s=args.ref_budget)
        cpu = {k: sample[k] for k in ("value", "unit", "cores", "kind", "sample", "cpu",
                                      "seconds_per_gate")}
        same_n = same_n_leg(args, nat, W, dev, sample)
    adjoint = None if (args.no_adjoint or world > 1) else adjoint_leg()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("c128 state; f64 arithmetic as float pairs on FP32/INT pipes" if args.mode == "fast"
                  and precision == nat.QGPU_C128 else f"{args.precision}/{args.mode}"),
        "data": "synthetic (seeded SplitMix64 angles)",
        "config": {"workload": f"brickwork+QFT {args.n}q {args.precision}: {args.layers} layers "
                               f"Rz Ry Rz + CNot bricks, {args.n}-qubit QFT + swaps",
                   "qubits": args.n, "gates": int(len(prog.ops)), "mode": args.mode,
                   "parallelism": f"replicas x{world}", "l2": "state 16 GiB > L2, no flush"},
        "value_counts": ("gate-equivalent bytes: 2 x 16 B x the amplitudes each of the circuit's "
                         "gates may change, per second (the bytes a gate-by-gate simulator such as "
                         "quantr moves); fusion moves fewer, so this exceeds HBM. The bytes the "
                         "passes really move are pct_peak x the measured HBM peak."),
        "pct_peak": (pass_bytes / (ms_max / 1e3) / 1e9) / peaks["hbm_gbs"],
        "hbm_gbs_moved": pass_bytes / (ms_max / 1e3) / 1e9,
        "gates_per_s": len(prog.ops) / (ms_max / 1e3),
        "roofline": roofline, "modes": precision_leg, "kernels": kernels,
        "cpu_baseline": cpu, "same_n": same_n, "e2e": e2e, "gpu_launches": launches,
        "adjoint": adjoint,
        "clocks": clocks.summary(),
        "result": {"norm": norm, "checksum": [checksum.real, checksum.imag]},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=30)
    ap.add_argument("--layers", type=int, default=20)
    ap.add_argument("--mode", choices=["fast", "f64", "exact"], default="fast")
    ap.add_argument("--precision", choices=["c128", "c64"], default="c128")
    ap.add_argument("--shots", type=int, default=10 ** 6)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--ref-n", type=int, default=14)
    ap.add_argument("--ref-budget", type=float, default=40.0,
                    help="seconds cap of the CPU sample (the whole 14-qubit circuit fits)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the f64/exact timings and the on-device comparison with them")
    ap.add_argument("--f64-steps", type=int, default=1)
    ap.add_argument("--sweep-max", type=int, default=20,
                    help="cpu-sweep config: largest brickwork+QFT size (even)")
    ap.add_argument("--sweep-gpu", action="store_true",
                    help="cpu-sweep config: also time the GPU on the same circuits")
    ap.add_argument("--config", choices=["headline", "precision", "batch", "adjoint", "cpu-sweep"],
                    default="headline",
                    help="headline: the 30q c128 line; precision: 33q c64 / 32q c128; batch: "
                         "4096 circuits of 10..24 qubits; adjoint: the differentiation leg alone; "
                         "cpu-sweep: the restated reference on whole circuits at n = 10..")
    ap.add_argument("--adjoint-reps", type=int, default=5)
    ap.add_argument("--adjoint-no-shift", action="store_true",
                    help="adjoint config: skip the parameter-shift comparison")
    ap.add_argument("--precision-layers", type=int, default=4)
    ap.add_argument("--precision-cross-only", action="store_true",
                    help="precision configuration: run only the 26-qubit cross-check")
    ap.add_argument("--batch-count", type=int, default=4096)
    args = ap.parse_args()
    if args.config == "precision":
        run_precision(args)
        return
    if args.config == "adjoint":
        print(json.dumps({"impl": "ours", "config": "adjoint",
                          **adjoint_leg(args.adjoint_reps, not args.adjoint_no_shift)}), flush=True)
        return
    if args.config == "batch":
        run_batch_leg(args)
        return
    if args.config == "cpu-sweep":
        run_cpu_sweep(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
