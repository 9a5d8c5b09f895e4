"""Batched energies and adjoint gradients for many independent circuits (qgpu_batch_run).

`batch_config(count, seed)` builds the batching workload: `count` circuits with qubit counts
uniform in 10..24, each the hardware-efficient ansatz (Ry Rz per wire + CNot ring) with 4 layers,
its own angles U[-pi, pi] and its own observable a_i, b_i ~ N(0, 1); circuit i draws from the
SplitMix64 stream seeded 5 * 2^32 + i.

Circuits are independent, so across GPUs they shard with no data-path collective:
`shard(circuits, world)` balances the estimated cost 2^n * gates over ranks and
`run_distributed` runs a rank's share and gathers (energy, gradient) pairs on every rank with one
all-reduce of flat arrays.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _native as nat
from .program import Program
from .rng import SplitMix64
from .workloads import Ansatz


class QgpuBatchItem(C.Structure):
    _fields_ = [("n_qubits", C.c_int32), ("n_ops", C.c_int32), ("op_offset", C.c_int64),
                ("obs_offset", C.c_int64), ("grad_offset", C.c_int64)]


@dataclass
class BatchCircuit:
    program: Program
    a: np.ndarray
    b: np.ndarray

    @property
    def n(self) -> int:
        return self.program.n

    def cost(self) -> float:
        return float(1 << self.n) * len(self.program.ops)


def batch_config(count: int = 4096, seed: int = 5, layers: int = 4, n_min: int = 10,
                 n_max: int = 24) -> list[BatchCircuit]:
    out = []
    for i in range(count):
        r = SplitMix64(seed * (1 << 32) + i)
        n = n_min + r.below(n_max - n_min + 1)
        params = np.array([r.uniform(-math.pi, math.pi) for _ in range(layers * n * 2)])
        a = np.array([r.normal() for _ in range(n)])
        b = np.array([r.normal() for _ in range(n)])
        an = Ansatz(n, layers, params.reshape(layers, n, 2), a, b)
        out.append(BatchCircuit(an.program(), a, b))
    return out


def run_batch(circuits: list[BatchCircuit], precision: int = nat.QGPU_C128):
    """Energies [len], per-circuit gradient arrays (one entry per op) and, per qubit count of
    the register-pass circuits, the autotuner's picks, all on the current GPU."""
    lib = nat.lib()
    items = (QgpuBatchItem * max(1, len(circuits)))()
    ops, obs = [], []
    op_off = obs_off = grad_off = 0
    for i, c in enumerate(circuits):
        items[i].n_qubits = c.n
        items[i].n_ops = len(c.program.ops)
        items[i].op_offset = op_off
        items[i].obs_offset = obs_off
        items[i].grad_offset = grad_off
        ops.append(c.program.ops)
        obs.extend([c.a, c.b])
        op_off += len(c.program.ops)
        obs_off += 2 * c.n
        grad_off += len(c.program.ops)
    all_ops = np.concatenate(ops) if ops else np.zeros(0, dtype=circuits[0].program.ops.dtype)
    all_obs = np.ascontiguousarray(np.concatenate(obs) if obs else np.zeros(0), dtype=np.float64)
    energies = np.zeros(len(circuits))
    grads = np.zeros(max(1, grad_off))
    tuned = (C.c_int * 41)()
    fn = lib.qgpu_batch_run
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int,
                   C.c_void_p, C.c_void_p, C.c_void_p]
    nat.check(fn(C.addressof(items), len(circuits), nat.ptr(all_ops), len(all_ops), nat.ptr(all_obs),
                 all_obs.size, int(precision), nat.ptr(energies), nat.ptr(grads), C.addressof(tuned)),
              "qgpu_batch_run")
    out_g = []
    for i, c in enumerate(circuits):
        out_g.append(grads[items[i].grad_offset: items[i].grad_offset + len(c.program.ops)].copy())
    # per size: the fusion budget (float-pair for complex128, f32 for complex64) and the adjoint
    # sweep form the autotuner picked
    picks = {q: {"fusion_budget": tuned[q] & 0xFFFF,
                 "adjoint_sweep": "grouped" if tuned[q] >> 16 else "per-wire"}
             for q in range(41) if tuned[q]}
    return energies, out_g, picks


def shard(circuits: list, world: int) -> list[list[int]]:
    """Greedy cost balance: largest first, each to the currently lightest rank."""
    loads = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    order = sorted(range(len(circuits)), key=lambda i: -circuits[i].cost())
    for i in order:
        r = min(range(world), key=lambda k: loads[k])
        parts[r].append(i)
        loads[r] += circuits[i].cost()
    return [sorted(p) for p in parts]


def run_distributed(circuits: list[BatchCircuit], runner=None):
    """Run this rank's share and gather every circuit's (energy, gradient) on all ranks.

    The gather is one all-reduce (sum) of two flat float64 arrays, every circuit's energy and
    its gradient slots written by the one rank that owns it and zero elsewhere: plain arrays, no
    pickled objects (on the device for NCCL, on the host for gloo)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size() if dist.is_initialized() else 1
    rank = dist.get_rank() if dist.is_initialized() else 0
    mine = shard(circuits, world)[rank]
    runner = runner or (lambda cs: run_batch(cs)[:2])
    e, g = runner([circuits[i] for i in mine]) if mine else (np.zeros(0), [])
    offs = np.zeros(len(circuits) + 1, dtype=np.int64)
    offs[1:] = np.cumsum([len(c.program.ops) for c in circuits])
    energies = np.zeros(len(circuits))
    flat = np.zeros(int(offs[-1]))
    for k, i in enumerate(mine):
        energies[i] = e[k]
        flat[offs[i]:offs[i + 1]] = g[k]
    if world > 1:
        dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" \
            else torch.device("cpu")
        buf = torch.from_numpy(np.concatenate([energies, flat])).to(dev)
        dist.all_reduce(buf, op=dist.ReduceOp.SUM)
        both = buf.cpu().numpy()
        energies, flat = both[:len(circuits)], both[len(circuits):]
    grads = [flat[offs[i]:offs[i + 1]].copy() for i in range(len(circuits))]
    return energies, grads
