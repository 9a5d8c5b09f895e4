"""Seeded synthetic circuit families (the benchmark workloads and parity cases).

All randomness comes from SplitMix64 (`rng.SplitMix64`) with doubles (x >> 11) * 2^-53, so the
same seed gives the same circuit everywhere (tests, benchmark, CPU baseline).

  random_columns(n=12, seed=1): 40 columns; each column gives every wire one gate drawn from
      {H, X, Y, Z, S, T, Rx, Ry, Rz, Phase} (angles U[0, 2pi)), then one CNot on a random distinct
      (control, target) pair, and every 5th column a Toffoli on random distinct wires.
  brickwork_qft(n=30, seed=2): 20 layers of Rz(a) Ry(b) Rz(c) on every wire (angles U[0, 2pi))
      followed by CNot(i -> i+1) on even i (even layers) or odd i (odd layers); then an n-qubit QFT
      in the gate pattern of quantr's examples/qft.rs:50-58 (H(i), then CRk(k) with control
      i+k-1 on target i for k = 2..n-i), then Swap(i, n-1-i) for i < n/2.
  ansatz(n=20, layers=10, seed=4): Ry(t) Rz(p) on every wire per layer + CNot ring i -> i+1 mod n;
      parameters U[-pi, pi]; observable coefficients a_i, b_i ~ N(0, 1) (Box-Muller).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .circuit import Circuit
from .gate import Gate
from .program import Program, ProgramBuilder, lower
from .rng import SplitMix64

TWO_PI = 2.0 * math.pi
_ONE_Q = ["H", "X", "Y", "Z", "S", "T", "Rx", "Ry", "Rz", "Phase"]


def _one_q_gate(name: str, r: SplitMix64) -> Gate:
    if name in ("Rx", "Ry", "Rz", "Phase"):
        return getattr(Gate, name)(r.uniform(0.0, TWO_PI))
    return getattr(Gate, name)


def _distinct(r: SplitMix64, n: int, count: int) -> list[int]:
    out: list[int] = []
    while len(out) < count:
        w = r.below(n)
        if w not in out:
            out.append(w)
    return out


def random_columns_circuit(n: int = 12, columns: int = 40, seed: int = 1) -> Circuit:
    r = SplitMix64(seed)
    qc = Circuit(n)
    for col in range(columns):
        qc.add_gates([_one_q_gate(_ONE_Q[r.below(len(_ONE_Q))], r) for _ in range(n)])
        c, t = _distinct(r, n, 2)
        qc.add_gate(Gate.CNot(c), t)
        if col % 5 == 4 and n >= 3:
            c1, c2, t = _distinct(r, n, 3)
            qc.add_gate(Gate.Toffoli(c1, c2), t)
    return qc


def random_columns(n: int = 12, columns: int = 40, seed: int = 1) -> Program:
    return lower(random_columns_circuit(n, columns, seed).get_gates(), n)


def brickwork_qft(n: int = 30, layers: int = 20, seed: int = 2, qft: bool = True) -> Program:
    r = SplitMix64(seed)
    b = ProgramBuilder(n)
    for layer in range(layers):
        angles = [(r.uniform(0.0, TWO_PI), r.uniform(0.0, TWO_PI), r.uniform(0.0, TWO_PI))
                  for _ in range(n)]
        for w in range(n):
            b.add("Rz", w, (), param=angles[w][0])
        for w in range(n):
            b.add("Ry", w, (), param=angles[w][1])
        for w in range(n):
            b.add("Rz", w, (), param=angles[w][2])
        for i in range(layer % 2, n - 1, 2):
            b.add("CNot", i + 1, (i,))
    if qft:
        for i in range(n):
            b.add("H", i, ())
            for k in range(2, n - i + 1):
                b.add("CRk", i, (i + k - 1,), k=k)
        for i in range(n // 2):
            b.add("Swap", i, (n - 1 - i,))
    return b.build()


def brickwork_qft_circuit(n: int, layers: int = 20, seed: int = 2) -> Circuit:
    """The same family built through the Circuit API (columns of Rz, Ry, Rz, then one CNot or
    gate per column): lowers to exactly the `brickwork_qft` program."""
    r = SplitMix64(seed)
    qc = Circuit(n)
    for layer in range(layers):
        angles = [(r.uniform(0.0, TWO_PI), r.uniform(0.0, TWO_PI), r.uniform(0.0, TWO_PI))
                  for _ in range(n)]
        qc.add_gates([Gate.Rz(angles[w][0]) for w in range(n)])
        qc.add_gates([Gate.Ry(angles[w][1]) for w in range(n)])
        qc.add_gates([Gate.Rz(angles[w][2]) for w in range(n)])
        for i in range(layer % 2, n - 1, 2):
            qc.add_gate(Gate.CNot(i), i + 1)
    for i in range(n):
        qc.add_gate(Gate.H, i)
        for k in range(2, n - i + 1):
            qc.add_gate(Gate.CRk(k, i + k - 1), i)
    for i in range(n // 2):
        qc.add_gate(Gate.Swap(n - 1 - i), i)
    return qc


@dataclass
class Ansatz:
    n: int
    layers: int
    params: np.ndarray   # [layers, n, 2]: (theta for Ry, phi for Rz)
    a: np.ndarray        # ZZ coefficients, a[i] couples wires i, (i+1) mod n
    b: np.ndarray        # X coefficients

    def program(self, params: np.ndarray | None = None) -> Program:
        p = self.params if params is None else params.reshape(self.layers, self.n, 2)
        b = ProgramBuilder(self.n)
        for l in range(self.layers):
            for w in range(self.n):
                b.add("Ry", w, (), param=p[l, w, 0])
            for w in range(self.n):
                b.add("Rz", w, (), param=p[l, w, 1])
            for i in range(self.n):
                b.add("CNot", (i + 1) % self.n, (i,))
        return b.build()


def ansatz(n: int = 20, layers: int = 10, seed: int = 4) -> Ansatz:
    r = SplitMix64(seed)
    params = np.array([r.uniform(-math.pi, math.pi) for _ in range(layers * n * 2)])
    a = np.array([r.normal() for _ in range(n)])
    bb = np.array([r.normal() for _ in range(n)])
    return Ansatz(n, layers, params.reshape(layers, n, 2), a, bb)


def energy_dense(state: np.ndarray, a: np.ndarray, b: np.ndarray) -> float:
    """<psi|H|psi> for H = sum_i a_i Z_i Z_{i+1} + sum_i b_i X_i (periodic), by numpy (small n)."""
    n = state.size.bit_length() - 1
    idx = np.arange(state.size)
    p = np.abs(state) ** 2
    e = 0.0
    for i in range(n):
        j = (i + 1) % n
        zi = 1 - 2 * ((idx >> (n - 1 - i)) & 1)
        zj = 1 - 2 * ((idx >> (n - 1 - j)) & 1)
        e += a[i] * float(np.sum(p * zi * zj))
        flipped = state[idx ^ (1 << (n - 1 - i))]
        e += b[i] * float(np.real(np.vdot(state, flipped)))
    return e
