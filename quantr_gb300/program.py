"""Lowering of quantr's flat gate list into `qgpu_op` records (include/qgpu.h).

`simulate_with_register` (src/circuit/simulation.rs:21-57) walks the flat column list, skipping
`Gate::Id` and placing each gate on wire `counter % num_qubits` (simulation.rs:43). `lower`
does the same walk and emits one record per non-identity gate. A `Gate::Custom` is tabulated
on the host: its function is called on each of the 2^k local basis states [controls..., target]
(simulation.rs:137-156) and the images become column j of a dense 2^k x 2^k block, with a
None flag per column.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from ._native import KIND, QGPU_MAX_OP_WIRES
from .errors import QuantrError
from .states import ProductState, SuperPosition

OP_DTYPE = np.dtype([("kind", "<i4"), ("target", "<i4"), ("n_controls", "<i4"), ("k", "<i4"),
                     ("controls", "<i4", (QGPU_MAX_OP_WIRES,)), ("param", "<f8"),
                     ("mat_offset", "<i8"), ("none_offset", "<i8")], align=True)
assert OP_DTYPE.itemsize == 80


@dataclass
class Program:
    n: int
    ops: np.ndarray                     # OP_DTYPE records
    mats: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    none: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint8))

    def __len__(self) -> int:
        return len(self.ops)


class ProgramBuilder:
    """Accumulates op records; used by `lower` and by the synthetic workload generators."""

    def __init__(self, n: int):
        self.n = n
        self._ops: list[tuple] = []
        self._mats: list[np.ndarray] = []
        self._none: list[np.ndarray] = []
        self._mat_len = 0
        self._none_len = 0

    def add(self, name: str, target: int, controls=(), param: float = 0.0, k: int = 0) -> None:
        c = list(controls) + [0] * (QGPU_MAX_OP_WIRES - len(controls))
        self._ops.append((KIND[name], int(target), len(controls), int(k), c, float(param), 0, 0))

    def add_custom(self, target: int, controls, block: np.ndarray, none: np.ndarray) -> None:
        d = 1 << (len(controls) + 1)
        blk = np.ascontiguousarray(block, dtype=np.complex128).reshape(d, d)  # [j, l] = column j
        c = list(controls) + [0] * (QGPU_MAX_OP_WIRES - len(controls))
        self._ops.append((KIND["Custom"], int(target), len(controls), 0, c, 0.0, self._mat_len,
                          self._none_len))
        flat = blk.reshape(-1).view(np.float64)
        self._mats.append(flat)
        self._none.append(np.asarray(none, dtype=np.uint8).reshape(d))
        self._mat_len += flat.size
        self._none_len += d

    def build(self) -> Program:
        ops = np.zeros(len(self._ops), dtype=OP_DTYPE)
        for i, rec in enumerate(self._ops):
            ops[i] = rec
        mats = np.concatenate(self._mats) if self._mats else np.zeros(0, np.float64)
        none = np.concatenate(self._none) if self._none else np.zeros(0, np.uint8)
        return Program(self.n, ops, mats, none)


def tabulate_custom(func, k: int):
    """Evaluate a Custom function on the 2^k local basis states (first qubit most significant)."""
    d = 1 << k
    block = np.zeros((d, d), dtype=np.complex128)
    none = np.zeros(d, dtype=np.uint8)
    for j in range(d):
        img = func(ProductState.binary_basis(j, k))
        if img is None:
            none[j] = 1
            continue
        if not isinstance(img, SuperPosition):
            raise QuantrError("A Custom gate function must return a SuperPosition or None.")
        amps = np.asarray(img.get_amplitudes(), dtype=np.complex128)
        if amps.size != d:
            raise QuantrError(f"The Custom gate acts on {k} qubits, so its image must have {d} "
                              f"amplitudes; it returned {amps.size}.")
        block[j] = amps
    return block, none


def lower(gates, n: int) -> Program:
    b = ProgramBuilder(n)
    counter = 0
    for gate in gates:
        if gate.name == "Id":
            counter += 1
            continue
        pos = counter % n
        a = gate.args
        if gate.name in ("Rx", "Ry", "Rz", "Phase"):
            b.add(gate.name, pos, (), param=a[0])
        elif gate.name in ("CNot", "Swap", "CZ", "CY"):
            b.add(gate.name, pos, (a[0],))
        elif gate.name == "CR":
            b.add("CR", pos, (a[1],), param=a[0])
        elif gate.name == "CRk":
            b.add("CRk", pos, (a[1],), k=a[0])
        elif gate.name == "Toffoli":
            b.add("Toffoli", pos, (a[0], a[1]))
        elif gate.name == "Custom":
            func, controls, _name = a
            if len(controls) + 1 > QGPU_MAX_OP_WIRES:
                raise QuantrError(f"Custom gates act on at most {QGPU_MAX_OP_WIRES} wires.")
            block, none = tabulate_custom(func, len(controls) + 1)
            b.add_custom(pos, controls, block, none)
        else:
            b.add(gate.name, pos, ())
        counter += 1
    return b.build()
