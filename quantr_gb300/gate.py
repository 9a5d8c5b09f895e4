"""`Gate` (src/circuit/gate.rs:19-106): the 25 variants, with the reference's equality.

Unit variants are instances (`Gate.H`, `Gate.CNot` is a constructor: `Gate.CNot(control)`).
`Gate.Custom(func, controls, name)` takes a Python function ProductState -> SuperPosition | None.
"""
from __future__ import annotations

from typing import Callable, Optional

from .errors import rust_debug_f64, rust_debug_str


class Gate:
    __slots__ = ("name", "args")

    # filled in below for the unit variants
    Id: "Gate"
    H: "Gate"
    X: "Gate"
    Y: "Gate"
    Z: "Gate"
    S: "Gate"
    Sdag: "Gate"
    T: "Gate"
    Tdag: "Gate"
    X90: "Gate"
    Y90: "Gate"
    MX90: "Gate"
    MY90: "Gate"

    def __init__(self, name: str, *args):
        self.name = name
        self.args = tuple(args)

    # ---- parametrised variants ---------------------------------------------------------------
    @staticmethod
    def Rx(angle: float) -> "Gate":
        return Gate("Rx", float(angle))

    @staticmethod
    def Ry(angle: float) -> "Gate":
        return Gate("Ry", float(angle))

    @staticmethod
    def Rz(angle: float) -> "Gate":
        return Gate("Rz", float(angle))

    @staticmethod
    def Phase(angle: float) -> "Gate":
        return Gate("Phase", float(angle))

    @staticmethod
    def CR(angle: float, control: int) -> "Gate":
        return Gate("CR", float(angle), int(control))

    @staticmethod
    def CRk(k: int, control: int) -> "Gate":
        return Gate("CRk", int(k), int(control))

    @staticmethod
    def CZ(control: int) -> "Gate":
        return Gate("CZ", int(control))

    @staticmethod
    def CY(control: int) -> "Gate":
        return Gate("CY", int(control))

    @staticmethod
    def CNot(control: int) -> "Gate":
        return Gate("CNot", int(control))

    @staticmethod
    def Swap(control: int) -> "Gate":
        return Gate("Swap", int(control))

    @staticmethod
    def Toffoli(c1: int, c2: int) -> "Gate":
        return Gate("Toffoli", int(c1), int(c2))

    @staticmethod
    def Custom(func: Callable, controls, name: str) -> "Gate":
        return Gate("Custom", func, tuple(int(c) for c in controls), str(name))

    # ---- gate.rs helpers ---------------------------------------------------------------------
    def get_nodes(self) -> Optional[list[int]]:  # gate.rs:110-138
        if self.name in ("CNot", "Swap", "CZ", "CY"):
            return [self.args[0]]
        if self.name in ("CR", "CRk"):
            return [self.args[1]]
        if self.name == "Toffoli":
            return [self.args[0], self.args[1]]
        if self.name == "Custom":
            return list(self.args[1])
        return None

    def is_single_gate(self) -> bool:  # gate.rs:173-201
        return self.get_nodes() is None

    def is_custom_gate(self) -> bool:
        return self.name == "Custom"

    def __eq__(self, other) -> bool:
        return isinstance(other, Gate) and self.name == other.name and self.args == other.args

    def __hash__(self) -> int:
        return hash((self.name, self.args))

    def __repr__(self) -> str:
        """`{:?}` of the Rust enum (the `#[derive(Debug)]` of gate.rs:18), as quantr's validation
        messages print it: "H", "Rx(0.5)", "CRk(3, 1)"; a Custom gate's function prints as an
        address, like a Rust function pointer."""
        if not self.args:
            return self.name
        if self.name == "Custom":
            nodes = ", ".join(str(int(c)) for c in self.args[1])
            return f"Custom({id(self.args[0]):#x}, [{nodes}], {rust_debug_str(self.args[2])})"
        parts = [rust_debug_f64(a) if isinstance(a, float) else str(a) for a in self.args]
        return f"{self.name}({', '.join(parts)})"


for _n in ("Id", "H", "X", "Y", "Z", "S", "Sdag", "T", "Tdag", "X90", "Y90", "MX90", "MY90"):
    setattr(Gate, _n, Gate(_n))
