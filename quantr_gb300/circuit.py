"""`Circuit` (src/circuit.rs), `SimulatedCircuit` (src/simulated_circuit.rs) and `Measurement`
(src/circuit/measurement.rs), with simulation on the GB300 engine.

The builder keeps quantr's flat column layout (`circuit_gates`: `num_qubits` entries per column,
padded with `Gate.Id`, multi-wire gates pushed to columns of their own by `push_multi_gates`,
circuit.rs:230-270) and its validation messages. `simulate` lowers the columns into a gate
program and runs it on a device-resident state; the amplitudes stay in HBM until `get_state`.
"""
from __future__ import annotations

import sys
from collections.abc import Mapping

import numpy as np

from . import _native as nat
from . import rng
from .errors import QuantrError
from .gate import Gate
from .program import lower
from .states import ZERO_MARGIN, ProductState, SuperPosition

_DEFAULTS = {"precision": nat.QGPU_C128, "mode": nat.QGPU_MODE_FAST}
_PRECISION = {"c128": nat.QGPU_C128, "c64": nat.QGPU_C64}
_MODE = {"fast": nat.QGPU_MODE_FAST, "exact": nat.QGPU_MODE_EXACT, "f64": nat.QGPU_MODE_F64}


def set_default_backend(precision: str | None = None, mode: str | None = None) -> None:
    """Engine options (not part of quantr's API): precision "c128"/"c64", mode
    "fast"/"exact"/"f64" (see QGPU_MODE_* in include/qgpu.h)."""
    if precision is not None:
        _DEFAULTS["precision"] = _PRECISION[precision]
    if mode is not None:
        _DEFAULTS["mode"] = _MODE[mode]


class Histogram(Mapping):
    """`HashMap<ProductState, usize>` of `measure_all`, backed by the sampler's sorted arrays:
    keys are materialised as `ProductState`s only when accessed."""

    def __init__(self, indices: np.ndarray, counts: np.ndarray, n: int):
        self.indices = np.asarray(indices, dtype=np.uint64)
        self.counts = np.asarray(counts, dtype=np.uint64)
        self.n = n

    def __len__(self) -> int:
        return int(self.indices.size)

    def __iter__(self):
        for i in self.indices:
            yield ProductState.binary_basis(int(i), self.n)

    def __getitem__(self, key: ProductState) -> int:
        # a key of another dimension is absent, as in the crate's HashMap (|101> is not |00101>)
        if not isinstance(key, ProductState) or key.num_qubits() != self.n:
            raise KeyError(key)
        j = np.searchsorted(self.indices, np.uint64(key.comp_basis()))
        if j < self.indices.size and int(self.indices[j]) == key.comp_basis():
            return int(self.counts[j])
        raise KeyError(key)

    def items(self):
        for i, c in zip(self.indices, self.counts):
            yield ProductState.binary_basis(int(i), self.n), int(c)

    def total(self) -> int:
        return int(self.counts.sum())


class Measurement:
    """`Measurement<T>`: Observable(T) | NonObservable(T)."""

    __slots__ = ("value",)

    def __init__(self, value):
        self.value = value

    def take(self):
        return self.value


class Observable(Measurement):
    pass


class NonObservable(Measurement):
    pass


class Circuit:
    def __init__(self, num_qubits: int):
        if num_qubits == 0:
            raise QuantrError("The initialised circuit must have at least one wire.")
        self.circuit_gates: list[Gate] = []
        self.num_qubits = int(num_qubits)
        self.register: SuperPosition | None = None
        self.config_progress = False
        self.precision = None
        self.mode = None

    @staticmethod
    def new(num_qubits: int) -> "Circuit":  # circuit.rs:48-62
        return Circuit(num_qubits)

    def get_num_qubits(self) -> int:
        return self.num_qubits

    def set_print_progress(self, progress: bool) -> None:
        self.config_progress = bool(progress)

    def set_backend(self, precision: str | None = None, mode: str | None = None) -> "Circuit":
        """Engine options for this circuit (not part of quantr's API)."""
        if precision is not None:
            self.precision = _PRECISION[precision]
        if mode is not None:
            self.mode = _MODE[mode]
        return self

    def get_gates(self) -> list[Gate]:
        return self.circuit_gates

    # ---- builders (circuit.rs:124-341) -------------------------------------------------------
    def add_gate(self, gate: Gate, position: int) -> "Circuit":
        return self.add_gates_with_positions({position: gate})

    def add_gates_with_positions(self, gates_with_positions: dict) -> "Circuit":
        for k in gates_with_positions:
            if not 0 <= k < self.num_qubits:  # (a usize in quantr: never negative)
                raise QuantrError(f"The position, {k}, is out of bounds for the circuit with "
                                  f"{self.num_qubits} qubits.")
        gates = [gates_with_positions.get(r, Gate.Id) for r in range(self.num_qubits)]
        self._has_overlapping_controls_and_target(gates, self.num_qubits)
        gates = self._push_multi_gates(gates)
        self.circuit_gates.extend(gates)
        return self

    def add_gates(self, gates) -> "Circuit":
        gates = list(gates)
        if len(gates) != self.num_qubits:
            raise QuantrError(f"The number of gates, {len(gates)}, does not match the number of "
                              f"wires, {self.num_qubits}. All wires must have gates added.")
        self._has_overlapping_controls_and_target(gates, self.num_qubits)
        gates = self._push_multi_gates(gates)
        self.circuit_gates.extend(gates)
        return self

    def add_repeating_gate(self, gate: Gate, positions) -> "Circuit":
        """circuit.rs:324-341. A position outside the register gets the out-of-bounds message of
        add_gates_with_positions (quantr's repeat scan indexes past its table and panics there)."""
        positions = list(positions)
        for p in positions:
            if not 0 <= p < self.num_qubits:
                raise QuantrError(f"The position, {p}, is out of bounds for the circuit with "
                                  f"{self.num_qubits} qubits.")
        if self._contains_repeating_values(self.num_qubits, positions):
            raise QuantrError(f"Attempted to add more than one gate onto a single wire. The "
                              f"positions in {positions} must all differ.")
        gates = [Gate.Id] * self.num_qubits
        for p in positions:
            gates[p] = gate
        return self.add_gates(gates)

    def change_register(self, super_pos: SuperPosition) -> "Circuit":  # circuit.rs:463-473
        if super_pos.product_dim != self.num_qubits:
            raise QuantrError(f"The custom register has a product state dimension of "
                              f"{super_pos.product_dim}, while the number of qubits is "
                              f"{self.num_qubits}. These must equal each other.")
        self.register = super_pos
        return self

    @staticmethod
    def _push_multi_gates(gates: list[Gate]) -> list[Gate]:  # circuit.rs:230-270
        found_multi = found_second = False
        for g in gates:
            if g.name == "Custom" and not g.args[2].isascii():
                raise QuantrError(f"The custom function name, {g.args[2]}, does not only use ASCII "
                                  "chars. This could lead to problems in printing the circuit "
                                  "diagram. This warning will be promoted to an Error in the next "
                                  "major release.")
            if g != Gate.Id:
                if found_multi:
                    found_second = True
                    break
                found_multi = True
        if not found_second:
            return list(gates)
        gates = list(gates)
        extended: list[Gate] = []
        positions = []
        for pos, g in enumerate(gates):
            if not g.is_single_gate():
                col = [Gate.Id] * len(gates)
                col[pos] = g
                extended.extend(col)
                positions.append(pos)
        for p in positions:
            gates[p] = Gate.Id
        return gates + extended

    @staticmethod
    def _has_overlapping_controls_and_target(gates, size: int) -> None:  # circuit.rs:272-293
        for pos, g in enumerate(gates):
            nodes = g.get_nodes()
            if nodes is None:
                continue
            for node in nodes:
                if not 0 <= node < size:  # (a usize in quantr: never negative)
                    raise QuantrError(f"The control node at position {node}, is greater than the "
                                      f"umnber of qubits {size}.")
            if Circuit._contains_repeating_values(size, nodes):
                raise QuantrError(f"The gate, {g!r}, has overlapping control nodes.")
            if pos in nodes:
                raise QuantrError(f"The gate, {g!r}, has a control node that equals the gate's "
                                  f"position {pos}.")

    @staticmethod
    def _contains_repeating_values(num_qubits: int, array) -> bool:
        seen = [False] * num_qubits
        for j in array:
            if not 0 <= j < num_qubits:
                raise IndexError(j)
            if seen[j]:
                return True
            seen[j] = True
        return False

    # ---- simulation -------------------------------------------------------------------------
    def _run(self, register: SuperPosition | None) -> "SimulatedCircuit":
        precision = self.precision if self.precision is not None else _DEFAULTS["precision"]
        mode = self.mode if self.mode is not None else _DEFAULTS["mode"]
        handle = nat.Handle(self.num_qubits, precision, mode)
        if register is not None:
            handle.upload(register.amplitudes)
        if self.config_progress:
            _print_log(self.circuit_gates, self.num_qubits)
        prog = lower(self.circuit_gates, self.num_qubits)
        handle.apply(prog.ops, prog.mats, prog.none)
        return SimulatedCircuit(list(self.circuit_gates), self.num_qubits, handle,
                                self.config_progress, precision, mode)

    def simulate(self) -> "SimulatedCircuit":  # circuit.rs:364-388
        reg, self.register = self.register, None
        return self._run(reg)

    def clone_and_simulate(self) -> "SimulatedCircuit":  # circuit.rs:411-435
        return self._run(self.register)


def _print_log(gates, n: int) -> None:  # simulation.rs:32-34, 183-200
    print("Starting circuit simulation...")
    total = len(gates)
    for counter, g in enumerate(gates):
        if g.name == "Id":
            continue
        print(f"Applying {g!r} on wire {counter % n} # {counter + 1}/{total} ")
        if counter + 1 == total:
            print("Finished circuit simulation.")


_WARN_CUSTOM = ("\x1b[93m[Quantr Warning] Custom gates were detected in the circuit. Measurements "
                "will be taken from a cached register in memory, and so if the Custom gate does NOT "
                "implement a unitary mapping, the measure_all method will most likely lead to wrong "
                "results. To simulate a circuit without cache, see "
                "SimulatedCircuit::measure_all_without_cache.\x1b[0m")
_WARN_NONE = ("\x1b[93m[Quantr Warning] The superposition failed to collapse to a state during "
              "repeat measurements. This is likely due to the use of Gate::Custom where the mapping "
              "is not unitary.\x1b[0m")


class SimulatedCircuit:
    """Result of `simulate`: the register stays on the device until `get_state`."""

    def __init__(self, gates, n, handle: nat.Handle, progress, precision, mode):
        self.circuit_gates = gates
        self.num_qubits = n
        self._handle = handle
        self._state: SuperPosition | None = None
        self.config_progress = progress
        self.disable_warnings = False
        self._precision = precision
        self._mode = mode

    @property
    def handle(self) -> nat.Handle:
        return self._handle

    def _register(self) -> SuperPosition:
        if self._state is None:
            self._state = SuperPosition(self._handle.download(), self.num_qubits)
        return self._state

    def measure_all(self, shots: int) -> Observable:  # simulated_circuit.rs:63-73
        if any(g.is_custom_gate() for g in self.circuit_gates) and not self.disable_warnings:
            print(_WARN_CUSTOM, file=sys.stderr)
        idx, cnt, failed = self._handle.measure(int(shots), rng.next_u64())
        if failed and not self.disable_warnings:
            for _ in range(failed):
                print(_WARN_NONE, file=sys.stderr)
        return Observable(Histogram(idx, cnt, self.num_qubits))

    def measure_all_without_cache(self, shots: int) -> Observable:  # simulated_circuit.rs:81-114
        """Shot 1 uses the cached register; every later shot re-simulates from |0...0>.

        Each later shot re-tabulates every `Custom` gate (its function is called again, so a
        function that draws random Kraus branches gets a fresh draw per shot, as in quantr). A
        run of consecutive shots whose tables come out identical yields the same register, so
        it is simulated once and sampled with one `measure` call for the whole run; a circuit
        without `Custom` gates is simulated once for shots 2..N."""
        if shots < 1:
            raise QuantrError("measure_all_without_cache needs at least one shot.")
        bins: dict = {}

        def add(count):
            idx, cnt, failed = self._handle.measure(int(count), rng.next_u64())
            if failed and not self.disable_warnings:
                for _ in range(failed):
                    print(_WARN_NONE, file=sys.stderr)
            for i, c in zip(idx, cnt):
                key = ProductState.binary_basis(int(i), self.num_qubits)
                bins[key] = bins.get(key, 0) + int(c)

        add(1)
        if self.config_progress:
            print(f"Measured state # 1/{shots}")
        stochastic = any(g.is_custom_gate() for g in self.circuit_gates)
        last_key, pending = None, 0
        prog = None
        for s in range(shots - 1):
            if prog is None or stochastic:
                prog = lower(self.circuit_gates, self.num_qubits)
            key = (prog.mats.tobytes(), prog.none.tobytes())
            if key != last_key:
                if pending:
                    add(pending)
                self._handle.set_zero()
                self._handle.apply(prog.ops, prog.mats, prog.none)
                self._state = None
                last_key, pending = key, 0
            pending += 1
            if self.config_progress:
                print("Register reset to zero state")
                print(f"Measured state # {s + 2}/{shots}")
        if pending:
            add(pending)
        return Observable(bins)

    def get_state(self) -> NonObservable:  # simulated_circuit.rs:158-160
        return NonObservable(self._register())

    def take_state(self) -> NonObservable:
        return NonObservable(self._register())

    def state_hash_map(self, margin: float = ZERO_MARGIN) -> dict:
        """`get_state().take().to_hash_map()` (super_positions.rs:315-323) computed on the device:
        only the surviving amplitudes cross PCIe/C2C, so a sparse 30-qubit register needs no
        16 GiB download."""
        idx, amp = self._handle.extract_nonzero(margin)
        return {ProductState.binary_basis(int(i), self.num_qubits): complex(a)
                for i, a in zip(idx, amp)}

    def print_warnings(self, printing: bool) -> None:
        # simulated_circuit.rs:163-165: the flag is stored as `disable_warnings`
        self.disable_warnings = bool(printing)

    def get_circuit_gates(self):
        return self.circuit_gates

    def get_num_qubits(self) -> int:
        return self.num_qubits

    def set_print_progress(self, printing: bool) -> None:
        self.config_progress = bool(printing)
