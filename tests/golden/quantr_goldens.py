"""Known-answer cases of the quantr crate's own tests, transcribed as fixtures.

Each case rebuilds the reference test's circuit through the Python mirror of quantr's API and
carries the test's expected amplitudes ("calculated by hand", src/circuit.rs:599-601) and its
tolerance: ERROR_MARGIN = 1e-6 in src/circuit.rs:485, 1e-8 in tests/qft.rs:19 and
tests/grovers.rs:19. These pin the CPU oracle (tests/test_oracle_golden.py) and the GPU engine
(tests/test_gpu_parity.py).
"""
from __future__ import annotations

import math

import numpy as np

from quantr_gb300 import Circuit, Gate, ProductState, Qubit, SuperPosition

R = 1.0 / math.sqrt(2.0)  # FRAC_1_SQRT_2
PI = math.pi


def example_cnot(prod: ProductState):
    """src/circuit.rs:504-512: a controlled-not written as a Custom function."""
    q = prod.get_qubits()
    if q == [Qubit.Zero, Qubit.Zero] or q == [Qubit.Zero, Qubit.One]:
        return None
    if q == [Qubit.One, Qubit.Zero]:
        return SuperPosition.new_with_amplitudes([0, 0, 0, 1])
    return SuperPosition.new_with_amplitudes([0, 0, 1, 0])


def qft(input_state: ProductState):
    """tests/qft.rs:51-67: a QFT Custom function that simulates a nested circuit."""
    n = input_state.num_qubits()
    mini = Circuit(n)
    for pos in range(n):
        mini.add_gate(Gate.H, pos)
        for k in range(2, n - pos + 1):
            mini.add_gate(Gate.CRk(k, pos + k - 1), pos)
    mini.change_register(SuperPosition.from_(input_state))
    return mini.simulate().take_state().take()


def multicnot(num_control: int):
    """tests/grovers.rs:157-172: a multi-controlled not on num_control qubits."""
    def f(input_state: ProductState):
        q = input_state.get_qubits()
        ones = [Qubit.One] * num_control
        last_zero = [Qubit.One] * (num_control - 1) + [Qubit.Zero]
        if q == ones:
            s = ProductState(q)
            s.get_mut_qubits()[num_control - 1] = Qubit.Zero
            return SuperPosition.from_(s)
        if q == last_zero:
            s = ProductState(q)
            s.get_mut_qubits()[num_control - 1] = Qubit.One
            return SuperPosition.from_(s)
        return None
    f.__name__ = f"multicnot{num_control}"
    return f


def cccnot(input_state: ProductState):
    """examples/custom_gate.rs:46-62: the CCC-not as a Custom function, None elsewhere."""
    q = input_state.get_qubits()
    if q == [Qubit.One, Qubit.One, Qubit.One, Qubit.Zero]:
        return SuperPosition.from_(ProductState([Qubit.One] * 4))
    if q == [Qubit.One] * 4:
        return SuperPosition.from_(ProductState([Qubit.One, Qubit.One, Qubit.One, Qubit.Zero]))
    return None


def post_select(state_in: ProductState):
    """examples/post_select.rs:39-49: a non-unitary Custom map (no golden in the reference)."""
    if state_in.get_qubits()[0] == Qubit.Zero:
        return SuperPosition.new_with_amplitudes_unchecked([math.sqrt(2.0), 0.0])
    return SuperPosition.new_with_amplitudes_unchecked([0.0, 0.0])


def _amps(n: int, entries: dict) -> np.ndarray:
    a = np.zeros(1 << n, dtype=np.complex128)
    for i, v in entries.items():
        a[i] = v
    return a


def _c_swap_conj():
    c = Circuit(2)
    c.add_gates([Gate.H, Gate.H]).add_gates([Gate.S, Gate.Sdag])
    return c


def _c_t_conj():
    c = Circuit(2)
    c.add_gates([Gate.H, Gate.H]).add_gates([Gate.T, Gate.Tdag])
    return c


def _c_custom():
    c = Circuit(3)
    c.add_gate(Gate.H, 2).add_gate(Gate.Custom(example_cnot, [2], "cNot"), 1)
    return c


def _c_toffoli():
    c = Circuit(4)
    c.add_gate(Gate.X, 0).add_gate(Gate.H, 3).add_gate(Gate.Y, 3).add_gate(Gate.Toffoli(3, 0), 1)
    return c


def _c_three_pauli():
    c = Circuit(4)
    c.add_gates([Gate.Z, Gate.Y, Gate.H, Gate.X])
    return c


def _c_hash_two():
    c = Circuit(3)
    c.add_gates_with_positions({0: Gate.X, 2: Gate.H})
    return c


def _c_two_h():
    c = Circuit(2)
    c.add_gates([Gate.H, Gate.H])
    return c


def _c_two_rows():
    c = Circuit(4)
    c.add_gates_with_positions({0: Gate.X}).add_gates_with_positions({3: Gate.X, 2: Gate.H})
    return c


def _c_cy_swap():
    c = Circuit(4)
    c.add_repeating_gate(Gate.X, [1, 2]).add_gate(Gate.CY(2), 0).add_gate(Gate.Swap(3), 2) \
        .add_gate(Gate.CY(0), 3)
    return c


def _c_cz_swap():
    c = Circuit(3)
    c.add_repeating_gate(Gate.X, [0, 2]).add_gate(Gate.Swap(1), 2).add_gate(Gate.CZ(1), 0)
    return c


def _c_cnot_simple():
    c = Circuit(2)
    c.add_gate(Gate.H, 0).add_gate(Gate.CNot(1), 0)
    return c


def _c_cnot_flipped():
    c = Circuit(2)
    c.add_gate(Gate.H, 0).add_gate(Gate.CNot(0), 1)
    return c


def _c_cnot_asym():
    c = Circuit(4)
    c.add_gate(Gate.H, 1).add_gate(Gate.CNot(1), 3).add_gate(Gate.Y, 1)
    return c


def _c_hh_then(gate, pos):
    def make():
        c = Circuit(2)
        c.add_gates([Gate.H, Gate.H]).add_gate(gate, pos)
        return c
    return make


def _c_x90():
    c = Circuit(2)
    c.add_gates([Gate.H, Gate.H]).add_gate(Gate.MX90, 0).add_gate(Gate.X90, 1)
    return c


def _c_y90():
    c = Circuit(2)
    c.add_gates([Gate.H, Gate.H]).add_gate(Gate.MY90, 0).add_gate(Gate.Y90, 1)
    return c


def _c_cr():
    c = Circuit(3)
    c.add_gates([Gate.X, Gate.X, Gate.X]).add_gate(Gate.CR(-PI * 0.5, 2), 1)
    return c


def _c_crk():
    c = Circuit(3)
    c.add_gates([Gate.X, Gate.X, Gate.X]).add_gate(Gate.CRk(2, 2), 1)
    return c


def _c_custom_register():
    c = Circuit(3)
    reg = SuperPosition.from_(ProductState([Qubit.One, Qubit.Zero, Qubit.One]))
    c.add_gate(Gate.X, 1).change_register(reg)
    return c


def _c_simple_qft():
    c = Circuit(3)
    c.add_repeating_gate(Gate.X, [1, 2]).add_gate(Gate.Custom(qft, [0, 1], "QFT"), 2)
    return c


def grovers_3qubit_circuit():
    """tests/grovers.rs:21-51."""
    c = Circuit(3)
    c.add_repeating_gate(Gate.H, [0, 1, 2])
    c.add_gate(Gate.CZ(1), 2)
    c.add_repeating_gate(Gate.H, [0, 1, 2]).add_repeating_gate(Gate.X, [0, 1, 2]) \
        .add_gate(Gate.H, 2).add_gate(Gate.Toffoli(0, 1), 2).add_gate(Gate.H, 2) \
        .add_repeating_gate(Gate.X, [0, 1, 2]).add_repeating_gate(Gate.H, [0, 1, 2])
    return c


def x3sudoko_circuit():
    """tests/grovers.rs:74-140 (10 qubits, multi-controlled Custom nots)."""
    qc = Circuit(10)
    qc.add_repeating_gate(Gate.H, [0, 1, 2, 3, 4, 5]).add_gate(Gate.X, 8).add_gate(Gate.X, 9) \
        .add_gate(Gate.H, 9)
    m4 = multicnot(4)
    m6 = multicnot(6)

    def oracle_half():
        for i in range(3):
            qc.add_gate(Gate.Toffoli(i, i + 3), 8)
        qc.add_gate(Gate.Custom(m4, [0, 1, 2], "X"), 6)
        for i in range(3):
            qc.add_gate(Gate.CNot(i), 6)
        qc.add_gate(Gate.Custom(m4, [3, 4, 5], "X"), 7)
        for i in range(3, 6):
            qc.add_gate(Gate.CNot(i), 7)

    oracle_half()
    qc.add_gate(Gate.Custom(m4, [6, 7, 8], "X"), 9)
    oracle_half()
    qc.add_repeating_gate(Gate.H, [0, 1, 2, 3, 4, 5]).add_repeating_gate(Gate.X, [0, 1, 2, 3, 4, 5]) \
        .add_gate(Gate.H, 5).add_gate(Gate.Custom(m6, [0, 1, 2, 3, 4], "X"), 5).add_gate(Gate.H, 5) \
        .add_repeating_gate(Gate.X, [0, 1, 2, 3, 4, 5]).add_repeating_gate(Gate.H, [0, 1, 2, 3, 4, 5])
    return qc


X3SUDOKO_SOLUTIONS = {"001100", "001010", "010100", "010001", "100010", "100001"}  # grovers.rs:143-152

# (name, builder, expected amplitudes, tolerance, citation)
AMPLITUDE_CASES = [
    ("swap_and_conjugate_gates", _c_swap_conj,
     _amps(2, {0: 0.5, 1: -0.5j, 2: 0.5j, 3: 0.5}), 1e-6, "src/circuit.rs:604-613"),
    ("t_and_conjugate_gates", _c_t_conj,
     _amps(2, {0: 0.5, 1: complex(0.5 * R, -0.5 * R), 2: complex(0.5 * R, 0.5 * R), 3: 0.5}),
     1e-6, "src/circuit.rs:616-625"),
    ("custom_gates", _c_custom, _amps(3, {0: R, 3: R}), 1e-6, "src/circuit.rs:629-641"),
    ("toffoli_gates", _c_toffoli, _amps(4, {8: -R * 1j, 13: R * 1j}), 1e-6, "src/circuit.rs:644-658"),
    ("runs_three_pauli_gates_with_hadamard", _c_three_pauli, _amps(4, {5: R * 1j, 7: R * 1j}), 1e-6,
     "src/circuit.rs:689-701"),
    ("hash_map_with_two_gates", _c_hash_two, _amps(3, {4: R, 5: R}), 1e-6, "src/circuit.rs:704-713"),
    ("two_hadamard_gates_work", _c_two_h, _amps(2, {0: 0.5, 1: 0.5, 2: 0.5, 3: 0.5}), 1e-6,
     "src/circuit.rs:723-731"),
    ("add_two_rows_single_gates", _c_two_rows, _amps(4, {9: R, 11: R}), 1e-6, "src/circuit.rs:734-748"),
    ("cy_and_swap_gates_work", _c_cy_swap, _amps(4, {12: 1.0}), 1e-6, "src/circuit.rs:751-768"),
    ("cz_and_swap_gates_work", _c_cz_swap, _amps(3, {6: -1.0}), 1e-6, "src/circuit.rs:771-786"),
    ("cnot_gate_simply_use_works", _c_cnot_simple, _amps(2, {0: R, 2: R}), 1e-6, "src/circuit.rs:789-802"),
    ("cnot_gate_simply_flipped", _c_cnot_flipped, _amps(2, {0: R, 3: R}), 1e-6, "src/circuit.rs:805-818"),
    ("cnot_gate_extended_control_works_asymmetric", _c_cnot_asym, _amps(4, {1: -R * 1j, 4: R * 1j}),
     1e-6, "src/circuit.rs:821-837"),
    ("rx_gate", _c_hh_then(Gate.Rx(PI), 0), _amps(2, {i: -0.5j for i in range(4)}), 1e-6,
     "src/circuit.rs:848-860"),
    ("ry_gate", _c_hh_then(Gate.Ry(PI), 0), _amps(2, {0: -0.5, 1: -0.5, 2: 0.5, 3: 0.5}), 1e-6,
     "src/circuit.rs:863-875"),
    ("rz_gate", _c_hh_then(Gate.Rz(PI), 0), _amps(2, {0: -0.5j, 1: -0.5j, 2: 0.5j, 3: 0.5j}), 1e-6,
     "src/circuit.rs:878-890"),
    ("global_gate", _c_hh_then(Gate.Phase(PI), 0), _amps(2, {i: 0.5j for i in range(4)}), 1e-6,
     "src/circuit.rs:893-905"),
    ("x90_and_mx90_gate", _c_x90, _amps(2, {i: 0.5 for i in range(4)}), 1e-6, "src/circuit.rs:908-921"),
    ("y90_and_my90_gate", _c_y90, _amps(2, {0: -0.5, 1: 0.5, 2: 0.5, 3: -0.5}), 1e-6,
     "src/circuit.rs:924-937"),
    ("cr_gate", _c_cr, _amps(3, {7: -1j}), 1e-6, "src/circuit.rs:940-952"),
    ("crk_gate", _c_crk, _amps(3, {7: 1j}), 1e-6, "src/circuit.rs:955-967"),
    ("custom_register", _c_custom_register, _amps(3, {7: 1.0}), 1e-6, "src/circuit.rs:970-982"),
    ("simple_qft", _c_simple_qft,
     _amps(3, {0: R * 0.5, 1: -R * 0.5, 2: -R * 0.5j, 3: R * 0.5j, 4: complex(-0.25, 0.25),
               5: complex(0.25, -0.25), 6: complex(0.25, 0.25), 7: complex(-0.25, -0.25)}),
     1e-8, "tests/qft.rs:21-47"),
    ("grovers_3qubit", grovers_3qubit_circuit, _amps(3, {3: -R, 7: -R}), 1e-8, "tests/grovers.rs:21-60"),
]

# src/circuit.rs:535-575: the flat layout after push_multi_gates
PUSHED_LAYOUT = [
    Gate.Id, Gate.Id, Gate.H,
    Gate.CNot(2), Gate.Id, Gate.Id,
    Gate.Id, Gate.CNot(0), Gate.Id,
    Gate.Id, Gate.H, Gate.Id,
    Gate.Toffoli(1, 2), Gate.Id, Gate.Id,
    Gate.Id, Gate.Id, Gate.CNot(0),
]
