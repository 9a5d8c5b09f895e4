"""The CPU oracle against the quantr crate's own known answers (no GPU).

The crate cannot be compiled here (no Rust toolchain), so its tests' goldens pin the restatement:
every amplitude case of src/circuit.rs, tests/qft.rs and tests/grovers.rs, through both oracle
engines (the literal HashMap algorithm and the dense one with the same accumulation order).
"""
import math

import numpy as np
import pytest

from golden import quantr_goldens as G
from quantr_gb300 import Circuit, Gate, ProductState, Qubit, SuperPosition
from quantr_gb300.program import ProgramBuilder, lower
from quantr_gb300 import workloads as W


def _oracle_qft(orc):
    """tests/qft.rs:51-67 with the nested circuit run on the oracle instead of the device."""
    def qft(input_state: ProductState):
        n = input_state.num_qubits()
        mini = Circuit(n)
        for pos in range(n):
            mini.add_gate(Gate.H, pos)
            for k in range(2, n - pos + 1):
                mini.add_gate(Gate.CRk(k, pos + k - 1), pos)
        reg = SuperPosition.from_(input_state).amplitudes
        out = orc.simulate(lower(mini.get_gates(), n), reg, engine=orc.HASHMAP)
        return SuperPosition(out, n)
    return qft


def _program_for_cpu(name, builder, orc):
    qc = builder()
    gates = list(qc.get_gates())
    if name == "simple_qft":
        gates = [Gate.Custom(_oracle_qft(orc), g.args[1], g.args[2]) if g.is_custom_gate() else g
                 for g in gates]
    reg = qc.register.amplitudes if qc.register is not None else None
    return lower(gates, qc.num_qubits), reg


@pytest.mark.parametrize("engine", [0, 1], ids=["hashmap", "dense"])
@pytest.mark.parametrize("case", G.AMPLITUDE_CASES, ids=[c[0] for c in G.AMPLITUDE_CASES])
def test_oracle_matches_reference_goldens(oracle, case, engine):
    name, builder, expected, tol, _cite = case
    prog, reg = _program_for_cpu(name, builder, oracle)
    out = oracle.simulate(prog, reg, engine=engine)
    assert np.max(np.abs(out.real - expected.real)) < tol
    assert np.max(np.abs(out.imag - expected.imag)) < tol


def test_engines_agree_value_for_value(oracle):
    """HashMap and dense engines: identical values on random columns with customs and None."""
    for seed in range(3):
        prog = W.random_columns(n=7, columns=12, seed=100 + seed)
        a = oracle.simulate(prog, engine=oracle.HASHMAP)
        b = oracle.simulate(prog, engine=oracle.DENSE)
        assert np.array_equal(a, b)
    qc = G.x3sudoko_circuit()
    prog = lower(qc.get_gates(), 10)
    a = oracle.simulate(prog, engine=oracle.HASHMAP)
    b = oracle.simulate(prog, engine=oracle.DENSE)
    assert np.array_equal(a, b)


def _custom_heavy(n, seed):
    """Rotations, CNot layers, a CRk row and Custom blocks with None entries (controls above and
    below the target, a non-unitary one-wire block, a six-wire permutation)."""
    rng = np.random.default_rng(seed)
    b = ProgramBuilder(n)
    for layer in range(3):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
        t, c1, c2 = (int(x) for x in rng.choice(n, size=3, replace=False))
        blk = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
        b.add_custom(t, [c1, c2], blk / 3, (rng.random(8) < 0.25).astype(np.uint8))
        b.add("H", 0)
        for k in range(2, n + 1):
            b.add("CRk", 0, (k - 1,), k=k)
        b.add_custom(int(rng.integers(0, n)), [], np.array([[1.2, 0.1j], [0, 0.8]], np.complex128),
                     np.array([0, layer % 2], np.uint8))
        b.add("Toffoli", int(rng.integers(2, n)), (0, 1))
    wires = [int(x) for x in rng.choice(n, size=6, replace=False)]
    perm = np.eye(64, dtype=np.complex128)[rng.permutation(64)] * np.exp(1j * rng.random(64))[:, None]
    b.add_custom(wires[2], wires[:2] + wires[3:], perm, (rng.random(64) < 0.2).astype(np.uint8))
    return b.build()


@pytest.mark.parametrize("threads", [3, 8])
def test_threaded_dense_engine_equals_dense_engine(oracle, monkeypatch, threads):
    """The threaded dense engine (used for the 20-22 qubit GPU parity cases) gives the dense
    engine's values exactly: custom-heavy circuits with None entries at 14 qubits (enough groups
    per gate for every thread), the brickwork + QFT family, and the 10-qubit sudoku."""
    monkeypatch.setenv("ORACLE_THREADS", str(threads))
    for prog in (_custom_heavy(14, 1), _custom_heavy(13, 2),
                 W.brickwork_qft(n=14, layers=3, seed=2), lower(G.x3sudoko_circuit().get_gates(), 10)):
        a = oracle.simulate(prog, engine=oracle.DENSE)
        b = oracle.simulate(prog, engine=oracle.DENSE_PAR)
        assert np.array_equal(a, b)


def test_non_unitary_post_select(oracle):
    """examples/post_select.rs: Custom with a scaled |0> image and a zero image."""
    qc = Circuit(3)
    qc.add_repeating_gate(Gate.H, [0, 1, 2]).add_gate(Gate.Custom(G.post_select, [], "P"), 1)
    out = oracle.simulate(lower(qc.get_gates(), 3), engine=oracle.HASHMAP)
    # H^3 |000> = all 1/sqrt(8); wire 1 = 0 -> * sqrt(2), wire 1 = 1 -> 0
    expect = np.array([0.5 if ((i >> 1) & 1) == 0 else 0.0 for i in range(8)])
    assert np.allclose(out, expect, atol=1e-15)


@pytest.mark.parametrize("engine", [0, 1], ids=["hashmap", "dense"])
def test_examples_custom_multi_controlled_nots(oracle, engine):
    """examples/custom_gate.rs (X on wires 0-2, then a Custom CCC-not on 3 with controls 0-2:
    |1111>) and examples/generalised_control_not_gate.rs (X on all 6 wires, then a Custom
    5-controlled not on wire 5: |111110>). Both Custom functions return None off their two
    inputs, so every other amplitude keeps its value under the None rule."""
    qc = Circuit(4)
    qc.add_repeating_gate(Gate.X, [0, 1, 2]).add_gate(Gate.Custom(G.cccnot, [0, 1, 2], "X"), 3)
    out = oracle.simulate(lower(qc.get_gates(), 4), engine=engine)
    assert np.array_equal(out, np.eye(16, dtype=np.complex128)[0b1111])
    qc = Circuit(6)
    qc.add_repeating_gate(Gate.X, list(range(6))).add_gate(
        Gate.Custom(G.multicnot(6), [0, 1, 2, 3, 4], "X"), 5)
    out = oracle.simulate(lower(qc.get_gates(), 6), engine=engine)
    assert np.array_equal(out, np.eye(64, dtype=np.complex128)[0b111110])


def test_none_overwrite_rule(oracle):
    """A None input keeps its amplitude even when other inputs' images land on it
    (simulation.rs:120-133)."""
    def f(prod):
        if prod.get_qubits()[0] == Qubit.Zero:
            return None
        return SuperPosition.new_with_amplitudes_unchecked([1.0, 1.0])  # |1> -> |0> + |1>
    qc = Circuit(1)
    qc.add_gate(Gate.Custom(f, [], "F"), 0)
    reg = np.array([0.6, 0.8], dtype=np.complex128)
    out = oracle.simulate(lower(qc.get_gates(), 1), reg, engine=oracle.HASHMAP)
    # input 0 -> None: out[0] = 0.6 overwrites the 0.8 mapped from input 1; out[1] = 0.8
    assert np.array_equal(out, np.array([0.6, 0.8], dtype=np.complex128))


def test_measure_linear_scan_and_search_agree(oracle):
    rng = np.random.default_rng(7)
    state = rng.normal(size=64) + 1j * rng.normal(size=64)
    state /= np.linalg.norm(state)
    u = rng.random(2000)
    fast = oracle.measure_uniforms(state, u)
    slow = np.array([oracle.measure_linear(state, x) for x in u])
    assert np.array_equal(fast, slow)
    # u beyond the total probability -> None
    half = state * math.sqrt(0.5)
    assert oracle.measure_linear(half, 0.75) == -1
    assert oracle.measure_uniforms(half, np.array([0.75]))[0] == -1


def test_crk_and_rz_use_reference_expressions(oracle):
    """Gate images come from the reference formulas: e.g. CRk(k) = exp(i 2pi / 2^k)."""
    b = ProgramBuilder(2)
    b.add("X", 0)
    b.add("X", 1)
    b.add("CRk", 1, (0,), k=3)
    out = oracle.simulate(b.build(), engine=oracle.HASHMAP)
    ang = (2.0 * math.pi) / 2.0 ** 3
    assert out[3] == complex(math.cos(ang), math.sin(ang))


def test_cfg1_state_is_normalised(oracle):
    prog = W.random_columns(n=12, seed=1)
    out = oracle.simulate(prog, engine=oracle.DENSE)
    assert abs(np.sum(np.abs(out) ** 2) - 1.0) < 1e-12
