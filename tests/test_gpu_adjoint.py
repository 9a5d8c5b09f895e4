"""Adjoint gradients (config: 20-qubit hardware-efficient ansatz, 400 parameters).

Bars: max |g_adjoint - g_FD| <= 1e-7 (central differences, h = 1e-6) and
max |g_adjoint - g_shift| <= 1e-9 (parameter shift +-pi/2), complex128. Small cases also check
against the CPU oracle with numpy finite differences.
"""
import math

import numpy as np
import pytest

from quantr_gb300 import QuantrError
from quantr_gb300 import _native as nat
from quantr_gb300 import gradients as GR
from quantr_gb300 import workloads as W
from quantr_gb300.program import ProgramBuilder, Program

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    yield


def _oracle_energy(orc, prog, a, b):
    return W.energy_dense(orc.simulate(prog, engine=orc.DENSE), a, b)


def _oracle_fd(orc, prog, a, b, h=1e-6):
    g = np.zeros(len(prog.ops))
    for i, k in enumerate(prog.ops["kind"]):
        if int(k) in GR.ROTATIONS:
            up = prog.ops.copy()
            up["param"][i] += h
            dn = prog.ops.copy()
            dn["param"][i] -= h
            g[i] = (_oracle_energy(orc, Program(prog.n, up, prog.mats, prog.none), a, b)
                    - _oracle_energy(orc, Program(prog.n, dn, prog.mats, prog.none), a, b)) / (2 * h)
    return g


def test_energy_matches_oracle(oracle):
    an = W.ansatz(n=8, layers=3, seed=4)
    prog = an.program()
    h = nat.Handle(8)
    e = GR.energy(h, prog, an.a, an.b)
    assert e == pytest.approx(_oracle_energy(oracle, prog, an.a, an.b), abs=1e-12)


@pytest.fixture(params=["gates", "pauli", "group"])
def sweep(request, monkeypatch):
    """The single-wire sweep forms: per-gate passes; one pass per wire with the gradients formed
    from Pauli sums; the same sums for the wires of a tile of up to 11 bits in one pass (the
    default)."""
    if request.param == "gates":
        monkeypatch.setenv("QGPU_ADJ_PAULI", "0")
    elif request.param == "pauli":
        monkeypatch.setenv("QGPU_ADJ_PAULI", "1")
        monkeypatch.setenv("QGPU_ADJ_GROUP", "0")
    else:
        monkeypatch.setenv("QGPU_ADJ_GROUP", "1")
    return request.param


def test_adjoint_all_gate_kinds_vs_oracle_fd(oracle, sweep):
    """Every invertible gate kind in the circuit (the sweep undoes each one)."""
    n = 6
    rng = np.random.default_rng(0)
    b = ProgramBuilder(n)
    for layer in range(2):
        for w in range(n):
            b.add(["Rx", "Ry", "Rz", "Phase"][(w + layer) % 4], w, (), param=rng.uniform(-3, 3))
        b.add("H", 0); b.add("S", 1); b.add("T", 2); b.add("Sdag", 3); b.add("Tdag", 4)
        b.add("X90", 5); b.add("Y90", 0); b.add("MX90", 1); b.add("MY90", 2); b.add("Y", 3)
        b.add("CNot", 1, (0,)); b.add("CZ", 2, (4,)); b.add("CY", 5, (3,)); b.add("Swap", 0, (5,))
        b.add("CR", 3, (1,), param=0.37); b.add("CRk", 4, (2,), k=3); b.add("Toffoli", 1, (3, 5))
        for w in range(n):
            b.add("Ry", w, (), param=rng.uniform(-3, 3))
    prog = b.build()
    a_c = rng.normal(size=n)
    b_c = rng.normal(size=n)
    h = nat.Handle(n)
    e, g = GR.energy_and_gradient(h, prog, a_c, b_c)
    assert e == pytest.approx(_oracle_energy(oracle, prog, a_c, b_c), abs=1e-12)
    fd = _oracle_fd(oracle, prog, a_c, b_c)
    assert np.max(np.abs(g - fd)) <= 1e-7


def test_adjoint_permutation_runs_vs_oracle_fd(oracle, sweep):
    """Runs of CNot / X / Swap between rotation layers (undone as one index permutation each,
    out of place): gradients against the oracle's finite differences, and the register still
    holds the final state afterwards."""
    n = 11
    rng = np.random.default_rng(12)
    b = ProgramBuilder(n)
    for layer in range(3):
        for w in range(n):
            b.add("Ry", w, (), param=rng.uniform(-3, 3))
            b.add("Rz", w, (), param=rng.uniform(-3, 3))
        for w in range(n):
            b.add("CNot", (w + 1) % n, (w,))      # ring: a chain of dependent gates
        b.add("X", 3)
        b.add("Swap", 2, (9,))
        b.add("CNot", 0, (7,))
        b.add("Swap", 5, (1,))
        b.add("X", 10)
    for w in range(n):
        b.add("Rx", w, (), param=rng.uniform(-3, 3))
    prog = b.build()
    a_c = rng.normal(size=n)
    b_c = rng.normal(size=n)
    h = nat.Handle(n)
    e, g = GR.energy_and_gradient(h, prog, a_c, b_c)
    assert e == pytest.approx(_oracle_energy(oracle, prog, a_c, b_c), abs=1e-12)
    fd = _oracle_fd(oracle, prog, a_c, b_c)
    assert np.max(np.abs(g - fd)) <= 1e-7
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    assert np.max(np.abs(h.download() - ref)) <= 1e-12


def test_adjoint_long_single_wire_runs_vs_parameter_shift(sweep):
    """Runs of up to seven single-wire gates on a wire (rotations of all kinds, Phase, and fixed
    gates between them) undone together: every rotation's gradient against parameter shift."""
    n = 9
    rng = np.random.default_rng(21)
    b = ProgramBuilder(n)
    kinds = ["Rx", "Ry", "Rz", "Phase"]
    for layer in range(2):
        for w in range(n):
            for q in range(1 + (w + layer) % 7):
                if q % 3 == 2:
                    b.add(["H", "S", "T", "X90", "MY90"][(w + q) % 5], w)
                else:
                    b.add(kinds[(w + q + layer) % 4], w, (), param=rng.uniform(-3, 3))
        for w in range(0, n - 1, 2):
            b.add("CNot", w + 1, (w,))
        b.add("CZ", 0, (n - 1,))
    prog = b.build()
    a_c = rng.normal(size=n)
    b_c = rng.normal(size=n)
    h = nat.Handle(n)
    e, g = GR.energy_and_gradient(h, prog, a_c, b_c)
    ps = GR.parameter_shift(h, prog, a_c, b_c)
    assert np.max(np.abs(g - ps)) <= 1e-9
    assert math.isfinite(e)


def test_adjoint_ansatz_22q_pauli_sweep_vs_parameter_shift():
    """22 qubits (the vectors leave L2; the sweep takes the Pauli-sum form by default)."""
    an = W.ansatz(n=22, layers=2, seed=7)
    prog = an.program()
    h = nat.Handle(22)
    e, g = GR.energy_and_gradient(h, prog, an.a, an.b)
    ps = GR.parameter_shift(h, prog, an.a, an.b)
    assert np.max(np.abs(g - ps)) <= 1e-9
    assert math.isfinite(e)


def test_adjoint_ansatz_20q_vs_fd_and_parameter_shift():
    """The differentiation config: 20 qubits, 10 layers of Ry Rz + CNot ring, 400 parameters."""
    an = W.ansatz(n=20, layers=10, seed=4)
    prog = an.program()
    h = nat.Handle(20)
    e, g = GR.energy_and_gradient(h, prog, an.a, an.b)
    rot = np.isin(prog.ops["kind"], list(GR.ROTATIONS))
    assert rot.sum() == 400
    fd = GR.finite_difference(h, prog, an.a, an.b, h=1e-6)
    ps = GR.parameter_shift(h, prog, an.a, an.b)
    assert np.max(np.abs(g - fd)) <= 1e-7
    assert np.max(np.abs(g - ps)) <= 1e-9
    assert math.isfinite(e)


@pytest.mark.parametrize("n,layers", [(16, 3), (23, 2)])
def test_grouped_sweep_equals_per_wire_passes(monkeypatch, n, layers):
    """k_adj_group (the wires of a tile of up to 11 bits per pass: at 23 qubits tiles of bits
    0..10, then bits 0..4 with six more wires, twice) against one pass per wire: the same
    Pauli sums in another summation order, so energies equal and gradients within 1e-11."""
    an = W.ansatz(n=n, layers=layers, seed=12)
    prog = an.program()
    h = nat.Handle(n)
    h.set_profiling(True)
    monkeypatch.setenv("QGPU_ADJ_GROUP", "1")
    e1, g1 = GR.energy_and_gradient(h, prog, an.a, an.b)
    prof = h.profile(reset=True)
    assert prof["k_adj_group"][0] == layers * (1 if n <= 11 else 1 + -(-(n - 11) // 6)), prof
    monkeypatch.setenv("QGPU_ADJ_GROUP", "0")
    monkeypatch.setenv("QGPU_ADJ_PAULI", "1")
    e2, g2 = GR.energy_and_gradient(h, prog, an.a, an.b)
    prof2 = h.profile(reset=True)
    assert "k_adj_group" not in prof2 and prof2["k_adj_tile"][0] == layers * n
    h.close()
    assert e1 == e2
    assert np.max(np.abs(g1 - g2)) <= 1e-11


@pytest.mark.parametrize("n,layers", [(9, 3), (14, 4), (21, 2)])
def test_complex64_energy_and_gradient(n, layers):
    """complex64 handles: the forward pass in f32, the sweep in k_adj_group_f32 (grouped passes
    at every size) and k_linperm for the CNot rings; energies within 1e-5 and gradients within
    1e-4 of the complex128 adjoint."""
    an = W.ansatz(n=n, layers=layers, seed=3)
    prog = an.program()
    h128 = nat.Handle(n)
    e128, g128 = GR.energy_and_gradient(h128, prog, an.a, an.b)
    h128.close()
    h64 = nat.Handle(n, nat.QGPU_C64)
    h64.set_profiling(True)
    e64, g64 = GR.energy_and_gradient(h64, prog, an.a, an.b)
    prof = h64.profile(reset=True)
    h64.close()
    assert prof["k_adj_group_f32"][0] >= layers, prof
    assert abs(e64 - e128) <= 1e-5
    assert np.max(np.abs(g64 - g128)) <= 1e-4


def test_complex64_all_gate_kinds_and_permutation_runs():
    """complex64 sweep on every invertible gate kind (fixed gates inside single-wire runs, the
    multi-wire kinds through the register passes) and on CNot rings / X / Swap runs (the index
    gather out of place, into and out of the third vector): energy and every gradient against
    the complex128 adjoint, 1e-5 / 1e-4; the register holds the final state afterwards."""
    n = 12
    rng = np.random.default_rng(31)
    b = ProgramBuilder(n)
    for layer in range(3):
        for w in range(n):
            b.add(["Rx", "Ry", "Rz", "Phase"][(w + layer) % 4], w, (), param=rng.uniform(-3, 3))
        b.add("H", 0); b.add("S", 1); b.add("T", 2); b.add("Sdag", 3); b.add("Tdag", 4)
        b.add("X90", 5); b.add("Y90", 6); b.add("MX90", 7); b.add("MY90", 8); b.add("Y", 9)
        b.add("CNot", 1, (0,)); b.add("CZ", 2, (4,)); b.add("CY", 5, (3,)); b.add("Swap", 0, (5,))
        b.add("CR", 3, (1,), param=0.37); b.add("CRk", 4, (2,), k=3); b.add("Toffoli", 1, (3, 5))
        for w in range(n):
            b.add("Ry", w, (), param=rng.uniform(-3, 3))
        for w in range(n):
            b.add("CNot", (w + 1) % n, (w,))
        b.add("X", 3); b.add("Swap", 2, (9,)); b.add("CNot", 0, (7,))
    prog = b.build()
    a_c = rng.normal(size=n)
    b_c = rng.normal(size=n)
    h128 = nat.Handle(n)
    e128, g128 = GR.energy_and_gradient(h128, prog, a_c, b_c)
    h64 = nat.Handle(n, nat.QGPU_C64)
    e64, g64 = GR.energy_and_gradient(h64, prog, a_c, b_c)
    assert abs(e64 - e128) <= 1e-5
    assert np.max(np.abs(g64 - g128)) <= 1e-4
    assert np.max(np.abs(h64.download() - h128.download())) <= 1e-5
    h64.close()
    h128.close()


def test_adjoint_rejects_custom():
    b = ProgramBuilder(3)
    b.add("H", 0)
    b.add_custom(1, [0], np.eye(4, dtype=np.complex128), np.zeros(4, np.uint8))
    prog = b.build()
    h = nat.Handle(3)
    with pytest.raises(QuantrError):
        h.adjoint_grad(prog.ops, prog.mats, prog.none, np.ones(3), np.ones(3))
