"""The fused-pass planner (quantr_gb300/csrc/plan.cpp) on the host: tests/cpp/plan_emulator.cpp
executes the planned passes in complex128 and the result is compared with the oracle.

Bar: max |a_plan - a_oracle| <= 1e-12 (the planner multiplies gate matrices together, so the
result is not value-equal to gate-by-gate application; the float-pair kernels add their own
rounding on top, checked by the GPU parity tests).
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from quantr_gb300 import workloads as W
from quantr_gb300.program import ProgramBuilder

ROOT = Path(__file__).resolve().parent.parent
TOL = 1e-12


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    exe = tmp_path_factory.mktemp("plan") / "plan_emulator"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "cpp" / "plan_emulator.cpp"),
           str(ROOT / "quantr_gb300" / "csrc" / "plan.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_plan(emulator, prog, tmp_path, pair=1, budget=280, arith_bits=2, group=1):
    f = {k: tmp_path / f"{k}.bin" for k in ("ops", "mats", "none", "out")}
    np.ascontiguousarray(prog.ops).tofile(f["ops"])
    np.ascontiguousarray(prog.mats, dtype=np.float64).tofile(f["mats"])
    np.ascontiguousarray(prog.none, dtype=np.uint8).tofile(f["none"])
    r = subprocess.run([str(emulator), str(prog.n), str(f["ops"]), str(f["mats"]), str(f["none"]),
                        str(f["out"]), str(pair), str(budget), str(arith_bits), "0", str(group)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    counts = dict(zip(r.stdout.split()[::2], map(int, r.stdout.split()[1::2])))
    return np.fromfile(f["out"], dtype=np.complex128), counts


@pytest.mark.parametrize("group", [0, 1])
@pytest.mark.parametrize("pair", [0, 1])
@pytest.mark.parametrize("budget", [140, 280])
@pytest.mark.parametrize("n", [6, 10, 11])
def test_brickwork_qft_plan(emulator, oracle, tmp_path, n, budget, pair, group):
    prog = W.brickwork_qft(n=n, layers=20, seed=2)
    out, counts = run_plan(emulator, prog, tmp_path, pair, budget, group=group)
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    assert np.max(np.abs(out - ref)) <= TOL
    if pair:
        # two layers of a wire pair and their CNot per block
        assert counts["pair"] + 2 * counts["pair2"] >= 10 * (n // 2) - n
    if pair and group and n % 2 == 0 and n // 2 - 1 >= 3:
        # blocks run two per pass; the CNot layers between brickwork layers (XOR passes of
        # n/2 - 1 terms) are folded into the double passes as register permutations, all but
        # the last layer's leftovers
        assert counts["pair2"] >= 10 * ((n // 2) // 2)
        assert counts["folded"] >= 9 * (n // 2 - 1)
        assert counts["xor"] <= 2


def test_double_pair_passes_fold_xor_terms(emulator, oracle, tmp_path):
    """Double pair passes with XOR terms folded before and after the blocks: CNots between and
    inside the tiles, swaps across two blocks, and a Toffoli whose bits span two tiles (left in
    an XOR pass)."""
    n = 8
    rng = np.random.default_rng(11)
    b = ProgramBuilder(n)
    for layer in range(8):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(0, n, 2):
            b.add("CNot", w + 1, (w,))
        for w in range(n):
            b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
        if layer % 2 == 0:
            b.add("CNot", 2, (1,))
            b.add("CNot", 4, (3,))
            b.add("CNot", 6, (5,))
            b.add("Toffoli", 7, (0, 3))
        else:
            b.add("Swap", 2, (5,))
            b.add("CNot", 1, (0,))
            b.add("CNot", 4, (3,))
            b.add("CNot", 7, (6,))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    for group in (0, 1):
        out, counts = run_plan(emulator, prog, tmp_path, 1, group=group)
        assert np.max(np.abs(out - ref)) <= TOL
        if group:
            assert counts["pair2"] > 0 and counts["folded"] > 0


@pytest.mark.parametrize("seed", [1, 11, 12])
def test_random_columns_plan(emulator, oracle, tmp_path, seed):
    prog = W.random_columns(n=9, columns=40, seed=seed)
    for pair in (0, 1):
        out, _ = run_plan(emulator, prog, tmp_path, pair)
        ref = oracle.simulate(prog, engine=oracle.DENSE)
        assert np.max(np.abs(out - ref)) <= TOL


@pytest.mark.parametrize("seed", [3, 4])
def test_double_pair_grouping_random_xor_layers(emulator, oracle, tmp_path, seed):
    """Random layers of wire-pair blocks separated by random commuting XOR runs (CNots with
    controls inside and outside the pair tiles, Toffolis, X): whatever the matching folds, the
    plan equals the oracle."""
    n = 12
    rng = np.random.default_rng(seed)
    b = ProgramBuilder(n)
    for layer in range(6):
        perm = rng.permutation(n)
        pairs = [(int(perm[2 * i]), int(perm[2 * i + 1])) for i in range(n // 2)]
        for a, c in pairs:  # two dense layers and a CNot per pair: one 4x4 block each
            for w in (a, c):
                b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
                b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("CNot", c, (a,))
            for w in (a, c):
                b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
        # a commuting XOR run (targets distinct, never controls): CNots joining neighbouring
        # pairs (foldable when the matching puts the two pairs in one tile), then X, CNot and
        # Toffoli on the remaining wires with controls anywhere
        targets, controls = set(), set()
        for i in range(0, len(pairs) - 1, 2):
            c, t = pairs[i][1], pairs[i + 1][0]
            b.add("CNot", t, (c,))
            targets.add(t)
            controls.add(c)
        free = [w for w in range(n) if w not in targets and w not in controls]
        for t in rng.permutation(free)[: 2]:
            t = int(t)
            targets.add(t)
            pool = [w for w in range(n) if w not in targets]
            k = int(rng.integers(0, 3))
            ctrls = tuple(int(x) for x in rng.choice(pool, size=k, replace=False))
            controls.update(ctrls)
            b.add(["X", "CNot", "Toffoli"][k], t, ctrls)
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    for group in (0, 1):
        out, counts = run_plan(emulator, prog, tmp_path, 1, group=group)
        assert np.max(np.abs(out - ref)) <= TOL
        if group:
            assert counts["pair2"] > 0 and counts["folded"] > 0


def test_every_gate_plan(emulator, oracle, tmp_path):
    """Each gate kind on each wire with controls above and below (no Custom)."""
    n = 6
    b = ProgramBuilder(n)
    for t in range(n):
        b.add("H", t)
    for t in range(n):
        for name in ("H", "X", "Y", "Z", "S", "Sdag", "T", "Tdag", "X90", "Y90", "MX90", "MY90"):
            b.add(name, t)
        for name in ("Rx", "Ry", "Rz", "Phase"):
            b.add(name, t, (), param=0.3 + t)
        for c in range(n):
            if c == t:
                continue
            b.add("CNot", t, (c,))
            b.add("Ry", c, (), param=0.1 * c + 0.2)
            b.add("CY", t, (c,))
            b.add("CZ", t, (c,))
            b.add("Swap", t, (c,))
            b.add("CR", t, (c,), param=0.7 * c - t)
            b.add("CRk", t, (c,), k=1 + (c + t) % 5)
            c2 = (c + 1 + t) % n
            if c2 not in (c, t):
                b.add("Toffoli", t, (c, c2))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    for pair in (0, 1):
        for arith_bits in (2, 3):
            out, _ = run_plan(emulator, prog, tmp_path, pair, 280, arith_bits)
            assert np.max(np.abs(out - ref)) <= TOL


def test_pair_blocks_interleaved_wires(emulator, oracle, tmp_path):
    """Blocks that must close when a gate reaches a third wire, merge when two single-wire
    blocks meet, and stay open across gates on other wires."""
    n = 7
    rng = np.random.default_rng(4)
    b = ProgramBuilder(n)
    for _ in range(6):
        for w in range(n):
            b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        b.add("CNot", 1, (0,))
        b.add("Ry", 0, (), param=float(rng.uniform(0, 6.3)))  # second layer on the 0-1 pair
        b.add("Ry", 1, (), param=float(rng.uniform(0, 6.3)))
        b.add("CZ", 3, (2,))
        b.add("CNot", 2, (1,))      # reaches across two open blocks
        b.add("Ry", 4, (), param=0.4)
        b.add("CNot", 5, (4,))
        b.add("CNot", 4, (5,))
        b.add("Toffoli", 6, (0, 5))  # not fusable: closes blocks on 0 and 5
        b.add("CRk", 3, (6,), k=3)
        b.add("Swap", 2, (5,))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    for group in (0, 1):
        out, counts = run_plan(emulator, prog, tmp_path, 1, group=group)
        assert counts["pair"] + counts["pair2"] > 0
        assert np.max(np.abs(out - ref)) <= TOL


@pytest.mark.parametrize("seed", [5, 6])
def test_custom_blocks_between_fused_passes(emulator, oracle, tmp_path, seed):
    """Custom gates (dense blocks with None entries, a non-unitary one-wire block, a permutation
    on six wires with controls above and below the target) inside runs of pair-fusable gates,
    phase rows and CNot layers: the planner must close every open block and table at a Custom
    gate and keep the gate order around it. (The None rule is folded into the tabulated matrix;
    blocks left in controlled-2x2 form join the ordinary passes.)"""
    n = 9
    rng = np.random.default_rng(seed)
    b = ProgramBuilder(n)
    customs = 0
    for layer in range(4):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
        t, c1, c2 = (int(x) for x in rng.choice(n, size=3, replace=False))
        blk = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
        none = (rng.random(8) < 0.25).astype(np.uint8)
        b.add_custom(t, [c1, c2], blk / 3, none)
        customs += 1
        for w in range(n):
            b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
        b.add("H", 0)
        for k in range(2, n + 1):
            b.add("CRk", 0, (k - 1,), k=k)
        w = int(rng.integers(0, n))
        b.add_custom(w, [], np.array([[1.2, 0.1j], [0, 0.8]], np.complex128),
                     np.array([0, layer % 2], np.uint8))
        customs += 1
    d = 1 << 6
    wires = [int(x) for x in rng.choice(n, size=6, replace=False)]
    perm = np.eye(d, dtype=np.complex128)[rng.permutation(d)] * np.exp(1j * rng.random(d))[:, None]
    b.add_custom(wires[2], wires[:2] + wires[3:], perm, np.zeros(d, np.uint8))
    customs += 1
    for w in range(n):
        b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    scale = max(1.0, float(np.max(np.abs(ref))))
    for pair in (0, 1):
        for group in (0, 1):
            out, counts = run_plan(emulator, prog, tmp_path, pair, group=group)
            # blocks in controlled-2x2 form (every one-wire block) run as ordinary gates
            assert 5 <= counts["custom"] <= customs
            assert np.max(np.abs(out - ref)) <= TOL * scale


def run_blocks(emulator, prog, tmp_path, block_qubits, max_gates):
    f = {k: tmp_path / f"{k}.bin" for k in ("ops", "mats", "none", "out")}
    np.ascontiguousarray(prog.ops).tofile(f["ops"])
    np.ascontiguousarray(prog.mats, dtype=np.float64).tofile(f["mats"])
    np.ascontiguousarray(prog.none, dtype=np.uint8).tofile(f["none"])
    r = subprocess.run([str(emulator), str(prog.n), str(f["ops"]), str(f["mats"]), str(f["none"]),
                        str(f["out"]), "1", "280", "2", "0", "1", str(block_qubits), str(max_gates)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    counts = dict(zip(r.stdout.split()[::2], map(int, r.stdout.split()[1::2])))
    return np.fromfile(f["out"], dtype=np.complex128), counts


@pytest.mark.parametrize("bq,mg", [(6, 12), (4, 5), (3, 4), (1, 1)])
def test_dense_block_fusion(emulator, oracle, tmp_path, bq, mg):
    """Dense-block fusion (build_blocks, the precision configuration's 6-qubit blocks of <= 12
    gates): consecutive gates multiplied on the host into one matrix per block, Custom blocks
    with None entries and a gate wider than the block limit (a block of its own) included. The
    blocks applied in complex128 equal the oracle; no block exceeds the limit unless one gate
    does; every non-identity gate lands in exactly one block."""
    n = 9
    rng = np.random.default_rng(17)
    b = ProgramBuilder(n)
    gates = 0
    for w in range(n):
        b.add("H", w)
        gates += 1
    for layer in range(3):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
            gates += 1
        for w in range(layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
            gates += 1
        b.add("Toffoli", 4, (8, 0))
        b.add_custom(2, [6], rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)),
                     np.array([0, 1, 0, 0], np.uint8))
        b.add("CRk", 1, (7,), k=4)
        b.add("Swap", 3, (5,))
        b.add("CR", 8, (2,), param=0.3)
        gates += 5
    d = 1 << 7
    perm = np.eye(d, dtype=np.complex128)[rng.permutation(d)]
    b.add_custom(5, [0, 1, 2, 3, 7, 8], perm, np.zeros(d, np.uint8))  # 7 wires
    gates += 1
    for w in range(n):
        b.add("Rx", w, (), param=0.2 * w + 0.1)
        gates += 1
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    out, counts = run_blocks(emulator, prog, tmp_path, bq, mg)
    assert np.max(np.abs(out - ref)) <= TOL * max(1.0, float(np.max(np.abs(ref))))
    assert counts["gates"] == gates
    assert counts["maxk"] <= max(bq, 7)
    assert counts["blocks"] >= -(-gates // mg)
