"""The headline metric's byte count (bench.gate_bytes) on the host: every gate kind counts
2 * S * T_gate bytes with T_gate the amplitudes it may change (2^n for the dense single-wire
gates and Custom, 2^(n-1) for S/T/Z/CNot/CY/Swap, 2^(n-2) for CZ/CR/CRk/Toffoli), and the 30-qubit
brickwork + QFT workload has 2 570 gates whose counts give the bytes the bench divides by the
step time."""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

from quantr_gb300 import workloads as W
from quantr_gb300._native import KINDS
from quantr_gb300.program import ProgramBuilder

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_every_kind_has_its_touched_fraction(bench):
    n = 6
    expect = {"H": 1, "X": 1, "Y": 1, "Rx": 1, "Ry": 1, "Rz": 1, "Phase": 1, "X90": 1, "Y90": 1,
              "MX90": 1, "MY90": 1, "Z": 0.5, "S": 0.5, "Sdag": 0.5, "T": 0.5, "Tdag": 0.5,
              "CNot": 0.5, "CY": 0.5, "Swap": 0.5, "CZ": 0.25, "CR": 0.25, "CRk": 0.25,
              "Toffoli": 0.25}
    for name, frac in expect.items():
        b = ProgramBuilder(n)
        controls = {"CNot": (0,), "CY": (0,), "CZ": (0,), "CR": (0,), "CRk": (0,),
                    "Toffoli": (0, 1), "Swap": (0,)}.get(name, ())
        b.add(name, 3, controls, param=0.3, k=2)
        for mult in (16, 8):
            assert bench.gate_bytes(b.build(), mult) == 2 * mult * (1 << n) * frac, name
    b = ProgramBuilder(n)
    b.add_custom(2, [4], np.eye(4, dtype=np.complex128), np.zeros(4, np.uint8))
    assert bench.gate_bytes(b.build()) == 2 * 16 * (1 << n)
    assert set(expect) | {"Custom"} == {k for k in KINDS if k != "Id"}


def test_headline_workload_bytes(bench):
    n = 30
    prog = W.brickwork_qft(n=n, layers=20, seed=2)
    names = [KINDS[int(k)] for k in prog.ops["kind"]]
    assert len(names) == 2570
    rot = 20 * n * 3                          # Rz Ry Rz on every wire, every layer
    cnot = sum(len(range(l % 2, n - 1, 2)) for l in range(20))
    crk = n * (n - 1) // 2                    # QFT controlled phases
    assert names.count("CNot") == cnot and names.count("CRk") == crk
    assert names.count("H") == n and names.count("Swap") == n // 2
    assert rot + cnot + n + crk + n // 2 == 2570
    full = 2 * 16 * float(1 << n)
    want = full * (rot + n) + full / 2 * (cnot + n // 2) + full / 4 * crk
    assert bench.gate_bytes(prog) == want
