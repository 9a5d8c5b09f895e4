"""ctypes wrapper of the CPU oracle (oracle/quantr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, always as the checker or the timed restated reference, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "quantr_oracle.cpp"
LIB = HERE / "_build" / "liboracle.so"

HASHMAP = 0  # literal HashMap-of-labels engine (the restated reference)
DENSE = 1    # same accumulation order on flat arrays
DENSE_PAR = 2  # the dense engine on all host cores (value for value equal to DENSE)

_lib = None


def build(force: bool = False) -> Path:
    LIB.parent.mkdir(exist_ok=True)
    stale = not LIB.exists() or LIB.stat().st_mtime < max(
        SRC.stat().st_mtime, (HERE.parent / "include" / "qgpu.h").stat().st_mtime)
    if force or stale:
        subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off",
                        "-pthread", str(SRC), "-o", str(LIB)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.oracle_simulate.restype = C.c_int
        L.oracle_simulate.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p,
                                      C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_measure_uniforms.restype = None
        L.oracle_measure_uniforms.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_void_p,
                                              C.c_void_p]
        L.oracle_measure_linear.restype = C.c_int64
        L.oracle_measure_linear.argtypes = [C.c_int, C.c_void_p, C.c_double]
        L.oracle_gate_image.restype = C.c_int
        L.oracle_gate_image.argtypes = [C.c_void_p, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None and a.size else C.c_void_p(0)


def simulate(program, state: np.ndarray | None = None, engine: int = DENSE) -> np.ndarray:
    """Run a `quantr_gb300.program.Program` on the oracle; returns the final amplitudes."""
    n = program.n
    if state is None:
        state = np.zeros(1 << n, dtype=np.complex128)
        state[0] = 1.0
    s = np.ascontiguousarray(state, dtype=np.complex128).copy()
    ops = np.ascontiguousarray(program.ops)
    st = lib().oracle_simulate(engine, n, _p(ops), len(ops), _p(program.mats), program.mats.size,
                               _p(program.none), program.none.size, _p(s))
    if st != 0:
        raise ValueError(lib().oracle_last_error().decode())
    return s


def measure_uniforms(state: np.ndarray, u: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(state, dtype=np.complex128)
    n = s.size.bit_length() - 1
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty(u.size, dtype=np.int64)
    lib().oracle_measure_uniforms(n, _p(s), u.size, _p(u), _p(out))
    return out


def measure_linear(state: np.ndarray, u: float) -> int:
    s = np.ascontiguousarray(state, dtype=np.complex128)
    n = s.size.bit_length() - 1
    return int(lib().oracle_measure_linear(n, _p(s), float(u)))
