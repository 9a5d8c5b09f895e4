"""Digit pair passes (quantr_gb300/csrc/digits.cu) on the GPU: runs of fused pair passes of
complex128 fast-mode registers executed on the tensor cores in fixed-point base-128 digits.

Bars: amplitudes within 1e-12 max-abs of the oracle for normalised registers (scaled by the
register's largest amplitude otherwise); the profile shows the digit kernels actually ran.
"""
import numpy as np
import pytest

from quantr_gb300 import _native as nat
from quantr_gb300 import workloads as W
from quantr_gb300.program import ProgramBuilder

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(autouse=True)
def _lib(gpu_lib, monkeypatch):
    # digit runs from 11 qubits here (the default starts at 20), so small registers exercise them
    monkeypatch.setenv("QGPU_DIGITS_MIN_QUBITS", "11")
    yield


def _run(prog, reg=None, profile=False):
    h = nat.Handle(prog.n, nat.QGPU_C128, nat.QGPU_MODE_FAST)
    if reg is not None:
        h.upload(reg)
    h.set_profiling(profile)
    h.apply(prog.ops, prog.mats, prog.none)
    out = h.download()
    prof = h.profile(reset=True) if profile else {}
    h.close()
    return out, prof


@pytest.mark.parametrize("n", [12, 14, 16])
def test_digit_passes_run_and_match_oracle(oracle, n):
    """The headline family (an even number of wires, so the brickwork's pair passes form one
    uninterrupted run): every pair pass runs as a digit pass."""
    prog = W.brickwork_qft(n=n, layers=8, seed=5)
    ref = oracle.simulate(prog, engine=oracle.DENSE_PAR)
    out, prof = _run(prog, profile=True)
    assert "k_dg2" in prof and "k_dg_from" in prof and "k_dg_to" in prof, prof
    assert not any(k.startswith("k_pair2<") for k in prof), prof
    assert np.max(np.abs(out - ref)) <= TOL


@pytest.mark.parametrize("scale", [7.25, 1e-20])
def test_digit_scale_follows_the_register(oracle, scale):
    """An uploaded register that is not normalised: the digits' fixed point is scaled by its norm,
    so large and tiny registers keep their relative accuracy."""
    n = 14
    rng = np.random.default_rng(3)
    reg = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    reg *= scale / np.linalg.norm(reg)
    prog = W.brickwork_qft(n=n, layers=6, seed=9, qft=False)
    ref = oracle.simulate(prog, reg, engine=oracle.DENSE_PAR)
    out, prof = _run(prog, reg=reg, profile=True)
    assert "k_dg2" in prof
    assert np.max(np.abs(out - ref)) <= TOL * scale


def test_digit_runs_after_non_unitary_custom(oracle):
    """A Custom gate that grows the register (x3 on one wire) before a run of pair passes: the
    amplitude bound carried through the plan keeps the digits in range."""
    n = 14
    b = ProgramBuilder(n)
    b.add_custom(4, [], np.array([[3.0, 0.0], [0.0, 3.0]], np.complex128), np.zeros(2, np.uint8))
    rng = np.random.default_rng(8)
    for layer in range(8):
        for w in range(n):
            b.add("Ry", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE_PAR)
    out, prof = _run(prog, profile=True)
    assert "k_dg2" in prof
    assert np.max(np.abs(out - ref)) <= TOL * 3


def test_digit_passes_with_measurement_and_norm(oracle):
    """Downstream kernels see complex128 after a digit run: norm, checksum and shots."""
    prog = W.brickwork_qft(n=16, layers=10, seed=2)
    ref = oracle.simulate(prog, engine=oracle.DENSE_PAR)
    h = nat.Handle(16)
    h.apply(prog.ops, prog.mats, prog.none)
    assert abs(h.norm() - 1.0) <= 1e-13
    cs = h.checksum()
    assert abs(cs - ref.sum()) <= 1e-11
    # the same state through the oracle's linear-scan rule: equal shots (the device sums in
    # another order, so a uniform within rounding of a cumulative boundary may differ)
    u = np.random.default_rng(1).random(2000)
    same = h.measure_uniforms(u) == oracle.measure_uniforms(h.download(), u)
    assert same.sum() >= 1998
    h.close()
