"""Dense-block fusion (precision configuration): 6-qubit blocks of up to 12 gates.

Bars: complex128 blocks within 1e-12 max-abs of the oracle; complex64 blocks and complex64 tile
passes: 1 - fidelity <= 1e-8 and max |delta a| <= 1e-5 against the complex128 path on identical
circuits (the 26-qubit cross-check of the configuration, reporting max error, 1 - F and norm
drift).
"""
import numpy as np
import pytest

from quantr_gb300 import _native as nat
from quantr_gb300 import workloads as W
from quantr_gb300.program import ProgramBuilder

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    yield


def run(prog, precision=nat.QGPU_C128, mode=nat.QGPU_MODE_FAST, blocks=0, gates=12):
    h = nat.Handle(prog.n, precision, mode)
    if blocks:
        h.set_fusion(blocks, gates)
    h.apply(prog.ops, prog.mats, prog.none)
    out = h.download()
    nrm = h.norm()
    h.close()
    return out, nrm


@pytest.mark.parametrize("bq,mg", [(6, 12), (3, 4), (1, 1)])
def test_c128_blocks_match_oracle(oracle, bq, mg):
    prog = W.brickwork_qft(n=12, layers=8, seed=7)
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    out, _ = run(prog, blocks=bq, gates=mg)
    assert np.max(np.abs(out - ref)) <= 1e-12


def test_blocks_with_customs_and_controls(oracle):
    n = 9
    rng = np.random.default_rng(11)
    b = ProgramBuilder(n)
    for w in range(n):
        b.add("H", w)
    b.add("Toffoli", 4, (8, 0))
    b.add_custom(2, [6], rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)),
                 np.array([0, 1, 0, 0], np.uint8))
    b.add("CRk", 1, (7,), k=4)
    b.add("Swap", 3, (5,))
    for w in range(n):
        b.add("Rx", w, (), param=0.2 * w + 0.1)
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    out, _ = run(prog, blocks=6)
    assert np.max(np.abs(out - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


def _cross(a, ref):
    fid = abs(np.vdot(ref, a)) ** 2 / (np.vdot(a, a).real * np.vdot(ref, ref).real)
    return float(np.max(np.abs(a - ref))), 1.0 - fid


def test_precision_cross_check_26q():
    """Identical 26-qubit circuits: c64 (blocks and tile passes) and c128 blocks against the
    complex128 tile path."""
    prog = W.brickwork_qft(n=26, layers=20, seed=3)
    ref, ref_norm = run(prog)
    assert abs(ref_norm - 1.0) <= 1e-12
    b128, n128 = run(prog, blocks=6)
    e, infid = _cross(b128, ref)
    assert e <= 1e-12 and abs(n128 - 1.0) <= 1e-12
    for blocks in (6, 0):
        a64, n64 = run(prog, precision=nat.QGPU_C64, blocks=blocks)
        e, infid = _cross(a64, ref)
        assert infid <= 1e-8, (blocks, infid)
        assert e <= 1e-5, (blocks, e)
        assert abs(n64 - 1.0) <= 1e-4, (blocks, n64)


@pytest.mark.parametrize("n,bq", [(13, 6), (16, 6), (14, 5), (12, 4), (10, 3)])
def test_c64_tensor_core_blocks(oracle, monkeypatch, n, bq):
    """complex64 blocks of 3-6 wires run on the tensor cores (k_block_tc, BF16x3 split): same
    bars as the CUDA-core blocks against the complex128 oracle, on circuits whose blocks sit on
    the lowest, the highest and scattered index bits; the CUDA-core path (QGPU_BLOCK_TC=0) is
    computed too and must differ in rounding (proof the tensor-core path ran)."""
    rng = np.random.default_rng(100 + n + bq)
    b = ProgramBuilder(n)
    for layer in range(6):
        for w in range(n):
            b.add("Rx", w, (), param=float(rng.uniform(0, 6.3)))
            b.add("Rz", w, (), param=float(rng.uniform(0, 6.3)))
        for w in range(layer % 2, n - 1, 2):
            b.add("CNot", w + 1, (w,))
        b.add("CRk", 0, (n - 1,), k=3)
        b.add("Toffoli", n // 2, (1, n - 2))
    prog = b.build()
    ref = oracle.simulate(prog, engine=oracle.DENSE)
    monkeypatch.setenv("QGPU_BLOCK_TC", "1")
    tc, _ = run(prog, precision=nat.QGPU_C64, blocks=bq)
    monkeypatch.setenv("QGPU_BLOCK_TC", "0")
    cc, _ = run(prog, precision=nat.QGPU_C64, blocks=bq)
    for a in (tc, cc):
        e, infid = _cross(a, ref)
        assert e <= 1e-5 and infid <= 1e-8, (e, infid)
    assert not np.array_equal(tc, cc)
