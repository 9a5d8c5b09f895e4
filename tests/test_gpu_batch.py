"""Batching configuration: many independent ansatz circuits, energies + adjoint gradients.

Bars: batched complex128 energies and gradients equal the per-circuit qgpu_adjoint_grad results
within 1e-10 (the in-shared-memory path uses f64 with a different reduction order); complex64
energies and gradients (shared-memory path up to 13 qubits, complex64 register passes and the f32
grouped sweep above) within 1e-4 of complex128.
"""
import numpy as np
import pytest

from quantr_gb300 import QuantrError
from quantr_gb300 import _native as nat
from quantr_gb300 import batch as B
from quantr_gb300 import gradients as GR
from quantr_gb300.program import ProgramBuilder

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    yield


def _reference(cs):
    es, gs = [], []
    for c in cs:
        h = nat.Handle(c.n)
        e, g = GR.energy_and_gradient(h, c.program, c.a, c.b)
        h.close()
        es.append(e)
        gs.append(g)
    return np.array(es), gs


def test_batch_c128_matches_per_circuit():
    cs = B.batch_config(count=40, seed=5, layers=3, n_min=4, n_max=15)
    assert {c.n for c in cs} & set(range(4, 13)) and {c.n for c in cs} & {13, 14, 15}
    e, g, tuned = B.run_batch(cs)
    re, rg = _reference(cs)
    assert np.max(np.abs(e - re)) <= 1e-10
    for a, b in zip(g, rg):
        assert np.max(np.abs(a - b)) <= 1e-10
    assert tuned and all(q > 12 for q in tuned)
    assert all(t["adjoint_sweep"] in ("grouped", "per-wire") and t["fusion_budget"] > 0 for t in tuned.values())


def test_batch_c64_energies_and_gradients():
    """complex64 batches (in shared memory up to 13 qubits, complex64 register passes and the f32
    grouped sweep above) against the complex128 per-circuit adjoint: energies and every gradient
    entry within 1e-4."""
    cs = B.batch_config(count=24, seed=6, layers=2, n_min=4, n_max=16)
    assert {c.n for c in cs} & {14, 15, 16}
    e64, g64, _ = B.run_batch(cs, precision=nat.QGPU_C64)
    re, rg = _reference(cs)
    assert np.max(np.abs(e64 - re)) <= 1e-4
    for a, b in zip(g64, rg):
        assert np.max(np.abs(a - b)) <= 1e-4


def test_batch_rejects_custom():
    b = ProgramBuilder(3)
    b.add_custom(0, [1], np.eye(4, dtype=np.complex128), np.zeros(4, np.uint8))
    c = B.BatchCircuit(b.build(), np.ones(3), np.ones(3))
    with pytest.raises(QuantrError):
        B.run_batch([c])
