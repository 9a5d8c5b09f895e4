"""Device-side `SuperPosition::to_hash_map` (super_positions.rs:315-323): qgpu_extract_nonzero
against the same rule applied on the host to the downloaded register.

Bar: bit-exact. The survivor set, its index order and every amplitude equal the host's
(the amplitudes are copied, not computed; for complex64 they are widened to f64 exactly).
"""
import numpy as np
import pytest

from quantr_gb300 import Circuit, Gate, QuantrError
from quantr_gb300 import _native as nat
from quantr_gb300.states import ZERO_MARGIN

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    yield


def host_rule(a: np.ndarray, margin: float):
    a = a.astype(np.complex128)
    p = a.real * a.real + a.imag * a.imag
    keep = np.nonzero(~((p > -margin) & (p < margin)))[0]
    return keep.astype(np.uint64), a[keep]


@pytest.mark.parametrize("precision", [nat.QGPU_C128, nat.QGPU_C64])
@pytest.mark.parametrize("n", [1, 5, 9, 10, 14, 20])
def test_extract_matches_host_rule(n, precision):
    rng = np.random.default_rng(100 + n)
    a = rng.normal(size=2**n) + 1j * rng.normal(size=2**n)
    # about half the amplitudes below the margin, some exactly zero, some right at it
    a[rng.random(2**n) < 0.5] *= 1e-5
    a[rng.random(2**n) < 0.1] = 0
    if n >= 5:
        a[3] = np.sqrt(ZERO_MARGIN)
    h = nat.Handle(n, precision)
    h.upload(a)
    reg = h.download()
    idx, amp = h.extract_nonzero(ZERO_MARGIN)
    ref_idx, ref_amp = host_rule(reg, ZERO_MARGIN)
    assert np.array_equal(idx, ref_idx)
    assert np.array_equal(amp, ref_amp)
    h.close()


def test_extract_cap_overflow_reports_count():
    n = 12
    h = nat.Handle(n)
    h.upload(np.full(2**n, 2 ** (-n / 2), dtype=np.complex128))
    with pytest.raises(QuantrError):
        h.extract_nonzero(ZERO_MARGIN, cap=100)
    idx, amp = h.extract_nonzero(ZERO_MARGIN)
    assert np.array_equal(idx, np.arange(2**n, dtype=np.uint64))
    h.close()


def test_state_hash_map_equals_to_hash_map():
    qc = Circuit(12)
    qc.add_gate(Gate.H, 0)
    for t in range(1, 12):
        qc.add_gate(Gate.CNot(0), t)
    qc.add_gate(Gate.Rx(0.3), 5)
    sim = qc.simulate()
    got = sim.state_hash_map()
    want = sim.get_state().take().to_hash_map()
    assert got == want
    assert len(got) == 4


def test_extract_sparse_28q():
    # 28-qubit GHZ-like state: 4 GiB register, 2 survivors; nothing but them is downloaded
    n = 28
    qc = Circuit(n)
    qc.add_gate(Gate.H, 0)
    for t in range(1, n):
        qc.add_gate(Gate.CNot(t - 1), t)
    sim = qc.simulate()
    before = sim.handle.io_bytes()[1]
    hm = sim.state_hash_map()
    moved = sim.handle.io_bytes()[1] - before
    assert len(hm) == 2
    for st, a in hm.items():
        assert abs(a - 2**-0.5) < 1e-12
        assert st.comp_basis() in (0, 2**n - 1)
    assert moved < 4096
