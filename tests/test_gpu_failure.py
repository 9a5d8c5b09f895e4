"""Failure detection without a GPU fault.

Device side: the pipelined passes bound every mbarrier wait; here one CTA waits on a phase that
nothing completes and must come back with QGPU_ERR_TIMEOUT, after which the same handle keeps
working. Host side: bad requests (an oversize register, a bad op, a Custom gate in the adjoint)
and an injected allocation failure (QGPU_INJECT_SCRATCH_OOM) come back as error statuses, never
as a device fault.
"""
import numpy as np
import pytest

from quantr_gb300 import QuantrError
from quantr_gb300 import _native as nat
from quantr_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(gpu_lib, oracle):
    h = nat.Handle(12)
    st = gpu_lib.qgpu_selftest_bounded_wait(h.raw, 256)
    assert st == nat.QGPU_ERR_TIMEOUT
    assert b"gave up" in gpu_lib.qgpu_last_error()
    prog = W.brickwork_qft(n=12, layers=3, seed=1)   # the handle and context still work
    h.apply(prog.ops, prog.mats, prog.none)
    assert np.max(np.abs(h.download() - oracle.simulate(prog, engine=oracle.DENSE))) <= 1e-12


def test_oversize_register_is_an_error_status(gpu_lib):
    with pytest.raises(QuantrError, match="qgpu_create"):
        nat.Handle(40)
    h = nat.Handle(3)  # later handles are unaffected
    assert h.download()[0] == 1


def test_injected_scratch_oom_is_an_error_status_and_recoverable(gpu_lib, oracle, monkeypatch):
    """Host-side fault injection: with QGPU_INJECT_SCRATCH_OOM=1 a scratch allocation fails as
    on a full device. The call returns QGPU_ERR_OOM (raised as QuantrError), the register is
    untouched, and once the variable is gone the same handle measures normally."""
    prog = W.brickwork_qft(n=10, layers=2, seed=3)
    h = nat.Handle(10)
    h.apply(prog.ops, prog.mats, prog.none)
    monkeypatch.setenv("QGPU_INJECT_SCRATCH_OOM", "1")
    with pytest.raises(QuantrError, match="injected"):
        h.measure(100, 7)  # a fresh handle's first measurement allocates its scratch
    monkeypatch.delenv("QGPU_INJECT_SCRATCH_OOM")
    idx, cnt, failed = h.measure(100, 7)
    assert int(cnt.sum()) == 100 and failed == 0
    assert np.max(np.abs(h.download() - oracle.simulate(prog, engine=oracle.DENSE))) <= 1e-12
