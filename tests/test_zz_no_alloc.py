"""qgpu_measure_uniforms_noalloc: the sampler for callers that cannot let the library allocate.

Such callers (a host framework whose own pool owns all device memory, or a loop that must not
enter the CUDA allocator) get the same sampling rule with the scratch in a fixed array inside
the library. This file is collected last so a run stopping at the first failure has run every
other test; it passes alone in a fresh process and after the rest of the suite.

Bar: indices equal, shot for shot, to qgpu_measure_uniforms (the same kernels on the same state),
on two calls in a row with different states and uniforms.
"""
import ctypes as C

import numpy as np
import pytest

from quantr_gb300 import _native as nat
from quantr_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(lib, h, u):
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.full(u.size, -7, dtype=np.int64)
    st = lib.qgpu_measure_uniforms_noalloc(h.raw, C.c_void_p(u.ctypes.data), u.size,
                                           C.c_void_p(out.ctypes.data))
    return st, out


def test_noalloc_sampler_matches_allocating_sampler(gpu_lib):
    lib = gpu_lib
    rng = np.random.default_rng(2024)
    for call, (n, seed, count) in enumerate([(20, 3, 50000), (12, 4, 65536)]):
        prog = W.random_columns(n=n, columns=12, seed=seed)
        h = nat.Handle(n)
        h.apply(prog.ops, prog.mats, prog.none)
        u = rng.random(count)
        want = h.measure_uniforms(u)
        st, got = _noalloc(lib, h, u)
        assert st == nat.QGPU_OK, lib.qgpu_last_error()
        assert np.array_equal(got, want), f"call {call + 1}"
        h.close()


@pytest.mark.parametrize("precision", [nat.QGPU_C128, nat.QGPU_C64])
def test_noalloc_sampler_at_its_limits_and_on_none_shots(gpu_lib, precision):
    """24 qubits (the largest register served, where the scan workspace is fullest) with the
    largest uniform count, then a register whose total probability is 0.6, so that uniforms at
    or above the total give None (-1); both precisions, two calls in a row each."""
    lib = gpu_lib
    rng = np.random.default_rng(77 + precision)
    prog = W.random_columns(n=24, columns=6, seed=5)
    h = nat.Handle(24, precision)
    h.apply(prog.ops, prog.mats, prog.none)
    u = rng.random(65536)
    u[:8] = [0.0, 1e-300, 0.25, 0.5, 0.999999, np.nextafter(1.0, 0.0), 0.0, 0.5]
    want = h.measure_uniforms(u)
    st, got = _noalloc(lib, h, u)
    assert st == nat.QGPU_OK, lib.qgpu_last_error()
    assert np.array_equal(got, want)
    h.close()

    n = 14
    amps = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    amps *= np.sqrt(0.6) / np.linalg.norm(amps)
    h = nat.Handle(n, precision)
    h.upload(amps)
    u = np.concatenate([rng.random(4000), [0.6 - 1e-9, 0.6 + 1e-9, np.nextafter(1.0, 0.0)]])
    want = h.measure_uniforms(u)
    assert (want == -1).sum() > 1000 and (want >= 0).sum() > 1000
    st, got = _noalloc(lib, h, u)
    assert st == nat.QGPU_OK, lib.qgpu_last_error()
    assert np.array_equal(got, want)
    h.close()


def test_noalloc_sampler_rejects_sizes_beyond_its_limits(gpu_lib):
    lib = gpu_lib
    h = nat.Handle(25)
    st, _ = _noalloc(lib, h, np.array([0.5]))
    assert st == nat.QGPU_ERR_INVALID
    assert b"at most 24" in lib.qgpu_last_error()
    h.close()
    h = nat.Handle(10)
    st, _ = _noalloc(lib, h, np.zeros(65537))
    assert st == nat.QGPU_ERR_INVALID
    assert b"65536" in lib.qgpu_last_error()
    h.close()
