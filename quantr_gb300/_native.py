"""ctypes binding of libquantr_gpu (include/qgpu.h).

The shared library is built in-tree by `quantr_gb300.build` (or `__graft_entry__.build()`).
There is no CPU fallback: if the library or a CUDA device is missing, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from .errors import QuantrError

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libquantr_gpu.so"

# status codes (qgpu.h)
QGPU_OK = 0
QGPU_ERR_INVALID = -1
QGPU_ERR_OOM = -2
QGPU_ERR_CUDA = -3
QGPU_ERR_TIMEOUT = -4
QGPU_ERR_UNSUPPORTED = -5
QGPU_ERR_NONUNITARY = -6

QGPU_C128 = 0
QGPU_C64 = 1
QGPU_MODE_FAST = 0
QGPU_MODE_EXACT = 1
QGPU_MODE_F64 = 2
QGPU_MAX_OP_WIRES = 10

# gate kinds, in quantr's Gate enum order (src/circuit/gate.rs:19-106)
KINDS = ["Id", "H", "X", "Y", "Z", "S", "Sdag", "T", "Tdag", "Rx", "Ry", "Rz", "X90", "Y90",
         "MX90", "MY90", "Phase", "CR", "CRk", "CZ", "CY", "CNot", "Swap", "Toffoli", "Custom"]
KIND = {name: i for i, name in enumerate(KINDS)}


class QgpuOp(C.Structure):
    _fields_ = [("kind", C.c_int32), ("target", C.c_int32), ("n_controls", C.c_int32),
                ("k", C.c_int32), ("controls", C.c_int32 * QGPU_MAX_OP_WIRES),
                ("param", C.c_double), ("mat_offset", C.c_int64), ("none_offset", C.c_int64)]


assert C.sizeof(QgpuOp) == 80, C.sizeof(QgpuOp)

_lib = None

_EXPORTS = {
    "qgpu_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "qgpu_destroy": (C.c_int, [C.c_void_p]),
    "qgpu_num_qubits": (C.c_int, [C.c_void_p]),
    "qgpu_set_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "qgpu_set_fusion": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qgpu_last_error": (C.c_char_p, []),
    "qgpu_set_zero": (C.c_int, [C.c_void_p]),
    "qgpu_upload": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "qgpu_download": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "qgpu_apply_program": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                                     C.c_void_p, C.c_size_t]),
    "qgpu_measure": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                               C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_uint64)]),
    "qgpu_measure_uniforms": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "qgpu_measure_uniforms_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "qgpu_extract_nonzero": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_size_t,
                                       C.POINTER(C.c_size_t)]),
    "qgpu_norm": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "qgpu_synchronize": (C.c_int, [C.c_void_p]),
    "qgpu_checksum": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "qgpu_compare": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                               C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "qgpu_expectation_zzx": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "qgpu_adjoint_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                                    C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_double), C.c_void_p]),
    "qgpu_selftest_bounded_wait": (C.c_int, [C.c_void_p, C.c_uint32]),
    "qgpu_stream": (C.c_void_p, [C.c_void_p]),
    "qgpu_launch_count": (C.c_uint64, [C.c_void_p]),
    "qgpu_io_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "qgpu_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "qgpu_profile_json": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t, C.c_int]),
}


def exported_symbols() -> list[str]:
    return list(_EXPORTS)


def load(path: Path | None = None) -> C.CDLL:
    """Load the shared library and declare every prototype (no device needed)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise QuantrError(f"libquantr_gpu is not built ({p} missing): run "
                          "`python -m quantr_gb300.build`")
    lib = C.CDLL(str(p))
    for name, (res, args) in _EXPORTS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def lib() -> C.CDLL:
    return load()


def check(status: int, what: str = "") -> None:
    if status != QGPU_OK:
        msg = (lib().qgpu_last_error() or b"").decode(errors="replace")
        raise QuantrError(f"{what + ': ' if what else ''}{msg} (status {status})")


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data) if a is not None and a.size else C.c_void_p(0)


class Handle:
    """One device state vector (a `qgpu_handle`)."""

    def __init__(self, n_qubits: int, precision: int = QGPU_C128, mode: int | None = None):
        self._h = C.c_void_p()
        check(lib().qgpu_create(int(n_qubits), int(precision), C.byref(self._h)), "qgpu_create")
        self.n = int(n_qubits)
        self.precision = precision
        if mode is None:
            mode = int(os.environ.get("QUANTR_GPU_MODE", QGPU_MODE_FAST))
        self.set_mode(mode)

    @property
    def raw(self) -> C.c_void_p:
        return self._h

    def set_mode(self, mode: int) -> None:
        check(lib().qgpu_set_mode(self._h, int(mode)), "qgpu_set_mode")
        self.mode = mode

    def set_fusion(self, block_qubits: int, max_gates: int = 12) -> None:
        """Dense-block fusion (0 = register-tile passes)."""
        check(lib().qgpu_set_fusion(self._h, int(block_qubits), int(max_gates)), "qgpu_set_fusion")

    def close(self) -> None:
        if self._h:
            lib().qgpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_zero(self) -> None:
        check(lib().qgpu_set_zero(self._h), "qgpu_set_zero")

    def upload(self, amps: np.ndarray) -> None:
        a = np.ascontiguousarray(amps, dtype=np.complex128)
        check(lib().qgpu_upload(self._h, ptr(a), a.size), "qgpu_upload")

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(1 << self.n, dtype=np.complex128)
        check(lib().qgpu_download(self._h, ptr(out), out.size), "qgpu_download")
        return out

    def apply(self, ops: np.ndarray, mats: np.ndarray, none: np.ndarray) -> None:
        check(lib().qgpu_apply_program(self._h, ptr(ops), len(ops), ptr(mats), mats.size,
                                       ptr(none), none.size), "qgpu_apply_program")

    def measure(self, shots: int, seed: int, cap: int | None = None):
        cap = int(min(shots, 1 << self.n) if cap is None else cap)
        idx = np.empty(max(cap, 1), dtype=np.uint64)
        cnt = np.empty(max(cap, 1), dtype=np.uint64)
        nu = C.c_size_t()
        nf = C.c_uint64()
        check(lib().qgpu_measure(self._h, int(shots), int(seed) & (2**64 - 1), ptr(idx), ptr(cnt),
                                 cap, C.byref(nu), C.byref(nf)), "qgpu_measure")
        return idx[:nu.value].copy(), cnt[:nu.value].copy(), int(nf.value)

    def measure_uniforms(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty(u.size, dtype=np.int64)
        check(lib().qgpu_measure_uniforms(self._h, ptr(u), u.size, ptr(out)),
              "qgpu_measure_uniforms")
        return out

    def extract_nonzero(self, margin: float = 1e-6, cap: int | None = None):
        """(indices, amplitudes) of |a|^2 not within `margin` of 0, ascending index order."""
        cnt = C.c_size_t()
        if cap is None:  # count first, then fetch exactly that many
            st = lib().qgpu_extract_nonzero(self._h, float(margin), None, None, 0, C.byref(cnt))
            if st not in (QGPU_OK, QGPU_ERR_INVALID):
                check(st, "qgpu_extract_nonzero")
            cap = cnt.value
        idx = np.empty(max(cap, 1), dtype=np.uint64)
        amp = np.empty(max(cap, 1), dtype=np.complex128)
        check(lib().qgpu_extract_nonzero(self._h, float(margin), ptr(idx), ptr(amp), cap,
                                         C.byref(cnt)), "qgpu_extract_nonzero")
        return idx[:cnt.value].copy(), amp[:cnt.value].copy()

    def synchronize(self) -> None:
        """Wait for every queued pass (apply returns once its passes are queued)."""
        check(lib().qgpu_synchronize(self._h), "qgpu_synchronize")

    def norm(self) -> float:
        v = C.c_double()
        check(lib().qgpu_norm(self._h, C.byref(v)), "qgpu_norm")
        return v.value

    def checksum(self) -> complex:
        re, im = C.c_double(), C.c_double()
        check(lib().qgpu_checksum(self._h, C.byref(re), C.byref(im)), "qgpu_checksum")
        return complex(re.value, im.value)

    def compare(self, other: "Handle") -> tuple[float, complex]:
        """(max_i |a_i - b_i|, sum_i conj(a_i) b_i) against another register, on the device."""
        mx, re, im = C.c_double(), C.c_double(), C.c_double()
        check(lib().qgpu_compare(self._h, other._h, C.byref(mx), C.byref(re), C.byref(im)),
              "qgpu_compare")
        return mx.value, complex(re.value, im.value)

    # ---- differentiation --------------------------------------------------------------------
    def expectation_zzx(self, a: np.ndarray, b: np.ndarray) -> float:
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        e = C.c_double()
        check(lib().qgpu_expectation_zzx(self._h, ptr(a), ptr(b), C.byref(e)),
              "qgpu_expectation_zzx")
        return e.value

    def adjoint_grad(self, ops, mats, none, a: np.ndarray, b: np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        g = np.zeros(len(ops), dtype=np.float64)
        e = C.c_double()
        check(lib().qgpu_adjoint_grad(self._h, ptr(ops), len(ops), ptr(mats), mats.size, ptr(none),
                                      none.size, ptr(a), ptr(b), C.byref(e), ptr(g)),
              "qgpu_adjoint_grad")
        return e.value, g

    # ---- introspection --------------------------------------------------------------------
    def stream(self) -> int:
        return int(lib().qgpu_stream(self._h) or 0)

    def launch_count(self) -> int:
        return int(lib().qgpu_launch_count(self._h))

    def io_bytes(self) -> tuple[int, int]:
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().qgpu_io_bytes(self._h, C.byref(a), C.byref(b)), "qgpu_io_bytes")
        return int(a.value), int(b.value)

    def set_profiling(self, on: bool) -> None:
        check(lib().qgpu_set_profiling(self._h, 1 if on else 0), "qgpu_set_profiling")

    def profile(self, reset: bool = False) -> dict:
        import json

        buf = C.create_string_buffer(1 << 16)
        check(lib().qgpu_profile_json(self._h, buf, len(buf), 1 if reset else 0),
              "qgpu_profile_json")
        return json.loads(buf.value.decode())
