//! The C ABI of libquantr_gpu, declaration for declaration as include/qgpu.h states it. Every
//! function returns QGPU_OK (0) or a negative QGPU_ERR_* status, with a thread-local message from
//! `qgpu_last_error`. Amplitudes cross as interleaved (re, im) f64 pairs, index i = sum over wires
//! w of bit_w << (n - 1 - w) (wire 0 most significant, quantr's `ProductState::binary_basis`).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const QGPU_OK: c_int = 0;
pub const QGPU_ERR_INVALID: c_int = -1;
pub const QGPU_ERR_OOM: c_int = -2;
pub const QGPU_ERR_CUDA: c_int = -3;
pub const QGPU_ERR_TIMEOUT: c_int = -4;
pub const QGPU_ERR_UNSUPPORTED: c_int = -5;
pub const QGPU_ERR_NONUNITARY: c_int = -6;

pub const QGPU_C128: c_int = 0;
pub const QGPU_C64: c_int = 1;

pub const QGPU_MODE_FAST: c_int = 0;
pub const QGPU_MODE_EXACT: c_int = 1;
pub const QGPU_MODE_F64: c_int = 2;

/// `enum qgpu_gate_kind`: one value per `quantr::Gate` variant, in declaration order.
pub const QGPU_GATE_ID: i32 = 0;
pub const QGPU_GATE_H: i32 = 1;
pub const QGPU_GATE_X: i32 = 2;
pub const QGPU_GATE_Y: i32 = 3;
pub const QGPU_GATE_Z: i32 = 4;
pub const QGPU_GATE_S: i32 = 5;
pub const QGPU_GATE_SDAG: i32 = 6;
pub const QGPU_GATE_T: i32 = 7;
pub const QGPU_GATE_TDAG: i32 = 8;
pub const QGPU_GATE_RX: i32 = 9;
pub const QGPU_GATE_RY: i32 = 10;
pub const QGPU_GATE_RZ: i32 = 11;
pub const QGPU_GATE_X90: i32 = 12;
pub const QGPU_GATE_Y90: i32 = 13;
pub const QGPU_GATE_MX90: i32 = 14;
pub const QGPU_GATE_MY90: i32 = 15;
pub const QGPU_GATE_PHASE: i32 = 16;
pub const QGPU_GATE_CR: i32 = 17;
pub const QGPU_GATE_CRK: i32 = 18;
pub const QGPU_GATE_CZ: i32 = 19;
pub const QGPU_GATE_CY: i32 = 20;
pub const QGPU_GATE_CNOT: i32 = 21;
pub const QGPU_GATE_SWAP: i32 = 22;
pub const QGPU_GATE_TOFFOLI: i32 = 23;
pub const QGPU_GATE_CUSTOM: i32 = 24;
pub const QGPU_GATE_COUNT: i32 = 25;

pub const QGPU_MAX_OP_WIRES: usize = 10;

/// `qgpu_op`: one non-identity gate of quantr's flat column list, in simulation order (80 bytes).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct QgpuOp {
    pub kind: i32,
    pub target: i32,
    pub n_controls: i32,
    pub k: i32,
    pub controls: [i32; QGPU_MAX_OP_WIRES],
    pub param: f64,
    pub mat_offset: i64,
    pub none_offset: i64,
}

/// `qgpu_batch_item`: one circuit of a `qgpu_batch_run` call.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct QgpuBatchItem {
    pub n_qubits: i32,
    pub n_ops: i32,
    pub op_offset: i64,
    pub obs_offset: i64,
    pub grad_offset: i64,
}

/// Opaque `qgpu_handle`: one device register and its CUDA stream.
#[repr(C)]
pub struct QgpuHandle {
    _private: [u8; 0],
}

extern "C" {
    pub fn qgpu_create(n_qubits: c_int, precision: c_int, out: *mut *mut QgpuHandle) -> c_int;
    pub fn qgpu_destroy(h: *mut QgpuHandle) -> c_int;
    pub fn qgpu_num_qubits(h: *const QgpuHandle) -> c_int;
    pub fn qgpu_set_mode(h: *mut QgpuHandle, mode: c_int) -> c_int;
    pub fn qgpu_set_fusion(h: *mut QgpuHandle, block_qubits: c_int, max_gates: c_int) -> c_int;
    pub fn qgpu_last_error() -> *const c_char;

    pub fn qgpu_set_zero(h: *mut QgpuHandle) -> c_int;
    pub fn qgpu_upload(h: *mut QgpuHandle, interleaved: *const f64, n_amplitudes: usize) -> c_int;
    pub fn qgpu_download(h: *mut QgpuHandle, interleaved_out: *mut f64, n_amplitudes: usize) -> c_int;

    pub fn qgpu_apply_program(h: *mut QgpuHandle, ops: *const QgpuOp, n_ops: usize,
                              mats: *const f64, n_mat_doubles: usize, none_flags: *const u8,
                              n_none_flags: usize) -> c_int;
    pub fn qgpu_synchronize(h: *mut QgpuHandle) -> c_int;

    pub fn qgpu_measure(h: *mut QgpuHandle, shots: u64, seed: u64, idx_out: *mut u64,
                        cnt_out: *mut u64, cap: usize, n_unique: *mut usize,
                        n_failed: *mut u64) -> c_int;
    pub fn qgpu_measure_uniforms(h: *mut QgpuHandle, u: *const f64, n: usize, out: *mut i64) -> c_int;
    pub fn qgpu_measure_uniforms_noalloc(h: *mut QgpuHandle, u: *const f64, n: usize,
                                         out: *mut i64) -> c_int;
    pub fn qgpu_extract_nonzero(h: *mut QgpuHandle, margin: f64, idx_out: *mut u64,
                                amp_out: *mut f64, cap: usize, count: *mut usize) -> c_int;

    pub fn qgpu_norm(h: *mut QgpuHandle, out: *mut f64) -> c_int;
    pub fn qgpu_checksum(h: *mut QgpuHandle, re_out: *mut f64, im_out: *mut f64) -> c_int;
    pub fn qgpu_compare(a: *mut QgpuHandle, b: *mut QgpuHandle, max_abs_diff: *mut f64,
                        inner_re: *mut f64, inner_im: *mut f64) -> c_int;

    pub fn qgpu_expectation_zzx(h: *mut QgpuHandle, a: *const f64, b: *const f64,
                                energy: *mut f64) -> c_int;
    pub fn qgpu_adjoint_grad(h: *mut QgpuHandle, ops: *const QgpuOp, n_ops: usize,
                             mats: *const f64, n_mat_doubles: usize, none_flags: *const u8,
                             n_none_flags: usize, a: *const f64, b: *const f64,
                             energy: *mut f64, grads: *mut f64) -> c_int;
    pub fn qgpu_batch_run(items: *const QgpuBatchItem, n_items: usize, ops: *const QgpuOp,
                          n_ops_total: usize, obs: *const f64, n_obs: usize, precision: c_int,
                          energies: *mut f64, grads: *mut f64, tuned_budget: *mut c_int) -> c_int;

    pub fn qgpu_stream(h: *mut QgpuHandle) -> *mut c_void;
    pub fn qgpu_selftest_bounded_wait(h: *mut QgpuHandle, polls: u32) -> c_int;
    pub fn qgpu_launch_count(h: *const QgpuHandle) -> u64;
    pub fn qgpu_io_bytes(h: *const QgpuHandle, h2d: *mut u64, d2h: *mut u64) -> c_int;
    pub fn qgpu_set_profiling(h: *mut QgpuHandle, on: c_int) -> c_int;
    pub fn qgpu_profile_json(h: *mut QgpuHandle, buf: *mut c_char, cap: usize, reset: c_int) -> c_int;
}
