//! A device register (one `qgpu_handle`): create, load, simulate, measure, read back. The handle
//! is freed when the register is dropped. A register may move between threads but is not shared
//! by them at once (the library's handles are not thread-safe).

use std::ffi::CStr;
use std::fmt;

use crate::ffi;
use crate::program::Program;

/// A non-zero status of the library with its message (`qgpu_last_error`).
#[derive(Clone, Debug, PartialEq)]
pub struct GpuError {
    pub status: i32,
    pub message: String,
}

impl fmt::Display for GpuError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "{} (status {})", self.message, self.status)
    }
}

impl std::error::Error for GpuError {}

pub(crate) fn check(status: i32) -> Result<(), GpuError> {
    if status == ffi::QGPU_OK {
        return Ok(());
    }
    let message = unsafe {
        let p = ffi::qgpu_last_error();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    };
    Err(GpuError { status, message })
}

#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Precision {
    Complex128,
    Complex64,
}

#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Mode {
    /// Fused passes, f64 carried as float pairs / fixed-point digits; within 1e-12 of quantr.
    Fast,
    /// One pass per gate with quantr's own arithmetic and order: equal value for value.
    Exact,
    /// Fused passes in native f64.
    F64,
}

pub struct Register {
    h: *mut ffi::QgpuHandle,
    n: usize,
}

unsafe impl Send for Register {}

impl Register {
    /// |0...0> on the current CUDA device.
    pub fn new(n_qubits: usize, precision: Precision) -> Result<Self, GpuError> {
        let mut h: *mut ffi::QgpuHandle = std::ptr::null_mut();
        let p = match precision {
            Precision::Complex128 => ffi::QGPU_C128,
            Precision::Complex64 => ffi::QGPU_C64,
        };
        check(unsafe { ffi::qgpu_create(n_qubits as i32, p, &mut h) })?;
        Ok(Register { h, n: n_qubits })
    }

    pub fn num_qubits(&self) -> usize {
        self.n
    }

    pub fn set_mode(&mut self, mode: Mode) -> Result<(), GpuError> {
        let m = match mode {
            Mode::Fast => ffi::QGPU_MODE_FAST,
            Mode::Exact => ffi::QGPU_MODE_EXACT,
            Mode::F64 => ffi::QGPU_MODE_F64,
        };
        check(unsafe { ffi::qgpu_set_mode(self.h, m) })
    }

    pub fn set_zero(&mut self) -> Result<(), GpuError> {
        check(unsafe { ffi::qgpu_set_zero(self.h) })
    }

    /// `interleaved`: 2^n (re, im) pairs (a `Vec<Complex64>` viewed as f64s).
    pub fn upload(&mut self, interleaved: &[f64]) -> Result<(), GpuError> {
        check(unsafe { ffi::qgpu_upload(self.h, interleaved.as_ptr(), interleaved.len() / 2) })
    }

    pub fn download(&mut self, interleaved: &mut [f64]) -> Result<(), GpuError> {
        check(unsafe { ffi::qgpu_download(self.h, interleaved.as_mut_ptr(), interleaved.len() / 2) })
    }

    pub fn apply(&mut self, program: &Program) -> Result<(), GpuError> {
        check(unsafe {
            ffi::qgpu_apply_program(self.h, program.ops.as_ptr(), program.ops.len(), program.mats.as_ptr(),
                                    program.mats.len(), program.none.as_ptr(), program.none.len())
        })
    }

    /// `shots` draws of `SuperPosition::measure`'s rule: the distinct basis indices observed (in
    /// increasing order) with their counts, and the number of shots that found no state (`None`).
    pub fn measure(&mut self, shots: u64, seed: u64) -> Result<(Vec<(u64, u64)>, u64), GpuError> {
        let cap = std::cmp::min(shots, 1u64 << std::cmp::min(self.n, 40)) as usize;
        let mut idx = vec![0u64; cap.max(1)];
        let mut cnt = vec![0u64; cap.max(1)];
        let (mut n_unique, mut n_failed) = (0usize, 0u64);
        check(unsafe {
            ffi::qgpu_measure(self.h, shots, seed, idx.as_mut_ptr(), cnt.as_mut_ptr(), cap, &mut n_unique,
                              &mut n_failed)
        })?;
        Ok((idx.into_iter().zip(cnt).take(n_unique).collect(), n_failed))
    }

    /// The (index, re, im) of every amplitude whose |a|^2 is not within `margin` of 0.
    pub fn extract_nonzero(&mut self, margin: f64) -> Result<Vec<(u64, f64, f64)>, GpuError> {
        let mut count = 0usize;
        let st = unsafe {
            ffi::qgpu_extract_nonzero(self.h, margin, std::ptr::null_mut(), std::ptr::null_mut(), 0, &mut count)
        };
        if st != ffi::QGPU_OK && st != ffi::QGPU_ERR_INVALID {
            check(st)?;
        }
        let mut idx = vec![0u64; count.max(1)];
        let mut amp = vec![0f64; 2 * count.max(1)];
        check(unsafe {
            ffi::qgpu_extract_nonzero(self.h, margin, idx.as_mut_ptr(), amp.as_mut_ptr(), count, &mut count)
        })?;
        Ok((0..count).map(|i| (idx[i], amp[2 * i], amp[2 * i + 1])).collect())
    }

    pub fn norm(&mut self) -> Result<f64, GpuError> {
        let mut v = 0f64;
        check(unsafe { ffi::qgpu_norm(self.h, &mut v) })?;
        Ok(v)
    }

    /// Runs `program` from the current register and returns <H> and dE/dangle per op for
    /// H = sum a_i Z_i Z_{i+1 mod n} + sum b_i X_i (the adjoint method).
    pub fn energy_and_gradient(&mut self, program: &Program, a: &[f64], b: &[f64]) -> Result<(f64, Vec<f64>), GpuError> {
        assert!(a.len() == self.n && b.len() == self.n, "a and b need one entry per wire");
        let mut e = 0f64;
        let mut g = vec![0f64; program.ops.len()];
        check(unsafe {
            ffi::qgpu_adjoint_grad(self.h, program.ops.as_ptr(), program.ops.len(), program.mats.as_ptr(),
                                   program.mats.len(), program.none.as_ptr(), program.none.len(), a.as_ptr(),
                                   b.as_ptr(), &mut e, g.as_mut_ptr())
        })?;
        Ok((e, g))
    }
}

impl Drop for Register {
    fn drop(&mut self) {
        unsafe {
            ffi::qgpu_destroy(self.h);
        }
    }
}
