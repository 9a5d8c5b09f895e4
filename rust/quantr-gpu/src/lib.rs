//! Rust binding of libquantr_gpu, the GB300 state-vector engine behind quantr's
//! `Circuit::simulate` / `SimulatedCircuit::measure_all`. `ffi` declares the C ABI of
//! include/qgpu.h; `Register` and `Program` wrap it safely. rust/quantr-backend/gpu.rs shows
//! the quantr side: lowering its gate list into a `Program` and running it on a `Register`.

pub mod ffi;
pub mod program;
pub mod register;

pub use program::Program;
pub use register::{GpuError, Mode, Precision, Register};
