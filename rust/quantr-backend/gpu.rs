//! GPU backend of quantr's simulate path. This file is the module a maintainer adds to the quantr
//! crate as `src/circuit/gpu.rs` (with `mod gpu;` in `src/circuit.rs` and `quantr-gpu` as a
//! dependency); it uses quantr's own types, so it only compiles inside that crate.
//!
//! * `Circuit::simulate_with_register_gpu` stands in for the body of `simulate_with_register`
//!   (src/circuit/simulation.rs:21-57): the flat gate list is walked the same way (identity
//!   skipped, `gate_pos = counter % num_qubits`, the same progress log), lowered into `qgpu_op`
//!   records with every `Gate::Custom` tabulated on the host, and run on a device register.
//! * `SimulatedCircuit::measure_all_gpu` stands in for `measure_all`
//!   (src/simulated_circuit.rs:63-73): the shots are drawn on the device with the rule of
//!   `SuperPosition::measure` (src/circuit/states/super_positions.rs:332-342), seeded from
//!   fastrand so that `fastrand::seed` still makes a run repeatable.
//!
//! `simulate` is infallible in quantr, so a device failure panics with the library's message.
//! Status: written against quantr 0.6.0 and the library's C ABI; not compiled here (no Rust
//! toolchain on this repository's hosts).

use std::collections::HashMap;

use num_complex::Complex64;
use quantr_gpu::ffi::*;
use quantr_gpu::{GpuError, Precision, Program, Register};

use super::measurement::Measurement;
use super::Circuit;
use crate::states::{ProductState, Qubit, SuperPosition};
use crate::{Gate, SimulatedCircuit};

fn as_f64(a: &[Complex64]) -> &[f64] {
    // num-complex's Complex<f64> is #[repr(C)] { re, im }
    unsafe { std::slice::from_raw_parts(a.as_ptr() as *const f64, 2 * a.len()) }
}

fn as_f64_mut(a: &mut [Complex64]) -> &mut [f64] {
    unsafe { std::slice::from_raw_parts_mut(a.as_mut_ptr() as *mut f64, 2 * a.len()) }
}

/// The image of each of the 2^k local basis states |j> (first qubit most significant, the order
/// `custom_gate_on_wires` builds, simulation.rs:137-156) as column j of a column-major block,
/// and the inputs for which the function returned `None`.
fn tabulate_custom(f: fn(ProductState) -> Option<SuperPosition>, k: usize) -> (Vec<f64>, Vec<u8>) {
    let d = 1usize << k;
    let mut block = vec![0f64; 2 * d * d];
    let mut none = vec![0u8; d];
    for j in 0..d {
        let qubits: Vec<Qubit> = (0..k)
            .map(|m| if (j >> (k - 1 - m)) & 1 == 1 { Qubit::One } else { Qubit::Zero })
            .collect();
        match f(ProductState::new_unchecked(&qubits)) {
            Some(image) => {
                for (l, amp) in image.amplitudes.iter().enumerate().take(d) {
                    block[2 * (j * d + l)] = amp.re;
                    block[2 * (j * d + l) + 1] = amp.im;
                }
            }
            None => none[j] = 1,
        }
    }
    (block, none)
}

/// quantr's flat gate list as a device program, in simulation order.
pub(crate) fn lower(gates: &[Gate], num_qubits: usize) -> Program {
    let mut p = Program::new();
    for (counter, gate) in gates.iter().enumerate() {
        let pos = counter % num_qubits;
        match gate {
            Gate::Id => {}
            Gate::H => { p.gate(QGPU_GATE_H, pos, &[], 0.0, 0); }
            Gate::X => { p.gate(QGPU_GATE_X, pos, &[], 0.0, 0); }
            Gate::Y => { p.gate(QGPU_GATE_Y, pos, &[], 0.0, 0); }
            Gate::Z => { p.gate(QGPU_GATE_Z, pos, &[], 0.0, 0); }
            Gate::S => { p.gate(QGPU_GATE_S, pos, &[], 0.0, 0); }
            Gate::Sdag => { p.gate(QGPU_GATE_SDAG, pos, &[], 0.0, 0); }
            Gate::T => { p.gate(QGPU_GATE_T, pos, &[], 0.0, 0); }
            Gate::Tdag => { p.gate(QGPU_GATE_TDAG, pos, &[], 0.0, 0); }
            Gate::Rx(t) => { p.gate(QGPU_GATE_RX, pos, &[], *t, 0); }
            Gate::Ry(t) => { p.gate(QGPU_GATE_RY, pos, &[], *t, 0); }
            Gate::Rz(t) => { p.gate(QGPU_GATE_RZ, pos, &[], *t, 0); }
            Gate::X90 => { p.gate(QGPU_GATE_X90, pos, &[], 0.0, 0); }
            Gate::Y90 => { p.gate(QGPU_GATE_Y90, pos, &[], 0.0, 0); }
            Gate::MX90 => { p.gate(QGPU_GATE_MX90, pos, &[], 0.0, 0); }
            Gate::MY90 => { p.gate(QGPU_GATE_MY90, pos, &[], 0.0, 0); }
            Gate::Phase(t) => { p.gate(QGPU_GATE_PHASE, pos, &[], *t, 0); }
            Gate::CR(t, c) => { p.gate(QGPU_GATE_CR, pos, &[*c], *t, 0); }
            Gate::CRk(k, c) => { p.gate(QGPU_GATE_CRK, pos, &[*c], 0.0, *k); }
            Gate::CZ(c) => { p.gate(QGPU_GATE_CZ, pos, &[*c], 0.0, 0); }
            Gate::CY(c) => { p.gate(QGPU_GATE_CY, pos, &[*c], 0.0, 0); }
            Gate::CNot(c) => { p.gate(QGPU_GATE_CNOT, pos, &[*c], 0.0, 0); }
            Gate::Swap(c) => { p.gate(QGPU_GATE_SWAP, pos, &[*c], 0.0, 0); }
            Gate::Toffoli(c1, c2) => { p.gate(QGPU_GATE_TOFFOLI, pos, &[*c1, *c2], 0.0, 0); }
            Gate::Custom(f, controls, _) => {
                let (block, none) = tabulate_custom(*f, controls.len() + 1);
                p.custom(pos, controls, &block, &none);
            }
        }
    }
    p
}

impl Circuit {
    /// The body of `simulate_with_register` on the GPU: `register` in, the simulated register out.
    pub(super) fn simulate_with_register_gpu(&self, register: &mut SuperPosition) {
        if self.config_progress {
            println!("Starting circuit simulation...");
            let number_gates = self.circuit_gates.len();
            for (counter, gate) in self.circuit_gates.iter().enumerate() {
                if *gate != Gate::Id {
                    Self::print_circuit_log(gate, &(counter % self.num_qubits), &counter, &number_gates);
                }
            }
        }
        let program = lower(&self.circuit_gates, self.num_qubits);
        let run = |register: &mut SuperPosition| -> Result<(), GpuError> {
            let mut reg = Register::new(self.num_qubits, Precision::Complex128)?;
            reg.upload(as_f64(&register.amplitudes))?;
            reg.apply(&program)?;
            reg.download(as_f64_mut(&mut register.amplitudes))
        };
        if let Err(e) = run(register) {
            panic!("{}", e.message);
        }
    }
}

impl SimulatedCircuit {
    /// `measure_all` with the shots drawn on the device from the cached register.
    pub fn measure_all_gpu(&self, shots: usize) -> Measurement<HashMap<ProductState, usize>> {
        if self.circuit_gates.iter().any(|x| x.is_custom_gate()) && !self.disable_warnings {
            eprintln!("\x1b[93m[Quantr Warning] Custom gates were detected in the circuit. Measurements will be taken from a cached register in memory, and so if the Custom gate does NOT implement a unitary mapping, the measure_all method will most likely lead to wrong results. To simulate a circuit without cache, see SimulatedCircuit::measure_all_without_cache.\x1b[0m")
        }
        let draw = || -> Result<(Vec<(u64, u64)>, u64), GpuError> {
            let mut reg = Register::new(self.num_qubits, Precision::Complex128)?;
            reg.upload(as_f64(&self.register.amplitudes))?;
            reg.measure(shots as u64, fastrand::u64(..))
        };
        let (bins, failed) = draw().unwrap_or_else(|e| panic!("{}", e.message));
        if !self.disable_warnings {
            for _ in 0..failed {
                eprintln!("\x1b[93m[Quantr Warning] The superposition failed to collapse to a state during repeat measurements. This is likely due to the use of Gate::Custom where the mapping is not unitary.\x1b[0m")
            }
        }
        let mut bin_count: HashMap<ProductState, usize> = HashMap::with_capacity(bins.len());
        for (index, count) in bins {
            bin_count.insert(ProductState::binary_basis(index as usize, self.num_qubits), count as usize);
        }
        Measurement::Observable(bin_count)
    }
}
