//! A gate program: quantr's flat gate list lowered to `qgpu_op` records (what
//! `simulate_with_register` walks, src/circuit/simulation.rs:37-56), with the tabulated blocks of
//! Custom gates.

use crate::ffi::{self, QgpuOp};

/// The ops, the Custom blocks (column-major 2^k x 2^k, interleaved re/im) and their None flags.
#[derive(Clone, Debug, Default)]
pub struct Program {
    pub ops: Vec<QgpuOp>,
    pub mats: Vec<f64>,
    pub none: Vec<u8>,
}

impl Program {
    pub fn new() -> Self {
        Self::default()
    }

    /// A standard gate of kind `kind` (ffi::QGPU_GATE_*) on wire `target`, its control wires in
    /// the variant's field order, `param` its angle (Rx/Ry/Rz/Phase/CR), `k` CRk's integer.
    pub fn gate(&mut self, kind: i32, target: usize, controls: &[usize], param: f64, k: i32) -> &mut Self {
        assert!(controls.len() < ffi::QGPU_MAX_OP_WIRES, "too many control wires");
        let mut op = QgpuOp { kind, target: target as i32, n_controls: controls.len() as i32, k, param, ..Default::default() };
        for (slot, &c) in op.controls.iter_mut().zip(controls) {
            *slot = c as i32;
        }
        self.ops.push(op);
        self
    }

    /// A Custom gate on [controls..., target] (first wire most significant): `block` holds image j
    /// of the 2^k local basis states as column j (column-major, (re, im) pairs, 2^k x 2^k complex
    /// entries) and `none[j]` marks the inputs whose function returned `None`.
    pub fn custom(&mut self, target: usize, controls: &[usize], block: &[f64], none: &[u8]) -> &mut Self {
        let k = controls.len() + 1;
        assert!(k <= ffi::QGPU_MAX_OP_WIRES, "a Custom gate acts on at most 10 wires");
        let d = 1usize << k;
        assert_eq!(block.len(), 2 * d * d, "block must hold 2^k x 2^k complex entries");
        assert_eq!(none.len(), d, "one None flag per local basis state");
        let mut op = QgpuOp {
            kind: ffi::QGPU_GATE_CUSTOM,
            target: target as i32,
            n_controls: controls.len() as i32,
            mat_offset: self.mats.len() as i64,
            none_offset: self.none.len() as i64,
            ..Default::default()
        };
        for (slot, &c) in op.controls.iter_mut().zip(controls) {
            *slot = c as i32;
        }
        self.mats.extend_from_slice(block);
        self.none.extend_from_slice(none);
        self.ops.push(op);
        self
    }
}
