/*
 * qgpu.h — C ABI of libquantr_gpu, the GB300 (sm_103a) state-vector engine behind
 * quantr's `Circuit::simulate` / `SimulatedCircuit::{get_state, measure_all}`.
 *
 * quantr (Rust crate 0.6.0) has no FFI of its own: the path it replaces is the crate-private
 * call chain `Circuit::simulate` (src/circuit.rs:364-388) -> `simulate_with_register`
 * (src/circuit/simulation.rs:21-57) -> `apply_gate` (src/circuit/simulation.rs:64-135), then
 * `SimulatedCircuit::measure_all` (src/simulated_circuit.rs:63-73) -> `SuperPosition::measure`
 * (src/circuit/states/super_positions.rs:332-342). Each entry point below names the reference
 * item it stands in for. A host binding (Rust `extern "C"` block, C++ `quantr.hpp`, Python
 * ctypes) lowers quantr's flat gate list into `qgpu_op` records and calls these functions.
 *
 * Conventions
 *  - Every function returns an `int` status: QGPU_OK (0) or a negative QGPU_ERR_* code.
 *    `qgpu_last_error()` returns a thread-local message for the last failure on this thread.
 *  - Amplitudes cross the boundary as interleaved (re, im) doubles, index i = sum over wires w
 *    of bit_w << (n-1-w): wire 0 is the most significant bit, as in quantr's
 *    `ProductState::binary_basis` (src/circuit/states/product_states.rs:205-215).
 *  - A handle owns one device state vector and one CUDA stream. Handles are not thread-safe;
 *    different handles may be driven from different threads. All calls are stream-ordered and
 *    synchronise before returning host-visible results.
 *  - No call falls back to a CPU implementation: a missing or failing device is an error.
 */
#ifndef QGPU_H
#define QGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define QGPU_OK               0
#define QGPU_ERR_INVALID     -1  /* bad argument: wire out of range, overlapping wires, size */
#define QGPU_ERR_OOM         -2  /* device allocation failed (e.g. 35 qubits of complex128)  */
#define QGPU_ERR_CUDA        -3  /* a CUDA runtime call or kernel launch failed               */
#define QGPU_ERR_TIMEOUT     -4  /* a bounded device-side wait ran out                        */
#define QGPU_ERR_UNSUPPORTED -5  /* valid request this build does not serve                  */
#define QGPU_ERR_NONUNITARY  -6  /* adjoint gradient asked for a circuit with Custom gates   */

/* ---- precision of the device state ----------------------------------------------------- */
#define QGPU_C128 0   /* complex128: quantr's `Complex64` amplitudes (num-complex f64 pairs) */
#define QGPU_C64  1   /* complex64: float pairs; reductions (norm, probabilities) stay in f64 */

/* ---- arithmetic mode for complex128 ------------------------------------------------------
 * QGPU_MODE_EXACT  one pass per gate, f64 products and sums without contraction, in the
 *                  reference's accumulation order (simulation.rs:168-179): amplitudes equal
 *                  the reference's value for value.
 * QGPU_MODE_FAST   gate fusion and GB300 kernels; f64 arithmetic carried on the FP32/INT
 *                  pipes as unevaluated float pairs (GB300 issues f64 at ~1/64 of the FP32
 *                  rate). Results stay within 1e-12 max-abs of the reference.
 * QGPU_MODE_F64    same fusion as FAST but native f64 FMA arithmetic (for comparison).       */
#define QGPU_MODE_FAST  0
#define QGPU_MODE_EXACT 1
#define QGPU_MODE_F64   2

/* ---- gate kinds: one per `quantr::Gate` variant (src/circuit/gate.rs:19-106) ---------- */
enum qgpu_gate_kind {
    QGPU_GATE_ID = 0,
    QGPU_GATE_H, QGPU_GATE_X, QGPU_GATE_Y, QGPU_GATE_Z,
    QGPU_GATE_S, QGPU_GATE_SDAG, QGPU_GATE_T, QGPU_GATE_TDAG,
    QGPU_GATE_RX, QGPU_GATE_RY, QGPU_GATE_RZ,
    QGPU_GATE_X90, QGPU_GATE_Y90, QGPU_GATE_MX90, QGPU_GATE_MY90,
    QGPU_GATE_PHASE,
    QGPU_GATE_CR, QGPU_GATE_CRK, QGPU_GATE_CZ, QGPU_GATE_CY, QGPU_GATE_CNOT, QGPU_GATE_SWAP,
    QGPU_GATE_TOFFOLI,
    QGPU_GATE_CUSTOM,
    QGPU_GATE_COUNT
};

/* Largest number of wires one Custom gate may act on (controls + target). The host tabulates
 * a Custom gate into a dense 2^k x 2^k block, so k = 10 is a 16 MiB matrix. */
#define QGPU_MAX_OP_WIRES 10

/* One non-identity gate of quantr's flat column list, in simulation order. `target` is the
 * gate's wire (`gate_pos = counter % num_qubits`, simulation.rs:43). `controls` hold the wires
 * of the variant's usize fields in declaration order: CNot/CY/CZ/Swap/CR/CRk -> [c],
 * Toffoli(c1, c2) -> [c1, c2], Custom(_, controls, _) -> controls. The gate then acts on the
 * local register [controls..., target], first entry most significant (simulation.rs:96-112).
 *
 * Custom gates (simulation.rs:102-105, 137-156): the host evaluates the user function on
 * each of the 2^k local basis states j and stores the image as column j of a column-major
 * 2^k x 2^k complex matrix at mats[mat_offset ...] (interleaved re, im: entry (l, j) at
 * mats[mat_offset + 2*(j*2^k + l)]), and none_flags[none_offset + j] = 1 where the function
 * returned `None`. Non-unitary blocks are allowed. */
typedef struct qgpu_op {
    int32_t kind;                          /* enum qgpu_gate_kind                        */
    int32_t target;                        /* wire of the gate                           */
    int32_t n_controls;                    /* used entries of controls[]                 */
    int32_t k;                             /* CRk's integer k                            */
    int32_t controls[QGPU_MAX_OP_WIRES];   /* control wires in variant order             */
    double  param;                         /* angle of Rx/Ry/Rz/Phase/CR                  */
    int64_t mat_offset;                    /* Custom: offset (in doubles) into mats       */
    int64_t none_offset;                   /* Custom: offset (in bytes) into none_flags   */
} qgpu_op;

typedef struct qgpu_handle qgpu_handle;

/* ---- lifetime --------------------------------------------------------------------------- */

/* Allocates a 2^n_qubits state on the current CUDA device, set to |0...0>.
 * Replaces `SuperPosition::new_unchecked` (src/circuit/states/super_positions_unchecked.rs:39-46).
 * precision: QGPU_C128 or QGPU_C64. Fails with QGPU_ERR_OOM when the state does not fit. */
int qgpu_create(int n_qubits, int precision, qgpu_handle** out);
int qgpu_destroy(qgpu_handle* h);
int qgpu_num_qubits(const qgpu_handle* h);
int qgpu_set_mode(qgpu_handle* h, int mode);             /* QGPU_MODE_*                  */
/* Dense-block fusion (no counterpart in quantr): when block_qubits is 1..6, qgpu_apply_program
 * multiplies runs of at most max_gates consecutive gates acting on at most block_qubits wires
 * into one 2^k x 2^k complex matrix on the host and applies each with one pass. 0 (default)
 * restores the register-tile passes. QGPU_MODE_EXACT ignores it. */
int qgpu_set_fusion(qgpu_handle* h, int block_qubits, int max_gates);
const char* qgpu_last_error(void);                        /* thread-local, never NULL     */

/* ---- register in / out ------------------------------------------------------------------ */

/* |0...0>: the default register of `Circuit::simulate` (circuit.rs:376-378). */
int qgpu_set_zero(qgpu_handle* h);
/* `Circuit::change_register` (circuit.rs:463-473): len must equal 2^n amplitudes. */
int qgpu_upload(qgpu_handle* h, const double* interleaved, size_t n_amplitudes);
/* `SimulatedCircuit::get_state` / `take_state` (src/simulated_circuit.rs:158-160, 185-187). */
int qgpu_download(qgpu_handle* h, double* interleaved_out, size_t n_amplitudes);

/* ---- simulation ------------------------------------------------------------------------- */

/* Applies ops[0..n_ops) in order: the loop of `simulate_with_register` (simulation.rs:37-56)
 * with one `apply_gate` (simulation.rs:64-135) per op. Identity ops are skipped. In the fused
 * modes the passes are queued on the handle's stream and the call returns once they are queued
 * (the host can plan the next circuit meanwhile); every later call on the handle is ordered
 * after them, and the ones that read results back (download, measure, norm, ...) wait for
 * them. A device fault in a queued pass is reported by the next call that synchronises. */
int qgpu_apply_program(qgpu_handle* h, const qgpu_op* ops, size_t n_ops,
                       const double* mats, size_t n_mat_doubles,
                       const uint8_t* none_flags, size_t n_none_flags);

/* Waits until every operation queued on the handle's stream has finished; returns the status of
 * that work (a device fault in a queued pass surfaces here). No counterpart in quantr. */
int qgpu_synchronize(qgpu_handle* h);

/* ---- measurement ------------------------------------------------------------------------ */

/* `SimulatedCircuit::measure_all(shots)` (simulated_circuit.rs:63-73): `shots` draws of
 * `SuperPosition::measure` (super_positions.rs:332-342) from a seeded counter-based generator.
 * Each shot returns the first index i with u < sum_{j<=i} |a_j|^2, or fails (`None`) when u is
 * at least the total. The histogram comes back sorted by index: idx_out[0..*n_unique) and
 * cnt_out[0..*n_unique); `cap` is the capacity of both arrays. *n_failed counts `None` shots. */
int qgpu_measure(qgpu_handle* h, uint64_t shots, uint64_t seed,
                 uint64_t* idx_out, uint64_t* cnt_out, size_t cap,
                 size_t* n_unique, uint64_t* n_failed);

/* The same sampling rule for caller-supplied uniforms u[0..n) in [0, 1): out[i] is the index
 * drawn for u[i], or -1 for `None`. Used to check the sampler shot by shot. */
int qgpu_measure_uniforms(qgpu_handle* h, const double* u, size_t n, int64_t* out);

/* No counterpart in quantr. qgpu_measure_uniforms for callers that cannot let the library
 * allocate device memory (all of the GPU's memory owned by a host framework's pool, or a loop
 * that must not enter the CUDA allocator): same arguments and results, but its scratch lives
 * in a fixed array inside the library's device image (about 1.5 MiB, held by every GPU that
 * loads the library until exit) and it calls no cudaMalloc/cudaFree. Limits: registers of at
 * most 24 qubits and at most 65536 uniforms per call; larger requests fail with
 * QGPU_ERR_INVALID. The first call on each device, and the first after that device's CUDA
 * context was re-created (cudaDeviceReset), looks up the array's device address, so make that
 * call before any stream capture. All calls share the one array: calls that overlap on
 * the GPU (other handles' streams on the same device) race. */
int qgpu_measure_uniforms_noalloc(qgpu_handle* h, const double* u, size_t n, int64_t* out);

/* `SuperPosition::to_hash_map` (src/circuit/states/super_positions.rs:315-323) without a full
 * download: the indices and amplitudes (interleaved re, im) of every amplitude whose |a|^2 is
 * not within `margin` of 0 (quantr uses 1e-6), in increasing index order. *count receives the
 * number of survivors; when it exceeds `cap`, the first `cap` are written and QGPU_ERR_INVALID is
 * returned. */
int qgpu_extract_nonzero(qgpu_handle* h, double margin, uint64_t* idx_out, double* amp_out,
                         size_t cap, size_t* count);

/* f64 reductions of the state: sum |a_i|^2, and the amplitude checksum sum a_i. */
int qgpu_norm(qgpu_handle* h, double* out);
int qgpu_checksum(qgpu_handle* h, double* re_out, double* im_out);

/* No counterpart in quantr (a parity check between two registers of the same size, e.g. one
 * simulated in QGPU_MODE_FAST and one in QGPU_MODE_EXACT, without downloading either):
 * *max_abs_diff = max_i |a_i - b_i| and (*inner_re, *inner_im) = sum_i conj(a_i) b_i, in f64 on
 * the device (deterministic order). The precisions may differ. Waits for b's queued passes. */
int qgpu_compare(qgpu_handle* a, qgpu_handle* b, double* max_abs_diff, double* inner_re,
                 double* inner_im);

/* ---- differentiation (no counterpart in quantr) ------------------------------------------
 * Observable H = sum_i a[i] Z_i Z_{(i+1) mod n} + sum_i b[i] X_i over the n wires (periodic),
 * a and b of length n. complex128 handles compute in f64 / float pairs; complex64 handles in f32
 * (the sums over the register in f64), gradients within about 1e-5 of the complex128 ones. */

/* <psi|H|psi> of the current register. */
int qgpu_expectation_zzx(qgpu_handle* h, const double* a, const double* b, double* energy);

/* Runs ops on the current register (leaving |psi_L> in it, like qgpu_apply_program), returns
 * E = <psi_L|H|psi_L> and dE/dtheta for every op by the adjoint method: grads[g] is the
 * derivative with respect to the angle of op g when it is Rx, Ry, Rz or Phase, else 0.
 * Circuits with Custom gates are rejected with QGPU_ERR_NONUNITARY (their maps need not be
 * invertible). Uses two state-sized work vectors, and a third one when the circuit has runs of
 * at least three CNot / X / Swap gates (each run is undone as one out-of-place index gather). */
int qgpu_adjoint_grad(qgpu_handle* h, const qgpu_op* ops, size_t n_ops,
                      const double* mats, size_t n_mat_doubles,
                      const uint8_t* none_flags, size_t n_none_flags,
                      const double* a, const double* b, double* energy, double* grads);

/* ---- batching (no counterpart in quantr) --------------------------------------------------
 * Many independent circuits, each started from |0...0>, each with its own ZZ+X observable:
 * energies[i] and d energy / d angle for every op (grads[grad_offset + g]). Circuits small
 * enough for shared memory (complex128 <= 12 qubits, complex64 <= 13) run in one persistent
 * launch replayed from a CUDA graph; larger ones run through the register-tile passes with a
 * per-size fusion budget and adjoint sweep form picked by timing (written to
 * tuned_budget[n_qubits] when not NULL, an int[41]: the budget, plus 65536 when the sweep takes
 * the single-wire gates of up to 11 wires per pass rather than one pass per wire; complex64
 * sweeps always do), in the batch's precision.
 * Custom gates are rejected (QGPU_ERR_NONUNITARY). */
typedef struct qgpu_batch_item {
    int32_t n_qubits;
    int32_t n_ops;
    int64_t op_offset;    /* first op in ops[]                                  */
    int64_t obs_offset;   /* a[n_qubits] then b[n_qubits] start at obs[...]     */
    int64_t grad_offset;  /* n_ops gradient slots start at grads[...]           */
} qgpu_batch_item;

int qgpu_batch_run(const qgpu_batch_item* items, size_t n_items, const qgpu_op* ops,
                   size_t n_ops_total, const double* obs, size_t n_obs, int precision,
                   double* energies, double* grads, int* tuned_budget);

/* ---- engine introspection (no counterpart in quantr) ------------------------------------ */

/* The handle's CUDA stream (a cudaStream_t), for callers that time or order work on it. */
void* qgpu_stream(qgpu_handle* h);
/* Failure-detection check: one CTA polls, at most `polls` times (1..2^20), an mbarrier phase
 * that nothing completes, the same bounded wait the pipelined passes use. Returns
 * QGPU_ERR_TIMEOUT with the device error word recorded and cleared; the context stays usable. */
int qgpu_selftest_bounded_wait(qgpu_handle* h, uint32_t polls);

/* Number of kernels this handle has launched since creation. */
uint64_t qgpu_launch_count(const qgpu_handle* h);
/* Bytes this handle has moved host->device (copies and kernel parameters) and device->host. */
int qgpu_io_bytes(const qgpu_handle* h, uint64_t* h2d, uint64_t* d2h);
/* When on, every pass of qgpu_apply_program is bracketed by CUDA events on the handle's stream
 * and its duration and algorithmic bytes (2 * sizeof(amplitude) * amplitudes the pass may
 * change) are accumulated per kernel. */
int qgpu_set_profiling(qgpu_handle* h, int on);
/* Writes the accumulated profile as JSON {"kernel": [launches, total_ms, bytes], ...} into buf
 * (NUL-terminated, truncated to cap) and, when reset != 0, clears it. */
int qgpu_profile_json(qgpu_handle* h, char* buf, size_t cap, int reset);

#ifdef __cplusplus
}
#endif
#endif /* QGPU_H */
