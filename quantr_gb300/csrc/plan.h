// plan.h — host-side gate tabulation and pass planning shared by the kernels' launchers.
#pragma once

#include <stdint.h>

#include <array>
#include <complex>
#include <string>
#include <vector>

#include "../../include/qgpu.h"

namespace qgpu {

using cd = std::complex<double>;

// ---------------------------------------------------------------------------------------------
// One gate as the reference applies it: a local register of k wires [controls..., target]
// (first = most significant local bit) and the 2^k images of its basis states.
// ---------------------------------------------------------------------------------------------
struct LocalGate {
    int k = 1;
    int wires[QGPU_MAX_OP_WIRES];  // acting positions, local bit order (MSB first)
    std::vector<cd> M;             // column-major: M[j * 2^k + l] = image of input j at output l
    std::vector<uint8_t> none;     // none[j] = 1 when the Custom function returned None for j
};

// Number of wires an op acts on; validates wires against n. Returns QGPU_OK or an error code
// with the message set.
int op_arity(const qgpu_op& op, int n, int* k_out);
// Tabulates an op with the reference's gate formulas (standard_gate_ops.rs:37-267) or the
// host-evaluated Custom table.
int tabulate(const qgpu_op& op, int n, const double* mats, size_t n_mats, const uint8_t* none,
             size_t n_none, LocalGate* out);

// Rotations (Rx, Ry, Rz, Phase: exp(-i theta P / 2) with P = X, Y, Z, -I), the gates with a
// gradient.
bool is_rotation(int kind);
// The inverse of a non-Custom op as another op (U^dagger), quantr's conventions.
qgpu_op inverse_op(const qgpu_op& op);

// A run of single-wire gates on one wire undone by the adjoint sweep in one pass. A rotation
// G = exp(-i theta P / 2) followed on its wire by V (the run's later gates) has gradient
// Im <lambda| V P V^dag |phi>, taken before the run is undone; V P V^dag = q0 I + qx X + qy Y + qz Z
// (real q: the product is Hermitian), so the gradient is a real combination of the sums
// Im <lambda| s |phi> over s = X, Y, Z, -I.
struct PauliRun {
    std::array<cd, 4> undo;  // row-major 2x2: G_1^dag ... G_k^dag (G_k^dag applied first)
    // per rotation: its op index and the coefficients of the sums (1 X, 2 Y, 3 Z, 4 -I)
    std::vector<std::pair<size_t, std::array<double, 5>>> rots;
    bool need[5] = {false, false, false, false, false};  // sums with a non-zero coefficient
};
// gw: the run's op indices into ops, in reverse order (gw[0] the run's last gate).
int pauli_run(const qgpu_op* ops, const std::vector<size_t>& gw, int n, PauliRun* out);

// The passes of a grouped adjoint sweep (the runs of single-wire gates of many wires per pass):
// wire bits in ascending order, each pass a tile of at most `max_bits` index bits that always
// holds bits 0..4 (32 consecutive amplitudes per load) and is filled up with the lowest other
// bits. Returns per pass the tile mask and the wires (indices into `bits`) it takes; every wire
// lands in exactly one pass.
constexpr int ADJ_GROUP_TILE_BITS = 11;
std::vector<std::pair<uint64_t, std::vector<size_t>>> adj_group_passes(const std::vector<int>& bits,
                                                                       int n, int max_bits);
// Whether ops (CNot, X, Swap only), applied in order, form an affine index map y -> A y + b over
// GF(2); if so, the gather tables of its inverse h for one out-of-place pass dst[y] = src[h(y)]:
// h(y) = *d xor tabs[c * 256 + byte c of y] over the 8-bit chunks c of y.
bool affine_tables(const qgpu_op* ops, size_t n_ops, int n, std::vector<uint64_t>* tabs,
                   uint64_t* d);

// ---------------------------------------------------------------------------------------------
// Fused passes for the fast kernels (QGPU_MODE_FAST / QGPU_MODE_F64 / complex64).
// ---------------------------------------------------------------------------------------------
enum StepType : uint8_t {
    ST_DENSE = 0,  // 2x2 complex on tile bit lb
    ST_REAL = 1,   // 2x2 real on tile bit lb
    ST_PERM = 2,   // monomial 2x2 with entries in {1, i, -1, -i} on tile bit lb (anti = swap)
    ST_SWAP = 3,   // exchange tile bits lb and lb2
    ST_PHASE = 4,  // v *= d where (index & cm) == cm (any bits; unit d uses no arithmetic)
    ST_DIAG = 5,   // v *= (index bit fb) ? d1 : d0, under (index & cm) == cm
    ST_TABLE = 6,  // v *= prod_f T_f[(index >> shift_f) & (2^width_f - 1)], under cm
    ST_DENSE4 = 7,  // 4x4 complex on two bits (a fused pair block; always a pass of its own)
};

constexpr int MAX_TILE_BITS = 3;
constexpr int MAX_STEPS = 24;
constexpr int MAX_TABLE_FIELDS = 3;
constexpr int MAX_TABLE_BITS = 14;  // widest table field the planner may form

// Step as seen by the device: FF constants (re_h, re_l, im_h, im_l per complex), f64 and f32
// copies, so one table serves every arithmetic policy.
struct DevStep {
    uint8_t type, lb, lb2, fb;
    uint8_t anti, u0, u1, unit;        // PERM: out0 = i^u0 * v[anti], out1 = i^u1 * v[!anti]
    uint64_t cm;                       // control mask on the full index
    uint32_t tab_off[MAX_TABLE_FIELDS];  // TABLE: entry offsets into the pass table buffer
    uint8_t tab_shift[MAX_TABLE_FIELDS], tab_width[MAX_TABLE_FIELDS];
    uint8_t nfields, pad[3];
    float ff[16];                      // up to 4 complex entries as float pairs
    double d[8];                       // the same entries in f64
    // Packed f32x2 operands of the float-pair kernels: term t of a Dot2 uses
    // pk[4t..4t+3] = (U_hi, U_lo, -U_hi, -U_lo), each lane pair (for the real, imag output).
    // DENSE: outputs 0 and 1, terms 0..3 each (slots 0..15, 16..31); REAL: terms 0..1 per
    // output; PHASE: one complex constant (slots 0..7); DIAG: two (slots 0..7, 8..15).
    uint64_t pk[32];
};

// A run of commuting controlled-X gates (X, CNot, Toffoli) and swaps whose targets are neither
// controls nor each other's targets (a swap's two bits belong to no other gate of the run): the
// run is the involution i -> i ^ f(i), with f built from terms. A grouped term (grouped = 1)
// covers single-bit controls that sit `shift` bits above their targets: f |= ((i & cm) >> shift);
// a plain term (0) is one gate: f |= tbit when (i & cm) == cm; a swap term (2) has cm = its two
// bits: f |= cm when exactly one of them is set.
constexpr int MAX_XOR_TERMS = 24;
struct XorPerm {
    int nterms = 0;
    uint64_t cm[MAX_XOR_TERMS];
    uint64_t tbit[MAX_XOR_TERMS];   // plain term: target bit mask
    int shift[MAX_XOR_TERMS];       // grouped term: control = target + shift (shift > 0)
    int grouped[MAX_XOR_TERMS];
};

// One term of an XOR run: a controlled X (flip = its target bit, applied where (i & cm) == cm)
// or a swap (swap = true, cm = flip = its two bits, applied where exactly one of them is set).
struct XTerm {
    uint64_t cm = 0, flip = 0;
    bool swap = false;
};
constexpr int MAX_PASS_BITS = 4;       // widest pass: two pair blocks on four bits
constexpr int MAX_TILE_XTERMS = 8;     // XOR terms a double pair pass applies before / after

struct Pass {
    int nbits = 0;                     // tile bits
    int bits[MAX_PASS_BITS];           // full-index bit positions, ascending
    bool xor_pass = false;             // the pass is one XorPerm (k_xor_perm)
    XorPerm xp;
    bool arith = false;                // needs float-pair / f64 arithmetic
    int cost = 0;                      // planner's ops-per-amplitude estimate
    double touched = 1.0;              // fraction of amplitudes the pass may change
    std::vector<DevStep> steps;
    int custom = -1;                   // >= 0: this pass is a Custom gate (group kernel)
    int pair = -1;                     // >= 0: this pass is pair block `pair` (k_pair kernel)
    // >= 0: a double pair pass (k_pair2): blocks `pair` and `pair2` on disjoint bit pairs of the
    // four tile bits, with the XOR terms `pre` applied before them and `post` after them (every
    // term's bits lie in the tile, so each thread permutes only its own 16 amplitudes)
    int pair2 = -1;
    std::vector<XTerm> pre, post;
};

// A 4x4 block over full-index bits hi > lo, local index l = 2 * bit(hi) + bit(lo).
// pk: packed Dot2 terms of the float-pair kernel, output r / input c at pk[32r + 8c ..+7]
// (terms (Re, Re) on x_c and (-Im, Im) on swap(x_c), 4 slots each as in DevStep::pk).
struct PairBlock {
    int hi = 0, lo = 0;
    cd m[4][4];                        // m[out][in]
    uint64_t pk[128];
};

struct Plan {
    std::vector<Pass> passes;
    std::vector<PairBlock> pairs;      // fused pair blocks
    std::vector<LocalGate> customs;    // Custom gates, run by the group kernel
    std::vector<float> table_ff;       // TABLE entries as float pairs (4 floats each)
    std::vector<double> table_f64;     // TABLE entries as f64 (2 doubles each)
};

enum ArithPolicy { POL_FF = 0, POL_F64 = 1, POL_F32 = 2 };

struct PlanOptions {
    int policy = POL_FF;               // arithmetic the passes will run in (sets step costs)
    int max_bits = MAX_TILE_BITS;      // tile width (register tile of 2^bits amplitudes)
    int max_arith_bits = MAX_TILE_BITS;  // tile width of passes that carry arithmetic
    int budget = 100;                  // arithmetic ops per amplitude a pass may carry
    bool merge_1q = true;              // multiply runs of single-wire gates into one matrix
    bool fuse_diagonal = true;         // fold diagonal runs into phase tables
    bool xor_runs = true;              // runs of >= 3 commuting controlled-X gates -> one pass
    bool pair_fusion = false;          // fuse gates on two wires into 4x4 blocks where cheaper
    int table_bits = 10;               // width of a phase-table field (<= MAX_TABLE_BITS)
    bool group_pairs = true;           // with pair_fusion: two pair blocks per pass, XOR terms folded in
};

// Elementary terms of an XOR pass, and the pass rebuilt from a subset of them (false when the
// terms need more than MAX_XOR_TERMS entries).
std::vector<XTerm> xor_terms(const XorPerm& xp);
bool xor_from_terms(const std::vector<XTerm>& ts, XorPerm* xp);

int build_plan(const qgpu_op* ops, size_t n_ops, int n, const double* mats, size_t n_mats,
               const uint8_t* none, size_t n_none, const PlanOptions& opt, Plan* plan);

// An unconditional ST_DENSE step for out0 = u00 a + u01 b, out1 = u10 a + u11 b (all constant
// forms filled in).
DevStep dense_step(cd u00, cd u01, cd u10, cd u11);

// ---------------------------------------------------------------------------------------------
// Dense-block fusion: consecutive gates whose wires fit in `block_qubits` wires (at most
// `max_gates` of them) are multiplied on the host into one 2^k x 2^k complex matrix.
// ---------------------------------------------------------------------------------------------
struct DenseBlock {
    int k = 0;
    int bits[QGPU_MAX_OP_WIRES];       // full-index bit of local bit m (local bit 0 = bits[0])
    std::vector<cd> M;                 // row-major: M[l * 2^k + j] = <l| U |j>
    int gates = 0;
};

int build_blocks(const qgpu_op* ops, size_t n_ops, int n, const double* mats, size_t n_mats,
                 const uint8_t* none, size_t n_none, int block_qubits, int max_gates,
                 std::vector<DenseBlock>* out);

}  // namespace qgpu
