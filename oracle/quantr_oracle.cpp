/*
 * quantr_oracle.cpp — CPU restatement of quantr 0.6.0's simulation path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity oracle and the timed CPU baseline. Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and only as the
 * checker. The product library (libquantr_gpu) never links, loads or calls it.
 *
 * What it restates (file:line inside the quantr crate):
 *  - `Circuit::apply_gate` (src/circuit/simulation.rs:64-135): every basis state of the
 *    register is turned into a ProductState, the gate's basis-image function is applied to the
 *    acting qubits, and the image is scattered into a HashMap keyed by ProductState with
 *    "first product, then +=" accumulation (simulation.rs:158-180). Custom gates returning
 *    `None` keep their amplitude and overwrite whatever was accumulated (simulation.rs:120-133).
 *    `set_amplitudes_from_states_unchecked` (super_positions_unchecked.rs:50-60) rebuilds the
 *    dense vector, absent keys becoming 0.
 *  - acting positions: Double [c, t], Triple [c1, c2, t], Custom [controls..., t]
 *    (simulation.rs:81-112); image labels are written back by `insert_qubits`
 *    (product_states.rs:112-123); label <-> index by `binary_basis` (product_states.rs:205-215,
 *    wire 0 = most significant bit).
 *  - gate images: src/circuit/standard_gate_ops.rs:37-267, entry by entry, with the same
 *    expressions (cos(0.5*angle), sin(0.5*angle), exp(i x) = (cos x, sin x) as num-complex's
 *    `from_polar(1, x)`, CRk angle (2*pi)/2^k).
 *  - complex arithmetic: num-complex 0.4.x (`Cargo.toml:16`, num-complex = "0.4.6") `Mul` is
 *    (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re) with self = gate image, other = register
 *    amplitude (simulation.rs:176-178); `norm_sqr` is re*re + im*im. Rust never contracts a*b+c
 *    into an FMA, so this file is compiled with -ffp-contract=off.
 *  - `SuperPosition::measure` (super_positions.rs:332-342): first index i with
 *    u < sum_{j<=i} |a_j|^2 (sequential f64 sum), else None. The uniform u comes from the
 *    caller: quantr draws it with `fastrand::f64()` (fastrand = "2.1.0", Cargo.toml:15), whose
 *    stream is not reproduced here.
 *
 * Engines with identical arithmetic:
 *  - oracle_simulate_hashmap: the literal HashMap-of-labels algorithm (std::unordered_map
 *    keyed by a byte vector, one heap-allocated label per basis state and image entry). It is
 *    the restated reference timed as the CPU baseline.
 *  - oracle_simulate_dense: the same per-key accumulation order on flat arrays (no hashing),
 *    used for larger parity cases. Tests check that both engines agree value for value.
 *  - a threaded form of the dense engine (independent groups of outputs on all host cores,
 *    each output's products in the same order) for the 20-22 qubit parity cases; tests check
 *    it against the dense engine value for value.
 *
 * Parity pinning: the restatement is checked against every amplitude golden of the crate's own
 * tests (src/circuit.rs:603-982, tests/qft.rs:30-39, tests/grovers.rs:124-133) and its layout
 * tests; the crate itself cannot be compiled here (no Rust toolchain).
 */
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../include/qgpu.h"

namespace {

struct Cx {
    double re, im;
};

// num-complex `Mul`: self * other.
inline Cx cmul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cx cadd(Cx a, Cx b) { return Cx{a.re + b.re, a.im + b.im}; }
// num-complex `exp` of (0, x): from_polar(exp(0) = 1, x) = (1*cos x, 1*sin x).
inline Cx expi(double x) { return Cx{1.0 * std::cos(x), 1.0 * std::sin(x)}; }

const double FRAC_1_SQRT_2 = 0.70710678118654752440;  // std::f64::consts::FRAC_1_SQRT_2
const double PI = 3.14159265358979323846;             // std::f64::consts::PI
const Cx ZERO{0.0, 0.0};
inline Cx re(double x) { return Cx{x, 0.0}; }
inline Cx im(double x) { return Cx{0.0, x}; }

thread_local std::string g_err;

// Number of wires the op acts on (local register size k).
int op_wires(const qgpu_op& op) {
    switch (op.kind) {
        case QGPU_GATE_CR: case QGPU_GATE_CRK: case QGPU_GATE_CZ: case QGPU_GATE_CY:
        case QGPU_GATE_CNOT: case QGPU_GATE_SWAP:
            return 2;
        case QGPU_GATE_TOFFOLI:
            return 3;
        case QGPU_GATE_CUSTOM:
            return op.n_controls + 1;
        default:
            return 1;
    }
}

// Acting positions, local bit order (first = most significant), simulation.rs:81-112.
void acting_positions(const qgpu_op& op, int* pos) {
    int k = op_wires(op);
    for (int m = 0; m < k - 1; ++m) pos[m] = op.controls[m];
    pos[k - 1] = op.target;
}

// Basis image of local input basis state j (bits MSB-first over the acting positions) ->
// 2^k amplitudes in `img`. Returns false for a Custom `None`. standard_gate_ops.rs:37-267.
bool gate_image(const qgpu_op& op, unsigned j, const double* mats, const uint8_t* none_flags,
                Cx* img) {
    const double half = 0.5 * op.param;  // `0.5f64.mul(angle)`
    switch (op.kind) {
        case QGPU_GATE_H:  // standard_gate_ops.rs:37-42
            img[0] = re(FRAC_1_SQRT_2);
            img[1] = j ? re(-FRAC_1_SQRT_2) : re(FRAC_1_SQRT_2);
            return true;
        case QGPU_GATE_RX: {  // :45-55
            Cx c = re(std::cos(half)), s = im(-std::sin(half));
            if (j == 0) { img[0] = c; img[1] = s; } else { img[0] = s; img[1] = c; }
            return true;
        }
        case QGPU_GATE_RY: {  // :58-69
            Cx c = re(std::cos(half)), sp = re(std::sin(half)), sn = re(-std::sin(half));
            if (j == 0) { img[0] = c; img[1] = sp; } else { img[0] = sn; img[1] = c; }
            return true;
        }
        case QGPU_GATE_RZ: {  // :72-82, `-angle*0.5` = (-angle)*0.5
            Cx ne = expi((-op.param) * 0.5), pe = expi(op.param * 0.5);
            if (j == 0) { img[0] = ne; img[1] = ZERO; } else { img[0] = ZERO; img[1] = pe; }
            return true;
        }
        case QGPU_GATE_PHASE: {  // global_phase :85-94
            Cx e = expi(op.param * 0.5);
            if (j == 0) { img[0] = e; img[1] = ZERO; } else { img[0] = ZERO; img[1] = e; }
            return true;
        }
        case QGPU_GATE_X90:  // :97-102
            if (j == 0) { img[0] = ZERO; img[1] = im(-1.0); } else { img[0] = im(-1.0); img[1] = ZERO; }
            return true;
        case QGPU_GATE_Y90:  // :105-110
            if (j == 0) { img[0] = ZERO; img[1] = re(-1.0); } else { img[0] = re(1.0); img[1] = ZERO; }
            return true;
        case QGPU_GATE_MX90:  // :113-118
            if (j == 0) { img[0] = ZERO; img[1] = im(1.0); } else { img[0] = im(1.0); img[1] = ZERO; }
            return true;
        case QGPU_GATE_MY90:  // :121-126
            if (j == 0) { img[0] = ZERO; img[1] = re(1.0); } else { img[0] = re(-1.0); img[1] = ZERO; }
            return true;
        case QGPU_GATE_T:  // :129-134
            if (j == 0) { img[0] = re(1.0); img[1] = ZERO; } else { img[0] = ZERO; img[1] = Cx{FRAC_1_SQRT_2, FRAC_1_SQRT_2}; }
            return true;
        case QGPU_GATE_TDAG:  // :137-142
            if (j == 0) { img[0] = re(1.0); img[1] = ZERO; } else { img[0] = ZERO; img[1] = Cx{FRAC_1_SQRT_2, -FRAC_1_SQRT_2}; }
            return true;
        case QGPU_GATE_S:  // phase :145-150
            if (j == 0) { img[0] = re(1.0); img[1] = ZERO; } else { img[0] = ZERO; img[1] = im(1.0); }
            return true;
        case QGPU_GATE_SDAG:  // phasedag :153-158
            if (j == 0) { img[0] = re(1.0); img[1] = ZERO; } else { img[0] = ZERO; img[1] = im(-1.0); }
            return true;
        case QGPU_GATE_X:  // :161-166
            if (j == 0) { img[0] = ZERO; img[1] = re(1.0); } else { img[0] = re(1.0); img[1] = ZERO; }
            return true;
        case QGPU_GATE_Y:  // :169-174
            if (j == 0) { img[0] = ZERO; img[1] = im(1.0); } else { img[0] = im(-1.0); img[1] = ZERO; }
            return true;
        case QGPU_GATE_Z:  // :177-182
            if (j == 0) { img[0] = re(1.0); img[1] = ZERO; } else { img[0] = ZERO; img[1] = re(-1.0); }
            return true;
        case QGPU_GATE_CNOT: {  // :189-196
            static const double t[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 0, 1}, {0, 0, 1, 0}};
            for (int l = 0; l < 4; ++l) img[l] = re(t[j][l]);
            return true;
        }
        case QGPU_GATE_CY: {  // :199-206
            static const double t[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 0, 1}, {0, 0, -1, 0}};
            for (int l = 0; l < 4; ++l) img[l] = (j < 2) ? re(t[j][l]) : im(t[j][l]);
            return true;
        }
        case QGPU_GATE_CZ: {  // :209-216
            static const double t[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, -1}};
            for (int l = 0; l < 4; ++l) img[l] = re(t[j][l]);
            return true;
        }
        case QGPU_GATE_SWAP: {  // :219-226
            static const double t[4][4] = {{1, 0, 0, 0}, {0, 0, 1, 0}, {0, 1, 0, 0}, {0, 0, 0, 1}};
            for (int l = 0; l < 4; ++l) img[l] = re(t[j][l]);
            return true;
        }
        case QGPU_GATE_CR:  // :229-237
        case QGPU_GATE_CRK: {  // :240-249, (2*pi).div(2.powi(k))
            if (j < 3) {
                for (int l = 0; l < 4; ++l) img[l] = re(l == (int)j ? 1.0 : 0.0);
            } else {
                double ang = (op.kind == QGPU_GATE_CR) ? op.param
                                                       : (2.0 * PI) / std::pow(2.0, (double)op.k);
                img[0] = ZERO; img[1] = ZERO; img[2] = ZERO; img[3] = expi(ang);
            }
            return true;
        }
        case QGPU_GATE_TOFFOLI: {  // :256-267
            unsigned out = (j == 6) ? 7u : (j == 7) ? 6u : j;
            for (int l = 0; l < 8; ++l) img[l] = re((unsigned)l == out ? 1.0 : 0.0);
            return true;
        }
        case QGPU_GATE_CUSTOM: {  // user fn, tabulated by the host
            int k = op.n_controls + 1;
            size_t dim = (size_t)1 << k;
            if (none_flags[op.none_offset + j]) return false;
            const double* col = mats + op.mat_offset + 2 * (size_t)j * dim;
            for (size_t l = 0; l < dim; ++l) img[l] = Cx{col[2 * l], col[2 * l + 1]};
            return true;
        }
        default:
            return false;
    }
}

int validate(int n, const qgpu_op* ops, size_t n_ops, size_t n_mat_doubles, size_t n_none) {
    if (n < 1 || n > 30) { g_err = "oracle supports 1..30 qubits"; return QGPU_ERR_INVALID; }
    for (size_t g = 0; g < n_ops; ++g) {
        const qgpu_op& op = ops[g];
        if (op.kind <= QGPU_GATE_ID || op.kind >= QGPU_GATE_COUNT) continue;
        int k = op_wires(op);
        if (k > QGPU_MAX_OP_WIRES || k > n) { g_err = "too many wires"; return QGPU_ERR_INVALID; }
        int pos[QGPU_MAX_OP_WIRES];
        acting_positions(op, pos);
        for (int m = 0; m < k; ++m) {
            if (pos[m] < 0 || pos[m] >= n) { g_err = "wire out of range"; return QGPU_ERR_INVALID; }
            for (int m2 = 0; m2 < m; ++m2)
                if (pos[m] == pos[m2]) { g_err = "overlapping wires"; return QGPU_ERR_INVALID; }
        }
        if (op.kind == QGPU_GATE_CUSTOM) {
            size_t dim = (size_t)1 << k;
            if (op.mat_offset < 0 || (size_t)op.mat_offset + 2 * dim * dim > n_mat_doubles ||
                op.none_offset < 0 || (size_t)op.none_offset + dim > n_none) {
                g_err = "custom table out of range";
                return QGPU_ERR_INVALID;
            }
        }
    }
    return QGPU_OK;
}

// ---------------------------------------------------------------------------------------
// Engine 1: the HashMap algorithm, literally.
// ---------------------------------------------------------------------------------------
using Label = std::vector<uint8_t>;  // a ProductState: one byte per qubit, wire order

struct LabelHash {
    size_t operator()(const Label& v) const noexcept {
        // FNV-1a over the bytes: any deterministic hash gives the same values; only the
        // per-key accumulation order matters and that follows the loop order below.
        uint64_t h = 1469598103934665603ull;
        for (uint8_t b : v) { h ^= b; h *= 1099511628211ull; }
        return (size_t)h;
    }
};

Label binary_basis(uint64_t index, int n) {  // product_states.rs:205-215
    Label q(n);
    for (int w = 0; w < n; ++w) q[w] = (uint8_t)((index >> (n - 1 - w)) & 1u);
    return q;
}

void apply_gate_hashmap(int n, const qgpu_op& op, const double* mats, const uint8_t* none_flags,
                        std::vector<Cx>& reg) {
    std::unordered_map<Label, Cx, LabelHash> mapped, untouched;
    const int k = op_wires(op);
    int pos[QGPU_MAX_OP_WIRES];
    acting_positions(op, pos);
    std::vector<Cx> img((size_t)1 << k);
    const uint64_t dim = (uint64_t)1 << n;
    for (uint64_t i = 0; i < dim; ++i) {  // `for (prod_state, amp) in register.into_iter()`
        Label prod = binary_basis(i, n);
        Cx amp = reg[i];
        unsigned j = 0;
        for (int m = 0; m < k; ++m) j = (j << 1) | prod[pos[m]];
        if (gate_image(op, j, mats, none_flags, img.data())) {
            for (size_t l = 0; l < img.size(); ++l) {  // insert_gate_image_into_product_state
                Label swapped = prod;
                for (int m = 0; m < k; ++m) swapped[pos[m]] = (uint8_t)((l >> (k - 1 - m)) & 1u);
                Cx p = cmul(img[l], amp);
                auto it = mapped.find(swapped);
                if (it != mapped.end()) it->second = cadd(it->second, p);
                else mapped.emplace(std::move(swapped), p);
            }
        } else {
            untouched[prod] = amp;
        }
    }
    for (auto& kv : untouched) mapped[kv.first] = kv.second;  // overwrite rule
    for (uint64_t i = 0; i < dim; ++i) {  // set_amplitudes_from_states_unchecked
        auto it = mapped.find(binary_basis(i, n));
        if (it != mapped.end()) { reg[i] = it->second; mapped.erase(it); }
        else reg[i] = ZERO;
    }
}

// ---------------------------------------------------------------------------------------
// Engine 2: same accumulation order, flat arrays.
// ---------------------------------------------------------------------------------------
void apply_gate_dense(int n, const qgpu_op& op, const double* mats, const uint8_t* none_flags,
                      std::vector<Cx>& reg, std::vector<Cx>& out, std::vector<uint8_t>& state) {
    const int k = op_wires(op);
    int pos[QGPU_MAX_OP_WIRES];
    acting_positions(op, pos);
    uint64_t bitmask[QGPU_MAX_OP_WIRES];
    uint64_t acting = 0;
    for (int m = 0; m < k; ++m) { bitmask[m] = 1ull << (n - 1 - pos[m]); acting |= bitmask[m]; }
    const size_t kd = (size_t)1 << k;
    std::vector<Cx> img(kd);
    std::vector<uint64_t> scatter(kd);
    for (size_t l = 0; l < kd; ++l) {
        uint64_t off = 0;
        for (int m = 0; m < k; ++m)
            if ((l >> (k - 1 - m)) & 1u) off |= bitmask[m];
        scatter[l] = off;
    }
    const uint64_t dim = (uint64_t)1 << n;
    // state: 0 = absent, 1 = mapped, 2 = untouched (overwrites mapped)
    std::fill(state.begin(), state.end(), 0);
    for (uint64_t i = 0; i < dim; ++i) {
        unsigned j = 0;
        for (int m = 0; m < k; ++m) j = (j << 1) | ((i & bitmask[m]) ? 1u : 0u);
        if (gate_image(op, j, mats, none_flags, img.data())) {
            uint64_t base = i & ~acting;
            for (size_t l = 0; l < kd; ++l) {
                uint64_t t = base | scatter[l];
                Cx p = cmul(img[l], reg[i]);
                if (state[t] == 1) out[t] = cadd(out[t], p);
                else if (state[t] == 0) { out[t] = p; state[t] = 1; }
                // state 2: an untouched entry wins whatever arrives later
            }
        } else {
            out[i] = reg[i];
            state[i] = 2;
        }
    }
    for (uint64_t i = 0; i < dim; ++i) reg[i] = state[i] ? out[i] : ZERO;
}

// ---------------------------------------------------------------------------------------
// Engine 3: engine 2 on all host cores, value for value. An output t receives products only
// from inputs that differ from t in the acting bits (its "group"), and engine 2 visits inputs
// in increasing full index, so processing each group on its own, its members in increasing
// full index, keeps every output's sequence of products and its None overwrite unchanged.
// Groups are independent and are split across threads.
// ---------------------------------------------------------------------------------------
void apply_gate_dense_parallel(int n, const qgpu_op& op, const double* mats,
                               const uint8_t* none_flags, std::vector<Cx>& reg, int threads) {
    const int k = op_wires(op);
    int pos[QGPU_MAX_OP_WIRES];
    acting_positions(op, pos);
    uint64_t bitmask[QGPU_MAX_OP_WIRES];
    uint64_t acting = 0;
    for (int m = 0; m < k; ++m) { bitmask[m] = 1ull << (n - 1 - pos[m]); acting |= bitmask[m]; }
    const size_t kd = (size_t)1 << k;
    std::vector<uint64_t> scatter(kd);  // local index -> offset of its acting bits
    for (size_t l = 0; l < kd; ++l) {
        uint64_t off = 0;
        for (int m = 0; m < k; ++m)
            if ((l >> (k - 1 - m)) & 1u) off |= bitmask[m];
        scatter[l] = off;
    }
    // members of a group in increasing full index: local indices sorted by their offsets
    std::vector<unsigned> visit(kd);
    for (size_t l = 0; l < kd; ++l) visit[l] = (unsigned)l;
    std::sort(visit.begin(), visit.end(),
              [&](unsigned a, unsigned b) { return scatter[a] < scatter[b]; });
    const uint64_t dim = (uint64_t)1 << n;
    const uint64_t free_mask = (dim - 1) & ~acting;
    const uint64_t groups = dim >> k;
    auto work = [&](uint64_t g0, uint64_t g1) {
        std::vector<Cx> img(kd), in(kd), out(kd);
        std::vector<uint8_t> state(kd);
        // base of group g0: deposit the bits of g0 into the free positions, low to high
        uint64_t base = 0;
        {
            uint64_t rest = g0;
            for (int b = 0; b < n && rest; ++b)
                if ((free_mask >> b) & 1u) { if (rest & 1u) base |= 1ull << b; rest >>= 1; }
        }
        for (uint64_t g = g0; g < g1; ++g) {
            for (size_t l = 0; l < kd; ++l) in[l] = reg[base | scatter[l]];
            std::fill(state.begin(), state.end(), 0);
            for (size_t v = 0; v < kd; ++v) {
                const unsigned j = visit[v];  // input base|scatter[j], local index j
                if (gate_image(op, j, mats, none_flags, img.data())) {
                    for (size_t l = 0; l < kd; ++l) {
                        Cx p = cmul(img[l], in[j]);
                        if (state[l] == 1) out[l] = cadd(out[l], p);
                        else if (state[l] == 0) { out[l] = p; state[l] = 1; }
                    }
                } else {
                    out[j] = in[j];
                    state[j] = 2;
                }
            }
            for (size_t l = 0; l < kd; ++l) reg[base | scatter[l]] = state[l] ? out[l] : ZERO;
            base = ((base | ~free_mask) + 1) & free_mask;  // next subset of the free bits
        }
    };
    if (threads <= 1 || groups < 256) {
        work(0, groups);
        return;
    }
    std::vector<std::thread> pool;
    const uint64_t per = (groups + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const uint64_t g0 = t * per, g1 = std::min<uint64_t>(groups, g0 + per);
        if (g0 >= g1) break;
        pool.emplace_back(work, g0, g1);
    }
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

/* Simulates ops on `state` (interleaved re/im, 2^n amplitudes) in place. engine 0 = HashMap,
 * 1 = dense, 2 = dense on all host cores (ORACLE_THREADS overrides the count). Returns QGPU_OK
 * or QGPU_ERR_INVALID. */
int oracle_simulate(int engine, int n, const qgpu_op* ops, size_t n_ops, const double* mats,
                    size_t n_mat_doubles, const uint8_t* none_flags, size_t n_none, double* state) {
    int st = validate(n, ops, n_ops, n_mat_doubles, n_none);
    if (st != QGPU_OK) return st;
    const uint64_t dim = (uint64_t)1 << n;
    std::vector<Cx> reg(dim);
    std::memcpy(reg.data(), state, dim * sizeof(Cx));
    std::vector<Cx> out;
    std::vector<uint8_t> flags;
    if (engine == 1) { out.resize(dim); flags.resize(dim); }
    int threads = 1;
    if (engine == 2) {
        threads = (int)std::thread::hardware_concurrency();
        if (const char* e = std::getenv("ORACLE_THREADS")) threads = std::atoi(e);
        if (threads < 1) threads = 1;
    }
    for (size_t g = 0; g < n_ops; ++g) {
        const qgpu_op& op = ops[g];
        if (op.kind <= QGPU_GATE_ID || op.kind >= QGPU_GATE_COUNT) continue;  // Identity skipped
        if (engine == 0) apply_gate_hashmap(n, op, mats, none_flags, reg);
        else if (engine == 1) apply_gate_dense(n, op, mats, none_flags, reg, out, flags);
        else apply_gate_dense_parallel(n, op, mats, none_flags, reg, threads);
    }
    std::memcpy(state, reg.data(), dim * sizeof(Cx));
    return QGPU_OK;
}

/* Basis image of one gate for local input j (for host-side table checks). Writes 2^k complex
 * values to img (interleaved). Returns 1 for an image, 0 for None, -1 for a bad op. */
int oracle_gate_image(const qgpu_op* op, unsigned j, const double* mats, const uint8_t* none_flags,
                      double* img) {
    if (op->kind <= QGPU_GATE_ID || op->kind >= QGPU_GATE_COUNT) return -1;
    return gate_image(*op, j, mats, none_flags, reinterpret_cast<Cx*>(img)) ? 1 : 0;
}

/* SuperPosition::measure for each uniform u[s]: first i with u < cumulative |a_i|^2, else -1. */
void oracle_measure_uniforms(int n, const double* state, size_t n_u, const double* u,
                             int64_t* out) {
    const uint64_t dim = (uint64_t)1 << n;
    // One pass builds the same sequential cumulative sums `measure` forms per shot.
    std::vector<double> cum(dim);
    double c = 0.0;
    for (uint64_t i = 0; i < dim; ++i) {
        double p = state[2 * i] * state[2 * i] + state[2 * i + 1] * state[2 * i + 1];
        c += p;
        cum[i] = c;
    }
    for (size_t s = 0; s < n_u; ++s) {
        // `dice_roll < cummalitive` at the first i: the cumulative sums are non-decreasing, so
        // this is the first i with cum[i] > u.
        uint64_t lo = 0, hi = dim;
        while (lo < hi) {
            uint64_t mid = (lo + hi) / 2;
            if (u[s] < cum[mid]) hi = mid; else lo = mid + 1;
        }
        out[s] = (lo < dim) ? (int64_t)lo : -1;
    }
}

/* The literal per-shot linear scan of `measure` (super_positions.rs:332-342), for pinning
 * oracle_measure_uniforms on small states. */
int64_t oracle_measure_linear(int n, const double* state, double u) {
    const uint64_t dim = (uint64_t)1 << n;
    double c = 0.0;
    for (uint64_t i = 0; i < dim; ++i) {
        c += state[2 * i] * state[2 * i] + state[2 * i + 1] * state[2 * i + 1];
        if (u < c) return (int64_t)i;
    }
    return -1;
}

}  // extern "C"
