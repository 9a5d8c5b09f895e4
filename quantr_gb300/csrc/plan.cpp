// plan.cpp — gate tabulation (the reference's formulas) and the fast-path pass planner.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace qgpu {

int fail(int code, const std::string& msg);  // state.cu

namespace {

const double FRAC_1_SQRT_2 = 0.70710678118654752440;  // std::f64::consts::FRAC_1_SQRT_2
const double PI = 3.14159265358979323846;             // std::f64::consts::PI

// exp(i x) as num-complex computes it: from_polar(exp(0) = 1, x) = (1*cos x, 1*sin x).
cd expi(double x) { return cd(1.0 * std::cos(x), 1.0 * std::sin(x)); }

// 2x2 column images of the single-wire gates, standard_gate_ops.rs:37-182.
// c0 = image of |0>, c1 = image of |1>.
void one_qubit_images(const qgpu_op& op, cd c0[2], cd c1[2]) {
    const double a = op.param;
    const cd O(0.0, 0.0);
    switch (op.kind) {
        case QGPU_GATE_H:
            c0[0] = cd(FRAC_1_SQRT_2, 0); c0[1] = cd(FRAC_1_SQRT_2, 0);
            c1[0] = cd(FRAC_1_SQRT_2, 0); c1[1] = cd(-FRAC_1_SQRT_2, 0);
            break;
        case QGPU_GATE_RX: {
            const cd c(std::cos(0.5 * a), 0), s(0, -std::sin(0.5 * a));
            c0[0] = c; c0[1] = s; c1[0] = s; c1[1] = c;
            break;
        }
        case QGPU_GATE_RY: {
            const cd c(std::cos(0.5 * a), 0), sp(std::sin(0.5 * a), 0), sn(-std::sin(0.5 * a), 0);
            c0[0] = c; c0[1] = sp; c1[0] = sn; c1[1] = c;
            break;
        }
        case QGPU_GATE_RZ:
            c0[0] = expi((-a) * 0.5); c0[1] = O; c1[0] = O; c1[1] = expi(a * 0.5);
            break;
        case QGPU_GATE_PHASE: {  // global phase exp(i a/2) * I
            const cd e = expi(a * 0.5);
            c0[0] = e; c0[1] = O; c1[0] = O; c1[1] = e;
            break;
        }
        case QGPU_GATE_X90:
            c0[0] = O; c0[1] = cd(0, -1); c1[0] = cd(0, -1); c1[1] = O;
            break;
        case QGPU_GATE_Y90:
            c0[0] = O; c0[1] = cd(-1, 0); c1[0] = cd(1, 0); c1[1] = O;
            break;
        case QGPU_GATE_MX90:
            c0[0] = O; c0[1] = cd(0, 1); c1[0] = cd(0, 1); c1[1] = O;
            break;
        case QGPU_GATE_MY90:
            c0[0] = O; c0[1] = cd(1, 0); c1[0] = cd(-1, 0); c1[1] = O;
            break;
        case QGPU_GATE_T:
            c0[0] = cd(1, 0); c0[1] = O; c1[0] = O; c1[1] = cd(FRAC_1_SQRT_2, FRAC_1_SQRT_2);
            break;
        case QGPU_GATE_TDAG:
            c0[0] = cd(1, 0); c0[1] = O; c1[0] = O; c1[1] = cd(FRAC_1_SQRT_2, -FRAC_1_SQRT_2);
            break;
        case QGPU_GATE_S:
            c0[0] = cd(1, 0); c0[1] = O; c1[0] = O; c1[1] = cd(0, 1);
            break;
        case QGPU_GATE_SDAG:
            c0[0] = cd(1, 0); c0[1] = O; c1[0] = O; c1[1] = cd(0, -1);
            break;
        case QGPU_GATE_X:
            c0[0] = O; c0[1] = cd(1, 0); c1[0] = cd(1, 0); c1[1] = O;
            break;
        case QGPU_GATE_Y:
            c0[0] = O; c0[1] = cd(0, 1); c1[0] = cd(0, -1); c1[1] = O;
            break;
        case QGPU_GATE_Z:
        default:
            c0[0] = cd(1, 0); c0[1] = O; c1[0] = O; c1[1] = cd(-1, 0);
            break;
    }
}

bool is_one_qubit(int kind) { return kind >= QGPU_GATE_H && kind <= QGPU_GATE_PHASE; }

}  // namespace

int op_arity(const qgpu_op& op, int n, int* k_out) {
    int k = 1;
    switch (op.kind) {
        case QGPU_GATE_CR: case QGPU_GATE_CRK: case QGPU_GATE_CZ: case QGPU_GATE_CY:
        case QGPU_GATE_CNOT: case QGPU_GATE_SWAP:
            k = 2;
            break;
        case QGPU_GATE_TOFFOLI:
            k = 3;
            break;
        case QGPU_GATE_CUSTOM:
            if (op.n_controls < 0 || op.n_controls >= QGPU_MAX_OP_WIRES)
                return fail(QGPU_ERR_INVALID, "Custom gate with " + std::to_string(op.n_controls) +
                                                  " controls: at most " +
                                                  std::to_string(QGPU_MAX_OP_WIRES - 1) + " supported");
            k = op.n_controls + 1;
            break;
        default:
            if (!is_one_qubit(op.kind))
                return fail(QGPU_ERR_INVALID, "unknown gate kind " + std::to_string(op.kind));
    }
    if (op.kind != QGPU_GATE_CUSTOM && op.n_controls != k - 1)
        return fail(QGPU_ERR_INVALID, "gate kind " + std::to_string(op.kind) + " takes " +
                                          std::to_string(k - 1) + " control(s), got " +
                                          std::to_string(op.n_controls));
    int wires[QGPU_MAX_OP_WIRES];
    for (int m = 0; m < k - 1; ++m) wires[m] = op.controls[m];
    wires[k - 1] = op.target;
    for (int m = 0; m < k; ++m) {
        // circuit.rs:157-166 / 284-288: positions and control nodes must lie on the register.
        if (wires[m] < 0 || wires[m] >= n)
            return fail(QGPU_ERR_INVALID, "The position, " + std::to_string(wires[m]) +
                                              ", is out of bounds for the circuit with " +
                                              std::to_string(n) + " qubits.");
        for (int m2 = 0; m2 < m; ++m2)
            if (wires[m] == wires[m2])  // circuit.rs:276-283
                return fail(QGPU_ERR_INVALID, "The gate has overlapping control nodes or a control "
                                              "node that equals the gate's position " +
                                                  std::to_string(wires[m]) + ".");
    }
    *k_out = k;
    return QGPU_OK;
}

int tabulate(const qgpu_op& op, int n, const double* mats, size_t n_mats, const uint8_t* none,
             size_t n_none, LocalGate* out) {
    int k = 0;
    int st = op_arity(op, n, &k);
    if (st != QGPU_OK) return st;
    out->k = k;
    for (int m = 0; m < k - 1; ++m) out->wires[m] = op.controls[m];
    out->wires[k - 1] = op.target;
    const size_t d = (size_t)1 << k;
    out->M.assign(d * d, cd(0, 0));
    out->none.assign(d, 0);
    auto M = [&](size_t j, size_t l) -> cd& { return out->M[j * d + l]; };
    if (is_one_qubit(op.kind)) {
        cd c0[2], c1[2];
        one_qubit_images(op, c0, c1);
        M(0, 0) = c0[0]; M(0, 1) = c0[1]; M(1, 0) = c1[0]; M(1, 1) = c1[1];
        return QGPU_OK;
    }
    switch (op.kind) {
        case QGPU_GATE_CNOT:  // standard_gate_ops.rs:189-196
            M(0, 0) = 1; M(1, 1) = 1; M(2, 3) = 1; M(3, 2) = 1;
            return QGPU_OK;
        case QGPU_GATE_CY:  // :199-206
            M(0, 0) = 1; M(1, 1) = 1; M(2, 3) = cd(0, 1); M(3, 2) = cd(0, -1);
            return QGPU_OK;
        case QGPU_GATE_CZ:  // :209-216
            M(0, 0) = 1; M(1, 1) = 1; M(2, 2) = 1; M(3, 3) = -1;
            return QGPU_OK;
        case QGPU_GATE_SWAP:  // :219-226
            M(0, 0) = 1; M(1, 2) = 1; M(2, 1) = 1; M(3, 3) = 1;
            return QGPU_OK;
        case QGPU_GATE_CR:    // :229-237
        case QGPU_GATE_CRK: {  // :240-249, angle (2*pi)/2^k
            M(0, 0) = 1; M(1, 1) = 1; M(2, 2) = 1;
            const double ang = op.kind == QGPU_GATE_CR ? op.param
                                                       : (2.0 * PI) / std::pow(2.0, (double)op.k);
            M(3, 3) = expi(ang);
            return QGPU_OK;
        }
        case QGPU_GATE_TOFFOLI:  // :256-267
            for (size_t j = 0; j < 8; ++j) M(j, j == 6 ? 7 : j == 7 ? 6 : j) = 1;
            return QGPU_OK;
        case QGPU_GATE_CUSTOM: {
            if (!mats || !none || op.mat_offset < 0 || op.none_offset < 0 ||
                (size_t)op.mat_offset + 2 * d * d > n_mats || (size_t)op.none_offset + d > n_none)
                return fail(QGPU_ERR_INVALID, "Custom gate table lies outside mats/none_flags");
            const double* src = mats + op.mat_offset;
            for (size_t j = 0; j < d; ++j) {
                out->none[j] = none[op.none_offset + j] ? 1 : 0;
                for (size_t l = 0; l < d; ++l)
                    M(j, l) = cd(src[2 * (j * d + l)], src[2 * (j * d + l) + 1]);
            }
            return QGPU_OK;
        }
        default:
            return fail(QGPU_ERR_INVALID, "unknown gate kind " + std::to_string(op.kind));
    }
}

// ---------------------------------------------------------------------------------------------
// Planner
// ---------------------------------------------------------------------------------------------
namespace {

// A gate reduced to "controlled 2x2 on one bit" form, a swap of two bits, or a generic block.
struct AGate {
    enum Kind { ONE, SWAP, BLOCK, PAIR } kind;
    int t = 0;          // target bit (full index)
    uint64_t cm = 0;    // control bits that must be 1
    cd u[2][2];         // u[out][in]
    int a = 0, b = 0;   // SWAP bits; PAIR: hi, lo bits
    int block = -1;     // BLOCK: index into plan.customs; PAIR: index into plan.pairs
    uint64_t support = 0;  // all bits the gate reads or writes
};

int unit_code(cd x) {
    if (x == cd(1, 0)) return 0;
    if (x == cd(0, 1)) return 1;
    if (x == cd(-1, 0)) return 2;
    if (x == cd(0, -1)) return 3;
    return -1;
}
bool is_zero(cd x) { return x.real() == 0.0 && x.imag() == 0.0; }

void put_ff(float* dst, cd x) {
    const float rh = (float)x.real();
    const float rl = (float)(x.real() - (double)rh);
    const float ih = (float)x.imag();
    const float il = (float)(x.imag() - (double)ih);
    dst[0] = rh; dst[1] = rl; dst[2] = ih; dst[3] = il;
}

DevStep blank_step(uint8_t type) {
    DevStep s;
    std::memset(&s, 0, sizeof(s));
    s.type = type;
    return s;
}

void set_entry(DevStep& s, int slot, cd x) {
    put_ff(s.ff + 4 * slot, x);
    s.d[2 * slot] = x.real();
    s.d[2 * slot + 1] = x.imag();
}

uint64_t pack2(float lane0, float lane1) {
    uint32_t a, b;
    std::memcpy(&a, &lane0, 4);
    std::memcpy(&b, &lane1, 4);
    return (uint64_t)a | ((uint64_t)b << 32);
}

// One Dot2 term with per-lane coefficients (c0 for the real output lane, c1 for the imaginary).
void set_term(DevStep& s, int term, double c0, double c1) {
    const float h0 = (float)c0, h1 = (float)c1;
    const float l0 = (float)(c0 - (double)h0), l1 = (float)(c1 - (double)h1);
    s.pk[4 * term + 0] = pack2(h0, h1);
    s.pk[4 * term + 1] = pack2(l0, l1);
    s.pk[4 * term + 2] = pack2(-h0, -h1);
    s.pk[4 * term + 3] = pack2(-l0, -l1);
}

// Packed terms of "out = c * x" for complex c: (re, im) = (cr, cr) (x.r, x.i) + (-ci, ci) (x.i, x.r)
void set_scalar_terms(DevStep& s, int first_term, cd c) {
    set_term(s, first_term, c.real(), c.real());
    set_term(s, first_term + 1, -c.imag(), c.imag());
}

// Packed constants of the float-pair kernels for a step whose entries are already set.
void set_packed(DevStep& s, const cd* e) {
    switch (s.type) {
        case ST_DENSE:  // out0 = e0 a + e1 b ; out1 = e2 a + e3 b
            set_scalar_terms(s, 0, e[0]);
            set_scalar_terms(s, 2, e[1]);
            set_scalar_terms(s, 4, e[2]);
            set_scalar_terms(s, 6, e[3]);
            break;
        case ST_REAL:
            set_term(s, 0, e[0].real(), e[0].real());
            set_term(s, 1, e[1].real(), e[1].real());
            set_term(s, 2, e[2].real(), e[2].real());
            set_term(s, 3, e[3].real(), e[3].real());
            break;
        case ST_PHASE:
            set_scalar_terms(s, 0, e[0]);
            break;
        case ST_DIAG:
            set_scalar_terms(s, 0, e[0]);
            set_scalar_terms(s, 2, e[1]);
            break;
        default:
            break;
    }
}

// Host-side step with its full-index bit(s) still unresolved to tile positions.
struct HStep {
    DevStep s;
    int need[2] = {-1, -1};  // full-index bits that must be tile bits
    bool diagonal = false;
    bool unit = false;       // no arithmetic
    // diagonal bookkeeping (PHASE/DIAG) for table fusion
    uint64_t dcm = 0;        // bits that must be 1
    int dfb = -1;            // DIAG: selecting bit
    cd d0 = 1, d1 = 1;       // DIAG entries; PHASE uses d1
};

int popcount64(uint64_t x) { return __builtin_popcountll(x); }

// Fraction of amplitudes a step may change (its algorithmic footprint).
double step_fraction(const HStep& h) {
    const DevStep& s = h.s;
    const double cond = std::ldexp(1.0, -popcount64(s.cm));
    switch (s.type) {
        case ST_SWAP: return 0.5;
        default: return cond;
    }
}

int step_cost(const HStep& h, int policy) {
    const DevStep& s = h.s;
    const int pc = popcount64(s.cm);
    const bool ff = policy == POL_FF;
    switch (s.type) {
        case ST_DENSE: return ff ? 95 : 8;
        case ST_REAL: return ff ? 45 : 4;
        case ST_PERM: return 2;
        case ST_SWAP: return 0;
        case ST_PHASE: return h.unit ? 3 : ((ff ? 45 : 4) >> std::min(pc, 4)) + 2;
        case ST_DIAG: return h.unit ? 4 : (ff ? 48 : 5);
        case ST_TABLE: return ((ff ? 55 : 8) * s.nfields >> std::min(pc, 4)) + 4;
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Pair fusion: gates confined to two wires become one 4x4 block when that costs less arithmetic
// than applying them one by one. Measured in complex multiply-adds per amplitude: a 4x4 costs 4,
// a dense 2x2 costs 2, a diagonal 1 (0.5 when one entry is 1), a permutation with unit phases 0,
// each halved per control bit. A brickwork of dense single-wire layers joined by CNot bricks
// fuses two layers of a wire pair and their CNot into one block (8 -> 4).
// ---------------------------------------------------------------------------------------------
double agate_macs(const AGate& g) {
    const cd u00 = g.u[0][0], u01 = g.u[0][1], u10 = g.u[1][0], u11 = g.u[1][1];
    double c;
    if (is_zero(u01) && is_zero(u10)) {
        const bool one0 = u00 == cd(1, 0), one1 = u11 == cd(1, 0);
        const bool unit = unit_code(u00) >= 0 && unit_code(u11) >= 0;
        c = unit ? 0.0 : ((one0 || one1) ? 0.5 : 1.0);
    } else if (is_zero(u00) && is_zero(u11)) {
        c = (unit_code(u01) >= 0 && unit_code(u10) >= 0) ? 0.0 : 1.0;
    } else {
        c = 2.0;
    }
    return std::ldexp(c, -popcount64(g.cm));
}

// 4x4 of a ONE gate whose support lies in {hi, lo}; local index l = 2 * bit(hi) + bit(lo).
void pair_matrix(const AGate& g, int hi, int lo, cd out[4][4]) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[r][c] = 0.0;
    auto full_of = [&](int l) -> uint64_t {
        return ((l >> 1) & 1 ? 1ull << hi : 0ull) | ((l & 1) ? 1ull << lo : 0ull);
    };
    auto local_of = [&](uint64_t f) -> int {
        return (int)(((f >> hi) & 1ull) << 1 | ((f >> lo) & 1ull));
    };
    for (int in = 0; in < 4; ++in) {
        const uint64_t f = full_of(in);
        if ((f & g.cm) != g.cm) {
            out[in][in] = 1.0;
            continue;
        }
        const int tb = (int)((f >> g.t) & 1ull);
        for (int ob = 0; ob < 2; ++ob) {
            const uint64_t fo = (f & ~(1ull << g.t)) | ((uint64_t)ob << g.t);
            out[local_of(fo)][in] += g.u[ob][tb];
        }
    }
}

void set_term_raw(uint64_t* pk4, double c0, double c1) {
    const float h0 = (float)c0, h1 = (float)c1;
    const float l0 = (float)(c0 - (double)h0), l1 = (float)(c1 - (double)h1);
    pk4[0] = pack2(h0, h1);
    pk4[1] = pack2(l0, l1);
    pk4[2] = pack2(-h0, -h1);
    pk4[3] = pack2(-l0, -l1);
}

std::vector<AGate> fuse_pairs(const std::vector<AGate>& gates, int n, Plan* plan) {
    struct Open {
        uint64_t bits = 0;
        std::vector<int> members;
        bool live = false;
        bool frozen = false;  // a standalone gate holding its wires: takes no further members
    };
    std::vector<Open> open;
    std::vector<int> owner(n, -1);
    std::vector<AGate> out;
    out.reserve(gates.size());
    auto close = [&](int oi) {
        Open& o = open[oi];
        for (int b = 0; b < n; ++b)
            if ((o.bits >> b) & 1ull) owner[b] = -1;
        o.live = false;
        double macs = 0.0;
        for (int gi : o.members) macs += agate_macs(gates[gi]);
        if (o.frozen || popcount64(o.bits) != 2 || macs <= 4.0 + 1e-9) {
            for (int gi : o.members) out.push_back(gates[gi]);
            return;
        }
        PairBlock pb;
        pb.hi = 63 - __builtin_clzll(o.bits);
        pb.lo = __builtin_ctzll(o.bits);
        cd acc[4][4];
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) acc[r][c] = r == c ? 1.0 : 0.0;
        for (int gi : o.members) {  // acc <- G * acc, in circuit order
            cd gm[4][4], nx[4][4];
            pair_matrix(gates[gi], pb.hi, pb.lo, gm);
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) {
                    cd v = 0.0;
                    for (int q = 0; q < 4; ++q) v += gm[r][q] * acc[q][c];
                    nx[r][c] = v;
                }
            std::memcpy(acc, nx, sizeof(acc));
        }
        std::memcpy(pb.m, acc, sizeof(acc));
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                set_term_raw(pb.pk + 32 * r + 8 * c, acc[r][c].real(), acc[r][c].real());
                set_term_raw(pb.pk + 32 * r + 8 * c + 4, -acc[r][c].imag(), acc[r][c].imag());
            }
        AGate a;
        a.kind = AGate::PAIR;
        a.a = pb.hi;
        a.b = pb.lo;
        a.block = (int)plan->pairs.size();
        a.support = o.bits;
        plan->pairs.push_back(pb);
        out.push_back(a);
    };
    for (size_t gi = 0; gi < gates.size(); ++gi) {
        const AGate& g = gates[gi];
        const bool fusable = g.kind == AGate::ONE && popcount64(g.support) <= 2;
        std::vector<int> os;
        for (int b = 0; b < n; ++b)
            if (((g.support >> b) & 1ull) && owner[b] >= 0 &&
                std::find(os.begin(), os.end(), owner[b]) == os.end())
                os.push_back(owner[b]);
        {  // standalone gates end when a later gate reaches one of their wires: all of them go
           // out together (they hold disjoint wires, so they commute) and stay one XOR run
            bool hit = false;
            std::vector<int> keep;
            for (int oi : os) {
                if (open[oi].frozen) hit = true;
                else keep.push_back(oi);
            }
            if (hit)
                for (size_t oi = 0; oi < open.size(); ++oi)
                    if (open[oi].live && open[oi].frozen) close((int)oi);
            os.swap(keep);
        }
        if (!fusable) {
            for (int oi : os) close(oi);
            out.push_back(g);
            continue;
        }
        // A two-wire diagonal gate (CZ, CR, CRk) only joins a block on exactly its two wires;
        // otherwise it goes out in place, so that diagonal runs keep their order and fold into
        // phase tables instead of lingering in blocks that are never fused.
        if (popcount64(g.support) == 2 && is_zero(g.u[0][1]) && is_zero(g.u[1][0]) &&
            !(os.size() == 1 && open[os[0]].bits == g.support)) {
            for (int oi : os) close(oi);
            out.push_back(g);
            continue;
        }
        uint64_t all = g.support;
        for (int oi : os) all |= open[oi].bits;
        if (popcount64(all) > 2) {  // blocks reaching outside this gate's wires end here
            if (agate_macs(g) < 1.0) {
                // A cheap two-wire gate (CNot, CZ, controlled phase) between blocks stays on its
                // own: opening a block with it would capture the next gates of both wires, which
                // pair better with the gates on their other neighbours (brickwork: the odd CNot
                // layer stands alone, each even CNot joins the dense layers around it). It is
                // emitted only when a later gate reaches its wires, so that standalone gates of
                // one layer come out next to each other (and form one XOR run). Diagonal gates
                // go out at once instead: they keep their order, and runs of them between two
                // non-diagonal gates fold into phase tables (QFT rows).
                for (int oi : os) close(oi);
                if (is_zero(g.u[0][1]) && is_zero(g.u[1][0])) {
                    out.push_back(g);
                    continue;
                }
                open.emplace_back();
                Open& f = open.back();
                f.live = f.frozen = true;
                f.bits = g.support;
                f.members.push_back((int)gi);
                for (int b = 0; b < n; ++b)
                    if ((f.bits >> b) & 1ull) owner[b] = (int)open.size() - 1;
                continue;
            }
            std::vector<int> keep;
            for (int oi : os) {
                if (open[oi].bits & ~g.support) close(oi);
                else keep.push_back(oi);
            }
            os.swap(keep);
        }
        int into;
        if (os.empty()) {
            open.emplace_back();
            into = (int)open.size() - 1;
            open[into].live = true;
        } else {
            into = os[0];
            for (size_t q = 1; q < os.size(); ++q) {  // disjoint blocks commute: concatenate
                Open& o = open[os[q]];
                open[into].bits |= o.bits;
                open[into].members.insert(open[into].members.end(), o.members.begin(),
                                          o.members.end());
                o.live = false;
                o.members.clear();
            }
        }
        open[into].bits |= g.support;
        open[into].members.push_back((int)gi);
        for (int b = 0; b < n; ++b)
            if ((open[into].bits >> b) & 1ull) owner[b] = into;
    }
    for (size_t oi = 0; oi < open.size(); ++oi)
        if (open[oi].live) close((int)oi);
    return out;
}

// Steps for a controlled 2x2 u on bit t under control mask cm.
void emit_one(const AGate& g, std::vector<HStep>& out) {
    const cd u00 = g.u[0][0], u01 = g.u[0][1], u10 = g.u[1][0], u11 = g.u[1][1];
    HStep h;
    if (is_zero(u01) && is_zero(u10)) {  // diagonal
        const int c0 = unit_code(u00), c1 = unit_code(u11);
        if (c0 == 0 && c1 == 0) return;  // identity
        h.diagonal = true;
        if (c0 == 0) {
            h.s = blank_step(ST_PHASE);
            h.s.cm = g.cm | (1ull << g.t);
            set_entry(h.s, 0, u11);
            set_packed(h.s, &u11);
            h.unit = c1 >= 0;
            h.s.unit = h.unit;
            h.s.u0 = (uint8_t)(c1 < 0 ? 0 : c1);
            h.dcm = h.s.cm;
            h.d1 = u11;
        } else {
            h.s = blank_step(ST_DIAG);
            h.s.cm = g.cm;
            h.s.fb = (uint8_t)g.t;
            set_entry(h.s, 0, u00);
            set_entry(h.s, 1, u11);
            const cd dd[2] = {u00, u11};
            set_packed(h.s, dd);
            h.unit = c0 >= 0 && c1 >= 0;
            h.s.unit = h.unit;
            h.s.u0 = (uint8_t)(c0 < 0 ? 0 : c0);
            h.s.u1 = (uint8_t)(c1 < 0 ? 0 : c1);
            h.dcm = g.cm;
            h.dfb = g.t;
            h.d0 = u00;
            h.d1 = u11;
        }
        out.push_back(h);
        return;
    }
    if (is_zero(u00) && is_zero(u11) && unit_code(u01) >= 0 && unit_code(u10) >= 0) {
        h.s = blank_step(ST_PERM);
        h.s.anti = 1;
        h.s.u0 = (uint8_t)unit_code(u01);
        h.s.u1 = (uint8_t)unit_code(u10);
        h.s.unit = 1;
        h.unit = true;
    } else if (u00.imag() == 0 && u01.imag() == 0 && u10.imag() == 0 && u11.imag() == 0) {
        h.s = blank_step(ST_REAL);
    } else {
        h.s = blank_step(ST_DENSE);
    }
    h.s.cm = g.cm;
    set_entry(h.s, 0, u00);
    set_entry(h.s, 1, u01);
    set_entry(h.s, 2, u10);
    set_entry(h.s, 3, u11);
    const cd ee[4] = {u00, u01, u10, u11};
    set_packed(h.s, ee);
    h.need[0] = g.t;
    out.push_back(h);
}

// Tries to fold a run of diagonal steps into one TABLE step. Returns false when the run's bits
// do not fit MAX_TABLE_FIELDS fields of table_bits contiguous bits.
bool fold_table(const std::vector<HStep>& run, Plan* plan, HStep* out, int table_bits) {
    uint64_t common = ~0ull;
    for (const HStep& h : run) common &= h.dcm;
    // bits each step depends on beyond the common condition
    std::vector<uint64_t> rest(run.size());
    uint64_t uni = 0;
    for (size_t i = 0; i < run.size(); ++i) {
        uint64_t r = run[i].dcm & ~common;
        if (run[i].dfb >= 0) r |= 1ull << run[i].dfb;
        rest[i] = r;
        uni |= r;
    }
    int lo[MAX_TABLE_FIELDS], width[MAX_TABLE_FIELDS], nf = 0;
    uint64_t left = uni;
    while (left) {
        if (nf == MAX_TABLE_FIELDS) return false;
        const int b = __builtin_ctzll(left);
        lo[nf] = b;
        int w = 0;
        for (int q = b; q < 64 && q < b + table_bits; ++q)
            if ((left >> q) & 1ull) w = q - b + 1;
        width[nf] = w;
        const uint64_t fm = (w >= 64) ? ~0ull : (((1ull << w) - 1ull) << b);
        left &= ~fm;
        ++nf;
    }
    if (nf == 0) {  // every step depends only on the common condition: one constant factor
        lo[0] = 0;
        width[0] = 0;
        nf = 1;
    }
    std::vector<int> field(run.size(), 0);
    for (size_t i = 0; i < run.size(); ++i) {
        if (!rest[i]) continue;
        int f = -1;
        for (int q = 0; q < nf; ++q) {
            const uint64_t fm = ((1ull << width[q]) - 1ull) << lo[q];
            if ((rest[i] & ~fm) == 0) { f = q; break; }
        }
        if (f < 0) return false;
        field[i] = f;
    }
    HStep h;
    h.s = blank_step(ST_TABLE);
    h.s.cm = common == ~0ull ? 0 : common;
    h.s.nfields = (uint8_t)nf;
    h.diagonal = true;
    using cl = std::complex<long double>;
    for (int q = 0; q < nf; ++q) {
        const size_t entries = (size_t)1 << width[q];
        h.s.tab_off[q] = (uint32_t)(plan->table_f64.size() / 2);
        h.s.tab_shift[q] = (uint8_t)lo[q];
        h.s.tab_width[q] = (uint8_t)width[q];
        std::vector<size_t> mine;  // the run's steps that live in this field
        bool single = true;        // each one a factor on a single bit (a controlled phase)
        for (size_t i = 0; i < run.size(); ++i) {
            if (field[i] != q) continue;
            mine.push_back(i);
            const uint64_t need = run[i].dcm & ~common;
            single = single && run[i].dfb < 0 && popcount64(need) == 1;
        }
        // single-bit factors: entry y is the product of the factors of y's set bits, built up
        // from the entry without y's lowest bit (one multiply per entry)
        std::vector<cl> tab(single ? entries : 0);
        if (single) {
            std::vector<cl> w(width[q], cl(1.0L, 0.0L));
            for (size_t i : mine) {
                const int b = __builtin_ctzll(run[i].dcm & ~common) - lo[q];
                w[b] *= cl(run[i].d1.real(), run[i].d1.imag());
            }
            tab[0] = cl(1.0L, 0.0L);
            for (size_t y = 1; y < entries; ++y)
                tab[y] = tab[y & (y - 1)] * w[__builtin_ctzll(y)];
        }
        for (size_t y = 0; y < entries; ++y) {
            const uint64_t idx = (uint64_t)y << lo[q];
            cl acc(1.0L, 0.0L);
            if (single) {
                acc = tab[y];
            } else {
                for (size_t i : mine) {
                    const HStep& s = run[i];
                    const uint64_t need = s.dcm & ~common;
                    if ((idx & need) != need) continue;
                    cd f = s.d1;
                    if (s.dfb >= 0) f = ((idx >> s.dfb) & 1ull) ? s.d1 : s.d0;
                    acc *= cl(f.real(), f.imag());
                }
            }
            const cd v((double)acc.real(), (double)acc.imag());
            plan->table_f64.push_back(v.real());
            plan->table_f64.push_back(v.imag());
            float ff[4];
            put_ff(ff, v);
            plan->table_ff.insert(plan->table_ff.end(), ff, ff + 4);
        }
    }
    *out = h;
    return true;
}

}  // namespace

std::vector<XTerm> xor_terms(const XorPerm& xp) {
    std::vector<XTerm> out;
    for (int e = 0; e < xp.nterms; ++e) {
        if (xp.grouped[e] == 2) {
            XTerm t;
            t.cm = t.flip = xp.cm[e];
            t.swap = true;
            out.push_back(t);
        } else if (xp.grouped[e] == 1) {  // controls at target + shift
            for (int c = 0; c < 64; ++c)
                if ((xp.cm[e] >> c) & 1ull) {
                    XTerm t;
                    t.cm = 1ull << c;
                    t.flip = 1ull << (c - xp.shift[e]);
                    out.push_back(t);
                }
        } else {
            XTerm t;
            t.cm = xp.cm[e];
            t.flip = xp.tbit[e];
            out.push_back(t);
        }
    }
    return out;
}

bool xor_from_terms(const std::vector<XTerm>& ts, XorPerm* xp) {
    *xp = XorPerm();
    for (const XTerm& t : ts) {
        int g = -1;
        if (t.swap) {
            if (xp->nterms == MAX_XOR_TERMS) return false;
            g = xp->nterms++;
            xp->grouped[g] = 2;
            xp->shift[g] = 0;
            xp->cm[g] = t.cm;
            xp->tbit[g] = 0;
            continue;
        }
        if (popcount64(t.cm) == 1) {
            const int shift = __builtin_ctzll(t.cm) - __builtin_ctzll(t.flip);
            for (int e = 0; e < xp->nterms; ++e)
                if (xp->grouped[e] == 1 && xp->shift[e] == shift) g = e;
            if (g < 0) {
                if (xp->nterms == MAX_XOR_TERMS) return false;
                g = xp->nterms++;
                xp->grouped[g] = 1;
                xp->shift[g] = shift;
                xp->cm[g] = 0;
                xp->tbit[g] = 0;
            }
            xp->cm[g] |= t.cm;
            xp->tbit[g] |= t.flip;
            continue;
        }
        if (xp->nterms == MAX_XOR_TERMS) return false;
        g = xp->nterms++;
        xp->grouped[g] = 0;
        xp->shift[g] = 0;
        xp->cm[g] = t.cm;
        xp->tbit[g] = t.flip;
    }
    return true;
}

// ---------------------------------------------------------------------------------------------
// Double pair passes. A float-pair pair block costs about as much arithmetic as its pass takes
// to stream the register, so two blocks on disjoint bit pairs share one pass (k_pair2: 16
// amplitudes per thread). Consecutive pair passes on pairwise disjoint bits commute and are
// matched two by two; an XOR pass next to such a run (the CNot layer between two brickwork
// layers) is split into its terms, and every term whose bits lie inside a matched tile becomes a
// register permutation of that tile: applied before the blocks when the XOR pass precedes the
// run, after them when it follows. The matching prefers tiles that take terms of the preceding
// XOR pass (they cannot wait), then tiles that take terms of the following one; terms no tile
// takes stay in a smaller XOR pass at the original position.
// ---------------------------------------------------------------------------------------------
namespace {

uint64_t xterm_bits(const XTerm& t) { return t.cm | t.flip; }

double xor_touched(const std::vector<XTerm>& ts) {
    double touched = 0.0;
    for (const XTerm& t : ts) touched += t.swap ? 0.5 : std::ldexp(1.0, -popcount64(t.cm));
    return std::min(1.0, touched);
}

bool push_xor_pass(const std::vector<XTerm>& ts, std::vector<Pass>& out) {
    if (ts.empty()) return true;
    Pass x;
    x.xor_pass = true;
    if (!xor_from_terms(ts, &x.xp)) return false;
    x.touched = xor_touched(ts);
    out.push_back(x);
    return true;
}

uint64_t pass_pair_bits(const Pass& p) { return (1ull << p.bits[0]) | (1ull << p.bits[1]); }

bool is_single_pair(const Pass& p) { return p.pair >= 0 && p.pair2 < 0; }

}  // namespace

void group_pair_passes(Plan* plan) {
    const std::vector<Pass> in = plan->passes;
    std::vector<Pass> out;
    std::vector<XTerm> pending;  // terms of the XOR pass just before the current run
    size_t i = 0;
    while (i < in.size()) {
        if (!is_single_pair(in[i])) {
            if (in[i].xor_pass && i + 1 < in.size() && is_single_pair(in[i + 1])) {
                pending = xor_terms(in[i].xp);  // placed by the run that follows
            } else {
                out.push_back(in[i]);
            }
            ++i;
            continue;
        }
        // the run: pair passes on pairwise disjoint bits
        size_t j = i;
        uint64_t used = 0;
        while (j < in.size() && is_single_pair(in[j]) && !(pass_pair_bits(in[j]) & used)) {
            used |= pass_pair_bits(in[j]);
            ++j;
        }
        const size_t m = j - i;
        std::vector<XTerm> next;
        const bool next_xor = j < in.size() && in[j].xor_pass;
        if (next_xor) next = xor_terms(in[j].xp);
        // greedy matching: heaviest tiles first (4 per preceding-XOR term, 1 per following)
        std::vector<int> mate(m, -1);
        struct Edge {
            int w, a, b;
        };
        std::vector<Edge> edges;
        if (m <= 64) {
            for (size_t a = 0; a < m; ++a)
                for (size_t b = a + 1; b < m; ++b) {
                    const uint64_t mask = pass_pair_bits(in[i + a]) | pass_pair_bits(in[i + b]);
                    int w = 0;
                    for (const XTerm& t : pending) w += (xterm_bits(t) & ~mask) ? 0 : 4;
                    for (const XTerm& t : next) w += (xterm_bits(t) & ~mask) ? 0 : 1;
                    if (w > 0) edges.push_back(Edge{w, (int)a, (int)b});
                }
            std::stable_sort(edges.begin(), edges.end(),
                             [](const Edge& x, const Edge& y) { return x.w > y.w; });
            for (const Edge& e : edges)
                if (mate[e.a] < 0 && mate[e.b] < 0) {
                    mate[e.a] = e.b;
                    mate[e.b] = e.a;
                }
        }
        for (size_t a = 0; a < m; ++a) {  // the rest two by two in order
            if (mate[a] >= 0) continue;
            for (size_t b = a + 1; b < m; ++b)
                if (mate[b] < 0) {
                    mate[a] = (int)b;
                    mate[b] = (int)a;
                    break;
                }
        }
        std::vector<Pass> groups;
        for (size_t a = 0; a < m; ++a) {
            if (mate[a] >= 0 && mate[a] < (int)a) continue;
            if (mate[a] < 0) {
                groups.push_back(in[i + a]);
                continue;
            }
            const Pass& pa = in[i + a];
            const Pass& pb = in[i + mate[a]];
            Pass g;
            int bits[4] = {pa.bits[0], pa.bits[1], pb.bits[0], pb.bits[1]};
            std::sort(bits, bits + 4);
            g.nbits = 4;
            for (int q = 0; q < 4; ++q) g.bits[q] = bits[q];
            g.arith = true;
            g.cost = pa.cost + pb.cost;
            g.touched = 1.0;
            g.pair = pa.pair;
            g.pair2 = pb.pair;
            groups.push_back(g);
        }
        auto place = [&](std::vector<XTerm>& terms, bool before) {
            std::vector<XTerm> rest;
            for (const XTerm& t : terms) {
                bool placed = false;
                for (Pass& g : groups) {
                    if (g.pair2 < 0) continue;
                    uint64_t mask = 0;
                    for (int q = 0; q < 4; ++q) mask |= 1ull << g.bits[q];
                    std::vector<XTerm>& dst = before ? g.pre : g.post;
                    if ((xterm_bits(t) & ~mask) == 0 && (int)dst.size() < MAX_TILE_XTERMS) {
                        dst.push_back(t);
                        placed = true;
                        break;
                    }
                }
                if (!placed) rest.push_back(t);
            }
            terms.swap(rest);
        };
        place(pending, true);
        if (!push_xor_pass(pending, out)) {  // cannot happen: a subset regroups into fewer entries
            plan->passes = in;
            return;
        }
        pending.clear();
        place(next, false);
        for (const Pass& g : groups) out.push_back(g);
        if (next_xor) {
            if (j + 1 < in.size() && is_single_pair(in[j + 1])) pending = next;
            else if (!push_xor_pass(next, out)) {
                plan->passes = in;
                return;
            }
            ++j;
        }
        i = j;
    }
    if (!pending.empty() && !push_xor_pass(pending, out)) {
        plan->passes = in;
        return;
    }
    plan->passes.swap(out);
}

DevStep dense_step(cd u00, cd u01, cd u10, cd u11) {
    DevStep s = blank_step(ST_DENSE);
    set_entry(s, 0, u00);
    set_entry(s, 1, u01);
    set_entry(s, 2, u10);
    set_entry(s, 3, u11);
    const cd e[4] = {u00, u01, u10, u11};
    set_packed(s, e);
    return s;
}

int build_plan(const qgpu_op* ops, size_t n_ops, int n, const double* mats, size_t n_mats,
               const uint8_t* none, size_t n_none, const PlanOptions& opt, Plan* plan) {
    plan->passes.clear();
    plan->pairs.clear();
    plan->customs.clear();
    plan->table_ff.clear();
    plan->table_f64.clear();
    const int max_bits = std::max(1, std::min(opt.max_bits, std::min(n, MAX_TILE_BITS)));

    // 1. ops -> AGates (controlled-2x2 form where possible), merging single-wire runs.
    std::vector<AGate> gates;
    std::vector<int> pending(n, -1);  // per bit: index in `gates` of an open single-wire run
    auto close_bits = [&](uint64_t mask) {
        for (int b = 0; b < n; ++b)
            if (((mask >> b) & 1ull) && pending[b] >= 0) pending[b] = -1;
    };
    for (size_t g = 0; g < n_ops; ++g) {
        const qgpu_op& op = ops[g];
        if (op.kind == QGPU_GATE_ID) continue;
        LocalGate lg;
        int st = tabulate(op, n, mats, n_mats, none, n_none, &lg);
        if (st != QGPU_OK) return st;
        const int k = lg.k;
        const size_t d = (size_t)1 << k;
        // Effective linear map of the gate (Custom None rule folded in, simulation.rs:120-133):
        // E[l][j] = none[l] ? delta(l, j) : (none[j] ? 0 : M[l][j]).
        std::vector<cd> E(d * d);
        for (size_t j = 0; j < d; ++j)
            for (size_t l = 0; l < d; ++l)
                E[j * d + l] = lg.none[l] ? cd(l == j ? 1.0 : 0.0, 0.0)
                                          : (lg.none[j] ? cd(0, 0) : lg.M[j * d + l]);
        uint64_t support = 0;
        int bitpos[QGPU_MAX_OP_WIRES];
        for (int m = 0; m < k; ++m) {
            bitpos[m] = n - 1 - lg.wires[m];
            support |= 1ull << bitpos[m];
        }
        // controlled-2x2 form: every column whose control bits are not all 1 is the identity
        bool controlled = op.kind != QGPU_GATE_SWAP;
        const size_t call = (d - 1) & ~(size_t)1;  // local index with every control bit set
        for (size_t j = 0; j < d && controlled; ++j)
            for (size_t l = 0; l < d && controlled; ++l) {
                const bool in_block = ((j & call) == call) && ((l & call) == call);
                if (in_block) continue;
                if (E[j * d + l] != cd(l == j ? 1.0 : 0.0, 0.0)) controlled = false;
            }
        if (op.kind == QGPU_GATE_SWAP) {
            close_bits(support);
            AGate a;
            a.kind = AGate::SWAP;
            a.a = bitpos[1];
            a.b = bitpos[0];
            a.support = support;
            gates.push_back(a);
            continue;
        }
        if (!controlled) {
            close_bits(support);
            AGate a;
            a.kind = AGate::BLOCK;
            a.block = (int)plan->customs.size();
            a.support = support;
            plan->customs.push_back(lg);
            gates.push_back(a);
            continue;
        }
        AGate a;
        a.kind = AGate::ONE;
        a.t = bitpos[k - 1];
        a.cm = support & ~(1ull << a.t);
        a.support = support;
        for (int lo = 0; lo < 2; ++lo)
            for (int in = 0; in < 2; ++in) a.u[lo][in] = E[(call | in) * d + (call | lo)];
        if (k == 1 && opt.merge_1q && pending[a.t] >= 0) {
            AGate& p = gates[pending[a.t]];  // new = a.u * p.u
            cd r[2][2];
            for (int lo = 0; lo < 2; ++lo)
                for (int in = 0; in < 2; ++in)
                    r[lo][in] = a.u[lo][0] * p.u[0][in] + a.u[lo][1] * p.u[1][in];
            std::memcpy(p.u, r, sizeof(r));
            continue;
        }
        close_bits(support);
        gates.push_back(a);
        if (k == 1 && opt.merge_1q) pending[a.t] = (int)gates.size() - 1;
    }

    if (opt.pair_fusion) gates = fuse_pairs(gates, n, plan);

    // 2. AGates -> steps.
    std::vector<HStep> steps;
    std::vector<int> block_at;  // steps index -> custom block (or -1)
    for (const AGate& g : gates) {
        if (g.kind == AGate::PAIR) {
            HStep h;
            h.s = blank_step(ST_DENSE4);
            h.need[0] = g.a;
            h.need[1] = g.b;
            h.s.tab_off[0] = (uint32_t)g.block;
            steps.push_back(h);
            continue;
        }
        if (g.kind == AGate::BLOCK) {
            HStep h;
            h.s = blank_step(0xFF);
            h.s.lb = 0;
            steps.push_back(h);
            block_at.resize(steps.size(), -1);
            block_at.back() = g.block;
            continue;
        }
        if (g.kind == AGate::SWAP) {
            HStep h;
            h.s = blank_step(ST_SWAP);
            h.need[0] = g.a;
            h.need[1] = g.b;
            h.unit = true;
            steps.push_back(h);
            continue;
        }
        emit_one(g, steps);
    }
    block_at.resize(steps.size(), -1);

    // 3. fold runs of diagonal steps into phase tables.
    if (opt.fuse_diagonal) {
        std::vector<HStep> folded;
        std::vector<int> folded_block;
        size_t i = 0;
        while (i < steps.size()) {
            if (!steps[i].diagonal || block_at[i] >= 0) {
                folded.push_back(steps[i]);
                folded_block.push_back(block_at[i]);
                ++i;
                continue;
            }
            size_t j = i;
            int general = 0;
            while (j < steps.size() && steps[j].diagonal && block_at[j] < 0) {
                general += steps[j].unit ? 0 : 1;
                ++j;
            }
            HStep t;
            std::vector<HStep> run(steps.begin() + i, steps.begin() + j);
            const int tb = std::max(1, std::min(opt.table_bits, MAX_TABLE_BITS));
            if (general >= 2 && fold_table(run, plan, &t, tb)) {
                folded.push_back(t);
                folded_block.push_back(-1);
            } else {
                for (size_t q = i; q < j; ++q) {
                    folded.push_back(steps[q]);
                    folded_block.push_back(-1);
                }
            }
            i = j;
        }
        steps.swap(folded);
        block_at.swap(folded_block);
    }

    // 4. group steps into register-tile passes.
    const int conv = opt.policy == POL_FF ? 40 : 0;
    Pass cur;
    std::vector<int> cur_bits;
    std::vector<HStep> cur_steps;
    int cur_cost = 0;
    bool cur_arith = false;
    auto flush = [&]() {
        if (cur_steps.empty()) return;
        Pass p;
        std::sort(cur_bits.begin(), cur_bits.end());
        if (cur_bits.empty()) cur_bits.push_back(0);
        p.nbits = (int)cur_bits.size();
        for (int m = 0; m < p.nbits; ++m) p.bits[m] = cur_bits[m];
        auto local = [&](int b) -> uint8_t {
            for (int m = 0; m < p.nbits; ++m)
                if (cur_bits[m] == b) return (uint8_t)m;
            return 0;
        };
        double touched = 0.0;
        for (HStep& h : cur_steps) {
            if (h.need[0] >= 0) h.s.lb = local(h.need[0]);
            if (h.need[1] >= 0) h.s.lb2 = local(h.need[1]);
            p.steps.push_back(h.s);
            touched += step_fraction(h);
        }
        p.touched = std::min(1.0, touched);
        p.arith = cur_arith;
        p.cost = cur_cost;
        plan->passes.push_back(p);
        cur_bits.clear();
        cur_steps.clear();
        cur_cost = 0;
        cur_arith = false;
    };
    // controlled-X step (X, CNot, Toffoli as a PERM without phases)
    auto is_cx = [&](size_t i) {
        const HStep& h = steps[i];
        return block_at[i] < 0 && h.s.type == ST_PERM && h.s.anti && h.s.u0 == 0 && h.s.u1 == 0 &&
               h.need[0] >= 0;
    };
    auto is_sw = [&](size_t i) { return block_at[i] < 0 && steps[i].s.type == ST_SWAP; };
    for (size_t i = 0; i < steps.size(); ++i) {
        if (block_at[i] >= 0) {
            flush();
            Pass p;
            p.custom = block_at[i];
            plan->passes.push_back(p);
            continue;
        }
        if (opt.xor_runs && (is_cx(i) || is_sw(i))) {
            // longest run of controlled-X / swap steps forming one involution
            uint64_t targets = 0, controls = 0, swapped = 0;
            size_t j = i;
            while (j < steps.size() && (is_cx(j) || is_sw(j))) {
                if (is_sw(j)) {
                    const uint64_t sb = (1ull << steps[j].need[0]) | (1ull << steps[j].need[1]);
                    if (sb & (targets | controls | swapped)) break;
                    swapped |= sb;
                } else {
                    const uint64_t tb = 1ull << steps[j].need[0], cm = steps[j].s.cm;
                    if ((targets & tb) || (targets & cm) || (controls & tb) || (swapped & (tb | cm)))
                        break;
                    targets |= tb;
                    controls |= cm;
                }
                ++j;
            }
            XorPerm xp;
            bool fits = j - i >= 3;
            for (size_t q = i; q < j && fits; ++q) {
                if (is_sw(q)) {
                    if (xp.nterms == MAX_XOR_TERMS) { fits = false; break; }
                    const int g = xp.nterms++;
                    xp.grouped[g] = 2;
                    xp.shift[g] = 0;
                    xp.cm[g] = (1ull << steps[q].need[0]) | (1ull << steps[q].need[1]);
                    xp.tbit[g] = 0;
                    continue;
                }
                const int t = steps[q].need[0];
                const uint64_t cm = steps[q].s.cm;
                if (popcount64(cm) == 1) {
                    const int c = __builtin_ctzll(cm);
                    const int shift = c - t;
                    int g = -1;
                    for (int e = 0; e < xp.nterms; ++e)
                        if (xp.grouped[e] && xp.shift[e] == shift) g = e;
                    if (g < 0) {
                        if (xp.nterms == MAX_XOR_TERMS) { fits = false; break; }
                        g = xp.nterms++;
                        xp.grouped[g] = 1;
                        xp.shift[g] = shift;
                        xp.cm[g] = 0;
                        xp.tbit[g] = 0;
                    }
                    xp.cm[g] |= cm;
                    xp.tbit[g] |= 1ull << t;
                } else {
                    if (xp.nterms == MAX_XOR_TERMS) { fits = false; break; }
                    const int g = xp.nterms++;
                    xp.grouped[g] = 0;
                    xp.shift[g] = 0;
                    xp.cm[g] = cm;
                    xp.tbit[g] = 1ull << t;
                }
            }
            if (fits) {
                flush();
                Pass p;
                p.xor_pass = true;
                p.xp = xp;
                double touched = 0.0;
                for (size_t q = i; q < j; ++q)
                    touched += is_sw(q) ? 0.5 : std::ldexp(1.0, -popcount64(steps[q].s.cm));
                p.touched = std::min(1.0, touched);
                plan->passes.push_back(p);
                i = j - 1;
                continue;
            }
        }
        const HStep& h = steps[i];
        if (h.s.type == ST_DENSE4) {  // a pair block is a pass of its own (k_pair)
            flush();
            Pass p;
            p.nbits = 2;
            p.bits[0] = std::min(h.need[0], h.need[1]);
            p.bits[1] = std::max(h.need[0], h.need[1]);
            p.arith = true;
            p.cost = 380;
            p.touched = 1.0;
            p.pair = (int)h.s.tab_off[0];
            plan->passes.push_back(p);
            continue;
        }
        std::vector<int> bits = cur_bits;
        for (int q = 0; q < 2; ++q)
            if (h.need[q] >= 0 && std::find(bits.begin(), bits.end(), h.need[q]) == bits.end())
                bits.push_back(h.need[q]);
        const int c = step_cost(h, opt.policy);
        const bool arith = !h.unit;
        const int new_cost = cur_cost + c + ((arith && !cur_arith) ? conv : 0);
        const int width = (arith || cur_arith) ? std::min(max_bits, std::max(1, opt.max_arith_bits))
                                               : max_bits;
        const bool fits = (int)bits.size() <= width && (int)cur_steps.size() < MAX_STEPS &&
                          (cur_steps.empty() || new_cost <= opt.budget);
        if (!fits) {
            flush();
            bits.clear();
            for (int q = 0; q < 2; ++q)
                if (h.need[q] >= 0 && std::find(bits.begin(), bits.end(), h.need[q]) == bits.end())
                    bits.push_back(h.need[q]);
        }
        cur_bits = bits;
        cur_cost += c + ((arith && !cur_arith) ? conv : 0);
        cur_arith = cur_arith || arith;
        cur_steps.push_back(h);
    }
    flush();
    if (opt.pair_fusion && opt.group_pairs) group_pair_passes(plan);
    return QGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Dense-block fusion
// ---------------------------------------------------------------------------------------------
namespace {

struct PendingGate {
    int kg;
    int bitpos[QGPU_MAX_OP_WIRES];  // full-index bit of gate wire m (gate-local bit kg-1-m)
    std::vector<cd> E;              // column-major effective matrix (None rule folded in)
};

// Multiplies the pending gates, in order, into a dense matrix over their sorted bits.
DenseBlock fuse_pending(const std::vector<PendingGate>& gs) {
    DenseBlock b;
    std::vector<int> bits;
    for (const PendingGate& g : gs)
        for (int m = 0; m < g.kg; ++m)
            if (std::find(bits.begin(), bits.end(), g.bitpos[m]) == bits.end()) bits.push_back(g.bitpos[m]);
    std::sort(bits.begin(), bits.end());
    b.k = (int)bits.size();
    for (int m = 0; m < b.k; ++m) b.bits[m] = bits[m];
    const size_t D = (size_t)1 << b.k;
    b.M.assign(D * D, cd(0, 0));
    for (size_t i = 0; i < D; ++i) b.M[i * D + i] = 1.0;
    std::vector<cd> col(D), out(D);
    for (const PendingGate& g : gs) {
        int lp[QGPU_MAX_OP_WIRES];  // block-local bit of gate wire m
        for (int m = 0; m < g.kg; ++m)
            lp[m] = (int)(std::find(bits.begin(), bits.end(), g.bitpos[m]) - bits.begin());
        const size_t dg = (size_t)1 << g.kg;
        size_t gmask = 0;
        for (int m = 0; m < g.kg; ++m) gmask |= (size_t)1 << lp[m];
        for (size_t c = 0; c < D; ++c) {  // new column c = G * (old column c)
            for (size_t x = 0; x < D; ++x) col[x] = b.M[x * D + c];
            std::fill(out.begin(), out.end(), cd(0, 0));
            for (size_t x = 0; x < D; ++x) {
                if (col[x] == cd(0, 0)) continue;
                size_t j = 0;
                for (int m = 0; m < g.kg; ++m) j = (j << 1) | ((x >> lp[m]) & 1u);
                const size_t rest = x & ~gmask;
                for (size_t l = 0; l < dg; ++l) {
                    const cd e = g.E[j * dg + l];
                    if (e == cd(0, 0)) continue;
                    size_t y = rest;
                    for (int m = 0; m < g.kg; ++m)
                        if ((l >> (g.kg - 1 - m)) & 1u) y |= (size_t)1 << lp[m];
                    out[y] += e * col[x];
                }
            }
            for (size_t x = 0; x < D; ++x) b.M[x * D + c] = out[x];
        }
    }
    b.gates = (int)gs.size();
    return b;
}

}  // namespace

int build_blocks(const qgpu_op* ops, size_t n_ops, int n, const double* mats, size_t n_mats,
                 const uint8_t* none, size_t n_none, int block_qubits, int max_gates,
                 std::vector<DenseBlock>* out) {
    out->clear();
    std::vector<PendingGate> cur;
    uint64_t cur_bits = 0;
    auto flush = [&]() {
        if (!cur.empty()) out->push_back(fuse_pending(cur));
        cur.clear();
        cur_bits = 0;
    };
    for (size_t g = 0; g < n_ops; ++g) {
        if (ops[g].kind == QGPU_GATE_ID) continue;
        LocalGate lg;
        int st = tabulate(ops[g], n, mats, n_mats, none, n_none, &lg);
        if (st != QGPU_OK) return st;
        PendingGate pg;
        pg.kg = lg.k;
        uint64_t gb = 0;
        for (int m = 0; m < lg.k; ++m) {
            pg.bitpos[m] = n - 1 - lg.wires[m];
            gb |= 1ull << pg.bitpos[m];
        }
        const size_t d = (size_t)1 << lg.k;
        pg.E.resize(d * d);
        for (size_t j = 0; j < d; ++j)
            for (size_t l = 0; l < d; ++l)
                pg.E[j * d + l] = lg.none[l] ? cd(l == j ? 1.0 : 0.0, 0.0)
                                             : (lg.none[j] ? cd(0, 0) : lg.M[j * d + l]);
        if (popcount64(cur_bits | gb) > std::max(block_qubits, lg.k) || (int)cur.size() >= max_gates)
            flush();
        cur.push_back(pg);
        cur_bits |= gb;
    }
    flush();
    return QGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Adjoint sweep helpers
// ---------------------------------------------------------------------------------------------
bool is_rotation(int kind) {
    return kind == QGPU_GATE_RX || kind == QGPU_GATE_RY || kind == QGPU_GATE_RZ ||
           kind == QGPU_GATE_PHASE;
}

qgpu_op inverse_op(const qgpu_op& op) {
    qgpu_op r = op;
    switch (op.kind) {
        case QGPU_GATE_S: r.kind = QGPU_GATE_SDAG; break;
        case QGPU_GATE_SDAG: r.kind = QGPU_GATE_S; break;
        case QGPU_GATE_T: r.kind = QGPU_GATE_TDAG; break;
        case QGPU_GATE_TDAG: r.kind = QGPU_GATE_T; break;
        case QGPU_GATE_X90: r.kind = QGPU_GATE_MX90; break;
        case QGPU_GATE_MX90: r.kind = QGPU_GATE_X90; break;
        case QGPU_GATE_Y90: r.kind = QGPU_GATE_MY90; break;
        case QGPU_GATE_MY90: r.kind = QGPU_GATE_Y90; break;
        case QGPU_GATE_RX: case QGPU_GATE_RY: case QGPU_GATE_RZ: case QGPU_GATE_PHASE:
        case QGPU_GATE_CR:
            r.param = -op.param;
            break;
        case QGPU_GATE_CRK:
            r.kind = QGPU_GATE_CR;
            r.param = -((2.0 * 3.14159265358979323846) / std::pow(2.0, (double)op.k));
            break;
        default:
            break;  // H, X, Y, Z, CNot, CY, CZ, Swap, Toffoli are self-inverse
    }
    return r;
}

std::vector<std::pair<uint64_t, std::vector<size_t>>> adj_group_passes(const std::vector<int>& bits,
                                                                       int n, int max_bits) {
    std::vector<size_t> order(bits.size());
    for (size_t w = 0; w < order.size(); ++w) order[w] = w;
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return bits[x] < bits[y]; });
    const int kmax = std::min(n, max_bits);
    const uint64_t low = (1ull << std::min(n, 5)) - 1;
    std::vector<std::pair<uint64_t, std::vector<size_t>>> out;
    size_t i = 0;
    while (i < order.size()) {
        uint64_t mask = low;
        std::vector<size_t> chosen;
        while (i < order.size() && (chosen.empty() ||
                                    __builtin_popcountll(mask | (1ull << bits[order[i]])) <= kmax)) {
            mask |= 1ull << bits[order[i]];  // (the first wire always: a pass takes at least one)
            chosen.push_back(order[i++]);
        }
        for (int b = 0; b < n && __builtin_popcountll(mask) < kmax; ++b) mask |= 1ull << b;
        out.emplace_back(mask, std::move(chosen));
    }
    return out;
}

int pauli_run(const qgpu_op* ops, const std::vector<size_t>& gw, int n, PauliRun* out) {
    const size_t k = gw.size();
    std::vector<std::array<cd, 4>> fwd(k), inv(k);  // row-major 2x2: m[2 l + j]
    for (size_t q = 0; q < k; ++q) {
        LocalGate a, b;
        int st = tabulate(ops[gw[q]], n, nullptr, 0, nullptr, 0, &a);
        if (st == QGPU_OK) st = tabulate(inverse_op(ops[gw[q]]), n, nullptr, 0, nullptr, 0, &b);
        if (st != QGPU_OK) return st;
        for (int l = 0; l < 2; ++l)
            for (int j = 0; j < 2; ++j) {
                fwd[q][2 * l + j] = a.M[j * 2 + l];
                inv[q][2 * l + j] = b.M[j * 2 + l];
            }
    }
    auto mul = [](const std::array<cd, 4>& x, const std::array<cd, 4>& y) {
        return std::array<cd, 4>{x[0] * y[0] + x[1] * y[2], x[0] * y[1] + x[1] * y[3],
                                 x[2] * y[0] + x[3] * y[2], x[2] * y[1] + x[3] * y[3]};
    };
    // V runs over the later gates
    std::array<cd, 4> undo{cd(1), cd(0), cd(0), cd(1)}, V{cd(1), cd(0), cd(0), cd(1)};
    out->rots.clear();
    for (int m = 0; m < 5; ++m) out->need[m] = false;
    for (size_t q = 0; q < k; ++q) {  // q = 0 is the last gate of the run
        undo = mul(inv[q], undo);
        const qgpu_op& op = ops[gw[q]];
        if (is_rotation(op.kind)) {
            std::array<cd, 4> P{cd(0), cd(0), cd(0), cd(0)};
            switch (op.kind) {
                case QGPU_GATE_RX: P = {cd(0), cd(1), cd(1), cd(0)}; break;
                case QGPU_GATE_RY: P = {cd(0), cd(0, -1), cd(0, 1), cd(0)}; break;
                case QGPU_GATE_RZ: P = {cd(1), cd(0), cd(0), cd(-1)}; break;
                default: P = {cd(-1), cd(0), cd(0), cd(-1)}; break;  // Phase: -I
            }
            const std::array<cd, 4> Vd{std::conj(V[0]), std::conj(V[2]), std::conj(V[1]),
                                       std::conj(V[3])};
            const std::array<cd, 4> Q = mul(mul(V, P), Vd);
            std::array<double, 5> c{};  // kinds 1 X, 2 Y, 3 Z, 4 -I
            c[1] = Q[2].real();
            c[2] = Q[2].imag();
            c[3] = 0.5 * (Q[0].real() - Q[3].real());
            c[4] = -0.5 * (Q[0].real() + Q[3].real());
            for (int m = 1; m <= 4; ++m) out->need[m] = out->need[m] || c[m] != 0.0;
            out->rots.emplace_back(gw[q], c);
        }
        V = mul(V, fwd[q]);  // the gates after the next one back
    }
    out->undo = undo;
    return QGPU_OK;
}

// Whether ops (applied in order) form an affine index map; if so, the gather tables of its
// inverse: tabs[c * 256 + v] = xor of the inverse map's columns for the set bits of v (bits
// 8c .. 8c+7), *d = inverse map of 0.
bool affine_tables(const qgpu_op* ops, size_t n_ops, int n, std::vector<uint64_t>* tabs,
                   uint64_t* d) {
    for (size_t g = 0; g < n_ops; ++g) {
        const int k = ops[g].kind;
        if (k != QGPU_GATE_CNOT && k != QGPU_GATE_X && k != QGPU_GATE_SWAP) return false;
    }
    // inverse of g_m ... g_1 is g_1 ... g_m (each gate is an involution): apply ops last to first
    auto inv = [&](uint64_t y) {
        for (size_t g = n_ops; g-- > 0;) {
            const qgpu_op& op = ops[g];
            const int t = n - 1 - op.target;
            if (op.kind == QGPU_GATE_X) {
                y ^= 1ull << t;
            } else if (op.kind == QGPU_GATE_CNOT) {
                const int c = n - 1 - op.controls[0];
                y ^= ((y >> c) & 1ull) << t;
            } else {  // Swap
                const int c = n - 1 - op.controls[0];
                const uint64_t bt = (y >> t) & 1ull, bc = (y >> c) & 1ull;
                if (bt != bc) y ^= (1ull << t) | (1ull << c);
            }
        }
        return y;
    };
    *d = inv(0);
    std::vector<uint64_t> col(n);
    for (int b = 0; b < n; ++b) col[b] = inv(1ull << b) ^ *d;
    const int nchunks = (n + 7) / 8;
    tabs->assign((size_t)nchunks * 256, 0);
    for (int c = 0; c < nchunks; ++c)
        for (int v = 0; v < 256; ++v) {
            uint64_t x = 0;
            for (int k = 0; k < 8; ++k)
                if (((v >> k) & 1) && 8 * c + k < n) x ^= col[8 * c + k];
            (*tabs)[(size_t)c * 256 + v] = x;
        }
    return true;
}

}  // namespace qgpu
