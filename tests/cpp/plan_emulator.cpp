// Host-side executor of the fused pass plan (quantr_gb300/csrc/plan.cpp) in complex128, so the
// planner's merging, pair fusion, table folding, XOR runs and pass grouping can be checked
// against the oracle on a machine without a GPU. Steps are applied with their f64 entries
// (DevStep::d) in the order and on the amplitudes the tile kernels use; Custom passes apply
// their tabulated block with the None rule.
//
// usage: plan_emulator n ops.bin mats.bin none.bin out.bin [pair_fusion budget max_arith_bits
//                                                          plan_only group block_qubits max_gates]
//   block_qubits > 0: dense-block fusion (build_blocks) instead of the pass plan
//   ops.bin: qgpu_op records; mats.bin: f64; none.bin: u8; out.bin receives 2^n complex128.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "../../quantr_gb300/csrc/plan.h"

namespace qgpu {
int fail(int code, const std::string& msg) {
    std::fprintf(stderr, "plan error: %s\n", msg.c_str());
    return code;
}
}  // namespace qgpu

using qgpu::cd;

template <class T>
static std::vector<T> read_all(const char* path) {
    std::ifstream f(path, std::ios::binary);
    std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<T> out(bytes.size() / sizeof(T));
    if (!out.empty()) std::memcpy(out.data(), bytes.data(), out.size() * sizeof(T));
    return out;
}

static uint64_t insert_zero(uint64_t x, int pos) {
    const uint64_t low = x & ((1ull << pos) - 1ull);
    return low | ((x >> pos) << (pos + 1));
}

static cd unit(int code) {
    static const cd u[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
    return u[code & 3];
}

static cd entry(const qgpu::DevStep& s, int slot) { return cd(s.d[2 * slot], s.d[2 * slot + 1]); }

static void apply_step(const qgpu::DevStep& s, const qgpu::Pass& p, const qgpu::Plan& plan,
                       std::vector<cd>& v, uint64_t base, const std::vector<uint64_t>& off) {
    const int T = (int)v.size();
    auto pairs = [&](int lb, auto&& fn) {
        for (int j = 0; j < T; ++j) {
            if ((j >> lb) & 1) continue;
            const int j1 = j | (1 << lb);
            if (s.cm && ((base | off[j]) & s.cm) != s.cm) continue;
            fn(j, j1);
        }
    };
    switch (s.type) {
        case qgpu::ST_DENSE:
            pairs(s.lb, [&](int j, int j1) {
                const cd a = v[j], b = v[j1];
                v[j] = entry(s, 0) * a + entry(s, 1) * b;
                v[j1] = entry(s, 2) * a + entry(s, 3) * b;
            });
            break;
        case qgpu::ST_REAL:
            pairs(s.lb, [&](int j, int j1) {
                const cd a = v[j], b = v[j1];
                v[j] = s.d[0] * a + s.d[2] * b;
                v[j1] = s.d[4] * a + s.d[6] * b;
            });
            break;
        case qgpu::ST_PERM:
            pairs(s.lb, [&](int j, int j1) {
                cd a = v[j], b = v[j1];
                if (s.anti) std::swap(a, b);
                v[j] = a * unit(s.u0);
                v[j1] = b * unit(s.u1);
            });
            break;
        case qgpu::ST_SWAP: {
            const int A = std::min(s.lb, s.lb2), B = std::max(s.lb, s.lb2);
            for (int j = 0; j < T; ++j)
                if (((j >> A) & 1) == 0 && ((j >> B) & 1) == 1) {
                    const int j2 = (j | (1 << A)) & ~(1 << B);
                    std::swap(v[j], v[j2]);
                }
            break;
        }
        case qgpu::ST_PHASE:
            for (int j = 0; j < T; ++j)
                if (((base | off[j]) & s.cm) == s.cm) v[j] *= s.unit ? unit(s.u0) : entry(s, 0);
            break;
        case qgpu::ST_DIAG:
            for (int j = 0; j < T; ++j) {
                const uint64_t idx = base | off[j];
                if ((idx & s.cm) != s.cm) continue;
                const int bit = (int)((idx >> s.fb) & 1ull);
                v[j] *= s.unit ? unit(bit ? s.u1 : s.u0) : entry(s, bit);
            }
            break;
        case qgpu::ST_TABLE:
            for (int j = 0; j < T; ++j) {
                const uint64_t idx = base | off[j];
                if ((idx & s.cm) != s.cm) continue;
                for (int f = 0; f < s.nfields; ++f) {
                    const uint64_t y = (idx >> s.tab_shift[f]) & ((1ull << s.tab_width[f]) - 1ull);
                    const size_t e = s.tab_off[f] + y;
                    v[j] *= cd(plan.table_f64[2 * e], plan.table_f64[2 * e + 1]);
                }
            }
            break;
        default:
            std::fprintf(stderr, "unknown step type %d\n", s.type);
            std::exit(3);
    }
    (void)p;
}

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s n ops mats none out [pair budget arith_bits plan_only group "
                             "block_qubits max_gates]\n", argv[0]);
        return 2;
    }
    const int n = std::atoi(argv[1]);
    auto ops = read_all<qgpu_op>(argv[2]);
    auto mats = read_all<double>(argv[3]);
    auto none = read_all<uint8_t>(argv[4]);
    qgpu::PlanOptions opt;
    opt.policy = qgpu::POL_FF;
    opt.pair_fusion = argc > 6 ? std::atoi(argv[6]) != 0 : true;
    opt.budget = argc > 7 ? std::atoi(argv[7]) : 280;
    opt.max_arith_bits = argc > 8 ? std::atoi(argv[8]) : 2;
    opt.group_pairs = argc > 10 ? std::atoi(argv[10]) != 0 : true;
    if (argc > 12 && std::atoi(argv[11]) > 0) {
        // dense-block fusion (build_blocks): each block's row-major matrix applied to the
        // amplitudes of its bits (local bit m <-> full-index bit bits[m])
        std::vector<qgpu::DenseBlock> blocks;
        if (qgpu::build_blocks(ops.data(), ops.size(), n, mats.data(), mats.size(), none.data(),
                               none.size(), std::atoi(argv[11]), std::atoi(argv[12]), &blocks) != QGPU_OK)
            return 1;
        const uint64_t dim = 1ull << n;
        std::vector<cd> st(dim);
        st[0] = 1.0;
        int maxk = 0, gates = 0;
        for (const qgpu::DenseBlock& b : blocks) {
            maxk = std::max(maxk, b.k);
            gates += b.gates;
            const size_t D = (size_t)1 << b.k;
            std::vector<uint64_t> off(D);
            uint64_t mask = 0;
            for (size_t c = 0; c < D; ++c) {
                uint64_t o = 0;
                for (int m = 0; m < b.k; ++m)
                    if ((c >> m) & 1u) o |= 1ull << b.bits[m];
                off[c] = o;
                mask |= o;
            }
            std::vector<cd> x(D);
            for (uint64_t base = 0; base < dim; ++base) {
                if (base & mask) continue;
                for (size_t c = 0; c < D; ++c) x[c] = st[base | off[c]];
                for (size_t l = 0; l < D; ++l) {
                    cd y = 0.0;
                    for (size_t c = 0; c < D; ++c) y += b.M[l * D + c] * x[c];
                    st[base | off[l]] = y;
                }
            }
        }
        std::ofstream out(argv[5], std::ios::binary);
        out.write(reinterpret_cast<const char*>(st.data()), (std::streamsize)(dim * sizeof(cd)));
        std::printf("blocks %zu maxk %d gates %d\n", blocks.size(), maxk, gates);
        return 0;
    }
    qgpu::Plan plan;
    if (qgpu::build_plan(ops.data(), ops.size(), n, mats.data(), mats.size(), none.data(),
                         none.size(), opt, &plan) != QGPU_OK)
        return 1;
    if (argc > 9 && std::atoi(argv[9]) == 2) {  // plan listing: one line per pass
        for (const qgpu::Pass& p : plan.passes) {
            if (p.pair2 >= 0) {
                std::printf("pair2 bits %d %d %d %d pre %zu post %zu\n", p.bits[0], p.bits[1],
                            p.bits[2], p.bits[3], p.pre.size(), p.post.size());
            } else if (p.pair >= 0) {
                std::printf("pair bits %d %d\n", p.bits[0], p.bits[1]);
            } else if (p.xor_pass) {
                std::printf("xor terms %d\n", p.xp.nterms);
            } else if (p.custom >= 0) {
                std::printf("custom\n");
            } else {
                std::printf("tile bits");
                for (int m = 0; m < p.nbits; ++m) std::printf(" %d", p.bits[m]);
                std::printf(" cost %d steps", p.cost);
                for (const qgpu::DevStep& d : p.steps) {
                    std::printf(" %d", d.type);
                    if (d.type == qgpu::ST_TABLE) {
                        std::printf("[");
                        for (int f = 0; f < d.nfields; ++f)
                            std::printf("%s%d+%d", f ? "," : "", d.tab_shift[f], d.tab_width[f]);
                        std::printf(" cm %llx]", (unsigned long long)d.cm);
                    }
                }
                std::printf("\n");
            }
        }
        return 0;
    }
    if (argc > 9 && std::atoi(argv[9]) != 0) {  // plan only: report the pass counts
        int counts[4] = {0, 0, 0, 0};
        size_t folded = 0;
        for (const qgpu::Pass& p : plan.passes) {
            ++counts[p.pair2 >= 0 ? 3 : (p.pair >= 0 ? 0 : (p.xor_pass ? 2 : 1))];
            folded += p.pre.size() + p.post.size();
        }
        std::printf("passes %zu pair %d tile %d xor %d pair2 %d folded %zu\n", plan.passes.size(),
                    counts[0], counts[1], counts[2], counts[3], folded);
        return 0;
    }
    const uint64_t dim = 1ull << n;
    std::vector<cd> st(dim);
    st[0] = 1.0;
    int npair = 0, ntile = 0, nxor = 0, npair2 = 0, ncustom = 0;
    size_t nfolded = 0;
    // a 4x4 block on bits (hi, lo), local index 2 * bit(hi) + bit(lo)
    auto apply_block = [&](const qgpu::PairBlock& pb) {
        for (uint64_t g = 0; g < (dim >> 2); ++g) {
            const uint64_t b = insert_zero(insert_zero(g, pb.lo), pb.hi);
            const uint64_t idx[4] = {b, b | (1ull << pb.lo), b | (1ull << pb.hi),
                                     b | (1ull << pb.lo) | (1ull << pb.hi)};
            cd x[4], y[4];
            for (int j = 0; j < 4; ++j) x[j] = st[idx[j]];
            for (int r = 0; r < 4; ++r) {
                y[r] = 0.0;
                for (int c = 0; c < 4; ++c) y[r] += pb.m[r][c] * x[c];
            }
            for (int j = 0; j < 4; ++j) st[idx[j]] = y[j];
        }
    };
    // i -> i ^ f(i) for XOR terms (each an involution; the terms commute)
    auto apply_terms = [&](const std::vector<qgpu::XTerm>& ts) {
        if (ts.empty()) return;
        std::vector<cd> nx(dim);
        for (uint64_t i = 0; i < dim; ++i) {
            uint64_t f = 0;
            for (const qgpu::XTerm& t : ts) {
                const uint64_t c = i & t.cm;
                if (t.swap ? (c != 0 && c != t.cm) : (c == t.cm)) f |= t.flip;
            }
            nx[i] = st[i ^ f];
        }
        st.swap(nx);
    };
    for (const qgpu::Pass& p : plan.passes) {
        if (p.pair2 >= 0) {
            ++npair2;
            nfolded += p.pre.size() + p.post.size();
            uint64_t mask = 0;
            for (int m = 0; m < p.nbits; ++m) mask |= 1ull << p.bits[m];
            for (const auto* ts : {&p.pre, &p.post})
                for (const qgpu::XTerm& t : *ts)
                    if ((t.cm | t.flip) & ~mask) {
                        std::fprintf(stderr, "folded XOR term outside its tile\n");
                        return 5;
                    }
            apply_terms(p.pre);
            apply_block(plan.pairs[p.pair]);
            apply_block(plan.pairs[p.pair2]);
            apply_terms(p.post);
            continue;
        }
        if (p.custom >= 0) {
            // quantr's apply_gate with the None rule (simulation.rs:64-135): an output whose
            // local input had no image keeps its amplitude; the others take the products of the
            // inputs that have one (M column-major: M[j * 2^k + l] = image of input j at l)
            ++ncustom;
            const qgpu::LocalGate& g = plan.customs[p.custom];
            const size_t kd = (size_t)1 << g.k;
            std::vector<uint64_t> scatter(kd);
            uint64_t acting = 0;
            for (size_t l = 0; l < kd; ++l) {
                uint64_t off = 0;
                for (int m = 0; m < g.k; ++m)
                    if ((l >> (g.k - 1 - m)) & 1u) off |= 1ull << (n - 1 - g.wires[m]);
                scatter[l] = off;
                acting |= off;
            }
            std::vector<cd> x(kd), y(kd);
            for (uint64_t b = 0; b < dim; ++b) {
                if (b & acting) continue;
                for (size_t l = 0; l < kd; ++l) x[l] = st[b | scatter[l]];
                for (size_t l = 0; l < kd; ++l) {
                    if (g.none[l]) {
                        y[l] = x[l];
                        continue;
                    }
                    y[l] = 0.0;
                    for (size_t j = 0; j < kd; ++j)
                        if (!g.none[j]) y[l] += g.M[j * kd + l] * x[j];
                }
                for (size_t l = 0; l < kd; ++l) st[b | scatter[l]] = y[l];
            }
            continue;
        }
        if (p.pair >= 0) {
            ++npair;
            const qgpu::PairBlock& pb = plan.pairs[p.pair];
            for (uint64_t g = 0; g < (dim >> 2); ++g) {
                const uint64_t b = insert_zero(insert_zero(g, pb.lo), pb.hi);
                const uint64_t idx[4] = {b, b | (1ull << pb.lo), b | (1ull << pb.hi),
                                         b | (1ull << pb.lo) | (1ull << pb.hi)};
                cd x[4], y[4];
                for (int j = 0; j < 4; ++j) x[j] = st[idx[j]];
                for (int r = 0; r < 4; ++r) {
                    y[r] = 0.0;
                    for (int c = 0; c < 4; ++c) y[r] += pb.m[r][c] * x[c];
                }
                for (int j = 0; j < 4; ++j) st[idx[j]] = y[j];
            }
            continue;
        }
        if (p.xor_pass) {
            ++nxor;
            const qgpu::XorPerm& xp = p.xp;
            for (uint64_t i = 0; i < dim; ++i) {
                uint64_t f = 0;
                for (int e = 0; e < xp.nterms; ++e) {
                    if (xp.grouped[e] == 1) {
                        const uint64_t c = i & xp.cm[e];
                        f |= xp.shift[e] > 0 ? (c >> xp.shift[e]) : (c << -xp.shift[e]);
                    } else if (xp.grouped[e] == 2) {
                        if (__builtin_popcountll(i & xp.cm[e]) == 1) f |= xp.cm[e];
                    } else if ((i & xp.cm[e]) == xp.cm[e]) {
                        f |= xp.tbit[e];
                    }
                }
                const uint64_t j = i ^ f;
                if (j > i) std::swap(st[i], st[j]);
            }
            continue;
        }
        ++ntile;
        const int K = p.nbits, T = 1 << K;
        std::vector<uint64_t> off(T);
        for (int j = 0; j < T; ++j) {
            uint64_t o = 0;
            for (int m = 0; m < K; ++m)
                if ((j >> m) & 1) o |= 1ull << p.bits[m];
            off[j] = o;
        }
        std::vector<cd> v(T);
        for (uint64_t g = 0; g < (dim >> K); ++g) {
            uint64_t b = g;
            for (int m = 0; m < K; ++m) b = insert_zero(b, p.bits[m]);
            for (int j = 0; j < T; ++j) v[j] = st[b | off[j]];
            for (const qgpu::DevStep& s : p.steps) apply_step(s, p, plan, v, b, off);
            for (int j = 0; j < T; ++j) st[b | off[j]] = v[j];
        }
    }
    std::ofstream out(argv[5], std::ios::binary);
    out.write(reinterpret_cast<const char*>(st.data()), (std::streamsize)(dim * sizeof(cd)));
    std::printf("passes %zu pair %d tile %d xor %d pair2 %d folded %zu custom %d\n",
                plan.passes.size(), npair, ntile, nxor, npair2, nfolded, ncustom);
    return 0;
}
