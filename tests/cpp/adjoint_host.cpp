// adjoint_host.cpp — the adjoint sweep's host-side algebra (quantr_gb300/csrc/plan.cpp) checked
// without a GPU:
//   * inverse_op: every non-Custom gate times its inverse is the identity (all 24 kinds, on
//     wires and controls of a 3-qubit register, through the library's own tabulation);
//   * pauli_run: for random runs of single-wire gates (every one-wire kind, random angles), the
//     undo matrix inverts the run, and each rotation's gradient formed from the Pauli sums
//     Im <lambda| s |phi> (s = X, Y, Z, -I) with the run's coefficients equals the central
//     difference of the energy <psi|H|psi> (random Hermitian H, random start state);
//   * affine_tables: a run of CNot / X / Swap as one gather through 8-bit chunk tables equals
//     the gates applied one by one;
//   * adj_group_passes: the grouped sweep's partition of a run's wires into tiles.
// Prints "fails <n>"; exit code 0 when there are none.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>

#include "../../quantr_gb300/csrc/plan.h"

namespace qgpu {
int fail(int code, const std::string& msg) {
    std::fprintf(stderr, "error: %s\n", msg.c_str());
    return code;
}
}  // namespace qgpu

using qgpu::cd;
using M2 = std::array<cd, 4>;  // row-major 2x2

static qgpu_op make_op(int kind, int target, std::initializer_list<int> controls, double param,
                       int k) {
    qgpu_op op;
    std::memset(&op, 0, sizeof(op));
    op.kind = kind;
    op.target = target;
    op.n_controls = (int32_t)controls.size();
    int i = 0;
    for (int c : controls) op.controls[i++] = c;
    op.param = param;
    op.k = k;
    return op;
}

static M2 mat_of(const qgpu_op& op) {
    qgpu::LocalGate g;
    if (qgpu::tabulate(op, 1, nullptr, 0, nullptr, 0, &g) != QGPU_OK) std::exit(2);
    M2 m;
    for (int l = 0; l < 2; ++l)
        for (int j = 0; j < 2; ++j) m[2 * l + j] = g.M[j * 2 + l];  // M: column-major images
    return m;
}

static M2 mul(const M2& x, const M2& y) {
    return {x[0] * y[0] + x[1] * y[2], x[0] * y[1] + x[1] * y[3], x[2] * y[0] + x[3] * y[2],
            x[2] * y[1] + x[3] * y[3]};
}

// adj_group_passes: every wire in exactly one pass; each tile at most max_bits bits of the
// register, holding the pass's wires and bits 0..4; a run over all n wires takes
// 1 + ceil((n - 11) / 6) passes from 12 qubits (one pass up to 11).
static int check_group_passes(std::mt19937_64& rng) {
    int fails = 0;
    for (int n = 1; n <= 34; ++n)
        for (int trial = 0; trial < 40; ++trial) {
            std::vector<int> bits;
            for (int b = 0; b < n; ++b)
                if (trial == 0 || (rng() & 1)) bits.push_back(b);
            std::shuffle(bits.begin(), bits.end(), rng);
            const auto passes = qgpu::adj_group_passes(bits, n, qgpu::ADJ_GROUP_TILE_BITS);
            std::vector<int> seen(bits.size(), 0);
            for (const auto& p : passes) {
                const uint64_t mask = p.first;
                const int kmax = std::min(n, qgpu::ADJ_GROUP_TILE_BITS);
                const uint64_t low = (1ull << std::min(n, 5)) - 1;
                if (__builtin_popcountll(mask) > kmax || (mask & low) != low || (mask >> n) != 0 ||
                    p.second.empty())
                    ++fails;
                for (size_t w : p.second) {
                    if (w >= bits.size() || !((mask >> bits[w]) & 1ull)) ++fails;
                    else ++seen[w];
                }
            }
            for (int c : seen)
                if (c != 1) ++fails;
            if (trial == 0) {
                const size_t want = n <= 11 ? 1 : 1 + (size_t)((n - 11 + 5) / 6);
                if (passes.size() != want) {
                    std::printf("n=%d: %zu passes, expected %zu\n", n, passes.size(), want);
                    ++fails;
                }
            }
        }
    return fails;
}

int main() {
    int fails = 0;
    {
        std::mt19937_64 grng(19);
        const int gf = check_group_passes(grng);
        std::printf("group_passes fails %d\n", gf);
        fails += gf;
    }
    // inverse_op on every kind, 3 qubits: U^dag U = I through the tabulated images
    {
        const int n = 3;
        std::vector<qgpu_op> ops;
        for (int kind = QGPU_GATE_H; kind <= QGPU_GATE_PHASE; ++kind) ops.push_back(make_op(kind, 1, {}, 0.7, 0));
        ops.push_back(make_op(QGPU_GATE_CR, 0, {2}, -1.3, 0));
        ops.push_back(make_op(QGPU_GATE_CRK, 2, {0}, 0.0, 3));
        ops.push_back(make_op(QGPU_GATE_CRK, 1, {2}, 0.0, 1));
        ops.push_back(make_op(QGPU_GATE_CZ, 2, {1}, 0.0, 0));
        ops.push_back(make_op(QGPU_GATE_CY, 0, {1}, 0.0, 0));
        ops.push_back(make_op(QGPU_GATE_CNOT, 1, {0}, 0.0, 0));
        ops.push_back(make_op(QGPU_GATE_SWAP, 2, {0}, 0.0, 0));
        ops.push_back(make_op(QGPU_GATE_TOFFOLI, 1, {2, 0}, 0.0, 0));
        for (const qgpu_op& op : ops) {
            qgpu::LocalGate a, b;
            if (qgpu::tabulate(op, n, nullptr, 0, nullptr, 0, &a) != QGPU_OK ||
                qgpu::tabulate(qgpu::inverse_op(op), n, nullptr, 0, nullptr, 0, &b) != QGPU_OK) {
                ++fails;
                continue;
            }
            const size_t d = (size_t)1 << a.k;
            double err = 0;
            bool same_wires = a.k == b.k;
            for (int m = 0; m < a.k && same_wires; ++m) same_wires = a.wires[m] == b.wires[m];
            for (size_t j = 0; j < d && same_wires; ++j)      // column j of B A
                for (size_t l = 0; l < d; ++l) {
                    cd s = 0;
                    for (size_t x = 0; x < d; ++x) s += b.M[x * d + l] * a.M[j * d + x];
                    err = std::max(err, std::abs(s - cd(l == j ? 1.0 : 0.0)));
                }
            if (!same_wires || err > 1e-14) {
                ++fails;
                std::printf("inverse_op kind %d: err %.3e\n", op.kind, err);
            }
        }
    }
    // pauli_run against central differences of the energy
    std::mt19937_64 rng(5);
    std::uniform_real_distribution<double> ang(-3.2, 3.2);
    std::normal_distribution<double> nd;
    const int one_wire[] = {QGPU_GATE_H, QGPU_GATE_X, QGPU_GATE_Y, QGPU_GATE_Z, QGPU_GATE_S,
                            QGPU_GATE_SDAG, QGPU_GATE_T, QGPU_GATE_TDAG, QGPU_GATE_X90,
                            QGPU_GATE_Y90, QGPU_GATE_MX90, QGPU_GATE_MY90, QGPU_GATE_RX,
                            QGPU_GATE_RY, QGPU_GATE_RZ, QGPU_GATE_PHASE};
    double worst = 0;
    int nrot = 0;
    for (int trial = 0; trial < 400; ++trial) {
        const int k = 1 + (int)(rng() % 8);
        std::vector<qgpu_op> ops;
        for (int q = 0; q < k; ++q) {
            // rotations three times as often as the others
            const int pick = (int)(rng() % 28);
            const int kind = pick < 12 ? one_wire[pick] : one_wire[12 + (pick - 12) % 4];
            ops.push_back(make_op(kind, 0, {}, ang(rng), 0));
        }
        std::vector<size_t> gw;
        for (int q = k - 1; q >= 0; --q) gw.push_back((size_t)q);
        qgpu::PauliRun pr;
        if (qgpu::pauli_run(ops.data(), gw, 1, &pr) != QGPU_OK) {
            ++fails;
            continue;
        }
        auto run = [&](const std::vector<qgpu_op>& o) {
            M2 U{cd(1), cd(0), cd(0), cd(1)};
            for (const qgpu_op& op : o) U = mul(mat_of(op), U);  // G_1 first
            return U;
        };
        const M2 U = run(ops);
        const M2 I = mul(pr.undo, U);
        const double uerr = std::max({std::abs(I[0] - 1.0), std::abs(I[1]), std::abs(I[2]),
                                      std::abs(I[3] - 1.0)});
        if (uerr > 1e-13) {
            ++fails;
            std::printf("trial %d: undo x run differs from I by %.3e\n", trial, uerr);
        }
        // random start state and Hermitian H
        cd p0[2] = {cd(nd(rng), nd(rng)), cd(nd(rng), nd(rng))};
        const double nrm = std::sqrt(std::norm(p0[0]) + std::norm(p0[1]));
        p0[0] /= nrm;
        p0[1] /= nrm;
        const double ha = nd(rng), hd = nd(rng);
        const cd hb(nd(rng), nd(rng));
        auto energy = [&](const M2& V) {
            const cd s0 = V[0] * p0[0] + V[1] * p0[1], s1 = V[2] * p0[0] + V[3] * p0[1];
            const cd h0 = ha * s0 + hb * s1, h1 = std::conj(hb) * s0 + hd * s1;
            return (std::conj(s0) * h0 + std::conj(s1) * h1).real();
        };
        const cd ps[2] = {U[0] * p0[0] + U[1] * p0[1], U[2] * p0[0] + U[3] * p0[1]};
        const cd lam[2] = {ha * ps[0] + hb * ps[1], std::conj(hb) * ps[0] + hd * ps[1]};
        // Im <lambda| s |phi> for s = X, Y, Z, -I
        const cd sx = std::conj(lam[0]) * ps[1] + std::conj(lam[1]) * ps[0];
        const cd sy = std::conj(lam[0]) * (cd(0, -1) * ps[1]) + std::conj(lam[1]) * (cd(0, 1) * ps[0]);
        const cd sz = std::conj(lam[0]) * ps[0] - std::conj(lam[1]) * ps[1];
        const cd si = -(std::conj(lam[0]) * ps[0] + std::conj(lam[1]) * ps[1]);
        const double S[5] = {0, sx.imag(), sy.imag(), sz.imag(), si.imag()};
        for (const auto& r : pr.rots) {
            ++nrot;
            double g = 0;
            for (int m = 1; m <= 4; ++m) {
                g += r.second[m] * S[m];
                if (r.second[m] != 0.0 && !pr.need[m]) ++fails;
            }
            const double h = 1e-6;
            std::vector<qgpu_op> up = ops, dn = ops;
            up[r.first].param += h;
            dn[r.first].param -= h;
            const double fd = (energy(run(up)) - energy(run(dn))) / (2 * h);
            const double e = std::fabs(g - fd);
            worst = std::max(worst, e);
            if (e > 1e-8) {
                ++fails;
                std::printf("trial %d op %zu (kind %d): gradient %.12f, central difference %.12f\n",
                            trial, r.first, ops[r.first].kind, g, fd);
            }
        }
    }
    std::printf("rotations %d, worst |gradient - central difference| %.3e\n", nrot, worst);

    // affine_tables: random runs of CNot / X / Swap (n = 3..17, chunks of 8 bits, a partial last
    // chunk); the one gather dst[y] = src[h(y)] equals the gates applied one by one through the
    // library's tabulated images; runs with any other gate are refused
    int gathers = 0;
    for (int trial = 0; trial < 60; ++trial) {
        const int n = 3 + trial % 15;
        const uint64_t dim = 1ull << n;
        std::vector<qgpu_op> ops;
        const int len = 1 + (int)(rng() % 12);
        for (int q = 0; q < len; ++q) {
            const int t = (int)(rng() % n);
            int c = (int)(rng() % (n - 1));
            if (c >= t) ++c;
            const int pick = (int)(rng() % 3);
            ops.push_back(pick == 0 ? make_op(QGPU_GATE_X, t, {}, 0, 0)
                                    : make_op(pick == 1 ? QGPU_GATE_CNOT : QGPU_GATE_SWAP, t, {c}, 0, 0));
        }
        std::vector<uint64_t> tabs;
        uint64_t d = 0;
        if (!qgpu::affine_tables(ops.data(), ops.size(), n, &tabs, &d)) {
            ++fails;
            continue;
        }
        std::vector<cd> src(dim), ref(dim), nx(dim);
        for (uint64_t i = 0; i < dim; ++i) src[i] = cd((double)i, -0.5 * (double)i);
        ref = src;
        for (const qgpu_op& op : ops) {  // dense application of each gate's image
            qgpu::LocalGate g;
            if (qgpu::tabulate(op, n, nullptr, 0, nullptr, 0, &g) != QGPU_OK) std::exit(2);
            const size_t kd = (size_t)1 << g.k;
            std::vector<uint64_t> sc(kd);
            uint64_t acting = 0;
            for (size_t l = 0; l < kd; ++l) {
                uint64_t off = 0;
                for (int m = 0; m < g.k; ++m)
                    if ((l >> (g.k - 1 - m)) & 1u) off |= 1ull << (n - 1 - g.wires[m]);
                sc[l] = off;
                acting |= off;
            }
            std::fill(nx.begin(), nx.end(), cd(0));
            for (uint64_t b = 0; b < dim; ++b) {
                if (b & acting) continue;
                for (size_t j = 0; j < kd; ++j)
                    for (size_t l = 0; l < kd; ++l) nx[b | sc[l]] += g.M[j * kd + l] * ref[b | sc[j]];
            }
            ref.swap(nx);
        }
        const int nch = (n + 7) / 8;
        bool ok = tabs.size() == (size_t)nch * 256;
        for (uint64_t y = 0; y < dim && ok; ++y) {
            uint64_t x = d;
            for (int c = 0; c < nch; ++c) x ^= tabs[(size_t)c * 256 + ((y >> (8 * c)) & 255u)];
            ok = x < dim && src[x] == ref[y];
        }
        if (!ok) {
            ++fails;
            std::printf("affine_tables: run %d (n %d, %d gates) differs\n", trial, n, len);
        }
        ++gathers;
    }
    {
        std::vector<qgpu_op> mixed = {make_op(QGPU_GATE_CNOT, 1, {0}, 0, 0), make_op(QGPU_GATE_TOFFOLI, 2, {0, 1}, 0, 0)};
        std::vector<uint64_t> tabs;
        uint64_t d = 0;
        if (qgpu::affine_tables(mixed.data(), mixed.size(), 3, &tabs, &d)) ++fails;
        mixed[1] = make_op(QGPU_GATE_H, 2, {}, 0, 0);
        if (qgpu::affine_tables(mixed.data(), mixed.size(), 3, &tabs, &d)) ++fails;
    }
    std::printf("affine gathers %d\n", gathers);
    std::printf("fails %d\n", fails);
    return fails != 0;
}
