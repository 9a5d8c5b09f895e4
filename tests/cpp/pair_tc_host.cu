// pair_tc_host.cu — the arithmetic of k_pair2_tc emulated on the host with the library's own
// image builder (quantr_gb300/csrc/pair_tc.cu): random 4x4 unitaries on all three bit layouts of
// a tile, slot permutations folded before and after, tiles spread over 12 octaves of magnitude;
// the 48-bit splitting (the kernel's own integer split, checked against round-to-nearest), the 26
// slice products of weight >= 4 (integer sums, as the tensor cores accumulate them exactly), the
// recombination and the rescaling must reproduce the complex128 product within 1e-12 of the
// tile's largest amplitude. Needs no GPU; exit code 0 on success.
#include "pair_tc.cu"

namespace qgpu {
int cuda_fail(cudaError_t, const char*) { return QGPU_ERR_CUDA; }
int fail(int code, const std::string&) { return code; }
}  // namespace qgpu
#include <cstdio>
#include <random>
using namespace qgpu;
static float bf16_to_f(uint16_t b) { uint32_t u = (uint32_t)b << 16; float f; memcpy(&f, &u, 4); return f; }
int main() {
    std::mt19937_64 rng(7);
    std::normal_distribution<double> nd;
    int fails = 0, split_fails = 0;
    for (int trial = 0; trial < 200; ++trial) {
        Plan plan;
        plan.pairs.resize(2);
        // random 4x4 unitaries via Gram-Schmidt
        for (int b = 0; b < 2; ++b) {
            cd m[4][4];
            for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) m[r][c] = cd(nd(rng), nd(rng));
            for (int c = 0; c < 4; ++c) {
                for (int p = 0; p < c; ++p) { cd d = 0; for (int r = 0; r < 4; ++r) d += std::conj(m[r][p]) * m[r][c]; for (int r = 0; r < 4; ++r) m[r][c] -= d * m[r][p]; }
                double nn = 0; for (int r = 0; r < 4; ++r) nn += std::norm(m[r][c]); nn = std::sqrt(nn);
                for (int r = 0; r < 4; ++r) m[r][c] /= nn;
            }
            for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) plan.pairs[b].m[r][c] = m[r][c];
        }
        Pass ps;
        ps.nbits = 4;
        int bits[4] = {1, 5, 9, 20};
        for (int m = 0; m < 4; ++m) ps.bits[m] = bits[m];
        const int part = trial % 3;  // which local bit pairs with bit 0
        int A1 = part + 1, B0 = part == 0 ? 2 : 1, B1 = part == 2 ? 2 : 3;
        plan.pairs[0].lo = bits[0]; plan.pairs[0].hi = bits[A1];
        plan.pairs[1].lo = bits[B0]; plan.pairs[1].hi = bits[B1];
        ps.pair = trial & 1 ? 1 : 0; ps.pair2 = 1 - ps.pair;
        // pre / post permutations: a CNot inside the tile (control local bit 3, target local 0)
        uint64_t pre_off[16], post_off[16];
        for (int j = 0; j < 16; ++j) {
            uint64_t o = 0; for (int m = 0; m < 4; ++m) if ((j >> m) & 1) o |= 1ull << bits[m];
            pre_off[j] = o; post_off[j] = o;
            if (trial % 2 && (o >> bits[3] & 1)) pre_off[j] = o ^ (1ull << bits[0]);
            if (trial % 4 == 3 && (o >> bits[1] & 1)) post_off[j] = o ^ (1ull << bits[2]);
        }
        static uint32_t img[PTC_B_BYTES / 4];
        build_pair_tc_image(plan, ps, pre_off, post_off, img);
        const uint16_t* h16 = reinterpret_cast<const uint16_t*>(img);
        // random tile (physical slots), magnitudes over 12 octaves
        cd x[16];
        for (int s = 0; s < 16; ++s) x[s] = cd(nd(rng), nd(rng)) * std::exp(-std::fabs(nd(rng)) * 4);
        // reference: logical transform
        auto lidx = [&](int b, int j) { int lo = -1, hi = -1; for (int m = 0; m < 4; ++m) { if (bits[m] == plan.pairs[b].lo) lo = m; if (bits[m] == plan.pairs[b].hi) hi = m; } return 2 * ((j >> hi) & 1) + ((j >> lo) & 1); };
        auto slot_of2 = [&](uint64_t off) { int j = 0; for (int m = 0; m < 4; ++m) if ((off >> bits[m]) & 1) j |= 1 << m; return j; };
        cd yin[16], yout[16];
        for (int c = 0; c < 16; ++c) yin[c] = x[slot_of2(pre_off[c])];
        for (int j = 0; j < 16; ++j) { cd acc = 0; for (int c = 0; c < 16; ++c) acc += plan.pairs[0].m[lidx(0, j)][lidx(0, c)] * plan.pairs[1].m[lidx(1, j)][lidx(1, c)] * yin[c]; yout[j] = acc; }
        cd ref[16]; for (int j = 0; j < 16; ++j) ref[slot_of2(post_off[j])] = yout[j];
        // kernel arithmetic: float pairs of x, exponent, X, slices, weights, recombination
        float h[32], l[32];
        for (int s = 0; s < 16; ++s) {
            double re = x[s].real(), im = x[s].imag();
            h[2*s] = (float)re; l[2*s] = (float)(re - (double)h[2*s]);
            h[2*s+1] = (float)im; l[2*s+1] = (float)(im - (double)h[2*s+1]);
        }
        int emax = 0;
        for (int q = 0; q < 32; ++q) { uint32_t u; memcpy(&u, &h[q], 4); emax = std::max(emax, (int)((u >> 23) & 0xFF)); }
        const int k = 173 - emax;
        long long X[32];
        for (int q = 0; q < 32; ++q) {
            X[q] = fixed48_bits(h[q], l[q], k);  // k_pair2_tc's own integer split
            // against round-to-nearest in double (both parts are exact there): equal but at ties
            for (float f : {h[q], l[q]}) {
                const double e = std::ldexp((double)f, k), r = (double)scaled_int(f, k);
                if (std::fabs(r - e) > 0.5 || (std::fabs(r - e) == 0.5 && std::fabs(r) < std::fabs(e))) ++split_fails;
            }
        }
        double out[32];
        for (int r = 0; r < 32; ++r) {
            double D[7] = {0};
            for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) {
                if (i + j < 4) continue;
                double sum = 0;
                for (int q = 0; q < 32; ++q) {
                    const long long xi = i < 5 ? ((X[q] >> (8 * i)) & 0xFF) : (X[q] >> 40);
                    const double bj = bf16_to_f(h16[ptc_off(32 * j + r, q, PTC_SBO_B) / 2]);
                    sum += (double)xi * bj;
                }
                D[i + j - 4] += sum;
            }
            double v = 0; for (int w = 6; w >= 0; --w) v = v * 256.0 + D[w];
            out[r] = std::ldexp(v, -14 - k);
        }
        double maxref = 0, err = 0;
        for (int s = 0; s < 16; ++s) {
            maxref = std::max(maxref, std::abs(ref[s]));
            err = std::max(err, std::abs(cd(out[2*s], out[2*s+1]) - ref[s]));
        }
        double xmax = 0; for (int s = 0; s < 16; ++s) xmax = std::max(xmax, std::abs(x[s]));
        if (err > 1e-12 * xmax) { ++fails; if (fails < 5) printf("trial %d err %.3e xmax %.3e\n", trial, err, xmax); }
        if (trial < 3) printf("trial %d rel err %.3e\n", trial, err / xmax);
    }
    // the split's corner cases: exact ties (away from zero), the largest and smallest shifts
    for (int k : {0, 1, 23, 24, 60, 150}) {
        for (float f : {0.5f, -0.5f, 1.5f, -2.5f, 1.0f, 0x1.fffffep-1f, 0x1.8p-24f, 0x1.p-25f, 3.0e-38f}) {
            const double e = std::ldexp((double)f, k);
            if (std::fabs(e) >= 0x1p47) continue;
            const double want = std::copysign(std::floor(std::fabs(e) + 0.5), e);
            if ((double)scaled_int(f, k) != want) {
                ++split_fails;
                printf("scaled_int(%a, %d) = %lld, want %.0f\n", f, k, scaled_int(f, k), want);
            }
        }
    }
    printf("split fails %d\n", split_fails);
    fails += split_fails;
    printf("fails %d\n", fails);
    return fails != 0;
}
