// digits_host.cu — the arithmetic of the digit pair passes (quantr_gb300/csrc/digits.cu) emulated
// on the host with the library's own pieces: its image builder (matrix digits in the B operand's
// shared-memory layout and the carry constants), the byte permutes that form the A operand, the
// MMA step table (every digit pair of weight >= 5 exactly once), integer sums standing in for
// the tensor cores' exact F32 accumulation, and the carry chain. Checked against the complex128
// product: random 16 x 16 unitaries and Kronecker products of 4 x 4 blocks with slot
// permutations, tiles of unit norm spread over many magnitudes, single-amplitude tiles, |x| = 1
// entries and the zero tile. Bar: |emulated - exact| <= 4 units of 2^-sx per real (the output is
// rounded to that grid). Also checks that the exactness bound rejects an oversized matrix and
// that the conversions' digit packing round-trips. Needs no GPU; exit code 0 on success.
#include "digits.cu"

namespace qgpu {
int cuda_fail(cudaError_t, const char*) { return QGPU_ERR_CUDA; }
int fail(int code, const std::string&) { return code; }
}  // namespace qgpu

#include <cstdio>
#include <random>

using namespace qgpu;
using cdd = std::complex<double>;

static float bf16_to_f(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

static void random_unitary(std::mt19937_64& rng, int d, std::vector<cdd>& m) {  // row-major
    std::normal_distribution<double> nd;
    m.assign((size_t)d * d, 0.0);
    for (auto& v : m) v = cdd(nd(rng), nd(rng));
    for (int c = 0; c < d; ++c) {  // Gram-Schmidt on columns
        for (int p = 0; p < c; ++p) {
            cdd dot = 0;
            for (int r = 0; r < d; ++r) dot += std::conj(m[r * d + p]) * m[r * d + c];
            for (int r = 0; r < d; ++r) m[r * d + c] -= dot * m[r * d + p];
        }
        double nn = 0;
        for (int r = 0; r < d; ++r) nn += std::norm(m[r * d + c]);
        nn = std::sqrt(nn);
        for (int r = 0; r < d; ++r) m[r * d + c] /= nn;
    }
}

// one tile through the emulated pass; returns the largest error in units of 2^-sx
static double run_tile(const cdd M[16][16], const uint32_t* bimg, const int32_t (*kap)[dg::KAP],
                       const cdd x[16], int sx, bool* bound_ok) {
    // digit layout of the tile
    uint32_t slot[16][4];
    for (int j = 0; j < 16; ++j) {
        const int64_t xr = std::llround(std::ldexp(x[j].real(), sx)), xi = std::llround(std::ldexp(x[j].imag(), sx));
        dg::pack_digits((uint64_t)(xr + dg::OFFSET), (uint64_t)(xi + dg::OFFSET), slot[j]);
        uint64_t ur, ui;
        dg::unpack_digits(slot[j], ur, ui);
        if ((int64_t)ur - dg::OFFSET != xr || (int64_t)ui - dg::OFFSET != xi) return 1e30;  // round trip
    }
    // A operand values a_i[k] (k = 2 slot + part) from the kernel's byte permute
    int64_t A[dg::DIGITS][32];
    for (int i = 0; i < dg::DIGITS; ++i)
        for (int j = 0; j < 16; ++j) {
            const uint32_t w = dg::a_word(slot[j][i >> 1], i & 1);
            const float re = bf16_to_f((uint16_t)(w & 0xFFFF)), im = bf16_to_f((uint16_t)(w >> 16));
            A[i][2 * j] = (int64_t)re;
            A[i][2 * j + 1] = (int64_t)im;
            if ((float)A[i][2 * j] != re || (float)A[i][2 * j + 1] != im || re < 128 || im < 128) return 1e30;
        }
    // matrix digits back from the B image
    auto rho = [&](int k, int c, int j) {
        const uint16_t* h16 = reinterpret_cast<const uint16_t*>(bimg);
        return (int64_t)bf16_to_f(h16[dg::op_off(32 * j + c, k, DG_SBO_B) / 2]);
    };
    // the MMA steps: integer sums per weight (the tensor cores' F32 accumulation is exact below 2^24)
    int64_t D[32][dg::NW];
    int cover[dg::DIGITS][dg::DIGITS] = {};
    for (int c = 0; c < 32; ++c)
        for (int w = 0; w < dg::NW; ++w) D[c][w] = 0;
    for (int s = 0; s < dg::NSTEPS; ++s) {
        const dg::MmaStep ms = dg::mma_step(s);
        for (int j = ms.jmin; j < ms.jend; ++j) {
            if (ms.i + j < dg::WMIN) return 1e30;
            cover[ms.i][j]++;
            for (int c = 0; c < 32; ++c) {
                int64_t sum = 0;
                for (int k = 0; k < 32; ++k) sum += A[ms.i][k] * rho(k, c, j);
                D[c][ms.i + j - dg::WMIN] += sum;
            }
        }
    }
    for (int i = 0; i < dg::DIGITS; ++i)
        for (int j = 0; j < dg::DIGITS; ++j)
            if (cover[i][j] != (i + j >= dg::WMIN ? 1 : 0)) return 1e30;
    for (int c = 0; c < 32; ++c)
        for (int w = 0; w < dg::NW; ++w)
            if (D[c][w] >= dg::DBOUND || D[c][w] <= -dg::DBOUND) *bound_ok = false;
    // carry chains and output digits
    double worst = 0.0;
    for (int u = 0; u < 16; ++u) {
        int32_t t[2][8];
        for (int part = 0; part < 2; ++part) {
            const int c = 2 * u + part;
            float d[dg::NW];
            for (int w = 0; w < dg::NW; ++w) d[w] = (float)(D[c][w] + (int64_t)dg::MAGIC_F);  // seeded accumulator
            dg::chain(d, kap[c], t[part]);
        }
        uint32_t w4[4];
        for (int m = 0; m < 4; ++m) w4[m] = dg::out_word(t[0][2 * m], t[1][2 * m], t[0][2 * m + 1], t[1][2 * m + 1]);
        uint64_t ur, ui;
        dg::unpack_digits(w4, ur, ui);
        // exact reference in units of 2^-sx: the rounded inputs times M, in extended precision
        long double wr = 0.0L, wi = 0.0L;
        for (int j = 0; j < 16; ++j) {
            const long double xr = (long double)std::llround(std::ldexp(x[j].real(), sx));
            const long double xi = (long double)std::llround(std::ldexp(x[j].imag(), sx));
            const long double mr = M[u][j].real(), mi = M[u][j].imag();
            wr += mr * xr - mi * xi;
            wi += mr * xi + mi * xr;
        }
        const long double gr = (long double)((int64_t)ur - dg::OFFSET);
        const long double gi = (long double)((int64_t)ui - dg::OFFSET);
        worst = std::max(worst, (double)std::fabs(gr - wr));
        worst = std::max(worst, (double)std::fabs(gi - wi));
    }
    return worst;
}

int main() {
    std::mt19937_64 rng(11);
    std::normal_distribution<double> nd;
    std::uniform_real_distribution<double> ud(0.0, 1.0);
    int fails = 0, rejected = 0;
    double worst = 0.0;
    static uint32_t bimg[DG_B_BYTES / 4];
    static int32_t kap[32][dg::KAP];
    for (int trial = 0; trial < 120; ++trial) {
        cdd M[16][16];
        if (trial % 3 == 0) {  // a general 16 x 16 unitary
            std::vector<cdd> u;
            random_unitary(rng, 16, u);
            for (int r = 0; r < 16; ++r)
                for (int c = 0; c < 16; ++c) M[r][c] = u[r * 16 + c];
        } else {  // Kronecker product of two 4 x 4 blocks, slots permuted before and after
            std::vector<cdd> a, b;
            random_unitary(rng, 4, a);
            random_unitary(rng, 4, b);
            int pin[16], pout[16];
            for (int j = 0; j < 16; ++j) pin[j] = pout[j] = j;
            std::shuffle(pin, pin + 16, rng);
            if (trial % 3 == 2) std::shuffle(pout, pout + 16, rng);
            for (int r = 0; r < 16; ++r)
                for (int c = 0; c < 16; ++c)
                    M[pout[r]][pin[c]] = a[(r & 3) * 4 + (c & 3)] * b[(r >> 2) * 4 + (c >> 2)];
            if (trial % 7 == 1)  // a permutation with phases (entries of modulus 1)
                for (int r = 0; r < 16; ++r)
                    for (int c = 0; c < 16; ++c) M[r][c] = (pin[c] == r) ? std::polar(1.0, 0.3 * r) : 0.0;
        }
        if (!dg_build_image(M, bimg, kap)) {
            ++rejected;
            continue;
        }
        for (int tt = 0; tt < 40; ++tt) {
            cdd x[16];
            const int kind = tt % 5;
            double nn = 0;
            for (int j = 0; j < 16; ++j) {
                x[j] = cdd(nd(rng), nd(rng)) * std::ldexp(1.0, -(int)(ud(rng) * 40));
                nn += std::norm(x[j]);
            }
            for (int j = 0; j < 16; ++j) x[j] /= std::sqrt(nn);
            if (kind == 1) {  // one amplitude of modulus 1
                for (int j = 0; j < 16; ++j) x[j] = 0.0;
                x[tt % 16] = std::polar(1.0, ud(rng) * 6.28);
            } else if (kind == 2) {  // +-1 on the real axis
                for (int j = 0; j < 16; ++j) x[j] = 0.0;
                x[(tt * 7) % 16] = (tt & 8) ? -1.0 : 1.0;
            } else if (kind == 3) {  // all zero
                for (int j = 0; j < 16; ++j) x[j] = 0.0;
            } else if (kind == 4) {  // tiny amplitudes (the tile of a large register)
                for (int j = 0; j < 16; ++j) x[j] *= std::ldexp(1.0, -15);
            }
            bool bound_ok = true;
            const double e = run_tile(M, bimg, kap, x, dg::SX_UNIT, &bound_ok);
            worst = std::max(worst, e);
            if (e > 4.0 || !bound_ok) {
                if (fails < 5) std::printf("trial %d tile %d: error %.3g units, bound %d\n", trial, tt, e, (int)bound_ok);
                ++fails;
            }
        }
    }
    // a matrix whose weights would overflow the exact range must be rejected
    // every real-form entry 2 - 64 (128^1 + ... + 128^6) / 2^56: top digit 256, digits 1..6 -64,
    // so weight 7 could reach 32 (255 * 256 + 5 * 255 * 64 + 255 * 64) > 2^22
    int64_t R = (int64_t)1 << 57;
    for (int j = 1; j <= 6; ++j) R -= 64ll << (7 * j);
    const double v = std::ldexp((double)R, -56);
    cdd big[16][16];
    for (int r = 0; r < 16; ++r)
        for (int c = 0; c < 16; ++c) big[r][c] = cdd(v, -v);
    const bool big_ok = dg_build_image(big, bimg, kap);
    std::printf("worst %.3f units rejected %d fails %d big_rejected %d\n", worst, rejected, fails, (int)!big_ok);
    if (big_ok) ++fails;
    if (rejected) ++fails;  // unitary passes must all be accepted
    std::printf("fails %d\n", fails);
    return fails ? 1 : 0;
}
