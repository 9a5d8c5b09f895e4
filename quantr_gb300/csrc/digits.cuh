// digits.cuh — the fixed-point digit arithmetic of the tensor-core pair passes (digits.cu),
// shared by the kernels and the host emulation (tests/cpp/digits_host.cu).
//
// Digit layout (a register layout of complex128 handles, used inside runs of pair passes): a
// 16-byte amplitude slot holds the real and imaginary parts as X = round(x 2^Sx), |X| <= 2^54,
// stored offset-binary as U = X + 2^55 in eight base-128 digits u_0..u_7 (7 bits each),
// interleaved: byte 2i = digit i of the real part, byte 2i + 1 = digit i of the imaginary part.
//
// One pass maps each 16-amplitude tile by a 16 x 16 complex matrix, in real form a 32 x 32 matrix
// r with R = round(r 2^56) split into balanced base-128 digits rho_0..rho_7 (|rho_j| <= 64 for
// j < 7, |rho_7| <= 256). The byte permute that turns a digit u into BF16 gives a = 128 + u
// exactly (exponent byte 0x43, the digit as the mantissa), so the tensor cores compute, per
// weight w = i + j, D_w = sum_{i+j=w} sum_k a_i[k] rho_j[k][c]: products of integers below 2^15,
// sums kept below 2^22 (checked on the host per pass), hence exact in the F32 accumulator.
// Then sum_w D_w 128^w = Y + (2^55 + 128 G) S_c with Y = sum_k X_k R_kc, G = sum_i 128^i and
// S_c = sum_k R_kc, and the output digits are those of
//   U' = floor((sum_w D_w 128^w + K_c) / 128^8) mod 128^8,  K_c = 2^111 + 2^55 - (2^55 + 128 G) S_c,
// i.e. X' = round(Y / 2^56), rebuilt by a carry chain over the weights. Weights below 5 are not
// formed (their total is below 2^51, 1/32 of the output's last place); the carry out of weights
// 5..7 is taken in float arithmetic (off by at most one last place). Per pass the error is at
// most ~2 units of 2^-Sx (about 1.1e-16 for Sx = 54), independent of the amplitudes' size.
#pragma once

#include <stdint.h>

namespace qgpu {
namespace dg {

constexpr int DIGITS = 8;                  // base-128 digits per real part (56 bits)
constexpr int WMIN = 5;                    // lowest digit-pair weight the MMAs form
constexpr int WMAX = 14;
constexpr int NW = WMAX - WMIN + 1;        // 10 accumulated weights
constexpr int SX_UNIT = 54;                // scale of a register whose amplitudes are at most 1
constexpr uint32_t MAGIC_BITS = 0x4B400000u;  // 1.5 * 2^23: x + MAGIC has x in its low bits
constexpr float MAGIC_F = 12582912.0f;
constexpr int64_t OFFSET = 1ll << 55;
constexpr int64_t XMAX = 1ll << 54;        // largest |X| a digit register holds
constexpr int KAP = 9;                     // carry constants per output real (see chain())
constexpr int32_t DBOUND = 1 << 22;        // |D_w| must stay below this (exact magic conversion)
constexpr int AMAX_LOW = 255;              // largest BF16 digit operand a = 128 + u ...
constexpr int AMAX_TOP = 224;              // ... and for the top digit (U < 3 2^54 + 2)

// Byte permute (PTX prmt, default mode; selectors here never set a nibble's top bit).
__host__ __device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
#ifdef __CUDA_ARCH__
    return __byte_perm(a, b, sel);
#else
    const uint64_t v = ((uint64_t)b << 32) | a;
    uint32_t r = 0;
    for (int k = 0; k < 4; ++k) r |= (uint32_t)((v >> (8 * ((sel >> (4 * k)) & 7u))) & 0xFFu) << (8 * k);
    return r;
#endif
}

__host__ __device__ __forceinline__ uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}
__host__ __device__ __forceinline__ float fma_rn(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
__host__ __device__ __forceinline__ float add_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

// A-operand word of digit i from a slot word holding digits (2m, 2m + 1): BF16 pair
// (128 + re digit, 128 + im digit), the real part in the low half.
__host__ __device__ __forceinline__ uint32_t a_word(uint32_t slot_word, int odd) {
    return prmt(slot_word, 0x43434343u, odd ? 0x4342u : 0x4140u);
}

// Byte offset of element (row, k) of a K-major BF16 operand (8-row x 16-byte core matrices, K
// core matrices 128 bytes apart, 8-row groups sbo apart), no swizzle.
__host__ __device__ __forceinline__ uint32_t op_off(int row, int k, uint32_t sbo) {
    return (uint32_t)((row % 8) * 16 + (k % 8) * 2 + (k / 8) * 128) + (uint32_t)(row / 8) * sbo;
}

// Slot of the digit layout from two offset-binary integers (real, imaginary).
__host__ __device__ __forceinline__ void pack_digits(uint64_t ur, uint64_t ui, uint32_t w[4]) {
    for (int m = 0; m < 4; ++m) {
        const uint32_t r0 = (uint32_t)(ur >> (14 * m)) & 127u, i0 = (uint32_t)(ui >> (14 * m)) & 127u;
        const uint32_t r1 = (uint32_t)(ur >> (14 * m + 7)) & 127u, i1 = (uint32_t)(ui >> (14 * m + 7)) & 127u;
        w[m] = r0 | (i0 << 8) | (r1 << 16) | (i1 << 24);
    }
}
__host__ __device__ __forceinline__ void unpack_digits(const uint32_t w[4], uint64_t& ur, uint64_t& ui) {
    ur = 0;
    ui = 0;
    for (int m = 0; m < 4; ++m) {
        ur |= (uint64_t)(w[m] & 127u) << (14 * m) | (uint64_t)((w[m] >> 16) & 127u) << (14 * m + 7);
        ui |= (uint64_t)((w[m] >> 8) & 127u) << (14 * m) | (uint64_t)((w[m] >> 24) & 127u) << (14 * m + 7);
    }
}

// Output word m of an amplitude from the chain values of positions 8 + 2m (p) and 9 + 2m (q),
// real and imaginary: bytes (re_p, im_p, re_q, im_q), each the value's low 7 bits.
__host__ __device__ __forceinline__ uint32_t out_word(int32_t pr, int32_t pi, int32_t qr, int32_t qi) {
    const uint32_t x = prmt((uint32_t)pr, (uint32_t)pi, 0x0040u);
    const uint32_t y = prmt((uint32_t)qr, (uint32_t)qi, 0x4000u);
    return ((x & 0x0000FFFFu) | (y & 0xFFFF0000u)) & 0x7F7F7F7Fu;
}

// Carry chain of one output real. The accumulators start at MAGIC_F (one MMA of a ones column
// against a row of MAGIC_F seeds them), so d[0..9] = MAGIC_F + D_5 .. MAGIC_F + D_14 exactly
// (|D_w| < 2^22) and their bits are MAGIC_BITS + D_w. kap[] holds the constants: kap[0] = bits
// of (float)(k5 + 128 k6 + 16384 k7 - 2^20 - 16513 MAGIC_F) (the low part, taken in float),
// kap[1] = k8 - 2 MAGIC_BITS, kap[2 + p - 9] = k_p - MAGIC_BITS for p = 9..14, kap[8] = k15 (k_p:
// the base-128 digits of K_c mod 2^112). t[0..7] receive the chain values of positions 8..15;
// their low 7 bits are the output digits. The kernels run the same operations.
__host__ __device__ __forceinline__ float chain_low(float d5, float d6, float d7, int32_t kap0) {
    float lo = add_rn(d5, u2f((uint32_t)kap0));
    lo = fma_rn(d6, 128.0f, lo);
    lo = fma_rn(d7, 16384.0f, lo);
    return fma_rn(lo, 1.0f / 2097152.0f, MAGIC_F);  // its bits: MAGIC + floor(low / 2^21) (+-1)
}
__host__ __device__ __forceinline__ int32_t chain_first(float d8, float low, int32_t kap1) {
    return (int32_t)(f2u(d8) + f2u(low) + (uint32_t)kap1);
}
__host__ __device__ __forceinline__ int32_t chain_next(float dp, int32_t prev, int32_t kapp) {
    return (int32_t)(f2u(dp) + (uint32_t)kapp + (uint32_t)(prev >> 7));
}
__host__ __device__ __forceinline__ void chain(const float d[NW], const int32_t kap[KAP], int32_t t[8]) {
    const float low = chain_low(d[0], d[1], d[2], kap[0]);
    t[0] = chain_first(d[3], low, kap[1]);
    for (int p = 9; p <= 14; ++p) t[p - 8] = chain_next(d[p - WMIN], t[p - 9], kap[2 + p - 9]);
    t[7] = kap[8] + (t[6] >> 7);
}

// The MMAs of one block: digit i of A times matrix digits j in [jmin, jend) into the weights
// i + j (N = 32 (jend - jmin) output columns), all accumulating onto the MAGIC_F seed. Every
// pair with i + j >= WMIN appears once (49 pairs), and each digit of A is read by one step.
struct MmaStep {
    int i, jmin, jend;
};
constexpr int NSTEPS = 8;
__host__ __device__ __forceinline__ MmaStep mma_step(int s) {
    const MmaStep tab[NSTEPS] = {{5, 0, 8}, {6, 0, 8}, {7, 0, 8}, {4, 1, 8},
                                 {3, 2, 8}, {2, 3, 8}, {1, 4, 8}, {0, 5, 8}};
    return tab[s];
}

}  // namespace dg
}  // namespace qgpu
