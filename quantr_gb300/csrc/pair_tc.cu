// pair_tc.cu — double pair passes (two 4x4 blocks on a 4-bit tile) of complex128 registers on the
// fifth-generation tensor cores.
//
// A double pair pass maps every 16-amplitude tile by one 16 x 16 complex matrix (the two blocks
// and the slot permutations folded around them), in real form a 32 x 32 matrix R. The float-pair
// arithmetic of k_pair2 spends 364 FP32-pipe operations per amplitude on it; here the products go
// to the tensor cores through the fixed-point splitting of Ozaki et al. (2012):
//   * each tile is scaled by a power of two to its largest component and rounded to 48-bit
//     integers X (|X| < 2^47), split into six 8-bit slices x_i (x_5 signed), exact in BF16;
//   * R is rounded to 46-bit integers and split the same way (slices r_j, prepared on the host);
//   * sum_i sum_j x_i r_j 2^(8(i+j)) is accumulated per weight s = i + j in F32 on the tensor
//     cores: every product is an integer below 2^16 and every weight's sum stays below 2^24, so
//     the accumulation is exact (tests/cuda/tc_probe.cu checks that bit for bit). Weights s < 4
//     are dropped: 26 of the 36 slice products remain, and a host emulation puts the error at
//     2^-45 of the tile's largest amplitude (the 48/46-bit rounding of the inputs sets that floor);
//   * the seven weights are recombined into a float pair with TwoSum and rescaled.
//
// k_pair2_tc: 8 warps per CTA, two CTAs per SM (84 KB of shared memory each keeps a third out, so
// the two 256-column tensor-memory accumulators always fit), persistent over blocks of 128 tiles.
// Per block: every thread loads half a tile (8 amplitudes, resident float-pair layout), the two
// halves agree on the tile's exponent through shared memory, the slices go to the A operand in the
// K-major core-matrix layout; one thread issues 10 MMAs (M = 128 tiles, K = 32, N = 32..192
// weights x outputs) and commits; after a bounded wait each thread reads its row's 7 weights for
// its 8 amplitudes from tensor memory, recombines and stores them. The two CTAs of an SM overlap
// each other's loads, MMAs and recombination.
//
// Status: correct (parity tests at 11-16 qubits; 30 qubits: norm drift 2.6e-14, checksum within
// 1.4e-13 of the float-pair path) and 38 % fewer instructions than k_pair2, but slower on GB300
// (12.9 against 11.4 ms per 30-qubit pass, 13.2 before the split moved to the integer pipes):
// with 16 warps per SM and the phases of a block in
// sequence it is latency-bound (issue 33 %, tensor pipe 11 %, DRAM 31 %). A version that staged
// the next block through cp.async was slower still (16.1 ms). It stays opt-in (QGPU_PAIR2_TC=1)
// until the phases run warp-specialised and double-buffered.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>

#include "internal.cuh"
#include "plan.h"
#include "tc.cuh"

namespace qgpu {

constexpr int PTC_M = 128;                             // tiles per block (MMA rows)
constexpr int PTC_THREADS = 256;
constexpr int PTC_K = 192;                             // 6 input slices x 32 reals
constexpr int PTC_NB = 192;                            // B rows: 6 matrix slices x 32 outputs
constexpr uint32_t PTC_SBO_A = (PTC_K / 8) * 128;      // 8-row groups of A
constexpr uint32_t PTC_SBO_B = (32 / 8) * 128;         // 8-row groups of B (K = 32)
constexpr uint32_t PTC_A_BYTES = PTC_M * PTC_K * 2;    // 48 KB
constexpr uint32_t PTC_B_BYTES = PTC_NB * 32 * 2;      // 12 KB
constexpr uint32_t PTC_TCOLS = 256;                    // 7 weights x 32 columns, rounded up
constexpr size_t PTC_SMEM = 84 * 1024;                 // > 228 KB / 3: at most two CTAs per SM
constexpr uint32_t PTC_WAIT_LIMIT = 1u << 22;

struct PairTcArgs {
    uint64_t ntiles;                  // dim / 16, a multiple of 128
    int bits[4];                      // tile bits, ascending (local slot bit m <-> bits[m])
    int* err;
    uint32_t bimg[PTC_B_BYTES / 4];   // B slices in the shared-memory layout (BF16 pairs)
};

// byte offset of element (row, k) of a K-major BF16 operand whose 8-row groups are sbo apart
__host__ __device__ __forceinline__ uint32_t ptc_off(int row, int k, uint32_t sbo) {
    return (uint32_t)((row % 8) * 16 + (k % 8) * 2 + (k / 8) * 128) + (uint32_t)(row / 8) * sbo;
}

// an integer 0..255 as a float, exactly (the 2^23 bias trick, no conversion instruction)
__device__ __forceinline__ float byte_f(long long b) {
    return __int_as_float(0x4B000000 | (int)b) - 8388608.0f;
}
// a signed top slice -128..127
__device__ __forceinline__ float sbyte_f(long long b) {
    return __int_as_float(0x4B000000 | (int)(b + 128)) - 8388736.0f;
}
__device__ __forceinline__ float pow2f(int e) {  // 2^e for -126 <= e <= 127
    return __int_as_float((e + 127) << 23);
}

// the float pair h + l scaled by f1 f2 (powers of two) and rounded to a 48-bit integer
__device__ __forceinline__ long long fixed48(float h, float l, float f1, float f2) {
    return __float2ll_rn((h * f1) * f2) + __float2ll_rn((l * f1) * f2);
}
// x 2^k rounded to the nearest integer (ties away from zero) for |x 2^k| < 2^47, from the
// float's bits on the integer pipes instead of the float-to-int64 conversion: the 24-bit
// mantissa shifted left, or right with the half added first. Measured in k_pair2_tc at 30
// qubits: 12.93 against 13.15 ms per launch with the conversions; k_pair2_ws keeps them (this
// form raises its spills).
__host__ __device__ __forceinline__ long long scaled_int(float x, int k) {
#ifdef __CUDA_ARCH__
    const uint32_t b = __float_as_uint(x);
#else
    uint32_t b;
    memcpy(&b, &x, 4);
#endif
    const int e = (int)((b >> 23) & 0xFFu);
    if (e == 0) return 0;  // zero or below 2^-126 (the float pairs flush those)
    const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u);
    const int sh = e - 150 + k;  // x 2^k = m 2^sh
    long long v;
    if (sh >= 0) v = m << sh;
    else if (sh >= -24) v = (m + (1ll << (-sh - 1))) >> (-sh);
    else v = 0;
    return (b >> 31) ? -v : v;
}
// the float pair h + l times 2^k, rounded to a 48-bit integer (integer pipes)
__host__ __device__ __forceinline__ long long fixed48_bits(float h, float l, int k) {
    return scaled_int(h, k) + scaled_int(l, k);
}
// slice i (8 bits; slice 5 signed) of the real and imaginary parts, as one BF16 pair
__device__ __forceinline__ uint32_t slice_pair(long long xr, long long xi, int i);

// weight w of a recombination: (ah, al) += t 2^(8 w) in float pairs (TwoSum), both lanes
__device__ __forceinline__ void add_weight(u64& ah, u64& al, float dr, float di, int w) {
    const float sc = pow2f(8 * w);
    const u64 t = pmul(p2(dr, di), p2(sc, sc));  // exact: a power of two
    if (w == 0) {
        ah = t;
        al = 0;
        return;
    }
    const u64 s = padd(ah, t);
    const u64 bb = psub(s, ah);
    const u64 q = padd(psub(ah, psub(s, bb)), psub(t, bb));
    ah = s;
    al = padd(al, q);
}
// the recombined pair normalised (FastTwoSum) and scaled by g1 g2 (powers of two)
__device__ __forceinline__ ffp finish_pair(u64 ah, u64 al, u64 g1, u64 g2) {
    const u64 hh = padd(ah, al);
    const u64 ll = psub(al, psub(hh, ah));
    ffp r;
    r.h = pmul(pmul(hh, g1), g2);
    r.l = pmul(pmul(ll, g1), g2);
    return r;
}

__device__ __forceinline__ uint32_t bf16pair(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&p);
}

__device__ __forceinline__ uint32_t slice_pair(long long xr, long long xi, int i) {
    const float br = i < 5 ? byte_f((xr >> (8 * i)) & 0xFF) : sbyte_f(xr >> 40);
    const float bi = i < 5 ? byte_f((xi >> (8 * i)) & 0xFF) : sbyte_f(xi >> 40);
    return bf16pair(br, bi);
}

__global__ void __launch_bounds__(PTC_THREADS, 2) k_pair2_tc(double2* __restrict__ st,
                                                             const __grid_constant__ PairTcArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + PTC_A_BYTES;
    uint8_t* tail = sB + PTC_B_BYTES;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tail);
    uint32_t* slot = reinterpret_cast<uint32_t*>(tail + 16);
    int* sexp = reinterpret_cast<int*>(tail + 64);  // [2][128]: each half-tile's largest exponent
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = tid & (PTC_M - 1), half = tid >> 7;  // row == 32 (warp % 4) + lane

    for (int i = tid; i < (int)(PTC_B_BYTES / 4); i += PTC_THREADS)
        reinterpret_cast<uint32_t*>(sB)[i] = a.bimg[i];
    const uint64_t o0 = 1ull << a.bits[0], o1 = 1ull << a.bits[1], o2 = 1ull << a.bits[2],
                   o3 = 1ull << a.bits[3];
    auto slot_off = [&](int j) {
        return ((j & 1) ? o0 : 0) | ((j & 2) ? o1 : 0) | ((j & 4) ? o2 : 0) | ((j & 8) ? o3 : 0);
    };
    if (tid == 0) {
        mbar_init(smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::alloc(smem_u32(slot), PTC_TCOLS);
    fence_proxy_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    uint32_t phase = 0;
    bool failed = false;
    const uint64_t nblocks = a.ntiles / PTC_M;
    auto tile_base = [&](uint64_t blk) {
        return insert_zero(
            insert_zero(insert_zero(insert_zero(blk * PTC_M + row, a.bits[0]), a.bits[1]), a.bits[2]),
            a.bits[3]);
    };
    for (uint64_t blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
        const uint64_t base = tile_base(blk);
        ffp v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = ffr_load(st[base | slot_off(8 * half + u)]);
        int emax = 0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            float rh, ih;
            up2(v[u].h, rh, ih);
            emax = max(emax, (int)((__float_as_uint(rh) >> 23) & 0xFFu));
            emax = max(emax, (int)((__float_as_uint(ih) >> 23) & 0xFFu));
        }
        sexp[half * PTC_M + row] = emax;
        __syncthreads();
        emax = max(sexp[row], sexp[PTC_M + row]);
        // X = v 2^k with |X| < 2^47 (the tile's largest |h| is below 2^(emax - 126)), built from
        // the floats' bits (k can exceed the largest float exponent)
        const int k = 173 - emax;
        long long xr[8], xi[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            float rh, ih, rl, il;
            up2(v[u].h, rh, ih);
            up2(v[u].l, rl, il);
            xr[u] = fixed48_bits(rh, rl, k);
            xi[u] = fixed48_bits(ih, il, k);
        }
        // slices into A: row = tile, k = 32 i + 2 slot + (re, im); 16 bytes = 4 slots of one slice
#pragma unroll
        for (int i = 0; i < 6; ++i) {
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q] = slice_pair(xr[4 * g + q], xi[4 * g + q], i);
                const int kk = 32 * i + 2 * (8 * half + 4 * g);
                *reinterpret_cast<uint4*>(sA + ptc_off(row, kk, PTC_SBO_A)) =
                    make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        fence_proxy_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            // weight s = i + j lands in columns 32 (s - 4); x_4 (weights 4..9) initialises them,
            // x_5 adds weights 5..9 and initialises weight 10, x_0..x_3 add their weights >= 4
            auto mma = [&](int i, int jmin, int jend, int s0, bool init) {
                const uint32_t idesc = tc::idesc_bf16(PTC_M, 32 * (jend - jmin));
#pragma unroll
                for (int kk = 0; kk < 2; ++kk) {
                    const uint64_t ad =
                        tc::smem_desc(smem_u32(sA) + (uint32_t)(4 * i) * 128 + kk * 256, 128, PTC_SBO_A);
                    const uint64_t bd =
                        tc::smem_desc(smem_u32(sB) + (uint32_t)(4 * jmin) * PTC_SBO_B + kk * 256, 128,
                                      PTC_SBO_B);
                    tc::mma_bf16(tmem + (uint32_t)(32 * (s0 - 4)), ad, bd, idesc,
                                 (init && kk == 0) ? 0u : 1u);
                }
            };
            mma(4, 0, 6, 4, true);
            mma(5, 0, 5, 5, false);
            mma(5, 5, 6, 10, true);
            for (int i = 0; i < 4; ++i) mma(i, 4 - i, 6, 4, false);
            tc::commit(smem_u32(bar));
        }
        const bool ok = mbar_wait_bounded(smem_u32(bar), phase, PTC_WAIT_LIMIT);
        phase ^= 1u;
        tc::fence_after_sync();
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(a.err, 3);
            failed = true;
            break;
        }
        // recombine: value = 2^(-14 - k) sum_w D_w 2^(8 w), w = s - 4 = 0..6, smallest first
        u64 ah[8], al[8];
#pragma unroll
        for (int w = 0; w < 7; ++w) {
            float d[16];
            tc::ld16(tmem + lane_base + (uint32_t)(32 * w + 16 * half), d);
#pragma unroll
            for (int u = 0; u < 8; ++u) add_weight(ah[u], al[u], d[2 * u], d[2 * u + 1], w);
        }
        const int c = -14 - k;
        const u64 g1 = p2(pow2f(c / 2), pow2f(c / 2)), g2 = p2(pow2f(c - c / 2), pow2f(c - c / 2));
#pragma unroll
        for (int u = 0; u < 8; ++u)
            st[base | slot_off(8 * half + u)] = ffr_store(finish_pair(ah[u], al[u], g1, g2));
        tc::fence_before_sync();
    }
    if (failed) {  // let an MMA still in flight finish (bounded) before freeing its accumulator
        mbar_wait_bounded(smem_u32(bar), phase ^ 1u, PTC_WAIT_LIMIT);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::dealloc(tmem, PTC_TCOLS);
}

// ---- warp-specialised version (QGPU_PAIR2_TC=2) ---------------------------------------------
// Status: correct (the same parity tests), slower on GB300: 15.4 ms per 30-qubit pass against
// 13.2 (k_pair2_tc) and 11.4 (k_pair2). With one warp of each role per SM sub-partition every role
// is latency-bound; the splitting (64-bit conversions and integer slicing) is the longest.
// One CTA per SM with three roles and two of everything (A operand, tensor-memory accumulator),
// so that block b+1 is split while block b is in the MMAs and block b-1 is recombined:
//   warps 0-3  producers: one thread per tile row, all 16 amplitudes (the next block's loads are
//              in flight while this one is split), writes A[s] and the row's scale exponent;
//   warp 4     lane 0 issues the block's MMAs into accumulator s once A[s] is full and the
//              consumers have released accumulator s, waits for them (bounded) and releases A[s]
//              to the producers and the accumulator to the consumers;
//   warps 5-8  consumers: one thread per tile row (tensor-memory lanes 32 (warp % 4) + lane),
//              read the 7 weights, recombine, store, release the accumulator.
// Hand-offs are mbarrier arrive (release) / bounded try_wait (acquire) pairs, counted per buffer
// use: full[s] (128 producer arrivals), done[s] and empty[s] (the MMA thread), tfree[s] (128
// consumer arrivals). Any wait that runs out sets the error word and stops that role; the others
// then run out too, and the CTA frees its tensor memory after a final bounded wait.
constexpr int PWS_THREADS = 288;
constexpr uint32_t PWS_A_BYTES = PTC_A_BYTES;         // per buffer
constexpr uint32_t PWS_TCOLS = 512;                   // two accumulators of 256 columns
constexpr size_t PWS_SMEM = 2 * PWS_A_BYTES + PTC_B_BYTES + 4096;

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(PWS_THREADS, 1) k_pair2_ws(double2* __restrict__ st,
                                                             const __grid_constant__ PairTcArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA0 = sm;
    uint8_t* sB = sm + 2 * PWS_A_BYTES;
    uint8_t* tail = sB + PTC_B_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(tail);  // full[2], empty[2], done[2], tfree[2], mma
    uint32_t* slot = reinterpret_cast<uint32_t*>(tail + 128);
    int* abort_flag = reinterpret_cast<int*>(tail + 132);
    // [4][128] scale exponents k of blocks it & 3: the producers of block it may only write once the
    // consumers of block it - 4 have read (they released accumulator s before the MMAs of block
    // it - 2, which released A[s] to the producers of block it)
    int* sexp = reinterpret_cast<int*>(tail + 256);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t b_full = smem_u32(bars), b_empty = smem_u32(bars + 2), b_done = smem_u32(bars + 4),
                   b_tfree = smem_u32(bars + 6), b_mma = smem_u32(bars + 8);

    for (int i = tid; i < (int)(PTC_B_BYTES / 4); i += PWS_THREADS)
        reinterpret_cast<uint32_t*>(sB)[i] = a.bimg[i];
    const uint64_t o0 = 1ull << a.bits[0], o1 = 1ull << a.bits[1], o2 = 1ull << a.bits[2],
                   o3 = 1ull << a.bits[3];
    auto slot_off = [&](int j) {
        return ((j & 1) ? o0 : 0) | ((j & 2) ? o1 : 0) | ((j & 4) ? o2 : 0) | ((j & 8) ? o3 : 0);
    };
    auto tile_base = [&](uint64_t blk, int r) {
        return insert_zero(
            insert_zero(insert_zero(insert_zero(blk * PTC_M + r, a.bits[0]), a.bits[1]), a.bits[2]),
            a.bits[3]);
    };
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(b_full + 8 * s, PTC_M);
            mbar_init(b_empty + 8 * s, 1);
            mbar_init(b_done + 8 * s, 1);
            mbar_init(b_tfree + 8 * s, PTC_M);
        }
        mbar_init(b_mma, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) tc::alloc(smem_u32(slot), PWS_TCOLS);
    fence_proxy_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint64_t nblocks = a.ntiles / PTC_M;
    const uint64_t nmine = (nblocks > blockIdx.x) ? (nblocks - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    auto fail_now = [&]() {
        atomicExch(a.err, 4);
        atomicExch(abort_flag, 1);
    };
    auto aborted = [&]() { return *(volatile int*)abort_flag != 0; };

    if (warp < 4) {  // ---------------------------------------------------------- producers
        const int row = tid;
        ffp nv[16];
        if (nmine > 0) {
            const uint64_t b0 = tile_base(blockIdx.x, row);
#pragma unroll
            for (int j = 0; j < 16; ++j) nv[j] = ffr_load(st[b0 | slot_off(j)]);
        }
        for (uint64_t it = 0; it < nmine; ++it) {
            const int s = (int)(it & 1);
            ffp v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = nv[j];
            if (it + 1 < nmine) {  // the next block's loads fly while this one is split
                const uint64_t bn = tile_base(blockIdx.x + (it + 1) * gridDim.x, row);
#pragma unroll
                for (int j = 0; j < 16; ++j) nv[j] = ffr_load(st[bn | slot_off(j)]);
            }
            if (it >= 2 && !mbar_wait_bounded(b_empty + 8 * s, (uint32_t)(((it >> 1) - 1) & 1),
                                              PTC_WAIT_LIMIT)) {
                fail_now();
                break;
            }
            if (aborted()) break;
            int emax = 0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float rh, ih;
                up2(v[j].h, rh, ih);
                emax = max(emax, (int)((__float_as_uint(rh) >> 23) & 0xFFu));
                emax = max(emax, (int)((__float_as_uint(ih) >> 23) & 0xFFu));
            }
            const int k = 173 - emax;
            const float f1 = pow2f(k / 2), f2 = pow2f(k - k / 2);
            uint8_t* sA = sA0 + s * PWS_A_BYTES;
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {  // 4 slots (16 bytes of one slice) at a time
                long long xr[4], xi[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float rh, ih, rl, il;
                    up2(v[4 * c4 + q].h, rh, ih);
                    up2(v[4 * c4 + q].l, rl, il);
                    xr[q] = fixed48(rh, rl, f1, f2);
                    xi[q] = fixed48(ih, il, f1, f2);
                }
#pragma unroll
                for (int i = 0; i < 6; ++i) {
                    uint32_t w4[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) w4[q] = slice_pair(xr[q], xi[q], i);
                    *reinterpret_cast<uint4*>(sA + ptc_off(row, 32 * i + 8 * c4, PTC_SBO_A)) =
                        make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
            }
            sexp[(int)(it & 3) * PTC_M + row] = k;
            fence_proxy_async_shared();  // the generic-proxy writes of A become visible to the MMAs
            mbar_arrive(b_full + 8 * s);
        }
    } else if (warp == 4) {  // ----------------------------------------------------- MMA issue
        if (lane == 0) {
            uint32_t mph = 0;
            for (uint64_t it = 0; it < nmine; ++it) {
                const int s = (int)(it & 1);
                if (!mbar_wait_bounded(b_full + 8 * s, (uint32_t)((it >> 1) & 1), PTC_WAIT_LIMIT) ||
                    (it >= 2 && !mbar_wait_bounded(b_tfree + 8 * s, (uint32_t)(((it >> 1) - 1) & 1),
                                                   PTC_WAIT_LIMIT))) {
                    fail_now();
                    break;
                }
                tc::fence_after_sync();
                const uint32_t sa = smem_u32(sA0 + s * PWS_A_BYTES), acc = tmem + 256u * (uint32_t)s;
                auto mma = [&](int i, int jmin, int jend, int s0, bool init) {
                    const uint32_t idesc = tc::idesc_bf16(PTC_M, 32 * (jend - jmin));
#pragma unroll
                    for (int kk = 0; kk < 2; ++kk) {
                        const uint64_t ad = tc::smem_desc(sa + (uint32_t)(4 * i) * 128 + kk * 256, 128, PTC_SBO_A);
                        const uint64_t bd = tc::smem_desc(
                            smem_u32(sB) + (uint32_t)(4 * jmin) * PTC_SBO_B + kk * 256, 128, PTC_SBO_B);
                        tc::mma_bf16(acc + (uint32_t)(32 * (s0 - 4)), ad, bd, idesc,
                                     (init && kk == 0) ? 0u : 1u);
                    }
                };
                mma(4, 0, 6, 4, true);
                mma(5, 0, 5, 5, false);
                mma(5, 5, 6, 10, true);
                for (int i = 0; i < 4; ++i) mma(i, 4 - i, 6, 4, false);
                tc::commit(b_mma);
                const bool ok = mbar_wait_bounded(b_mma, mph, PTC_WAIT_LIMIT);
                mph ^= 1u;
                if (!ok) {
                    fail_now();
                    mbar_wait_bounded(b_mma, mph ^ 1u, PTC_WAIT_LIMIT);  // let it drain (bounded)
                    break;
                }
                tc::fence_after_sync();
                mbar_arrive(b_empty + 8 * s);  // A[s] may be rewritten
                mbar_arrive(b_done + 8 * s);   // accumulator s holds block it
            }
        }
    } else {  // ------------------------------------------------------------------- consumers
        const int row = 32 * (warp & 3) + lane;
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        for (uint64_t it = 0; it < nmine; ++it) {
            const int s = (int)(it & 1);
            if (!mbar_wait_bounded(b_done + 8 * s, (uint32_t)((it >> 1) & 1), PTC_WAIT_LIMIT)) {
                fail_now();
                break;
            }
            tc::fence_after_sync();
            const int k = sexp[(int)(it & 3) * PTC_M + row];
            const uint64_t base = tile_base(blockIdx.x + it * gridDim.x, row);
            const int c = -14 - k;
            const u64 g1 = p2(pow2f(c / 2), pow2f(c / 2)), g2 = p2(pow2f(c - c / 2), pow2f(c - c / 2));
#pragma unroll 1
            for (int half = 0; half < 2; ++half) {
                u64 ah[8], al[8];
#pragma unroll
                for (int w = 0; w < 7; ++w) {
                    float d[16];
                    tc::ld16(tmem + 256u * (uint32_t)s + lane_base + (uint32_t)(32 * w + 16 * half), d);
#pragma unroll
                    for (int u = 0; u < 8; ++u) add_weight(ah[u], al[u], d[2 * u], d[2 * u + 1], w);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    st[base | slot_off(8 * half + u)] = ffr_store(finish_pair(ah[u], al[u], g1, g2));
            }
            tc::fence_before_sync();
            mbar_arrive(b_tfree + 8 * s);  // accumulator s may be overwritten
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 4) tc::dealloc(tmem, PWS_TCOLS);
}

namespace {

using cd = std::complex<double>;

uint16_t bf16_exact(double v) {  // v: an integer with |v| <= 256 (exact in BF16)
    const float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (uint16_t)(u >> 16);
}

// full-index offset -> local slot index of a tile
int slot_of(const int bits[4], uint64_t off) {
    int j = 0;
    for (int m = 0; m < 4; ++m)
        if ((off >> bits[m]) & 1ull) j |= 1 << m;
    return j;
}

}  // namespace

bool pair2_tc_supported(const qgpu_handle* h) {
    return h->precision == QGPU_C128 && (h->dim >> 4) % PTC_M == 0;
}

// The pass as one 16 x 16 complex matrix over the tile's physical slots, in real form, split into
// the B operand's six BF16 slices (shared-memory layout).
static void build_pair_tc_image(const Plan& plan, const Pass& ps, const uint64_t pre_off[16],
                                const uint64_t post_off[16], uint32_t* img) {
    const PairBlock* blk[2] = {&plan.pairs[ps.pair], &plan.pairs[ps.pair2]};
    int lo[2], hi[2];  // local bit positions of each block
    for (int b = 0; b < 2; ++b)
        for (int m = 0; m < 4; ++m) {
            if (ps.bits[m] == blk[b]->lo) lo[b] = m;
            if (ps.bits[m] == blk[b]->hi) hi[b] = m;
        }
    auto lidx = [&](int b, int j) { return 2 * ((j >> hi[b]) & 1) + ((j >> lo[b]) & 1); };
    cd M16[16][16];
    for (int j = 0; j < 16; ++j)
        for (int c = 0; c < 16; ++c) M16[j][c] = 0.0;
    for (int j = 0; j < 16; ++j)        // logical output slot
        for (int c = 0; c < 16; ++c) {  // logical input slot
            const cd kv = blk[0]->m[lidx(0, j)][lidx(0, c)] * blk[1]->m[lidx(1, j)][lidx(1, c)];
            M16[slot_of(ps.bits, post_off[j])][slot_of(ps.bits, pre_off[c])] = kv;
        }
    uint16_t* h16 = reinterpret_cast<uint16_t*>(img);
    std::memset(img, 0, PTC_B_BYTES);
    for (int r = 0; r < 32; ++r)
        for (int q = 0; q < 32; ++q) {
            const cd m = M16[r / 2][q / 2];
            const int o = r & 1, i = q & 1;  // [[Re, -Im], [Im, Re]][o][i]
            const double val = (o == i) ? m.real() : (o == 0 ? -m.imag() : m.imag());
            const long long X = std::llround(std::ldexp(val, 46));
            for (int sl = 0; sl < 6; ++sl) {
                const long long b = sl < 5 ? ((X >> (8 * sl)) & 0xFF) : (X >> 40);
                h16[ptc_off(32 * sl + r, q, PTC_SBO_B) / 2] = bf16_exact((double)b);
            }
        }
}

int launch_pair2_tc(qgpu_handle* h, const Plan& plan, const Pass& ps, const uint64_t pre_off[16],
                    const uint64_t post_off[16], int variant) {
    const cudaError_t attr = smem_opt_in((const void*)k_pair2_tc, PTC_SMEM);
    QGPU_CUDA(attr);
    const cudaError_t attr_ws = smem_opt_in((const void*)k_pair2_ws, PWS_SMEM);
    QGPU_CUDA(attr_ws);
    PairTcArgs a;
    std::memset(&a, 0, sizeof(a));
    a.ntiles = h->dim >> 4;
    for (int m = 0; m < 4; ++m) a.bits[m] = ps.bits[m];
    a.err = h->d_err;
    build_pair_tc_image(plan, ps, pre_off, post_off, a.bimg);
    if (variant == 2) {  // warp-specialised: one CTA per SM
        const uint64_t blocks =
            std::max<uint64_t>(1, std::min<uint64_t>(a.ntiles / PTC_M, (uint64_t)h->sm_count));
        k_pair2_ws<<<(unsigned)blocks, PWS_THREADS, PWS_SMEM, h->stream>>>((double2*)cur_state(h), a);
        QGPU_CHECK_LAUNCH("k_pair2_ws");
    } else {
        const uint64_t blocks =
            std::max<uint64_t>(1, std::min<uint64_t>(a.ntiles / PTC_M, (uint64_t)h->sm_count * 2));
        k_pair2_tc<<<(unsigned)blocks, PTC_THREADS, PTC_SMEM, h->stream>>>((double2*)cur_state(h), a);
        QGPU_CHECK_LAUNCH("k_pair2_tc");
    }
    h->launches++;
    h->h2d_bytes += sizeof(a);
    return QGPU_OK;
}

}  // namespace qgpu
