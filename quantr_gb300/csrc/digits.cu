// digits.cu — complex128 double pair passes on the fifth-generation tensor cores in fixed-point
// base-128 digits (the arithmetic is described in digits.cuh).
//
// Inside a run of pair passes the register stays in the digit layout; k_dg_from converts into it
// (from complex128 or the resident float pairs) before the run and k_dg_to converts back after
// it. A pass k_dg2 maps every 16-amplitude tile by one 16 x 16 complex matrix (two fused 4 x 4
// blocks with the XOR terms around them folded in, or one block on two of the tile's bits): the
// same work as k_pair2, which spends 364 FP32-pipe operations per amplitude on float-pair Dot2
// sums. Here the products go to the tensor cores (49 digit-pair MMAs per tile, exact F32
// accumulation) and the CUDA cores only permute bytes into BF16 operands (8 byte permutes per
// amplitude) and run the carry chains (about 70 operations per amplitude).
//
// k_dg2: one CTA per SM, persistent over blocks of 128 tiles, warp-specialised:
//   warp 0      lane 0 issues the MMAs of a block into the one 320-column accumulator (10 weights
//               x 32 output reals): two seed MMAs (every column := 1.5 * 2^23), then for each digit
//               i of A one MMA per K half over the matrix digits j it pairs with (M = 128 tiles,
//               K = 16, N = 32 per digit, up to 256), so every A slice is read once per block;
//   warps 1-4   converters, one tile row each: copy the tile's 16 slots (digit layout) to shared
//               memory with cp.async two blocks ahead, byte-permute them into the A operand
//               (K = 8 digits x 32 reals, BF16) of one of two buffers;
//   warps 5-20  consumers: every block, each thread one tile row and output reals 4 s .. 4 s + 3 and
//               16 + 4 s .. 16 + 4 s + 3: read their 10 weights from tensor memory (all loads, then
//               one wait), run the carry chains, pack the digits and store the 4 amplitudes.
// Hand-offs are mbarriers: a_full[2] (128 converter arrivals), a_empty[2] (MMA commit after the
// block), acc_full (MMA commit), acc_empty (512 consumer arrivals once their tensor-memory loads
// completed). Every wait is bounded: a wait that runs out sets the error word and an abort flag
// that stops every role; the MMA thread drains its MMAs (bounded) before the CTA frees its
// tensor memory. Shared memory per block read by the tensor cores: A 80 KB, B 100 KB (the chunked
// form, which re-read A per 16 outputs, was bound by shared-memory bandwidth).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>

#include "digits.cuh"
#include "internal.cuh"
#include "plan.h"
#include "tc.cuh"

namespace qgpu {

constexpr int DG_M = 128;                               // tiles per block (MMA rows)
constexpr int DG_THREADS = 672;                         // 21 warps: 6 on some SM sub-partition, so 80 registers
constexpr int DG_K = 256;                               // A: 8 digits x 32 reals
constexpr uint32_t DG_SBO_A = (DG_K / 8) * 128;         // 4096: 8-row groups of A
constexpr uint32_t DG_A_BYTES = DG_M * DG_K * 2;        // 64 KB per buffer
constexpr uint32_t DG_SBO_B = (32 / 8) * 128;           // 512: 8-row groups of B (K = 32)
constexpr uint32_t DG_B_BYTES = 256 * 32 * 2;           // 16 KB: rows 32 j + c (8 digits x 32 outputs)
constexpr uint32_t DG_ACC_COLS = 32 * dg::NW;           // 320 columns: weight-major, 32 outputs each
constexpr uint32_t DG_TCOLS = 512;
constexpr int DG_CONSUMERS = 512;                       // 16 consumer warps
constexpr uint32_t DG_STAGE_BYTES = DG_M * 16 * 16;    // 32 KB: one block's slots
constexpr uint32_t DG_SBO_SEED = (16 / 8) * 128;      // 256: 8-row groups of the K = 16 seed operands
constexpr uint32_t DG_ONE_BYTES = DG_M * 16 * 2;        // 4 KB: A of the seed MMA (a ones column)
constexpr uint32_t DG_SEED_N = DG_ACC_COLS / 2;         // two seed MMAs of N = 160
constexpr uint32_t DG_MAGIC_BYTES = DG_SEED_N * 16 * 2;  // 5 KB: B of the seed MMA (MAGIC_F row)
constexpr size_t DG_SMEM = 2 * DG_A_BYTES + DG_B_BYTES + 2 * DG_STAGE_BYTES + DG_ONE_BYTES +
                           DG_MAGIC_BYTES + 2048 + 32 * dg::KAP * 4;
constexpr uint32_t DG_WAIT_LIMIT = 1u << 22;

struct DgArgs {
    uint64_t nblocks;                  // dim / 16 / 128
    int bits[4];                       // tile bits, ascending (slot bit m <-> bits[m])
    int* err;
    int32_t kap[32][dg::KAP];          // carry constants per output real
    uint32_t bimg[DG_B_BYTES / 4];     // matrix digits, both chunks, shared-memory layout
};

// ---- tensor-memory loads without the wait (the wait names the registers it completes) ------
__device__ __forceinline__ void tm_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tm_wait(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                   "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                   "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}
__device__ __forceinline__ void dg_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tm_ld4(uint32_t taddr, uint32_t (&r)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}

// Consumer side of one job for 4 output reals (2 amplitudes: re, im, re, im) of one tile row:
// the 10 weights of each from tensor memory at taddr (column 32 w' + output), all loads issued
// before the one wait; arrives on `release` (when not 0) once they completed; then the carry chains (kap:
// the outputs' constants in shared memory, [KAP][32] from the first of them, the same for every
// lane) and the packed slots.
__device__ __forceinline__ void dg_consume4(uint32_t taddr, const int32_t* __restrict__ kap,
                                            uint32_t release, uint4 (&out)[2]) {
    uint32_t d[dg::NW][4];
#pragma unroll
    for (int w = 0; w < dg::NW; ++w) tm_ld4(taddr + (uint32_t)(32 * w), d[w]);
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(d[0][0]), "+r"(d[0][1]), "+r"(d[0][2]), "+r"(d[0][3]), "+r"(d[1][0]),
                   "+r"(d[1][1]), "+r"(d[1][2]), "+r"(d[1][3]), "+r"(d[2][0]), "+r"(d[2][1]),
                   "+r"(d[2][2]), "+r"(d[2][3]), "+r"(d[3][0]), "+r"(d[3][1]), "+r"(d[3][2]),
                   "+r"(d[3][3]), "+r"(d[4][0]), "+r"(d[4][1]), "+r"(d[4][2]), "+r"(d[4][3]),
                   "+r"(d[5][0]), "+r"(d[5][1]), "+r"(d[5][2]), "+r"(d[5][3]), "+r"(d[6][0]),
                   "+r"(d[6][1]), "+r"(d[6][2]), "+r"(d[6][3]), "+r"(d[7][0]), "+r"(d[7][1]),
                   "+r"(d[7][2]), "+r"(d[7][3])
                 :
                 : "memory");
    asm volatile("" : "+r"(d[8][0]), "+r"(d[8][1]), "+r"(d[8][2]), "+r"(d[8][3]), "+r"(d[9][0]),
                      "+r"(d[9][1]), "+r"(d[9][2]), "+r"(d[9][3])::"memory");
    if (release) {
        tc::fence_before_sync();
        dg_arrive(release);
    }
    // the four chains run position by position; kap is [KAP][32] in shared memory, so one 16-byte
    // load gives constant i of the thread's four outputs
    const int4* k4 = reinterpret_cast<const int4*>(kap);
    auto kc = [](const int4& v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; };
    float low[4];
    int32_t tp[4], tq[4];
    uint32_t w4[2][4];
    {
        const int4 k0 = k4[0];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            low[c] = dg::chain_low(__uint_as_float(d[0][c]), __uint_as_float(d[1][c]), __uint_as_float(d[2][c]), kc(k0, c));
        const int4 k1 = k4[8];
#pragma unroll
        for (int c = 0; c < 4; ++c) tp[c] = dg::chain_first(__uint_as_float(d[3][c]), low[c], kc(k1, c));
    }
#pragma unroll
    for (int p = 9; p <= 15; p += 2) {  // positions p (odd) and p + 1 (even, or none after 15)
        const int4 kp = k4[8 * (2 + p - 9)];
#pragma unroll
        for (int c = 0; c < 4; ++c)
            tq[c] = p < 15 ? dg::chain_next(__uint_as_float(d[p - dg::WMIN][c]), tp[c], kc(kp, c))
                           : kc(kp, c) + (tp[c] >> 7);
#pragma unroll
        for (int u = 0; u < 2; ++u)
            w4[u][(p - 9) / 2] = dg::out_word(tp[2 * u], tp[2 * u + 1], tq[2 * u], tq[2 * u + 1]);
        if (p < 15) {
            const int4 kn = k4[8 * (2 + p + 1 - 9)];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                tp[c] = p + 1 < 15 ? dg::chain_next(__uint_as_float(d[p + 1 - dg::WMIN][c]), tq[c], kc(kn, c))
                                   : kc(kn, c) + (tq[c] >> 7);
        }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) out[u] = make_uint4(w4[u][0], w4[u][1], w4[u][2], w4[u][3]);
}

__global__ void __launch_bounds__(DG_THREADS, 1) k_dg2(uint4* __restrict__ st,
                                                       const __grid_constant__ DgArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + 2 * DG_A_BYTES;
    uint8_t* sStage = sB + DG_B_BYTES;  // 2 x 32 KB: converters' staging of the state
    uint8_t* sOne = sStage + 2 * DG_STAGE_BYTES;
    uint8_t* sMagic = sOne + DG_ONE_BYTES;
    uint8_t* tail = sMagic + DG_MAGIC_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(tail);  // a_full[2] a_empty[2] acc_full[3] acc_empty[3] drain
    uint32_t* slot = reinterpret_cast<uint32_t*>(tail + 128);
    int* abort_flag = reinterpret_cast<int*>(tail + 132);
    int32_t* skap = reinterpret_cast<int32_t*>(tail + 2048);  // carry constants [KAP][32]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t b_afull = smem_u32(bars), b_aempty = smem_u32(bars + 2),
                   b_accfull = smem_u32(bars + 4), b_accempty = smem_u32(bars + 7),
                   b_drain = smem_u32(bars + 10);

    for (int i = tid; i < (int)(DG_B_BYTES / 4); i += DG_THREADS)
        reinterpret_cast<uint32_t*>(sB)[i] = a.bimg[i];
    for (int i = tid; i < 32 * dg::KAP; i += DG_THREADS) skap[i] = a.kap[i % 32][i / 32];
    // seed operands: A = e_0 in every row (BF16 1.0 at k = 0), B = MAGIC_F at k = 0 in every row
    for (int i = tid; i < (int)((DG_ONE_BYTES + DG_MAGIC_BYTES) / 2); i += DG_THREADS) {
        const bool one = i < (int)(DG_ONE_BYTES / 2);
        const int e = one ? i : i - (int)(DG_ONE_BYTES / 2);
        const int row = e / 16, k = e % 16;
        const uint16_t v = k != 0 ? 0 : (one ? 0x3F80 : 0x4B40);  // BF16 1.0 / 1.5 * 2^23
        *reinterpret_cast<uint16_t*>((one ? sOne : sMagic) + dg::op_off(row, k, DG_SBO_SEED)) = v;
    }
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(b_afull + 8 * s, DG_M);
            mbar_init(b_aempty + 8 * s, 1);
        }
        mbar_init(b_accfull, 1);
        mbar_init(b_accempty, DG_CONSUMERS);
        mbar_init(b_drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::alloc(smem_u32(slot), DG_TCOLS);
    fence_proxy_async_shared();  // B (generic-proxy writes) visible to the MMAs
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint64_t nmine =
        (a.nblocks > blockIdx.x) ? (a.nblocks - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const uint64_t o0 = 1ull << a.bits[0], o1 = 1ull << a.bits[1], o2 = 1ull << a.bits[2],
                   o3 = 1ull << a.bits[3];
    auto slot_off = [&](int j) {
        return ((j & 1) ? o0 : 0) | ((j & 2) ? o1 : 0) | ((j & 4) ? o2 : 0) | ((j & 8) ? o3 : 0);
    };
    auto tile_base = [&](uint64_t blk, int r) {
        return insert_zero(
            insert_zero(insert_zero(insert_zero(blk * DG_M + r, a.bits[0]), a.bits[1]), a.bits[2]),
            a.bits[3]);
    };
    auto fail_now = [&](int code) {
        atomicExch(a.err, code);
        atomicExch(abort_flag, 1);
    };
    auto aborted = [&]() { return *(volatile int*)abort_flag != 0; };

    if (warp == 0) {  // ------------------------------------------------------------ MMA issue
        if (lane == 0) {
            bool issued = false;
            const uint64_t a_desc0 = tc::smem_desc(smem_u32(sA), 128, DG_SBO_A);
            const uint64_t b_desc0 = tc::smem_desc(smem_u32(sB), 128, DG_SBO_B);
            const uint64_t one_desc = tc::smem_desc(smem_u32(sOne), 128, DG_SBO_SEED);
            const uint64_t magic_desc = tc::smem_desc(smem_u32(sMagic), 128, DG_SBO_SEED);
            for (uint64_t it = 0; it < nmine; ++it) {
                const int s = (int)(it & 1);
                if (!mbar_wait_bounded(b_afull + 8 * s, (uint32_t)((it >> 1) & 1), DG_WAIT_LIMIT)) {
                    fail_now(5);
                    break;
                }
                if (it >= 1 && !mbar_wait_bounded(b_accempty, (uint32_t)((it - 1) & 1), DG_WAIT_LIMIT)) {
                    fail_now(6);
                    break;
                }
                if (aborted()) break;
                tc::fence_after_sync();
                const uint32_t acc = tmem;
                // descriptors: base + the operand's byte offset / 16 (the start-address field)
                const uint64_t ad0 = a_desc0 + (uint64_t)((s * DG_A_BYTES) >> 4);
                tc::mma_bf16(acc, one_desc, magic_desc, tc::idesc_bf16(DG_M, (int)DG_SEED_N), 0u);
                tc::mma_bf16(acc + DG_SEED_N, one_desc, magic_desc, tc::idesc_bf16(DG_M, (int)DG_SEED_N), 0u);
#pragma unroll
                for (int k = 0; k < dg::NSTEPS; ++k) {
                    const dg::MmaStep ms = dg::mma_step(k);
                    const uint32_t idesc = tc::idesc_bf16(DG_M, 32 * (ms.jend - ms.jmin));
#pragma unroll
                    for (int kk = 0; kk < 2; ++kk)
                        tc::mma_bf16(acc + (uint32_t)(32 * (ms.i + ms.jmin - dg::WMIN)),
                                     ad0 + (uint64_t)(((4 * ms.i + 2 * kk) * 128) >> 4),
                                     b_desc0 + (uint64_t)((ms.jmin * 2048 + kk * 256) >> 4), idesc, 1u);
                }
                issued = true;
                tc::commit(b_accfull);
                tc::commit(b_aempty + 8 * s);
            }
            if (issued) {  // every MMA completed before the tensor memory is freed
                tc::commit(b_drain);
                if (!mbar_wait_bounded(b_drain, 0, DG_WAIT_LIMIT)) atomicExch(a.err, 7);
            }
        }
        __syncwarp();
    } else if (warp <= 4) {  // ------------------------------------------------------ converters
        // Each thread copies its tile row's 16 slots global -> shared with cp.async into one of two
        // stages (slot j of row r at stage[j * 128 + r]: conflict-free for the warp), two blocks
        // ahead of the block it converts, so no registers are held while the loads fly.
        const int r = tid - 32;
        auto issue = [&](uint64_t it) {
            const uint64_t b0 = tile_base(blockIdx.x + it * gridDim.x, r);
            uint8_t* dst = sStage + (uint32_t)(it & 1) * DG_STAGE_BYTES;
#pragma unroll
            for (int j = 0; j < 16; ++j)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst + (j * DG_M + r) * 16)),
                             "l"(st + (b0 | slot_off(j)))
                             : "memory");
        };
        if (nmine > 0) issue(0);
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (nmine > 1) issue(1);
        asm volatile("cp.async.commit_group;" ::: "memory");
        for (uint64_t it = 0; it < nmine; ++it) {
            const int s = (int)(it & 1);
            asm volatile("cp.async.wait_group 1;" ::: "memory");  // block it's group is complete
            if (it >= 2 && !mbar_wait_bounded(b_aempty + 8 * s, (uint32_t)(((it >> 1) - 1) & 1), DG_WAIT_LIMIT)) {
                fail_now(8);
                break;
            }
            if (aborted()) break;
            const uint8_t* src = sStage + (uint32_t)s * DG_STAGE_BYTES;
            uint8_t* A = sA + (uint32_t)s * DG_A_BYTES;
#pragma unroll
            for (int g = 0; g < 4; ++g) {  // slots 4g..4g+3: one 16-byte row of each digit's core matrix
                uint4 v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) v[q] = *reinterpret_cast<const uint4*>(src + ((4 * g + q) * DG_M + r) * 16);
#pragma unroll
                for (int i = 0; i < dg::DIGITS; ++i) {
                    uint32_t w[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint32_t sw = (i >> 1) == 0 ? v[q].x : (i >> 1) == 1 ? v[q].y : (i >> 1) == 2 ? v[q].z : v[q].w;
                        w[q] = dg::a_word(sw, i & 1);
                    }
                    *reinterpret_cast<uint4*>(A + dg::op_off(r, 32 * i + 8 * g, DG_SBO_A)) =
                        make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
            fence_proxy_async_shared();  // the generic-proxy writes of A visible to the MMAs
            dg_arrive(b_afull + 8 * s);
            if (it + 2 < nmine) issue(it + 2);  // refills the stage just read
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        asm volatile("cp.async.wait_group 0;" ::: "memory");  // nothing in flight at exit
    } else {  // ------------------------------------------------------------------- consumers
        // warp 5 + 4 sub + k: tensor-memory lanes 32 (warp % 4) (the tile rows it may read) and
        // output reals 4 sub .. 4 sub + 3 of every job's chunk (amplitudes 2 sub, 2 sub + 1)
        const int sub = (warp - 5) >> 2;
        const int quad = warp & 3;
        const int r = 32 * quad + lane;
        for (uint64_t it = 0; it < nmine; ++it) {
            const uint64_t base = tile_base(blockIdx.x + it * gridDim.x, r);
            if (!mbar_wait_bounded(b_accfull, (uint32_t)(it & 1), DG_WAIT_LIMIT)) {
                fail_now(9);
                break;
            }
            if (aborted()) break;
            tc::fence_after_sync();
#pragma unroll 1
            for (int q = 0; q < 2; ++q) {  // output reals 16 q + 4 sub ..; the second releases
                const uint32_t taddr = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(16 * q + 4 * sub);
                uint4 out[2];
                dg_consume4(taddr, skap + 16 * q + 4 * sub, q == 1 ? b_accempty : 0u, out);
                st[base | slot_off(8 * q + 2 * sub)] = out[0];
                st[base | slot_off(8 * q + 2 * sub + 1)] = out[1];
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::dealloc(tmem, DG_TCOLS);
}

// ---- layout conversions -----------------------------------------------------------------------
// x (f64) -> round(x 2^sx) from the double's bits (integer pipes), clamped to |X| <= 2^54 (a value
// outside that range sets the error word: the host's bound on the amplitudes was wrong).
__device__ __forceinline__ long long dg_fixed_f64(double x, int sx, int* err) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FFu);
    if (e == 0) return 0;  // zero or subnormal
    const long long m = (long long)((b & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    const int sh = e - 1075 + sx;
    long long v;
    if (sh > 2) {
        v = dg::XMAX + 1;
    } else if (sh >= 0) {
        v = m << sh;
    } else if (sh >= -60) {
        v = (m + (1ll << (-sh - 1))) >> (-sh);
    } else {
        v = 0;
    }
    if (v > dg::XMAX) {
        v = dg::XMAX;
        atomicExch(err, 10);
    }
    return (b >> 63) ? -v : v;
}
// the float pair h + l times 2^sx, rounded (integer pipes)
__device__ __forceinline__ long long dg_scaled_f32(float x, int sx) {
    const uint32_t b = __float_as_uint(x);
    const int e = (int)((b >> 23) & 0xFFu);
    if (e == 0) return 0;
    const long long m = (long long)((b & 0x7FFFFFu) | 0x800000u);
    const int sh = e - 150 + sx;
    long long v;
    if (sh > 31) v = dg::XMAX + 1;
    else if (sh >= 0) v = m << sh;
    else if (sh >= -30) v = (m + (1ll << (-sh - 1))) >> (-sh);
    else v = 0;
    return (b >> 31) ? -v : v;
}
__device__ __forceinline__ long long dg_clamp(long long v, int* err) {
    if (v > dg::XMAX || v < -dg::XMAX) {
        atomicExch(err, 10);
        v = v > 0 ? dg::XMAX : -dg::XMAX;
    }
    return v;
}

// from = 0: complex128 -> digits; from = 1: resident float pairs -> digits
template <int FROM>
__global__ void k_dg_from(uint4* __restrict__ st, uint64_t dim, int sx, int* err) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (; i < dim; i += stride) {
        const uint4 v = st[i];
        long long xr, xi;
        if (FROM == 0) {
            xr = dg_fixed_f64(__hiloint2double((int)v.y, (int)v.x), sx, err);
            xi = dg_fixed_f64(__hiloint2double((int)v.w, (int)v.z), sx, err);
        } else {  // (re_h, im_h | re_l, im_l)
            xr = dg_clamp(dg_scaled_f32(__uint_as_float(v.x), sx) + dg_scaled_f32(__uint_as_float(v.z), sx), err);
            xi = dg_clamp(dg_scaled_f32(__uint_as_float(v.y), sx) + dg_scaled_f32(__uint_as_float(v.w), sx), err);
        }
        uint32_t w[4];
        dg::pack_digits((uint64_t)(xr + dg::OFFSET), (uint64_t)(xi + dg::OFFSET), w);
        st[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// to = 0: digits -> complex128; to = 1: digits -> resident float pairs
template <int TO>
__global__ void k_dg_to(uint4* __restrict__ st, uint64_t dim, int sx) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const double scale = ldexp(1.0, -sx);
    for (; i < dim; i += stride) {
        const uint4 v = st[i];
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        uint64_t ur, ui;
        dg::unpack_digits(w, ur, ui);
        const long long xr = (long long)ur - dg::OFFSET, xi = (long long)ui - dg::OFFSET;
        if (TO == 0) {
            const double re = __ll2double_rn(xr) * scale, im = __ll2double_rn(xi) * scale;
            st[i] = make_uint4((uint32_t)__double2loint(re), (uint32_t)__double2hiint(re),
                               (uint32_t)__double2loint(im), (uint32_t)__double2hiint(im));
        } else {
            // X = H + L with H = X rounded to 24 bits (exact as a float) and L = X - H
            const float hr = __ll2float_rn(xr), hi = __ll2float_rn(xi);
            const float lr = __ll2float_rn(xr - __float2ll_rn(hr)), li = __ll2float_rn(xi - __float2ll_rn(hi));
            const float fs = (float)scale;  // a power of two within the float range
            float rh = hr * fs, ih = hi * fs, rl = lr * fs, il = li * fs;
            // the float pairs flush magnitudes below 2^-126 (as split_f64 does)
            if ((__float_as_uint(rh) & 0x7F800000u) == 0) rh = rl = 0.0f;
            if ((__float_as_uint(ih) & 0x7F800000u) == 0) ih = il = 0.0f;
            if ((__float_as_uint(rl) & 0x7F800000u) == 0) rl = 0.0f;
            if ((__float_as_uint(il) & 0x7F800000u) == 0) il = 0.0f;
            st[i] = make_uint4(__float_as_uint(rh), __float_as_uint(ih), __float_as_uint(rl),
                               __float_as_uint(il));
        }
    }
}

// ---- host side ----------------------------------------------------------------------------------
namespace {

uint16_t dg_bf16(int v) {  // |v| <= 256: exact in BF16
    const float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (uint16_t)(u >> 16);
}

}  // namespace

// The pass's 16 x 16 complex matrix (M[out slot][in slot], physical slots) as the B operand's
// digits and the carry constants. False when the matrix's digits could make a weight's sum reach
// 2^22 (the F32 accumulation and the magic conversion would no longer be exact) or a digit would
// not be exact in BF16; the caller then keeps the float-pair kernels.
bool dg_build_image(const std::complex<double> M[16][16], uint32_t* bimg, int32_t (*kap)[dg::KAP]) {
    using i128 = __int128;
    std::memset(bimg, 0, DG_B_BYTES);
    uint16_t* h16 = reinterpret_cast<uint16_t*>(bimg);
    int64_t S[32];
    int32_t rho[32][32][dg::DIGITS];  // [k][c][j]
    for (int c = 0; c < 32; ++c) {
        S[c] = 0;
        for (int k = 0; k < 32; ++k) {
            const std::complex<double> m = M[c / 2][k / 2];
            const int o = c & 1, ii = k & 1;  // [[Re, -Im], [Im, Re]][o][ii]
            const double val = (o == ii) ? m.real() : (o == 0 ? -m.imag() : m.imag());
            if (!(std::fabs(val) <= 2.0)) return false;
            int64_t R = std::llround(std::ldexp(val, 56));
            S[c] += R;
            for (int j = 0; j < dg::DIGITS - 1; ++j) {
                int64_t d = R & 127;
                if (d >= 64) d -= 128;
                rho[k][c][j] = (int32_t)d;
                R = (R - d) >> 7;
            }
            if (R > 256 || R < -256) return false;
            rho[k][c][dg::DIGITS - 1] = (int32_t)R;
        }
    }
    // exactness: every weight's sum stays below 2^22 for any register digits
    for (int c = 0; c < 32; ++c) {
        int64_t colsum[dg::DIGITS];
        for (int j = 0; j < dg::DIGITS; ++j) {
            colsum[j] = 0;
            for (int k = 0; k < 32; ++k) colsum[j] += std::llabs(rho[k][c][j]);
        }
        for (int w = dg::WMIN; w <= dg::WMAX; ++w) {
            int64_t b = 0;
            for (int i = 0; i < dg::DIGITS; ++i) {
                const int j = w - i;
                if (j < 0 || j >= dg::DIGITS) continue;
                b += (int64_t)(i == dg::DIGITS - 1 ? dg::AMAX_TOP : dg::AMAX_LOW) * colsum[j];
            }
            if (b >= dg::DBOUND) return false;
        }
    }
    // B: row 32 j + c (digit j of output real c), K = input real k
    for (int c = 0; c < 32; ++c)
        for (int j = 0; j < dg::DIGITS; ++j)
            for (int k = 0; k < 32; ++k)
                h16[dg::op_off(32 * j + c, k, DG_SBO_B) / 2] =
                    dg_bf16(rho[k][c][j]);
    // carry constants: K_c = 2^111 + 2^55 - (2^55 + 128 G) S_c, taken mod 2^112
    i128 G = 0;
    for (int i = 0; i < dg::DIGITS; ++i) G += (i128)1 << (7 * i);
    const i128 Z = ((i128)1 << 55) + 128 * G;
    const i128 MOD = (i128)1 << 112;
    for (int c = 0; c < 32; ++c) {
        i128 K = ((i128)1 << 111) + ((i128)1 << 55) - Z * (i128)S[c];
        K %= MOD;
        if (K < 0) K += MOD;
        int32_t kp[16];
        for (int p = 0; p < 16; ++p) kp[p] = (int32_t)((K >> (7 * p)) & 127);
        const float lowc = (float)((double)(kp[5] + 128 * kp[6] + 16384 * kp[7] - (1 << 20)) -
                                   16513.0 * (double)dg::MAGIC_F);
        uint32_t lb;
        std::memcpy(&lb, &lowc, 4);
        kap[c][0] = (int32_t)lb;
        kap[c][1] = (int32_t)((uint32_t)kp[8] - 2u * dg::MAGIC_BITS);
        for (int p = 9; p <= 14; ++p) kap[c][2 + p - 9] = (int32_t)((uint32_t)kp[p] - dg::MAGIC_BITS);
        kap[c][8] = kp[15];
    }
    return true;
}

bool dg_supported(const qgpu_handle* h) {
    // tuning knobs, read per call: QGPU_DIGITS=0 keeps the float-pair kernels; digit runs are
    // used from QGPU_DIGITS_MIN_QUBITS qubits (default 20: below that the register sits in L2
    // and the two layout conversions cost more than the passes save)
    const char* e = std::getenv("QGPU_DIGITS");
    const char* m = std::getenv("QGPU_DIGITS_MIN_QUBITS");
    const int on = e ? std::atoi(e) : 1;
    const int min_qubits = std::max(11, m ? std::atoi(m) : 20);
    return on != 0 && h->precision == QGPU_C128 && h->mode == QGPU_MODE_FAST &&
           (h->dim >> 4) % DG_M == 0 && h->n_qubits >= min_qubits;
}

int dg_launch_pass(qgpu_handle* h, const int bits[4], const uint32_t* bimg,
                   const int32_t (*kap)[dg::KAP]) {
    const cudaError_t attr = smem_opt_in((const void*)k_dg2, DG_SMEM);
    QGPU_CUDA(attr);
    DgArgs a;
    a.nblocks = (h->dim >> 4) / DG_M;
    for (int m = 0; m < 4; ++m) a.bits[m] = bits[m];
    a.err = h->d_err;
    std::memcpy(a.kap, kap, sizeof(a.kap));
    std::memcpy(a.bimg, bimg, sizeof(a.bimg));
    const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(a.nblocks, (uint64_t)h->sm_count));
    k_dg2<<<(unsigned)grid, DG_THREADS, DG_SMEM, h->stream>>>((uint4*)cur_state(h), a);
    QGPU_CHECK_LAUNCH("k_dg2");
    h->launches++;
    h->h2d_bytes += sizeof(a);
    return QGPU_OK;
}

// from_layout / to_layout: 0 complex128, 1 resident float pairs
int dg_convert(qgpu_handle* h, bool into_digits, int other_layout, int sx) {
    const int threads = 256;
    uint64_t blocks = (h->dim + threads - 1) / threads;
    blocks = std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)h->sm_count * 16));
    uint4* s = (uint4*)cur_state(h);
    if (into_digits) {
        if (other_layout == 0) k_dg_from<0><<<(unsigned)blocks, threads, 0, h->stream>>>(s, h->dim, sx, h->d_err);
        else k_dg_from<1><<<(unsigned)blocks, threads, 0, h->stream>>>(s, h->dim, sx, h->d_err);
        QGPU_CHECK_LAUNCH("k_dg_from");
    } else {
        if (other_layout == 0) k_dg_to<0><<<(unsigned)blocks, threads, 0, h->stream>>>(s, h->dim, sx);
        else k_dg_to<1><<<(unsigned)blocks, threads, 0, h->stream>>>(s, h->dim, sx);
        QGPU_CHECK_LAUNCH("k_dg_to");
    }
    h->launches++;
    return QGPU_OK;
}

}  // namespace qgpu
