// blocks_tc.cu — complex64 dense blocks (3 to 6 wires) on the fifth-generation tensor cores.
//
// A block U (D x D complex, D = 2^k) maps every group of D amplitudes that share their non-block
// bits. In real form that is one GEMM per 128-group tile: Y (128 x 2D) = X (128 x 2D) * B^T with
// B[2l + o][2c + i] = (Re U, -Im U; Im U, Re U)[o][i] at (l, c). Both operands are split into three
// BF16 slices (x = x0 + x1 + x2, exact in F32), and the six slice products whose weight is above
// 2^-24 (x2 b0, x1 b1, x0 b2, x1 b0, x0 b1, x0 b0; smallest first) accumulate in one F32 tensor-
// memory accumulator: F32-level accuracy at BF16 tensor rate (split precision).
//
// k_block_tc: one CTA of 8 warps per SM, persistent over tiles. The three B slices (the block's
// matrix, identical for every tile) are copied into shared memory once, already in the MMA's
// K-major core-matrix layout (prepared on the host). Per tile:
//   1. gather: address bits 0-4 always vary inside a tile (they are block bits or among the 7
//      lowest group bits), so lane = address bits 0-4 and a per-CTA table enumerates the other
//      k + 2 varying bits: every warp load is 32 consecutive amplitudes (256 bytes);
//   2. split each float into three BF16 slices, written straight into the A-operand layout;
//   3. one thread issues 6 x (2D / 16) MMAs (M = 128, N = 2D, K = 16) and commits to an
//      mbarrier; all threads wait (bounded);
//   4. tcgen05.ld moves the accumulator to registers, through a padded shared staging tile;
//   5. scatter back with the same coalesced mapping.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"
#include "plan.h"
#include "tc.cuh"

namespace qgpu {

constexpr int TCB_M = 128;
constexpr int TCB_THREADS = 256;
constexpr int TCB_SLICES = 3;
constexpr uint32_t TCB_WAIT_LIMIT = 1u << 22;

struct TcBlockArgs {
    uint64_t ntiles;     // groups / 128
    int k;
    int bits[6];         // block bits, ascending: local bit m <-> bits[m]
    const uint8_t* bimg; // 3 B slices in shared-memory layout
    int* err;
};

template <int D>
struct TcbShape {
    static constexpr int K = 2 * D, N = 2 * D;
    static constexpr uint32_t LBO = 128;                  // K-adjacent core matrices
    static constexpr uint32_t SBO = (K / 8) * 128;        // next 8 rows (A: groups, B: outputs)
    static constexpr uint32_t A_SLICE = TCB_M * K * 2;    // bytes
    static constexpr uint32_t B_SLICE = N * K * 2;
    static constexpr int NI = 4 * D;                      // 32-amplitude chunks per tile
    static constexpr uint32_t TCOLS = N < 32 ? 32 : N;    // tensor-memory columns
    static constexpr int OSTRIDE = D + 1;                 // staging row stride (float2)
    static constexpr size_t SMEM = (size_t)TCB_SLICES * (A_SLICE + B_SLICE) + 64 + 10 * NI;
};

// byte offset of element (row, k) of a K-major BF16 operand with K columns
__host__ __device__ __forceinline__ uint32_t tcb_off(int row, int k, uint32_t sbo) {
    return (uint32_t)((row % 8) * 16 + (k % 8) * 2 + (k / 8) * 128) + (uint32_t)(row / 8) * sbo;
}

__device__ __forceinline__ void split3(float x, __nv_bfloat16 (&s)[3]) {
    s[0] = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(s[0]);
    s[1] = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(s[1]);
    s[2] = __float2bfloat16_rn(r2);
}

template <int D>
__global__ void __launch_bounds__(TCB_THREADS, 1) k_block_tc(float2* __restrict__ st,
                                                             const __grid_constant__ TcBlockArgs a) {
    using SH = TcbShape<D>;
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sB = sm;
    uint8_t* sA = sm + TCB_SLICES * SH::B_SLICE;
    float2* stage = reinterpret_cast<float2*>(sA);  // reused once the MMAs of a tile are done
    uint8_t* tail = sA + TCB_SLICES * SH::A_SLICE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tail);
    uint32_t* slot = reinterpret_cast<uint32_t*>(tail + 16);
    uint64_t* ioff = reinterpret_cast<uint64_t*>(tail + 64);
    uint16_t* iloc = reinterpret_cast<uint16_t*>(tail + 64 + 8 * SH::NI);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    {  // the block's matrix slices, already laid out for the MMA
        const uint4* src = reinterpret_cast<const uint4*>(a.bimg);
        uint4* dst = reinterpret_cast<uint4*>(sB);
        for (int i = tid; i < (int)(TCB_SLICES * SH::B_SLICE / 16); i += TCB_THREADS) dst[i] = src[i];
    }
    uint64_t bmask = 0;
    for (int m = 0; m < a.k; ++m) bmask |= 1ull << a.bits[m];
    int gpos[7];
    for (int b = 0, q = 0; q < 7; ++b)
        if (!((bmask >> b) & 1ull)) gpos[q++] = b;
    auto local_of = [&](int b, uint32_t& l, uint32_t& g) {  // adds full bit b to (l, g)
        if ((bmask >> b) & 1ull) {
            for (int m = 0; m < a.k; ++m)
                if (a.bits[m] == b) l |= 1u << m;
        } else {
            for (int q = 0; q < 7; ++q)
                if (gpos[q] == b) g |= 1u << q;
        }
    };
    uint32_t l_lane = 0, g_lane = 0;
    for (int b = 0; b < 5; ++b)
        if ((lane >> b) & 1) local_of(b, l_lane, g_lane);
    if (tid < SH::NI) {
        uint64_t vmask = bmask;
        for (int q = 0; q < 7; ++q) vmask |= 1ull << gpos[q];
        uint64_t off = 0;
        uint32_t li = 0, gi = 0;
        for (int b = 5, j = 0; b < 64; ++b) {
            if (!((vmask >> b) & 1ull)) continue;
            if ((tid >> j) & 1) {
                off |= 1ull << b;
                local_of(b, li, gi);
            }
            ++j;
        }
        ioff[tid] = off;
        iloc[tid] = (uint16_t)((gi << 8) | li);
    }
    if (tid == 0) {
        mbar_init(smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::alloc(smem_u32(slot), SH::TCOLS);
    fence_proxy_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t idesc = tc::idesc_bf16(TCB_M, SH::N);
    uint32_t phase = 0;

    // Software pipeline: the tile's amplitudes sit in registers (PER per thread) while the
    // previous tile's MMAs, accumulator read-out and stores run, so a whole tile of loads is in
    // flight at once.
    constexpr int PER = SH::NI / (TCB_THREADS / 32);
    auto tile_base = [&](uint64_t tile) {  // first group of the tile, spread over non-block bits
        uint64_t b = tile * TCB_M;
        for (int m = 0; m < a.k; ++m) b = insert_zero(b, a.bits[m]);
        return b;
    };
    float2 pv[PER];
    uint64_t tile = blockIdx.x;
    uint64_t base = tile_base(tile);
    if (tile < a.ntiles) {
#pragma unroll
        for (int j = 0; j < PER; ++j) pv[j] = st[base | ioff[warp + 8 * j] | (uint64_t)lane];
    }
    for (; tile < a.ntiles; tile += gridDim.x) {
#pragma unroll
        for (int j = 0; j < PER; ++j) {  // split into the three A slices
            const uint32_t loc = iloc[warp + 8 * j];
            const int g = (int)((loc >> 8) | g_lane), l = (int)((loc & 0xFFu) | l_lane);
            __nv_bfloat16 re[3], im[3];
            split3(pv[j].x, re);
            split3(pv[j].y, im);
            const uint32_t off = tcb_off(g, 2 * l, SH::SBO);
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                __nv_bfloat162 p;
                p.x = re[s];
                p.y = im[s];
                *reinterpret_cast<__nv_bfloat162*>(sA + s * SH::A_SLICE + off) = p;
            }
        }
        fence_proxy_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
            uint32_t acc = 0;
            for (int p = 0; p < 6; ++p)
                for (int kk = 0; kk < SH::K / 16; ++kk) {
                    const uint64_t ad =
                        tc::smem_desc(smem_u32(sA + pa[p] * SH::A_SLICE) + kk * 2 * SH::LBO, SH::LBO, SH::SBO);
                    const uint64_t bd =
                        tc::smem_desc(smem_u32(sB + pb[p] * SH::B_SLICE) + kk * 2 * SH::LBO, SH::LBO, SH::SBO);
                    tc::mma_bf16(tmem, ad, bd, idesc, acc);
                    acc = 1;
                }
            tc::commit(smem_u32(bar));
        }
        const uint64_t next = tile + gridDim.x;
        const uint64_t nbase = tile_base(next);
        if (next < a.ntiles) {  // next tile's loads overlap this tile's MMAs and stores
#pragma unroll
            for (int j = 0; j < PER; ++j) pv[j] = st[nbase | ioff[warp + 8 * j] | (uint64_t)lane];
        }
        const bool ok = mbar_wait_bounded(smem_u32(bar), phase, TCB_WAIT_LIMIT);
        phase ^= 1u;
        tc::fence_after_sync();
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicExch(a.err, 2);
            break;
        }
        {  // accumulator -> staging: warp w reads lanes 32 (w % 4) .., columns of half w / 4
            const int q = warp & 3, row = 32 * q + lane;
            for (int c0 = (warp >> 2) * 16; c0 < SH::N; c0 += 32) {
                float v[16];
                tc::ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    stage[row * SH::OSTRIDE + c0 / 2 + j] = make_float2(v[2 * j], v[2 * j + 1]);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int i = warp + 8 * j;
            const uint32_t loc = iloc[i];
            const int g = (int)((loc >> 8) | g_lane), l = (int)((loc & 0xFFu) | l_lane);
            st[base | ioff[i] | (uint64_t)lane] = stage[g * SH::OSTRIDE + l];
        }
        __syncthreads();
        base = nbase;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::dealloc(tmem, SH::TCOLS);
}

namespace {

uint16_t bf16_bits(float f) {  // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7FFFFFFFu) > 0x7F800000u) return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
double bf16_value(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return (double)f;
}

// The three BF16 slices of B for block b, in the shared-memory layout k_block_tc copies.
void build_bimg(const DenseBlock& b, std::vector<uint8_t>& img, size_t at) {
    const int D = 1 << b.k, K = 2 * D;
    const uint32_t sbo = (uint32_t)(K / 8) * 128, slice = (uint32_t)(2 * D * K * 2);
    for (int lo = 0; lo < D; ++lo)
        for (int c = 0; c < D; ++c) {
            const cd u = b.M[(size_t)lo * D + c];
            const double v[2][2] = {{u.real(), -u.imag()}, {u.imag(), u.real()}};  // [o][i]
            for (int o = 0; o < 2; ++o)
                for (int i = 0; i < 2; ++i) {
                    double r = v[o][i];
                    const uint32_t off = tcb_off(2 * lo + o, 2 * c + i, sbo);
                    for (int s = 0; s < 3; ++s) {
                        const uint16_t h = bf16_bits((float)r);
                        r -= bf16_value(h);
                        std::memcpy(img.data() + at + s * slice + off, &h, 2);
                    }
                }
        }
}

template <int D>
int launch_tc(qgpu_handle* h, const DenseBlock& b, const uint8_t* dev_img) {
    using SH = TcbShape<D>;
    // set once per kernel instance; a function-local static initialises once even when
    // several host threads launch concurrently
    const cudaError_t attr = smem_opt_in((const void*)k_block_tc<D>, SH::SMEM);
    QGPU_CUDA(attr);
    TcBlockArgs a;
    std::memset(&a, 0, sizeof(a));
    a.k = b.k;
    for (int m = 0; m < b.k; ++m) a.bits[m] = b.bits[m];
    a.ntiles = (h->dim >> b.k) / TCB_M;
    a.bimg = dev_img;
    a.err = h->d_err;
    const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>(a.ntiles, (uint64_t)h->sm_count));
    k_block_tc<D><<<(unsigned)blocks, TCB_THREADS, SH::SMEM, h->stream>>>((float2*)cur_state(h), a);
    QGPU_CHECK_LAUNCH("k_block_tc");
    h->launches++;
    h->h2d_bytes += sizeof(TcBlockArgs);
    return QGPU_OK;
}

}  // namespace

bool block_tc_supported(const qgpu_handle* h, const DenseBlock& b) {
    return h->precision == QGPU_C64 && b.k >= 3 && b.k <= 6 && h->n_qubits >= b.k + 7;
}

// Applies complex64 blocks on the tensor cores (every block must pass block_tc_supported).
int apply_blocks_tc(qgpu_handle* h, const std::vector<DenseBlock>& blocks) {
    std::vector<size_t> offs(blocks.size());
    size_t total = 0;
    for (size_t i = 0; i < blocks.size(); ++i) {
        const size_t D = (size_t)1 << blocks[i].k;
        offs[i] = total;
        total += (size_t)TCB_SLICES * (2 * D) * (2 * D) * 2;
        total = (total + 255) / 256 * 256;
    }
    std::vector<uint8_t> img(total ? total : 256, 0);
    for (size_t i = 0; i < blocks.size(); ++i) build_bimg(blocks[i], img, offs[i]);
    int st = h->tables.ensure(img.size());
    if (st != QGPU_OK) return st;
    QGPU_CUDA(copy_async(h, h->tables.ptr, img.data(), img.size(), cudaMemcpyHostToDevice));
    QGPU_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    std::vector<std::string> names;
    std::vector<double> bytes;
    size_t ev_base = 0;
    if (h->profile) {
        st = prof_events(h, blocks.size(), &ev_base);
        if (st != QGPU_OK) return st;
    }
    for (size_t i = 0; i < blocks.size(); ++i) {
        const uint8_t* dimg = (const uint8_t*)h->tables.ptr + offs[i];
        if (h->profile) {
            QGPU_CUDA(cudaEventRecord(h->events[2 * (ev_base + i)], h->stream));
            names.push_back("k_block_tc<" + std::to_string(1 << blocks[i].k) + ">");
            bytes.push_back(2.0 * (double)h->amp_bytes * (double)h->dim);
        }
        switch (blocks[i].k) {
            case 3: st = launch_tc<8>(h, blocks[i], dimg); break;
            case 4: st = launch_tc<16>(h, blocks[i], dimg); break;
            case 5: st = launch_tc<32>(h, blocks[i], dimg); break;
            default: st = launch_tc<64>(h, blocks[i], dimg); break;
        }
        if (st != QGPU_OK) return st;
        if (h->profile) QGPU_CUDA(cudaEventRecord(h->events[2 * (ev_base + i) + 1], h->stream));
    }
    int err = 0;
    QGPU_CUDA(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (h->profile) {
        st = prof_collect(h, names, bytes);
        if (st != QGPU_OK) return st;
    }
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    if (err) return fail(QGPU_ERR_TIMEOUT, "k_block_tc gave up waiting for its tensor-core MMAs");
    return QGPU_OK;
}

}  // namespace qgpu
