// blocks.cu — dense-block fusion: runs of consecutive gates on at most 6 wires, multiplied on the
// host into one 2^k x 2^k complex matrix, applied in one pass (the precision configuration's
// "6-qubit blocks of up to 12 gates").
//
// k_block: a CTA owns GT = 64 groups (a group = the 2^k amplitudes that share all non-block
// bits). It stages the block matrix and the 64 groups in shared memory (loads ordered so that
// consecutive threads read consecutive groups: coalesced whenever the low index bits are not
// block bits), each thread accumulates a 4 x 4 register tile of outputs (4 matrix rows x 4
// groups) over the 2^k inputs, then the results go back through shared memory to coalesced
// stores. complex64 accumulates in f32 FMA (or runs on the tensor cores, blocks_tc.cu);
// complex128 uses float-pair Dot2 arithmetic in the fast mode (k_block_ff) and f64 FMA in
// QGPU_MODE_F64. A dense 64 x 64 block costs 256 real multiply-adds per amplitude, so on GB300
// these CUDA-core versions are compute-bound; the register-tile passes of program.cu apply the
// same gates one by one at 8-16 multiply-adds per gate per amplitude.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"
#include "plan.h"

namespace qgpu {

constexpr int BLK_GT = 64;      // groups per CTA tile
constexpr int BLK_THREADS = 256;

struct BlockArgs {
    uint64_t ngroups;
    int k;
    int bits[QGPU_MAX_OP_WIRES];  // sorted ascending; local bit m <-> bits[m]
    const void* M;                // row-major D x D complex (float2 or double2)
};

template <class T>
struct Cplx;
template <>
struct Cplx<float2> {
    using R = float;
    static __device__ __forceinline__ float2 mla(float2 acc, float2 m, float2 x) {
        return make_float2(fmaf(m.x, x.x, fmaf(-m.y, x.y, acc.x)), fmaf(m.x, x.y, fmaf(m.y, x.x, acc.y)));
    }
};
template <>
struct Cplx<double2> {
    using R = double;
    static __device__ __forceinline__ double2 mla(double2 acc, double2 m, double2 x) {
        return make_double2(fma(m.x, x.x, fma(-m.y, x.y, acc.x)), fma(m.x, x.y, fma(m.y, x.x, acc.y)));
    }
};

template <class T, int D>
__global__ void __launch_bounds__(BLK_THREADS) k_block(T* __restrict__ st, const __grid_constant__ BlockArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    T* sM = reinterpret_cast<T*>(smem);           // [D][D]
    T* sA = sM + D * D;                           // [D][BLK_GT]
    const T* gM = reinterpret_cast<const T*>(a.M);
    for (int t = threadIdx.x; t < D * D; t += BLK_THREADS) sM[t] = gM[t];
    constexpr int RL = D >= 64 ? 4 : (D >= 16 ? D / 16 : 1);  // rows per thread
    constexpr int RG = 4;                                     // groups per thread
    constexpr int TX = BLK_GT / RG;                           // 16 thread columns
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;   // ty in [0, 16)
    const uint64_t ntiles = (a.ngroups + BLK_GT - 1) / BLK_GT;
    __syncthreads();
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t g0 = tile * BLK_GT;
        // load: consecutive threads take consecutive groups of the same local index j
        for (int t = threadIdx.x; t < D * BLK_GT; t += BLK_THREADS) {
            const int j = t / BLK_GT, gl = t % BLK_GT;
            const uint64_t g = g0 + gl;
            if (g >= a.ngroups) continue;
            uint64_t base = g;
            for (int m = 0; m < a.k; ++m) base = insert_zero(base, a.bits[m]);
            uint64_t off = 0;
            for (int m = 0; m < a.k; ++m)
                if ((j >> m) & 1) off |= 1ull << a.bits[m];
            sA[j * BLK_GT + gl] = st[base | off];
        }
        __syncthreads();
        T acc[RL][RG];
        if (ty * RL < D) {
#pragma unroll
            for (int r = 0; r < RL; ++r)
#pragma unroll
                for (int c = 0; c < RG; ++c) acc[r][c] = T{0, 0};
            for (int j = 0; j < D; ++j) {
                T m[RL], x[RG];
#pragma unroll
                for (int r = 0; r < RL; ++r) m[r] = sM[(ty * RL + r) * D + j];
#pragma unroll
                for (int c = 0; c < RG; ++c) x[c] = sA[j * BLK_GT + tx * RG + c];
#pragma unroll
                for (int r = 0; r < RL; ++r)
#pragma unroll
                    for (int c = 0; c < RG; ++c) acc[r][c] = Cplx<T>::mla(acc[r][c], m[r], x[c]);
            }
        }
        __syncthreads();
        if (ty * RL < D) {
#pragma unroll
            for (int r = 0; r < RL; ++r)
#pragma unroll
                for (int c = 0; c < RG; ++c) sA[(ty * RL + r) * BLK_GT + tx * RG + c] = acc[r][c];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < D * BLK_GT; t += BLK_THREADS) {
            const int j = t / BLK_GT, gl = t % BLK_GT;
            const uint64_t g = g0 + gl;
            if (g >= a.ngroups) continue;
            uint64_t base = g;
            for (int m = 0; m < a.k; ++m) base = insert_zero(base, a.bits[m]);
            uint64_t off = 0;
            for (int m = 0; m < a.k; ++m)
                if ((j >> m) & 1) off |= 1ull << a.bits[m];
            st[base | off] = sA[j * BLK_GT + gl];
        }
        __syncthreads();
    }
}

// complex128 blocks in float-pair arithmetic (QGPU_MODE_FAST): the matrix sits in shared memory
// as float pairs (re_h, re_l, im_h, im_l), the tile's inputs are split once into packed pairs,
// and every output is one packed Dot2 over its 2D terms (M[l][j] x_j and the swapped lanes).
// A thread owns RL rows x 4 groups; the CTA covers BFF_GT groups.
constexpr int BFF_GT = 32;

template <int D>
__global__ void __launch_bounds__(BLK_THREADS) k_block_ff(double2* __restrict__ st,
                                                          const __grid_constant__ BlockArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    float4* sM = reinterpret_cast<float4*>(smem);  // [D][D]
    ffp* sA = reinterpret_cast<ffp*>(sM + D * D);   // [D][BFF_GT] inputs
    double2* sO = reinterpret_cast<double2*>(sA);   // [D][BFF_GT] outputs (after the inputs)
    const float4* gM = reinterpret_cast<const float4*>(a.M);
    for (int t = threadIdx.x; t < D * D; t += BLK_THREADS) sM[t] = gM[t];
    constexpr int RG = 4, TX = BFF_GT / RG, TY = BLK_THREADS / TX;
    constexpr int RL = D / TY > 0 ? D / TY : 1;
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const bool active = ty * RL < D;
    const uint64_t ntiles = (a.ngroups + BFF_GT - 1) / BFF_GT;
    __syncthreads();
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t g0 = tile * BFF_GT;
        for (int t = threadIdx.x; t < D * BFF_GT; t += BLK_THREADS) {
            const int j = t / BFF_GT, gl = t % BFF_GT;
            const uint64_t g = g0 + gl;
            if (g >= a.ngroups) continue;
            uint64_t base = g;
            for (int m = 0; m < a.k; ++m) base = insert_zero(base, a.bits[m]);
            uint64_t off = 0;
            for (int m = 0; m < a.k; ++m)
                if ((j >> m) & 1) off |= 1ull << a.bits[m];
            sA[j * BFF_GT + gl] = to_ffp(st[base | off]);
        }
        __syncthreads();
        PDot2 acc[RL][RG];
        if (active) {
            for (int j = 0; j < D; ++j) {
                u64 c[RL][8];
#pragma unroll
                for (int r = 0; r < RL; ++r) {
                    const float4 m = sM[(ty * RL + r) * D + j];
                    c[r][0] = p2(m.x, m.x);
                    c[r][1] = p2(m.y, m.y);
                    c[r][2] = p2(-m.x, -m.x);
                    c[r][3] = p2(-m.y, -m.y);
                    c[r][4] = p2(-m.z, m.z);
                    c[r][5] = p2(-m.w, m.w);
                    c[r][6] = p2(m.z, -m.z);
                    c[r][7] = p2(m.w, -m.w);
                }
#pragma unroll
                for (int q = 0; q < RG; ++q) {
                    const ffp x = sA[j * BFF_GT + tx * RG + q];
                    const u64 xsh = pswap(x.h), xsl = pswap(x.l);
#pragma unroll
                    for (int r = 0; r < RL; ++r) {
                        if (j == 0) acc[r][q].first(c[r], x.h, x.l);
                        else acc[r][q].add(c[r], x.h, x.l);
                        acc[r][q].add(c[r] + 4, xsh, xsl);
                    }
                }
            }
        }
        __syncthreads();
        if (active) {
#pragma unroll
            for (int r = 0; r < RL; ++r)
#pragma unroll
                for (int q = 0; q < RG; ++q) {
                    ffp o;
                    acc[r][q].result(o.h, o.l);
                    sO[(ty * RL + r) * BFF_GT + tx * RG + q] = from_ffp(o);
                }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < D * BFF_GT; t += BLK_THREADS) {
            const int j = t / BFF_GT, gl = t % BFF_GT;
            const uint64_t g = g0 + gl;
            if (g >= a.ngroups) continue;
            uint64_t base = g;
            for (int m = 0; m < a.k; ++m) base = insert_zero(base, a.bits[m]);
            uint64_t off = 0;
            for (int m = 0; m < a.k; ++m)
                if ((j >> m) & 1) off |= 1ull << a.bits[m];
            st[base | off] = sO[j * BFF_GT + gl];
        }
        __syncthreads();
    }
}

template <int D>
static int launch_block_ff_t(qgpu_handle* h, const BlockArgs& a) {
    const size_t smem = (size_t)(D * D + D * BFF_GT) * 16;
    // set once per kernel instance; a function-local static initialises once even when
    // several host threads launch concurrently
    const cudaError_t attr = smem_opt_in((const void*)k_block_ff<D>, smem);
    QGPU_CUDA(attr);
    const uint64_t ntiles = (a.ngroups + BFF_GT - 1) / BFF_GT;
    uint64_t blocks = std::min<uint64_t>(ntiles, (uint64_t)h->sm_count * 2);
    if (blocks < 1) blocks = 1;
    k_block_ff<D><<<(unsigned)blocks, BLK_THREADS, smem, h->stream>>>((double2*)cur_state(h), a);
    QGPU_CHECK_LAUNCH("k_block_ff");
    h->launches++;
    h->h2d_bytes += sizeof(BlockArgs);
    return QGPU_OK;
}

static int launch_block_ff(qgpu_handle* h, const BlockArgs& a) {
    switch (a.k) {
        case 1: return launch_block_ff_t<2>(h, a);
        case 2: return launch_block_ff_t<4>(h, a);
        case 3: return launch_block_ff_t<8>(h, a);
        case 4: return launch_block_ff_t<16>(h, a);
        case 5: return launch_block_ff_t<32>(h, a);
        case 6: return launch_block_ff_t<64>(h, a);
        default: return fail(QGPU_ERR_UNSUPPORTED, "dense blocks act on at most 6 wires");
    }
}

template <class T, int D>
static int launch_block_t(qgpu_handle* h, const BlockArgs& a) {
    const size_t smem = (size_t)(D * D + D * BLK_GT) * sizeof(T);
    // set once per kernel instance; a function-local static initialises once even when
    // several host threads launch concurrently
    const cudaError_t attr = smem_opt_in((const void*)k_block<T, D>, smem);
    QGPU_CUDA(attr);
    const uint64_t ntiles = (a.ngroups + BLK_GT - 1) / BLK_GT;
    uint64_t blocks = std::min<uint64_t>(ntiles, (uint64_t)h->sm_count * 2);
    if (blocks < 1) blocks = 1;
    k_block<T, D><<<(unsigned)blocks, BLK_THREADS, smem, h->stream>>>((T*)cur_state(h), a);
    QGPU_CHECK_LAUNCH("k_block");
    h->launches++;
    h->h2d_bytes += sizeof(BlockArgs);
    return QGPU_OK;
}

template <class T>
static int launch_block(qgpu_handle* h, const BlockArgs& a) {
    switch (a.k) {
        case 1: return launch_block_t<T, 2>(h, a);
        case 2: return launch_block_t<T, 4>(h, a);
        case 3: return launch_block_t<T, 8>(h, a);
        case 4: return launch_block_t<T, 16>(h, a);
        case 5: return launch_block_t<T, 32>(h, a);
        case 6: return launch_block_t<T, 64>(h, a);
        default: return fail(QGPU_ERR_UNSUPPORTED, "dense blocks act on at most 6 wires");
    }
}

bool block_tc_supported(const qgpu_handle* h, const DenseBlock& b);               // blocks_tc.cu
int apply_blocks_tc(qgpu_handle* h, const std::vector<DenseBlock>& blocks);       // blocks_tc.cu

// Blocks on the CUDA cores (k_block), in order.
static int apply_blocks_cc(qgpu_handle* h, const std::vector<DenseBlock>& blocks) {
    int st = QGPU_OK;
    // complex128 in the fast mode: float-pair kernel (k_block_ff); QGPU_MODE_F64: f64 FMA
    const bool ff = h->precision == QGPU_C128 && h->mode != QGPU_MODE_F64;
    // all block matrices in one upload
    const size_t esz = h->precision == QGPU_C128 ? 16 : 8;
    std::vector<size_t> offs(blocks.size());
    size_t total = 0;
    for (size_t i = 0; i < blocks.size(); ++i) {
        offs[i] = total;
        total += ((size_t)1 << (2 * blocks[i].k)) * esz;
        total = (total + 255) / 256 * 256;
    }
    std::vector<uint8_t> host(total ? total : 1);
    for (size_t i = 0; i < blocks.size(); ++i) {
        const size_t D2 = (size_t)1 << (2 * blocks[i].k);
        for (size_t e = 0; e < D2; ++e) {
            const cd v = blocks[i].M[e];
            if (ff) {  // (re_h, re_l, im_h, im_l)
                const float rh = (float)v.real(), ih = (float)v.imag();
                const float4 q = make_float4(rh, (float)(v.real() - (double)rh), ih,
                                             (float)(v.imag() - (double)ih));
                std::memcpy(host.data() + offs[i] + e * 16, &q, 16);
            } else if (esz == 16) {
                double2 d = make_double2(v.real(), v.imag());
                std::memcpy(host.data() + offs[i] + e * 16, &d, 16);
            } else {
                float2 f = make_float2((float)v.real(), (float)v.imag());
                std::memcpy(host.data() + offs[i] + e * 8, &f, 8);
            }
        }
    }
    st = h->tables.ensure(total ? total : 256);
    if (st != QGPU_OK) return st;
    QGPU_CUDA(copy_async(h, h->tables.ptr, host.data(), total, cudaMemcpyHostToDevice));
    std::vector<std::string> names;
    std::vector<double> bytes;
    size_t ev_base = 0;
    if (h->profile) {
        st = prof_events(h, blocks.size(), &ev_base);
        if (st != QGPU_OK) return st;
    }
    for (size_t i = 0; i < blocks.size(); ++i) {
        if (h->profile) {
            QGPU_CUDA(cudaEventRecord(h->events[2 * (ev_base + i)], h->stream));
            names.push_back((ff ? "k_block_ff<" : "k_block<") + std::to_string(1 << blocks[i].k) + ">");
            bytes.push_back(2.0 * (double)h->amp_bytes * (double)h->dim);
        }
        BlockArgs a;
        std::memset(&a, 0, sizeof(a));
        a.k = blocks[i].k;
        for (int m = 0; m < a.k; ++m) a.bits[m] = blocks[i].bits[m];
        a.ngroups = h->dim >> a.k;
        a.M = (const uint8_t*)h->tables.ptr + offs[i];
        st = ff ? launch_block_ff(h, a)
                : (h->precision == QGPU_C128) ? launch_block<double2>(h, a) : launch_block<float2>(h, a);
        if (st != QGPU_OK) return st;
        if (h->profile) QGPU_CUDA(cudaEventRecord(h->events[2 * (ev_base + i) + 1], h->stream));
    }
    if (h->profile) {
        st = prof_collect(h, names, bytes);
        if (st != QGPU_OK) return st;
    }
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

// Applies ops as fused dense blocks of at most `bq` wires / `mg` gates: complex64 blocks of 3 to 6
// wires on the tensor cores (k_block_tc; QGPU_BLOCK_TC=0 keeps them on the CUDA cores), the rest
// with k_block, in circuit order.
int apply_blocks(qgpu_handle* h, const qgpu_op* ops, size_t n_ops, const double* mats,
                 size_t n_mats, const uint8_t* none, size_t n_none, int bq, int mg) {
    std::vector<DenseBlock> blocks;
    int st = build_blocks(ops, n_ops, h->n_qubits, mats, n_mats, none, n_none, bq, mg, &blocks);
    if (st != QGPU_OK) return st;
    for (const DenseBlock& b : blocks)
        if (b.k > 6)
            return fail(QGPU_ERR_UNSUPPORTED, "dense-block fusion: a gate acts on more than 6 wires");
    const char* env = std::getenv("QGPU_BLOCK_TC");
    const bool use_tc = !(env && env[0] == '0');
    size_t i = 0;
    while (i < blocks.size()) {  // consecutive runs of one kind
        const bool tc = use_tc && block_tc_supported(h, blocks[i]);
        size_t j = i + 1;
        while (j < blocks.size() && (use_tc && block_tc_supported(h, blocks[j])) == tc) ++j;
        std::vector<DenseBlock> run(blocks.begin() + i, blocks.begin() + j);
        st = tc ? apply_blocks_tc(h, run) : apply_blocks_cc(h, run);
        if (st != QGPU_OK) return st;
        i = j;
    }
    return QGPU_OK;
}

}  // namespace qgpu
