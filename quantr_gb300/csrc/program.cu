// program.cu — qgpu_apply_program: the device side of `simulate_with_register`
// (src/circuit/simulation.rs:21-57) and `apply_gate` (simulation.rs:64-135).
//
// Two execution paths:
//  * QGPU_MODE_EXACT (complex128): one launch of k_group per gate. Each CTA stages whole
//    gate groups (the 2^k amplitudes that share all non-acting bits) in shared memory and writes
//    out[l] = none[l] ? a[l] : sum over non-None inputs j, in increasing full index, of
//    M[l][j] * a[j] — f64 products and sums without contraction, first product assigned then
//    added to (simulation.rs:168-179) — so amplitudes equal the reference's.
//  * fused (QGPU_MODE_FAST / QGPU_MODE_F64 / complex64): the planner (plan.cpp) turns the gate
//    list into register-tile passes. k_tile<K> gives each thread 2^K amplitudes that differ in
//    the pass's K tile bits, applies every step of the pass in registers and writes them back:
//    one HBM round trip per pass.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "digits.cuh"
#include "internal.cuh"
#include "plan.h"

namespace qgpu {

// =============================================================================================
// Exact group kernel
// =============================================================================================
struct GroupArgs {
    uint64_t ngroups;
    int k;
    int nbits_sorted;
    int sorted_bits[QGPU_MAX_OP_WIRES];   // acting bit positions, ascending (for base insertion)
    const uint64_t* scatter;              // [2^k] offset of local index l
    const int* order;                     // [2^k] local inputs in increasing full index
    const double2* M;                     // [2^k * 2^k] column-major images
    const uint8_t* none;                  // [2^k]
    int groups_per_block;
};

template <class S>
__device__ __forceinline__ double2 ld_amp(const S* s, uint64_t i) {
    return make_double2((double)s[i].x, (double)s[i].y);
}
__device__ __forceinline__ void st_amp(double2* s, uint64_t i, double2 v) { s[i] = v; }
__device__ __forceinline__ void st_amp(float2* s, uint64_t i, double2 v) {
    s[i] = make_float2((float)v.x, (float)v.y);
}

template <class S>
__global__ void __launch_bounds__(256) k_group(S* __restrict__ st, GroupArgs a) {
    extern __shared__ double2 sh[];
    const int dk = 1 << a.k;
    const int per = a.groups_per_block * dk;
    for (uint64_t g0 = (uint64_t)blockIdx.x * a.groups_per_block; g0 < a.ngroups;
         g0 += (uint64_t)gridDim.x * a.groups_per_block) {
        for (int t = threadIdx.x; t < per; t += blockDim.x) {
            const uint64_t g = g0 + (t >> a.k);
            if (g >= a.ngroups) continue;
            uint64_t base = g;
            for (int m = 0; m < a.nbits_sorted; ++m) base = insert_zero(base, a.sorted_bits[m]);
            sh[t] = ld_amp(st, base | a.scatter[t & (dk - 1)]);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < per; t += blockDim.x) {
            const uint64_t g = g0 + (t >> a.k);
            if (g >= a.ngroups) continue;
            const int l = t & (dk - 1);
            const double2* grp = sh + (t >> a.k) * dk;
            double2 out = grp[l];
            if (!a.none[l]) {
                bool first = true;
                for (int q = 0; q < dk; ++q) {
                    const int j = a.order[q];
                    if (a.none[j]) continue;
                    const double2 m = a.M[(size_t)j * dk + l];
                    const double2 x = grp[j];
                    // num-complex Mul (image * amplitude), no FMA contraction
                    const double pr = __dsub_rn(__dmul_rn(m.x, x.x), __dmul_rn(m.y, x.y));
                    const double pi = __dadd_rn(__dmul_rn(m.x, x.y), __dmul_rn(m.y, x.x));
                    if (first) {
                        out = make_double2(pr, pi);
                        first = false;
                    } else {
                        out = make_double2(__dadd_rn(out.x, pr), __dadd_rn(out.y, pi));
                    }
                }
            }
            uint64_t base = g;
            for (int m = 0; m < a.nbits_sorted; ++m) base = insert_zero(base, a.sorted_bits[m]);
            st_amp(st, base | a.scatter[l], out);
        }
        __syncthreads();
    }
}

// Device copy of one gate's tables, laid out in the handle's gate scratch.
struct GroupTables {
    size_t scatter_off, order_off, m_off, none_off, bytes;
};

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

static GroupTables group_layout(int k, size_t at) {
    const size_t d = (size_t)1 << k;
    GroupTables t;
    t.scatter_off = align_up(at, 256);
    t.order_off = align_up(t.scatter_off + d * 8, 16);
    t.m_off = align_up(t.order_off + d * 4, 16);
    t.none_off = align_up(t.m_off + d * d * 16, 16);
    t.bytes = align_up(t.none_off + d, 256) - at;
    return t;
}

static void group_fill(const LocalGate& g, int n, std::vector<uint8_t>& host, size_t at,
                       const GroupTables& t, GroupArgs* args) {
    const int k = g.k;
    const size_t d = (size_t)1 << k;
    uint64_t* scatter = (uint64_t*)(host.data() + t.scatter_off);
    int* order = (int*)(host.data() + t.order_off);
    double2* M = (double2*)(host.data() + t.m_off);
    uint8_t* none = host.data() + t.none_off;
    for (size_t l = 0; l < d; ++l) {
        uint64_t off = 0;
        for (int m = 0; m < k; ++m)
            if ((l >> (k - 1 - m)) & 1u) off |= 1ull << (n - 1 - g.wires[m]);
        scatter[l] = off;
        order[l] = (int)l;
        none[l] = g.none[l];
    }
    std::sort(order, order + d, [&](int x, int y) { return scatter[x] < scatter[y]; });
    for (size_t j = 0; j < d; ++j)
        for (size_t l = 0; l < d; ++l)
            M[j * d + l] = make_double2(g.M[j * d + l].real(), g.M[j * d + l].imag());
    args->k = k;
    args->nbits_sorted = k;
    int sb[QGPU_MAX_OP_WIRES];
    for (int m = 0; m < k; ++m) sb[m] = n - 1 - g.wires[m];
    std::sort(sb, sb + k);
    for (int m = 0; m < k; ++m) args->sorted_bits[m] = sb[m];
    (void)at;
}

static int launch_group(qgpu_handle* h, const GroupArgs& a0, const uint8_t* dev_base,
                        const GroupTables& t) {
    GroupArgs a = a0;
    a.scatter = (const uint64_t*)(dev_base + t.scatter_off);
    a.order = (const int*)(dev_base + t.order_off);
    a.M = (const double2*)(dev_base + t.m_off);
    a.none = dev_base + t.none_off;
    const int dk = 1 << a.k;
    a.groups_per_block = dk >= 256 ? 1 : 256 / dk;
    a.ngroups = h->dim >> a.k;
    if ((uint64_t)a.groups_per_block > a.ngroups) a.groups_per_block = (int)a.ngroups;
    const size_t smem = (size_t)a.groups_per_block * dk * sizeof(double2);
    uint64_t blocks = (a.ngroups + a.groups_per_block - 1) / a.groups_per_block;
    const uint64_t cap = (uint64_t)h->sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (smem > 48 * 1024) {
        cudaError_t e = (h->precision == QGPU_C128) ? smem_opt_in((const void*)k_group<double2>, smem)
                                                    : smem_opt_in((const void*)k_group<float2>, smem);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_group)");
    }
    if (h->precision == QGPU_C128)
        k_group<double2><<<(unsigned)blocks, 256, smem, h->stream>>>((double2*)cur_state(h), a);
    else
        k_group<float2><<<(unsigned)blocks, 256, smem, h->stream>>>((float2*)cur_state(h), a);
    QGPU_CHECK_LAUNCH("k_group");
    h->launches++;
    h->h2d_bytes += sizeof(GroupArgs);
    return QGPU_OK;
}

// Uploads the tables of `gates` and runs one k_group launch per gate.
static int run_groups(qgpu_handle* h, const std::vector<const LocalGate*>& gates) {
    if (gates.empty()) return QGPU_OK;
    std::vector<GroupTables> lay(gates.size());
    size_t at = 0;
    for (size_t i = 0; i < gates.size(); ++i) {
        lay[i] = group_layout(gates[i]->k, at);
        at = align_up(lay[i].none_off + ((size_t)1 << gates[i]->k), 256);
    }
    std::vector<uint8_t> host(at, 0);
    std::vector<GroupArgs> args(gates.size());
    for (size_t i = 0; i < gates.size(); ++i) {
        std::memset(&args[i], 0, sizeof(GroupArgs));
        group_fill(*gates[i], h->n_qubits, host, 0, lay[i], &args[i]);
    }
    int st = h->gates.ensure(at);
    if (st != QGPU_OK) return st;
    QGPU_CUDA(copy_async(h, h->gates.ptr, host.data(), at, cudaMemcpyHostToDevice));
    for (size_t i = 0; i < gates.size(); ++i) {
        st = launch_group(h, args[i], (const uint8_t*)h->gates.ptr, lay[i]);
        if (st != QGPU_OK) return st;
    }
    // the host staging buffer must outlive the async copy
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

// =============================================================================================
// Register-tile kernels
// =============================================================================================
struct TileParams {
    uint64_t ngroups;
    const float4* tab_ff;     // TABLE entries, float pairs
    const double2* tab_f64;   // TABLE entries, f64
    int prefetch;             // prefetch the next grid-stride iteration into L2
    int streaming;            // register loads/stores with the evict-first (streaming) hint
    int nbits;
    int bits[MAX_TILE_BITS];
    int nsteps;
    DevStep steps[MAX_STEPS];
};

// multiply by i^code on any complex representation
template <class R>
__device__ __forceinline__ void unit_mul(R& a, int code);

template <>
__device__ __forceinline__ void unit_mul<ffp>(ffp& a, int code) {
    if (code == 0) return;
    float rh, ih, rl, il;
    up2(a.h, rh, ih);
    up2(a.l, rl, il);
    if (code == 1) {  // (re, im) -> (-im, re)
        a.h = p2(-ih, rh);
        a.l = p2(-il, rl);
    } else if (code == 2) {
        a.h = p2(-rh, -ih);
        a.l = p2(-rl, -il);
    } else {  // (re, im) -> (im, -re)
        a.h = p2(ih, -rh);
        a.l = p2(il, -rl);
    }
}
template <>
__device__ __forceinline__ void unit_mul<double2>(double2& a, int code) {
    if (code == 1) a = make_double2(-a.y, a.x);
    else if (code == 2) a = make_double2(-a.x, -a.y);
    else if (code == 3) a = make_double2(a.y, -a.x);
}
template <>
__device__ __forceinline__ void unit_mul<float2>(float2& a, int code) {
    if (code == 1) a = make_float2(-a.y, a.x);
    else if (code == 2) a = make_float2(-a.x, -a.y);
    else if (code == 3) a = make_float2(a.y, -a.x);
}

// ---- float-pair policy: complex128 storage, f64 arithmetic emulated on FP32/INT pipes -------
// Each complex value is two packed registers (ffp); one Dot2 computes the real and imaginary
// output lanes together: out = sum_t (c_t lanes) * (x_t lanes) with x_t = a, swap(a), b, swap(b).
struct PolFF {
    using S = double2;
    using R = ffp;
    static __device__ __forceinline__ R load(S a) { return to_ffp(a); }
    static __device__ __forceinline__ S store(const R& r) { return from_ffp(r); }
    // out0 = u00 a + u01 b ; out1 = u10 a + u11 b (packed terms, DevStep::pk)
    static __device__ __forceinline__ void dense(R& a, R& b, const DevStep& s) {
        ff_dense(a, b, s.pk);
    }
    static __device__ __forceinline__ void real(R& a, R& b, const DevStep& s) {
        const u64* c = s.pk;
        PDot2 d;
        R o0, o1;
        d.first(c + 0, a.h, a.l);
        d.add(c + 4, b.h, b.l);
        d.result(o0.h, o0.l);
        d.first(c + 8, a.h, a.l);
        d.add(c + 12, b.h, b.l);
        d.result(o1.h, o1.l);
        a = o0;
        b = o1;
    }
    // a *= c, with c's two packed terms at c[0..7]
    static __device__ __forceinline__ void mul_pk(R& a, const u64* c) {
        PDot2 d;
        d.first(c, a.h, a.l);
        d.add(c + 4, pswap(a.h), pswap(a.l));
        d.result(a.h, a.l);
    }
    static __device__ __forceinline__ void mul_slot(R& a, const DevStep& s, int slot) {
        mul_pk(a, s.pk + 8 * slot);
    }
    static __device__ __forceinline__ void mul_table(R& a, const TileParams& p, uint32_t e) {
        const float4 v = __ldg(p.tab_ff + e);  // (re_h, re_l, im_h, im_l)
        const u64 c[8] = {p2(v.x, v.x), p2(v.y, v.y), p2(-v.x, -v.x), p2(-v.y, -v.y),
                          p2(-v.z, v.z), p2(-v.w, v.w), p2(v.z, -v.z), p2(v.w, -v.w)};
        mul_pk(a, c);
    }
};

// ---- native f64 policy (FMA), for comparison ----------------------------------------------
struct PolF64 {
    using S = double2;
    using R = double2;
    static __device__ __forceinline__ R load(S a) { return a; }
    static __device__ __forceinline__ S store(const R& r) { return r; }
    static __device__ __forceinline__ double2 cmla(double2 acc, double ur, double ui, double2 x) {
        return make_double2(fma(ur, x.x, fma(-ui, x.y, acc.x)), fma(ur, x.y, fma(ui, x.x, acc.y)));
    }
    static __device__ __forceinline__ void dense(R& a, R& b, const DevStep& s) {
        const double* m = s.d;
        double2 o0 = cmla(cmla(make_double2(0, 0), m[0], m[1], a), m[2], m[3], b);
        double2 o1 = cmla(cmla(make_double2(0, 0), m[4], m[5], a), m[6], m[7], b);
        a = o0;
        b = o1;
    }
    static __device__ __forceinline__ void real(R& a, R& b, const DevStep& s) {
        const double* m = s.d;
        double2 o0 = make_double2(fma(m[0], a.x, m[2] * b.x), fma(m[0], a.y, m[2] * b.y));
        double2 o1 = make_double2(fma(m[4], a.x, m[6] * b.x), fma(m[4], a.y, m[6] * b.y));
        a = o0;
        b = o1;
    }
    static __device__ __forceinline__ void mul(R& a, double cr, double ci) {
        a = make_double2(fma(cr, a.x, -ci * a.y), fma(cr, a.y, ci * a.x));
    }
    static __device__ __forceinline__ void mul_slot(R& a, const DevStep& s, int slot) {
        mul(a, s.d[2 * slot], s.d[2 * slot + 1]);
    }
    static __device__ __forceinline__ void mul_table(R& a, const TileParams& p, uint32_t e) {
        const double2 c = __ldg(p.tab_f64 + e);
        mul(a, c.x, c.y);
    }
};

// ---- complex64 policy ------------------------------------------------------------------------
struct PolF32 {
    using S = float2;
    using R = float2;
    static __device__ __forceinline__ R load(S a) { return a; }
    static __device__ __forceinline__ S store(const R& r) { return r; }
    static __device__ __forceinline__ float2 cmla(float2 acc, float ur, float ui, float2 x) {
        return make_float2(fmaf(ur, x.x, fmaf(-ui, x.y, acc.x)), fmaf(ur, x.y, fmaf(ui, x.x, acc.y)));
    }
    static __device__ __forceinline__ void dense(R& a, R& b, const DevStep& s) {
        // hi parts of the float-pair entries are the entries rounded to f32
        const float* m = s.ff;
        float2 o0 = cmla(cmla(make_float2(0, 0), m[0], m[2], a), m[4], m[6], b);
        float2 o1 = cmla(cmla(make_float2(0, 0), m[8], m[10], a), m[12], m[14], b);
        a = o0;
        b = o1;
    }
    static __device__ __forceinline__ void real(R& a, R& b, const DevStep& s) {
        const float* m = s.ff;
        float2 o0 = make_float2(fmaf(m[0], a.x, m[4] * b.x), fmaf(m[0], a.y, m[4] * b.y));
        float2 o1 = make_float2(fmaf(m[8], a.x, m[12] * b.x), fmaf(m[8], a.y, m[12] * b.y));
        a = o0;
        b = o1;
    }
    static __device__ __forceinline__ void mul(R& a, float cr, float ci) {
        a = make_float2(fmaf(cr, a.x, -ci * a.y), fmaf(cr, a.y, ci * a.x));
    }
    static __device__ __forceinline__ void mul_slot(R& a, const DevStep& s, int slot) {
        mul(a, s.ff[4 * slot], s.ff[4 * slot + 2]);
    }
    static __device__ __forceinline__ void mul_table(R& a, const TileParams& p, uint32_t e) {
        const float4 c = __ldg(p.tab_ff + e);
        mul(a, c.x, c.z);
    }
};

// ---- data-movement-only policy (passes of permutations and +-1/+-i phases) -------------------
template <class T>
struct PolRaw {
    using S = T;
    using R = T;
    static __device__ __forceinline__ R load(S a) { return a; }
    static __device__ __forceinline__ S store(const R& r) { return r; }
};

// ---- resident float-pair layout ---------------------------------------------------------------
// During a run of float-pair passes the register can stay in float-pair form: each 16-byte
// amplitude slot holds (re_h, im_h | re_l, im_l) instead of (re, im) as doubles. Loads and stores
// are then plain register moves (no split, no join on the FP64 pipe); k_ff_layout converts the
// whole register once before the run and once after it.

struct PolFFR : PolFF {
    static __device__ __forceinline__ R load(S a) { return ffr_load(a); }
    static __device__ __forceinline__ S store(const R& r) { return ffr_store(r); }
};

// The first and the last arithmetic pass of a resident plan convert the layout themselves
// (instead of a separate streaming pass each way): PolFFIn reads complex128 and writes the
// resident layout, PolFFOut reads the resident layout and writes complex128.
struct PolFFIn : PolFF {
    static __device__ __forceinline__ S store(const R& r) { return ffr_store(r); }
};
struct PolFFOut : PolFF {
    static __device__ __forceinline__ R load(S a) { return ffr_load(a); }
};

// moves and +-1/+-i phases on the resident layout (a phase of i swaps and negates both halves)
struct PolRawFFR {
    using S = double2;
    using R = ffp;
    static __device__ __forceinline__ R load(S a) { return ffr_load(a); }
    static __device__ __forceinline__ S store(const R& r) { return ffr_store(r); }
};

// to_pairs: complex128 -> resident float pairs; otherwise back (in place, one pass each)
template <bool TO_PAIRS>
__global__ void __launch_bounds__(256) k_ff_layout(double2* __restrict__ st, uint64_t dim) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < dim; i += stride) {
        const double2 a = st[i];
        st[i] = TO_PAIRS ? ffr_store(to_ffp(a)) : from_ffp(ffr_load(a));
    }
}

// ---- pair blocks: a 4x4 complex matrix on two bits (fused gates on a wire pair) -------------
struct PairParams {
    uint64_t ngroups;
    int lo, hi;                // full-index bits, lo < hi; local index l = 2 * bit(hi) + bit(lo)
    uint64_t pk[128];          // PairBlock::pk
};

// v[r] <- sum_c m[r][c] v[c]: one 8-term packed Dot2 per output (terms x_c and swap(x_c))
__device__ __forceinline__ void ff_pair(ffp v[4], const u64* c) {
    ffp sw[4], o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        sw[q].h = pswap(v[q].h);
        sw[q].l = pswap(v[q].l);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const u64* cr = c + 32 * r;
        PDot2 d;
        d.first(cr, v[0].h, v[0].l);
        d.add(cr + 4, sw[0].h, sw[0].l);
#pragma unroll
        for (int q = 1; q < 4; ++q) {
            d.add(cr + 8 * q, v[q].h, v[q].l);
            d.add(cr + 8 * q + 4, sw[q].h, sw[q].l);
        }
        d.result(o[r].h, o[r].l);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = o[q];
}

// VARIANT 0: one quad per thread per iteration. 1: the next iteration's quad is loaded into
// registers before the current one is computed (loads in flight during the arithmetic).
// 2: two quads per thread per iteration (constants read once for both).
template <class P, int VARIANT>
__global__ void __launch_bounds__(256) k_pair(typename P::S* __restrict__ st,
                                              const __grid_constant__ PairParams p) {
    using S = typename P::S;
    const uint64_t olo = 1ull << p.lo, ohi = 1ull << p.hi;
    auto quad = [&](uint64_t g, uint64_t idx[4]) {
        const uint64_t b = insert_zero(insert_zero(g, p.lo), p.hi);
        idx[0] = b;
        idx[1] = b | olo;
        idx[2] = b | ohi;
        idx[3] = b | olo | ohi;
    };
    auto compute = [&](const S raw[4], const uint64_t idx[4]) {
        ffp v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = P::load(raw[j]);
        ff_pair(v, p.pk);
#pragma unroll
        for (int j = 0; j < 4; ++j) st[idx[j]] = P::store(v[j]);
    };
    if constexpr (VARIANT == 2) {
        const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * 2;
        for (uint64_t g0 = blockIdx.x * (uint64_t)blockDim.x * 2 + threadIdx.x; g0 < p.ngroups;
             g0 += stride) {
            const uint64_t g1 = g0 + blockDim.x;
            const bool has1 = g1 < p.ngroups;
            uint64_t i0[4], i1[4];
            quad(g0, i0);
            quad(has1 ? g1 : g0, i1);
            S r0[4], r1[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) r0[j] = st[i0[j]];
#pragma unroll
            for (int j = 0; j < 4; ++j) r1[j] = st[i1[j]];
            ffp v0[4], v1[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                v0[j] = P::load(r0[j]);
                v1[j] = P::load(r1[j]);
            }
            ff_pair(v0, p.pk);
            ff_pair(v1, p.pk);
#pragma unroll
            for (int j = 0; j < 4; ++j) st[i0[j]] = P::store(v0[j]);
            if (has1) {
#pragma unroll
                for (int j = 0; j < 4; ++j) st[i1[j]] = P::store(v1[j]);
            }
        }
    } else if constexpr (VARIANT == 1) {
        const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
        uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
        if (g >= p.ngroups) return;
        uint64_t idx[4];
        quad(g, idx);
        S raw[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) raw[j] = st[idx[j]];
        for (;;) {
            const uint64_t gn = g + stride;
            const bool more = gn < p.ngroups;
            uint64_t nidx[4];
            S nraw[4];
            if (more) {
                quad(gn, nidx);
#pragma unroll
                for (int j = 0; j < 4; ++j) nraw[j] = st[nidx[j]];
            }
            compute(raw, idx);
            if (!more) break;
            g = gn;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                idx[j] = nidx[j];
                raw[j] = nraw[j];
            }
        }
    } else {
        const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
        for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < p.ngroups;
             g += stride) {
            uint64_t idx[4];
            quad(g, idx);
            S raw[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) raw[j] = st[idx[j]];
            compute(raw, idx);
        }
    }
}

template <class P>
struct IsArith { static constexpr bool value = true; };
template <class T>
struct IsArith<PolRaw<T>> { static constexpr bool value = false; };
template <>
struct IsArith<PolRawFFR> { static constexpr bool value = false; };

// Applies step s to the 2^K amplitudes v of one tile (full indices base | off[j]).
template <int K, int B, class P>
__device__ __forceinline__ void step_on_bit(typename P::R* v, const DevStep& s, uint64_t base,
                                            const uint64_t* off) {
    constexpr int T = 1 << K;
    const bool controlled = s.cm != 0;
#pragma unroll
    for (int j = 0; j < T; ++j) {
        if ((j >> B) & 1) continue;
        const int j1 = j | (1 << B);
        if (controlled && ((base | off[j]) & s.cm) != s.cm) continue;
        if (s.type == ST_PERM) {
            typename P::R a = v[j], b = v[j1];
            if (s.anti) {
                v[j] = b;
                v[j1] = a;
            }
            unit_mul(v[j], s.u0);
            unit_mul(v[j1], s.u1);
        } else {
            if constexpr (IsArith<P>::value) {
                if (s.type == ST_DENSE) P::dense(v[j], v[j1], s);
                else P::real(v[j], v[j1], s);
            }
        }
    }
}

// Exchange the amplitudes whose tile bits (A, B) read (0, 1) and (1, 0): the Swap gate.
template <int K, int A, int B, class P>
__device__ __forceinline__ void swap_bits(typename P::R* v) {
#pragma unroll
    for (int j = 0; j < (1 << K); ++j) {
        if (((j >> A) & 1) == 0 && ((j >> B) & 1) == 1) {
            const int j2 = (j | (1 << A)) & ~(1 << B);
            typename P::R t = v[j];
            v[j] = v[j2];
            v[j2] = t;
        }
    }
}

template <int K, class P>
__device__ __forceinline__ void step_tile(typename P::R* v, const DevStep& s, uint64_t base,
                                          const uint64_t* off, const TileParams& p) {
    constexpr int T = 1 << K;
    switch (s.type) {
        case ST_DENSE:
        case ST_REAL:
        case ST_PERM:
            if (s.lb == 0) step_on_bit<K, 0, P>(v, s, base, off);
            if constexpr (K > 1) if (s.lb == 1) step_on_bit<K, (K > 1 ? 1 : 0), P>(v, s, base, off);
            if constexpr (K > 2) if (s.lb == 2) step_on_bit<K, (K > 2 ? 2 : 0), P>(v, s, base, off);
            break;
        case ST_SWAP: {
            const int lo = s.lb < s.lb2 ? s.lb : s.lb2, hi = s.lb < s.lb2 ? s.lb2 : s.lb;
            if constexpr (K >= 2) {
                if (lo == 0 && hi == 1) swap_bits<K, 0, 1, P>(v);
            }
            if constexpr (K >= 3) {
                if (lo == 0 && hi == 2) swap_bits<K, 0, (K >= 3 ? 2 : 1), P>(v);
                if (lo == 1 && hi == 2) swap_bits<K, 1, (K >= 3 ? 2 : 1), P>(v);
            }
            break;
        }
        case ST_PHASE:
#pragma unroll
            for (int j = 0; j < T; ++j) {
                if (((base | off[j]) & s.cm) != s.cm) continue;
                if (s.unit) unit_mul(v[j], s.u0);
                else if constexpr (IsArith<P>::value) P::mul_slot(v[j], s, 0);
            }
            break;
        case ST_DIAG:
#pragma unroll
            for (int j = 0; j < T; ++j) {
                const uint64_t idx = base | off[j];
                if ((idx & s.cm) != s.cm) continue;
                const int bit = (int)((idx >> s.fb) & 1ull);
                if (s.unit) unit_mul(v[j], bit ? s.u1 : s.u0);
                else if constexpr (IsArith<P>::value) P::mul_slot(v[j], s, bit);
            }
            break;
        case ST_TABLE:
            if constexpr (IsArith<P>::value) {
#pragma unroll
                for (int j = 0; j < T; ++j) {
                    const uint64_t idx = base | off[j];
                    if ((idx & s.cm) != s.cm) continue;
                    for (int f = 0; f < s.nfields; ++f) {
                        const uint32_t y =
                            (uint32_t)((idx >> s.tab_shift[f]) & ((1ull << s.tab_width[f]) - 1ull));
                        P::mul_table(v[j], p, s.tab_off[f] + y);
                    }
                }
            }
            break;
        default:
            break;
    }
}

// Register traffic of the tile kernels; with `streaming` the cache-streaming forms keep the
// once-touched amplitudes from evicting phase-table lines out of L1.
template <class S>
__device__ __forceinline__ S tile_load(const S* p, int streaming) {
    return streaming ? __ldcs(p) : *p;
}
template <class S>
__device__ __forceinline__ void tile_store(S* p, S v, int streaming) {
    if (streaming) __stcs(p, v);
    else *p = v;
}

// ONE >= 0: the pass is exactly one unconditional step of that type on tile bit 0 (the common
// single fused gate), applied as straight-line code without the step loop or its dispatch.
template <int K, int U, class P, int ONE = -1>
__global__ void __launch_bounds__(256) k_tile(typename P::S* __restrict__ st, const __grid_constant__ TileParams p) {
    constexpr int T = 1 << K;
    uint64_t off[T];
#pragma unroll
    for (int j = 0; j < T; ++j) {
        uint64_t o = 0;
#pragma unroll
        for (int m = 0; m < K; ++m)
            if ((j >> m) & 1) o |= 1ull << p.bits[m];
        off[j] = o;
    }
    const uint64_t chunk = (uint64_t)blockDim.x * U;
    for (uint64_t g0 = (uint64_t)blockIdx.x * chunk; g0 < p.ngroups; g0 += (uint64_t)gridDim.x * chunk) {
        uint64_t base[U];
        typename P::S raw[U][T];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t g = g0 + (uint64_t)u * blockDim.x + threadIdx.x;
            uint64_t b = g;
#pragma unroll
            for (int m = 0; m < K; ++m) b = insert_zero(b, p.bits[m]);
            base[u] = b;
            if (g < p.ngroups) {
#pragma unroll
                for (int j = 0; j < T; ++j) raw[u][j] = tile_load(st + (b | off[j]), p.streaming);
            }
        }
        if (p.prefetch) {  // the next iteration's amplitudes head for L2 while this one computes
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint64_t g = g0 + (uint64_t)gridDim.x * chunk + (uint64_t)u * blockDim.x + threadIdx.x;
                if (g >= p.ngroups) continue;
                uint64_t b = g;
#pragma unroll
                for (int m = 0; m < K; ++m) b = insert_zero(b, p.bits[m]);
#pragma unroll
                for (int j = 0; j < T; ++j)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(st + (b | off[j])));
            }
        }
        typename P::R v[U][T];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int j = 0; j < T; ++j) v[u][j] = P::load(raw[u][j]);
        // step-major: each step's constants and dispatch are read once for all U groups
        if constexpr (ONE == ST_DENSE && IsArith<P>::value && K == 1) {
#pragma unroll
            for (int u = 0; u < U; ++u) P::dense(v[u][0], v[u][1], p.steps[0]);
        } else if constexpr (ONE == ST_DENSE && IsArith<P>::value && K == 2) {
            // every step an unconditional dense 2x2 on tile bit 0 or 1 (fused single-wire gates)
            for (int s = 0; s < p.nsteps; ++s) {
                const DevStep& sp = p.steps[s];
                if (sp.lb == 0) {
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        P::dense(v[u][0], v[u][1], sp);
                        P::dense(v[u][2], v[u][3], sp);
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        P::dense(v[u][0], v[u][2], sp);
                        P::dense(v[u][1], v[u][3], sp);
                    }
                }
            }
        } else if constexpr (ONE == ST_REAL && IsArith<P>::value) {
#pragma unroll
            for (int u = 0; u < U; ++u) P::real(v[u][0], v[u][1], p.steps[0]);
        } else if constexpr (ONE == ST_TABLE && IsArith<P>::value) {
            // QFT rows and rotation layers: unconditional REAL / DENSE steps, +-1/+-i monomials and
            // phase tables only (no dispatch over the other step kinds, no control test on the
            // 2x2 steps)
            for (int s = 0; s < p.nsteps; ++s) {
                const DevStep& sp = p.steps[s];
                if (sp.type == ST_PERM) {  // +-1 / +-i monomial under its control mask
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (sp.lb == 0) step_on_bit<K, 0, P>(v[u], sp, base[u], off);
                        if constexpr (K > 1) if (sp.lb == 1) step_on_bit<K, (K > 1 ? 1 : 0), P>(v[u], sp, base[u], off);
                    }
                } else if (sp.type == ST_TABLE) {
#pragma unroll
                    for (int u = 0; u < U; ++u)
#pragma unroll
                        for (int j = 0; j < T; ++j) {
                            const uint64_t idx = base[u] | off[j];
                            if ((idx & sp.cm) != sp.cm) continue;
#pragma unroll
                            for (int f = 0; f < MAX_TABLE_FIELDS; ++f) {
                                if (f >= sp.nfields) break;
                                const uint32_t y = (uint32_t)((idx >> sp.tab_shift[f]) &
                                                              ((1ull << sp.tab_width[f]) - 1ull));
                                P::mul_table(v[u][j], p, sp.tab_off[f] + y);
                            }
                        }
                } else {
                    const bool dense = sp.type == ST_DENSE;
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if constexpr (K == 1) {
                            if (dense) P::dense(v[u][0], v[u][1], sp);
                            else P::real(v[u][0], v[u][1], sp);
                        } else if (sp.lb == 0) {
                            if (dense) {
                                P::dense(v[u][0], v[u][1], sp);
                                P::dense(v[u][2], v[u][3], sp);
                            } else {
                                P::real(v[u][0], v[u][1], sp);
                                P::real(v[u][2], v[u][3], sp);
                            }
                        } else {
                            if (dense) {
                                P::dense(v[u][0], v[u][2], sp);
                                P::dense(v[u][1], v[u][3], sp);
                            } else {
                                P::real(v[u][0], v[u][2], sp);
                                P::real(v[u][1], v[u][3], sp);
                            }
                        }
                    }
                }
            }
        } else {
            for (int s = 0; s < p.nsteps; ++s) {
                const DevStep& sp = p.steps[s];
#pragma unroll
                for (int u = 0; u < U; ++u) step_tile<K, P>(v[u], sp, base[u], off, p);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t g = g0 + (uint64_t)u * blockDim.x + threadIdx.x;
            if (g >= p.ngroups) continue;
#pragma unroll
            for (int j = 0; j < T; ++j) tile_store(st + (base[u] | off[j]), P::store(v[u][j]), p.streaming);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// k_tile1_pipe: the 1-bit tile pass with bulk-copy (TMA) staging.
// The register is cut into chunks of PIPE_CH amplitude pairs (32 KB of complex128). Chunk c of a
// pass on bit q is either one contiguous run of 2*PIPE_CH amplitudes (q < log2 PIPE_CH: both
// halves of every pair interleave inside it) or two runs of PIPE_CH amplitudes 2^q apart. Each
// persistent CTA owns chunks blockIdx.x + i*gridDim.x; one thread keeps PIPE_STAGES-1 chunks in
// flight with cp.async.bulk (mbarrier completion) while all threads compute the current chunk
// from shared memory and store results straight to global memory (coalesced).
// ---------------------------------------------------------------------------------------------
constexpr int PIPE_LOG_CH = 10;
constexpr int PIPE_CH = 1 << PIPE_LOG_CH;  // amplitude pairs per chunk
constexpr int PIPE_STAGES = 2;
constexpr int PIPE_THREADS = 256;
constexpr uint32_t PIPE_WAIT_LIMIT = 1u << 24;  // polls before a wait is declared failed

template <class P>
__global__ void __launch_bounds__(PIPE_THREADS, 3)
k_tile1_pipe(typename P::S* __restrict__ st, const __grid_constant__ TileParams p, uint64_t nchunks,
             int* __restrict__ err) {
    using S = typename P::S;
    extern __shared__ __align__(128) unsigned char smem[];
    S* stage = reinterpret_cast<S*>(smem);
    __shared__ __align__(8) uint64_t bars[PIPE_STAGES];
    const int q = p.bits[0];
    const bool two_runs = q >= PIPE_LOG_CH;
    const uint32_t chunk_bytes = 2u * PIPE_CH * (uint32_t)sizeof(S);
    if (threadIdx.x == 0) {
        for (int s = 0; s < PIPE_STAGES; ++s) mbar_init(smem_u32(&bars[s]), 1);
        fence_proxy_async_shared();
    }
    __syncthreads();
    const uint64_t my_n =
        nchunks > blockIdx.x ? (nchunks - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    auto chunk_of = [&](uint64_t i) -> uint64_t { return blockIdx.x + i * gridDim.x; };
    auto issue = [&](uint64_t i, int s) {  // thread 0 only
        const uint64_t c = chunk_of(i);
        const uint32_t dst = smem_u32(stage + (size_t)s * 2 * PIPE_CH);
        const uint32_t bar = smem_u32(&bars[s]);
        mbar_arrive_expect_tx(bar, chunk_bytes);
        if (two_runs) {
            const uint64_t b0 = insert_zero(c * PIPE_CH, q);
            bulk_g2s(dst, st + b0, chunk_bytes / 2, bar);
            bulk_g2s(dst + chunk_bytes / 2, st + b0 + (1ull << q), chunk_bytes / 2, bar);
        } else {
            bulk_g2s(dst, st + c * 2 * PIPE_CH, chunk_bytes, bar);
        }
    };
    if (threadIdx.x == 0)
        for (int s = 0; s < PIPE_STAGES && (uint64_t)s < my_n; ++s) issue(s, s);
    uint64_t off[2] = {0, 1ull << q};
    bool failed = false;
    uint64_t i = 0;
    for (; i < my_n; ++i) {
        const int s = (int)(i % PIPE_STAGES);
        if (i > 0) {
            __syncthreads();  // every thread is done with chunk i-1: refill its stage
            if (threadIdx.x == 0 && i - 1 + PIPE_STAGES < my_n)
                issue(i - 1 + PIPE_STAGES, (int)((i - 1) % PIPE_STAGES));
        }
        const bool ok = mbar_wait_bounded(smem_u32(&bars[s]), (uint32_t)((i / PIPE_STAGES) & 1),
                                          PIPE_WAIT_LIMIT);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        const S* src = stage + (size_t)s * 2 * PIPE_CH;
        const uint64_t c = chunk_of(i);
#pragma unroll
        for (int k = 0; k < PIPE_CH / PIPE_THREADS; ++k) {
            const int lp = threadIdx.x + k * PIPE_THREADS;  // pair within the chunk
            int l0, l1;
            uint64_t g0;
            if (two_runs) {
                l0 = lp;
                l1 = PIPE_CH + lp;
                g0 = insert_zero(c * PIPE_CH, q) + lp;
            } else {
                l0 = (int)insert_zero((uint64_t)lp, q);
                l1 = l0 + (1 << q);
                g0 = c * 2 * PIPE_CH + l0;
            }
            typename P::R v[2] = {P::load(src[l0]), P::load(src[l1])};
            for (int t = 0; t < p.nsteps; ++t) step_tile<1, P>(v, p.steps[t], g0, off, p);
            st[g0] = P::store(v[0]);
            st[g0 + (1ull << q)] = P::store(v[1]);
        }
    }
    if (failed) {
        // record the failure, then let this CTA's copies still in flight land before exiting
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            for (uint64_t j = i; j < my_n && j < i + PIPE_STAGES; ++j)
                mbar_wait_bounded(smem_u32(&bars[j % PIPE_STAGES]), (uint32_t)((j / PIPE_STAGES) & 1),
                                  PIPE_WAIT_LIMIT);
        }
        __syncthreads();
    }
}

template <class P>
static int launch_tile1_pipe(qgpu_handle* h, const TileParams& p) {
    using S = typename P::S;
    const size_t smem = (size_t)PIPE_STAGES * 2 * PIPE_CH * sizeof(S);
    QGPU_CUDA(smem_opt_in((const void*)k_tile1_pipe<P>, smem));
    const uint64_t nchunks = h->dim / (2ull * PIPE_CH);
    uint64_t blocks = std::min<uint64_t>(nchunks, (uint64_t)h->sm_count * 3);
    if (blocks < 1) blocks = 1;
    k_tile1_pipe<P><<<(unsigned)blocks, PIPE_THREADS, smem, h->stream>>>(
        (S*)cur_state(h), p, nchunks, h->d_err);
    QGPU_CHECK_LAUNCH("k_tile1_pipe");
    h->launches++;
    h->h2d_bytes += sizeof(TileParams);
    return QGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// k_xor_perm: a run of commuting controlled-X gates as one involution i -> j = i ^ f(i). f only
// reads control bits, which no gate of the run changes, so f(j) = f(i): the thread with the
// smaller index of each pair swaps it, the other does nothing. Amplitudes no gate moves are not
// touched.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t xor_f(uint64_t i, const XorPerm& xp) {
    uint64_t f = 0;
    for (int e = 0; e < xp.nterms; ++e) {
        if (xp.grouped[e] == 1) {
            const uint64_t c = i & xp.cm[e];
            f |= xp.shift[e] > 0 ? (c >> xp.shift[e]) : (c << -xp.shift[e]);
        } else if (xp.grouped[e] == 2) {
            if (__popcll(i & xp.cm[e]) == 1) f |= xp.cm[e];  // swap of two differing bits
        } else if ((i & xp.cm[e]) == xp.cm[e]) {
            f |= xp.tbit[e];
        }
    }
    return f;
}

// U indices per thread (blockDim apart, so each of the U rounds is a coalesced warp access):
// all loads of a thread are issued before its stores, U x the memory-level parallelism of one
// index per thread (half the threads of a round have nothing to do: j < i).
template <class S, int U>
__global__ void __launch_bounds__(256) k_xor_perm(S* __restrict__ st, uint64_t dim,
                                                  const __grid_constant__ XorPerm xp) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * U;
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x * U + threadIdx.x; i0 < dim; i0 += stride) {
        uint64_t ii[U], jj[U];
        bool act[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t i = i0 + (uint64_t)u * blockDim.x;
            ii[u] = i;
            jj[u] = i < dim ? (i ^ xor_f(i, xp)) : i;
            act[u] = jj[u] > i;
        }
        S a[U], b[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (act[u]) {
                a[u] = st[ii[u]];
                b[u] = st[jj[u]];
            }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (act[u]) {
                st[ii[u]] = b[u];
                st[jj[u]] = a[u];
            }
    }
}

// ---------------------------------------------------------------------------------------------
// k_bitperm: a run of disjoint swaps (a QFT's final bit reversal) permutes index bits: amplitude
// x moves to pi(x), pi an involution on bit positions. Scattered one-by-one swaps of such a run
// touch a different far-away DRAM page per lane; this kernel tiles instead. Tile bits B = the 5
// lowest bits and their images (|B| <= 10, closed under pi); a tile = the 2^|B| amplitudes that
// share all other bits (a base). pi maps tile(base) onto tile(pi(base)): a CTA owns both tiles of
// a pair (or one tile that maps onto itself), stages them in shared memory with coalesced loads
// (low bits fastest) and writes each destination tile with coalesced stores, in place. Tile slot
// l sits at l ^ ((l >> 5) & 31) in shared memory: the loads (32 consecutive l per warp) and the
// gather of a bit reversal (which sends the lane bits to the tile's high bits) both touch every
// bank group equally instead of the gather hitting one.
// ---------------------------------------------------------------------------------------------
constexpr int BP_MAX_BITS = 10;

struct BitPermArgs {
    int nb;                    // |B|
    int bits[BP_MAX_BITS];     // B, ascending: tile-local bit m <-> bits[m]
    int perm[64];              // pi(b) for every index bit b
    int n;
    uint64_t nbases;           // 2^(n - nb)
};

__device__ __forceinline__ int bp_swz(int l) { return l ^ ((l >> 5) & 31); }

template <class S>
__global__ void __launch_bounds__(256) k_bitperm(S* __restrict__ st, const __grid_constant__ BitPermArgs p) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int T = 1 << p.nb;
    S* tA = reinterpret_cast<S*>(smem);
    S* tB = tA + T;
    uint64_t* offB = reinterpret_cast<uint64_t*>(tB + T);  // [T] spread of local index l over B
    uint16_t* pl = reinterpret_cast<uint16_t*>(offB + T);   // [T] local index of pi(spread(l))
    for (int l = threadIdx.x; l < T; l += blockDim.x) {
        uint64_t o = 0;
        int q = 0;
        for (int m = 0; m < p.nb; ++m)
            if ((l >> m) & 1) {
                o |= 1ull << p.bits[m];
                const int pb = p.perm[p.bits[m]];
                for (int r = 0; r < p.nb; ++r)
                    if (p.bits[r] == pb) q |= 1 << r;
            }
        offB[l] = o;
        pl[l] = (uint16_t)q;
    }
    __syncthreads();
    for (uint64_t bi = blockIdx.x; bi < p.nbases; bi += gridDim.x) {
        uint64_t base = bi;
        for (int m = 0; m < p.nb; ++m) base = insert_zero(base, p.bits[m]);
        uint64_t pbase = 0;  // pi(base): non-B bits map to non-B bits
        for (int b = 0; b < p.n; ++b)
            if ((base >> b) & 1ull) pbase |= 1ull << p.perm[b];
        if (pbase < base) continue;  // the partner tile's CTA moves this pair
        const bool self = pbase == base;
        for (int l = threadIdx.x; l < T; l += blockDim.x) {
            tA[bp_swz(l)] = st[base | offB[l]];
            if (!self) tB[bp_swz(l)] = st[pbase | offB[l]];
        }
        __syncthreads();
        // destination d = base | spread(l) receives pi(d) = pbase | spread(pl[l])
        for (int l = threadIdx.x; l < T; l += blockDim.x) {
            const int q = bp_swz(pl[l]);
            st[base | offB[l]] = self ? tA[q] : tB[q];
            if (!self) st[pbase | offB[l]] = tA[q];
        }
        __syncthreads();
    }
}

// Whether an XOR pass is a run of swaps only; fills the bit permutation if so.
static bool xor_as_bitperm(const qgpu_handle* h, const XorPerm& xp, BitPermArgs* a) {
    if (xp.nterms == 0) return false;
    std::memset(a, 0, sizeof(*a));
    a->n = h->n_qubits;
    for (int b = 0; b < 64; ++b) a->perm[b] = b;
    for (int e = 0; e < xp.nterms; ++e) {
        if (xp.grouped[e] != 2 || __builtin_popcountll(xp.cm[e]) != 2) return false;
        const int b0 = __builtin_ctzll(xp.cm[e]), b1 = 63 - __builtin_clzll(xp.cm[e]);
        if (a->perm[b0] != b0 || a->perm[b1] != b1) return false;  // swaps must be disjoint
        a->perm[b0] = b1;
        a->perm[b1] = b0;
    }
    uint64_t B = 0;
    for (int b = 0; b < 5 && b < a->n; ++b) B |= (1ull << b) | (1ull << a->perm[b]);
    a->nb = __builtin_popcountll(B);
    if (a->nb > BP_MAX_BITS) return false;
    for (int b = 0, m = 0; b < 64; ++b)
        if ((B >> b) & 1ull) a->bits[m++] = b;
    a->nbases = h->dim >> a->nb;
    return true;
}

static int launch_bitperm(qgpu_handle* h, const BitPermArgs& a) {
    const int T = 1 << a.nb;
    const size_t smem = (size_t)T * (2 * h->amp_bytes + 8 + 2);
    uint64_t blocks = std::min<uint64_t>(a.nbases, (uint64_t)h->sm_count * 8);
    if (blocks < 1) blocks = 1;
    if (h->precision == QGPU_C128)
        k_bitperm<double2><<<(unsigned)blocks, 256, smem, h->stream>>>((double2*)cur_state(h), a);
    else
        k_bitperm<float2><<<(unsigned)blocks, 256, smem, h->stream>>>((float2*)cur_state(h), a);
    QGPU_CHECK_LAUNCH("k_bitperm");
    h->launches++;
    h->h2d_bytes += sizeof(BitPermArgs);
    return QGPU_OK;
}

static int launch_xor(qgpu_handle* h, const XorPerm& xp) {
    BitPermArgs bp;
    if (xor_as_bitperm(h, xp, &bp)) return launch_bitperm(h, bp);
    constexpr int U = 4;
    uint64_t blocks = (h->dim + 256 * U - 1) / (256 * U);
    const uint64_t cap = (uint64_t)h->sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (h->precision == QGPU_C128)
        k_xor_perm<double2, U><<<(unsigned)blocks, 256, 0, h->stream>>>((double2*)cur_state(h), h->dim, xp);
    else
        k_xor_perm<float2, U><<<(unsigned)blocks, 256, 0, h->stream>>>((float2*)cur_state(h), h->dim, xp);
    QGPU_CHECK_LAUNCH("k_xor_perm");
    h->launches++;
    h->h2d_bytes += sizeof(XorPerm);
    return QGPU_OK;
}

static int env_int(const char* name, int dflt);

// Bulk-copy staging for 1-bit tiles (QGPU_PIPE=1). Its kernel reports bounded-wait timeouts
// through the handle's error word, so plans run with it are synchronised at the end.
static int pipe_enabled() {
    static const int on = env_int("QGPU_PIPE", 0);
    return on;
}

template <int K, int U, class P>
static int launch_tile_t(qgpu_handle* h, const TileParams& p) {
    const uint64_t per_block = 256ull * U;
    uint64_t blocks = (p.ngroups + per_block - 1) / per_block;
    const uint64_t cap = (uint64_t)h->sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    typename P::S* s = (typename P::S*)cur_state(h);
    bool launched = false;
    if constexpr (K == 1 && IsArith<P>::value) {
        if (p.nsteps == 1 && p.steps[0].cm == 0) {
            if (p.steps[0].type == ST_DENSE) {
                k_tile<K, U, P, ST_DENSE><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
                launched = true;
            } else if (p.steps[0].type == ST_REAL) {
                k_tile<K, U, P, ST_REAL><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
                launched = true;
            }
        }
    }
    if constexpr (K == 2 && IsArith<P>::value) {
        static const int straight = env_int("QGPU_K2_STRAIGHT", 1);
        bool all_dense = straight != 0;
        for (int i = 0; i < p.nsteps && all_dense; ++i)
            all_dense = p.steps[i].type == ST_DENSE && p.steps[i].cm == 0;
        if (all_dense) {
            k_tile<K, U, P, ST_DENSE><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
            launched = true;
        }
    }
    if constexpr ((K == 1 || K == 2) && IsArith<P>::value) {
        // passes of unconditional 2x2 steps, monomials and phase tables only (the QFT rows,
        // rotation layers with their CNots): straight-line variant; tuning knob
        // QGPU_TABLE_STRAIGHT=0 keeps the step loop
        static const int straight_tab = env_int("QGPU_TABLE_STRAIGHT", 1);
        bool ok = !launched && straight_tab != 0, any_table = false;
        for (int i = 0; i < p.nsteps && ok; ++i) {
            const DevStep& d = p.steps[i];
            any_table = any_table || d.type == ST_TABLE;
            ok = d.type == ST_TABLE || d.type == ST_PERM ||
                 ((d.type == ST_DENSE || d.type == ST_REAL) && d.cm == 0);
        }
        if (ok && (any_table || p.nsteps > 1)) {
            k_tile<K, U, P, ST_TABLE><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
            launched = true;
        }
    }
    if (!launched) k_tile<K, U, P><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
    QGPU_CHECK_LAUNCH("k_tile");
    h->launches++;
    h->h2d_bytes += sizeof(TileParams);
    return QGPU_OK;
}

template <class P>
static int launch_tile_k(qgpu_handle* h, const TileParams& p) {
    // Groups per thread: 4 amplitudes live per thread (8 for 3-bit tiles) keeps the float-pair
    // passes near 56 registers and 4 CTAs per SM; measured on GB300, 2 groups of a 1-bit tile
    // ran 17 % faster than 4.
    static const int k1_groups = env_int("QGPU_K1_GROUPS", 2);  // tuning knob: 2 or 4
    // Bulk-copy staging for 1-bit tiles (k_tile1_pipe): correct and measured, but on GB300 its
    // shared-memory footprint lowers occupancy below what the float-pair arithmetic needs, so the
    // register-tile kernel stays the default (QGPU_PIPE=1 selects the pipeline).
    static const int use_pipe = pipe_enabled();
    switch (p.nbits) {
        case 1:
            if (use_pipe && h->n_qubits >= 13) return launch_tile1_pipe<P>(h, p);
            return k1_groups == 4 ? launch_tile_t<1, 4, P>(h, p) : launch_tile_t<1, 2, P>(h, p);
        case 2: {
            static const int k2_groups = env_int("QGPU_K2_GROUPS", 1);  // tuning knob: 1 or 2
            return k2_groups == 2 ? launch_tile_t<2, 2, P>(h, p) : launch_tile_t<2, 1, P>(h, p);
        }
        default: return launch_tile_t<3, 1, P>(h, p);
    }
}

static int policy_of(const qgpu_handle* h) {
    if (h->precision == QGPU_C64) return POL_F32;
    return h->mode == QGPU_MODE_F64 ? POL_F64 : POL_FF;
}

static int env_int(const char* name, int dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    return std::atoi(v);
}

static int launch_pass(qgpu_handle* h, const Pass& ps, int pol, int lay,
                       const float4* tab_ff, const double2* tab_f64, TileParams& tp);

static int launch_ff_layout(qgpu_handle* h, bool to_pairs) {
    uint64_t blocks = (h->dim + 255) / 256;
    const uint64_t cap = (uint64_t)h->sm_count * 8;
    if (blocks > cap) blocks = cap;
    double2* s = (double2*)cur_state(h);
    if (to_pairs) k_ff_layout<true><<<(unsigned)blocks, 256, 0, h->stream>>>(s, h->dim);
    else k_ff_layout<false><<<(unsigned)blocks, 256, 0, h->stream>>>(s, h->dim);
    QGPU_CHECK_LAUNCH("k_ff_layout");
    h->launches++;
    return QGPU_OK;
}

// complex64 pair blocks: the 4x4 in f32 FMA, 16 complex multiply-adds per quad (memory-bound)
struct PairParams32 {
    uint64_t ngroups;
    int lo, hi;
    float2 m[4][4];  // m[out][in]
};

__global__ void __launch_bounds__(256) k_pair_f32(float2* __restrict__ st,
                                                  const __grid_constant__ PairParams32 p) {
    const uint64_t olo = 1ull << p.lo, ohi = 1ull << p.hi;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < p.ngroups; g += stride) {
        const uint64_t b = insert_zero(insert_zero(g, p.lo), p.hi);
        const uint64_t idx[4] = {b, b | olo, b | ohi, b | olo | ohi};
        float2 x[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) x[j] = st[idx[j]];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float re = 0.f, im = 0.f;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float2 u = p.m[r][c];
                re = fmaf(u.x, x[c].x, fmaf(-u.y, x[c].y, re));
                im = fmaf(u.x, x[c].y, fmaf(u.y, x[c].x, im));
            }
            st[idx[r]] = make_float2(re, im);
        }
    }
}

// Layout of a float-pair pass: LAY_PLAIN (complex128 in and out), LAY_RES (resident in and out),
// LAY_IN (complex128 in, resident out), LAY_OUT (resident in, complex128 out).
enum PassLayout { LAY_PLAIN = 0, LAY_RES = 1, LAY_IN = 2, LAY_OUT = 3 };

static int launch_pair(qgpu_handle* h, const PairBlock& pb, int lay) {
    const bool resident = lay == LAY_RES;
    if (h->precision == QGPU_C64) {
        PairParams32 q;
        q.ngroups = h->dim >> 2;
        q.lo = pb.lo;
        q.hi = pb.hi;
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c)
                q.m[r][c] = make_float2((float)pb.m[r][c].real(), (float)pb.m[r][c].imag());
        uint64_t blocks = std::min<uint64_t>((q.ngroups + 255) / 256, (uint64_t)h->sm_count * 8);
        if (blocks < 1) blocks = 1;
        k_pair_f32<<<(unsigned)blocks, 256, 0, h->stream>>>((float2*)cur_state(h), q);
        QGPU_CHECK_LAUNCH("k_pair_f32");
        h->launches++;
        h->h2d_bytes += sizeof(PairParams32);
        return QGPU_OK;
    }
    PairParams p;
    p.ngroups = h->dim >> 2;
    p.lo = pb.lo;
    p.hi = pb.hi;
    std::memcpy(p.pk, pb.pk, sizeof(p.pk));
    uint64_t blocks = (p.ngroups + 255) / 256;
    const uint64_t cap = (uint64_t)h->sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    double2* s = (double2*)cur_state(h);
    static const int variant = env_int("QGPU_PAIR_VARIANT", 0);  // tuning knob: 0, 1 or 2
    if (variant == 2 && (lay == LAY_RES || lay == LAY_PLAIN)) {
        blocks = std::max<uint64_t>(1, std::min<uint64_t>((p.ngroups + 511) / 512, cap));
        if (resident) k_pair<PolFFR, 2><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
        else k_pair<PolFF, 2><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
    } else if (variant == 1 && (lay == LAY_RES || lay == LAY_PLAIN)) {
        if (resident) k_pair<PolFFR, 1><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
        else k_pair<PolFF, 1><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
    } else if (lay == LAY_IN) {
        k_pair<PolFFIn, 0><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
    } else if (lay == LAY_OUT) {
        k_pair<PolFFOut, 0><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
    } else {
        if (resident) k_pair<PolFFR, 0><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
        else k_pair<PolFF, 0><<<(unsigned)blocks, 256, 0, h->stream>>>(s, p);
    }
    QGPU_CHECK_LAUNCH("k_pair");
    h->launches++;
    h->h2d_bytes += sizeof(PairParams);
    return QGPU_OK;
}

// ---- double pair passes: two 4x4 blocks on disjoint bit pairs of a 4-bit tile --------------
// A tile is 16 amplitudes (full indices base | combinations of the 4 bits). Its amplitudes are
// gathered through the slot permutation of the XOR terms folded before the blocks, block A (the
// one on local bit 0) and block B are applied, and they are scattered through the permutation of
// the terms folded after them. Every term flips only tile bits, so sources and destinations are
// the tile's own 16 slots and the pass stays in place. complex128 (float pairs): four threads
// share a tile (k_pair2); complex64: one thread holds it (k_pair2_f32).
struct Pair2Params {
    uint64_t ngroups;                   // dim / 16
    int bits[4];                        // full-index bits, ascending
    // full-index offset, within the tile, that local slot j is read from / written to: the
    // identity, or the permutation of the XOR terms folded before / after the blocks (their bits
    // all lie in the tile, so the permutation is the same for every tile)
    uint64_t pre_off[16], post_off[16];
};
struct Pair2ParamsFF : Pair2Params {
    uint64_t pka[128], pkb[128];        // PairBlock::pk of blocks A and B
};
struct Pair2Params32 : Pair2Params {
    float2 ma[4][4], mb[4][4];          // m[out][in] of blocks A and B
};

// PART: which local bits block A holds with local bit 0 (0: bit 1, 1: bit 2, 2: bit 3); block B
// holds the other two.
template <int PART>
struct Pair2Layout {
    static constexpr int A0 = 0, A1 = PART + 1;
    static constexpr int B0 = PART == 0 ? 2 : 1, B1 = PART == 2 ? 2 : 3;
};

// Four lanes share a tile: lane `sub` first holds the quad over block A's bits at B-combination
// sub (four loads), applies A, and the tile is transposed through shared memory so that it then
// holds the quad over block B's bits at A-combination sub; it applies B and stores. A thread so
// keeps one quad in registers, like k_pair. Shared layout per tile: 20 16-byte units (4 of
// padding), element (a, b) at unit 4a + (b ^ a): the stores of one a and the loads of one b both
// hit eight distinct bank groups per quarter warp.
constexpr int PAIR2_THREADS = 256;
constexpr int PAIR2_UNITS = 20;

// Applies fn(w[4]) to the four quads of v[16] over local bits (X0 < X1), quad order
// l = 2 bit(X1) + bit(X0), for every combination of the other two local bits (Y0, Y1).
template <int X0, int X1, int Y0, int Y1, class V, class F>
__device__ __forceinline__ void tile_quads(V* v, F&& fn) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int jb = ((q & 1) << Y0) | ((q >> 1) << Y1);
        V w[4] = {v[jb], v[jb | (1 << X0)], v[jb | (1 << X1)], v[jb | (1 << X0) | (1 << X1)]};
        fn(w);
        v[jb] = w[0];
        v[jb | (1 << X0)] = w[1];
        v[jb | (1 << X1)] = w[2];
        v[jb | (1 << X0) | (1 << X1)] = w[3];
    }
}

template <class P, int PART, class Prm, class Apply>
__device__ __forceinline__ void pair2_body(typename P::S* __restrict__ st, const Prm& p,
                                           Apply&& apply) {
    using L = Pair2Layout<PART>;
    using R = typename P::R;
    __shared__ R xs[PAIR2_THREADS / 4][PAIR2_UNITS];
    const int sub = threadIdx.x & 3;
    const int tl = threadIdx.x >> 2;
    // local slot of A-combination a and B-combination b
    auto slot = [](int a, int b) {
        return ((a & 1) << L::A0) | ((a >> 1) << L::A1) | ((b & 1) << L::B0) | ((b >> 1) << L::B1);
    };
    const uint64_t tiles_per_cta = PAIR2_THREADS / 4;
    const uint64_t tstride = (uint64_t)gridDim.x * tiles_per_cta;
    // every warp runs the same number of iterations (shared-memory exchange inside)
    const uint64_t wfirst = blockIdx.x * tiles_per_cta + (tl & ~7);
    for (uint64_t g0 = wfirst; g0 < p.ngroups; g0 += tstride) {
        const uint64_t g = g0 + (tl & 7);
        const bool active = g < p.ngroups;
        const uint64_t base =
            insert_zero(insert_zero(insert_zero(insert_zero(active ? g : g0, p.bits[0]), p.bits[1]),
                                    p.bits[2]),
                        p.bits[3]);
        R w[4];
        // the slot offsets are re-read from the parameter bank every iteration (hoisted out of
        // the loop they would take 16 registers and spill under the 64-register bound)
        int ls;
        asm volatile("mov.b32 %0, %1;" : "=r"(ls) : "r"(sub));
        if (active) {
#pragma unroll
            for (int a = 0; a < 4; ++a) w[a] = P::load(st[base | p.pre_off[slot(a, ls)]]);
            apply(w, 0);
#pragma unroll
            for (int a = 0; a < 4; ++a) xs[tl][4 * a + (sub ^ a)] = w[a];
        }
        __syncwarp();
        if (active) {
#pragma unroll
            for (int b = 0; b < 4; ++b) w[b] = xs[tl][4 * sub + (b ^ sub)];
        }
        __syncwarp();
        if (active) {
            apply(w, 1);
#pragma unroll
            for (int b = 0; b < 4; ++b) st[base | p.post_off[slot(ls, b)]] = P::store(w[b]);
        }
    }
}

template <class P, int PART>
// 64 registers on the resident layout (4 CTAs per SM; unbounded, the compiler keeps block
// constants in registers across tiles, about 100 registers and 2 CTAs per SM); 80 with the
// split and join of the plain layout.
__global__ void __launch_bounds__(PAIR2_THREADS, std::is_same<P, PolFFR>::value ? 4 : 3) k_pair2(typename P::S* __restrict__ st,
                                                  const __grid_constant__ Pair2ParamsFF p) {
    pair2_body<P, PART>(st, p, [&](ffp w[4], int blk) { ff_pair(w, blk ? p.pkb : p.pka); });
}

struct PolPlainF32 {
    using S = float2;
    using R = float2;
    static __device__ __forceinline__ R load(S a) { return a; }
    static __device__ __forceinline__ S store(R a) { return a; }
};

__device__ __forceinline__ void f32_pair(float2 x[4], const float2 (*m)[4]) {
    float2 y[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float2 u = m[r][c];
            re = fmaf(u.x, x[c].x, fmaf(-u.y, x[c].y, re));
            im = fmaf(u.x, x[c].y, fmaf(u.y, x[c].x, im));
        }
        y[r] = make_float2(re, im);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) x[r] = y[r];
}

template <int PART>
// complex64: the pass is bound by HBM, not arithmetic, so one thread holds a whole tile (16
// amplitudes, 32 registers) and a warp's load of one slot covers 32 consecutive tiles; the
// blocks run on the tile's quads in registers.
__global__ void __launch_bounds__(PAIR2_THREADS) k_pair2_f32(float2* __restrict__ st,
                                                   const __grid_constant__ Pair2Params32 p) {
    using L = Pair2Layout<PART>;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < p.ngroups; g += stride) {
        const uint64_t base =
            insert_zero(insert_zero(insert_zero(insert_zero(g, p.bits[0]), p.bits[1]), p.bits[2]),
                        p.bits[3]);
        float2 v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = st[base | p.pre_off[j]];
        tile_quads<L::A0, L::A1, L::B0, L::B1>(v, [&](float2 w[4]) { f32_pair(w, p.ma); });
        tile_quads<L::B0, L::B1, L::A0, L::A1>(v, [&](float2 w[4]) { f32_pair(w, p.mb); });
#pragma unroll
        for (int j = 0; j < 16; ++j) st[base | p.post_off[j]] = v[j];
    }
}

// Offsets of the 16 tile slots after the permutation i -> i ^ f(i) of XOR terms whose bits all
// lie in the tile (the permutation does not depend on the tile's base).
static void slot_offsets(const int bits[4], const std::vector<XTerm>& ts, uint64_t off[16]) {
    for (int j = 0; j < 16; ++j) {
        uint64_t i = 0;
        for (int m = 0; m < 4; ++m)
            if ((j >> m) & 1) i |= 1ull << bits[m];
        uint64_t f = 0;
        for (const XTerm& t : ts) {
            const uint64_t c = i & t.cm;
            if (t.swap ? (c != 0 && c != t.cm) : (c == t.cm)) f |= t.flip;
        }
        off[j] = i ^ f;
    }
}

template <class P>
static void launch_pair2_pol(qgpu_handle* h, int part, uint64_t blocks, double2* s,
                             const Pair2ParamsFF& q) {
    if (part == 0) k_pair2<P, 0><<<(unsigned)blocks, PAIR2_THREADS, 0, h->stream>>>(s, q);
    else if (part == 1) k_pair2<P, 1><<<(unsigned)blocks, PAIR2_THREADS, 0, h->stream>>>(s, q);
    else k_pair2<P, 2><<<(unsigned)blocks, PAIR2_THREADS, 0, h->stream>>>(s, q);
}

bool pair2_tc_supported(const qgpu_handle* h);  // pair_tc.cu
int launch_pair2_tc(qgpu_handle* h, const Plan& plan, const Pass& ps, const uint64_t pre_off[16],
                    const uint64_t post_off[16], int variant);

// Double pair passes on the tensor cores (k_pair2_tc, complex128 resident layout): tuning knob
// QGPU_PAIR2_TC=1, read per call. Its kernel reports bounded-wait timeouts through the handle's
// error word, so plans run with it are synchronised at the end.
static int pair2_tc_variant() {  // 0 off, 1 k_pair2_tc, 2 warp-specialised k_pair2_ws
    const char* e = std::getenv("QGPU_PAIR2_TC");
    return (e && (e[0] == '1' || e[0] == '2')) ? e[0] - '0' : 0;
}
static bool pair2_tc_enabled() { return pair2_tc_variant() != 0; }

static int launch_pair2(qgpu_handle* h, const Plan& plan, const Pass& ps, int lay) {
    // block A holds local bit 0 (the lowest tile bit)
    const PairBlock* a = &plan.pairs[ps.pair];
    const PairBlock* b = &plan.pairs[ps.pair2];
    if (b->lo == ps.bits[0]) std::swap(a, b);
    int part = -1;
    for (int q = 1; q < 4; ++q)
        if (a->hi == ps.bits[q]) part = q - 1;
    uint64_t tile = 0;
    for (int m = 0; m < 4; ++m) tile |= 1ull << ps.bits[m];
    bool inside = true;
    for (const auto* ts : {&ps.pre, &ps.post})
        for (const XTerm& t : *ts) inside = inside && ((t.cm | t.flip) & ~tile) == 0;
    if (a->lo != ps.bits[0] || part < 0 || !inside)
        return fail(QGPU_ERR_UNSUPPORTED, "double pair pass: blocks or terms outside the tile");
    auto fill = [&](Pair2Params& q) {
        std::memset(&q, 0, sizeof(Pair2Params));
        q.ngroups = h->dim >> 4;
        for (int m = 0; m < 4; ++m) q.bits[m] = ps.bits[m];
        slot_offsets(ps.bits, ps.pre, q.pre_off);
        slot_offsets(ps.bits, ps.post, q.post_off);
    };
    if (lay == LAY_RES && pair2_tc_enabled() && pair2_tc_supported(h)) {  // tensor cores
        uint64_t pre_off[16], post_off[16];
        slot_offsets(ps.bits, ps.pre, pre_off);
        slot_offsets(ps.bits, ps.post, post_off);
        return launch_pair2_tc(h, plan, ps, pre_off, post_off, pair2_tc_variant());
    }
    // four threads per 16-amplitude tile
    uint64_t blocks = std::max<uint64_t>(
        1, std::min<uint64_t>(((h->dim >> 4) + PAIR2_THREADS / 4 - 1) / (PAIR2_THREADS / 4),
                              (uint64_t)h->sm_count * 8));
    if (h->precision == QGPU_C64) {
        Pair2Params32 q;
        fill(q);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                q.ma[r][c] = make_float2((float)a->m[r][c].real(), (float)a->m[r][c].imag());
                q.mb[r][c] = make_float2((float)b->m[r][c].real(), (float)b->m[r][c].imag());
            }
        float2* s = (float2*)cur_state(h);
        blocks = std::max<uint64_t>(
            1, std::min<uint64_t>((q.ngroups + PAIR2_THREADS - 1) / PAIR2_THREADS,
                                  (uint64_t)h->sm_count * 8));
        if (part == 0) k_pair2_f32<0><<<(unsigned)blocks, PAIR2_THREADS, 0, h->stream>>>(s, q);
        else if (part == 1) k_pair2_f32<1><<<(unsigned)blocks, PAIR2_THREADS, 0, h->stream>>>(s, q);
        else k_pair2_f32<2><<<(unsigned)blocks, PAIR2_THREADS, 0, h->stream>>>(s, q);
        QGPU_CHECK_LAUNCH("k_pair2_f32");
        h->launches++;
        h->h2d_bytes += sizeof(q);
        return QGPU_OK;
    }
    Pair2ParamsFF q;
    fill(q);
    std::memcpy(q.pka, a->pk, sizeof(q.pka));
    std::memcpy(q.pkb, b->pk, sizeof(q.pkb));
    double2* s = (double2*)cur_state(h);
    switch (lay) {
        case LAY_RES: launch_pair2_pol<PolFFR>(h, part, blocks, s, q); break;
        case LAY_IN: launch_pair2_pol<PolFFIn>(h, part, blocks, s, q); break;
        case LAY_OUT: launch_pair2_pol<PolFFOut>(h, part, blocks, s, q); break;
        default: launch_pair2_pol<PolFF>(h, part, blocks, s, q); break;
    }
    QGPU_CHECK_LAUNCH("k_pair2");
    h->launches++;
    h->h2d_bytes += sizeof(q);
    return QGPU_OK;
}

// ---- digit passes (digits.cu) ------------------------------------------------------------------
bool dg_supported(const qgpu_handle* h);
bool dg_build_image(const std::complex<double> M[16][16], uint32_t* bimg, int32_t (*kap)[dg::KAP]);
int dg_launch_pass(qgpu_handle* h, const int bits[4], const uint32_t* bimg,
                   const int32_t (*kap)[dg::KAP]);
int dg_convert(qgpu_handle* h, bool into_digits, int other_layout, int sx);

// A pair pass as a digit pass: its tile bits and the B operand / carry constants of its 16 x 16
// matrix over the tile's physical slots.
struct DgPass {
    int bits[4];
    std::vector<uint32_t> bimg;
    std::vector<int32_t> kap;
};

static int slot_of(const int bits[4], uint64_t off) {
    int j = 0;
    for (int m = 0; m < 4; ++m)
        if ((off >> bits[m]) & 1ull) j |= 1 << m;
    return j;
}

// False when the pass cannot run as a digit pass (the matrix fails the exactness bound).
static bool dg_pass_image(const Plan& plan, const Pass& ps, int n, DgPass* out) {
    cd M16[16][16];
    for (int j = 0; j < 16; ++j)
        for (int c = 0; c < 16; ++c) M16[j][c] = 0.0;
    if (ps.pair2 >= 0) {
        for (int m = 0; m < 4; ++m) out->bits[m] = ps.bits[m];
        const PairBlock* blk[2] = {&plan.pairs[ps.pair], &plan.pairs[ps.pair2]};
        int lo[2] = {-1, -1}, hi[2] = {-1, -1};
        for (int b = 0; b < 2; ++b)
            for (int m = 0; m < 4; ++m) {
                if (ps.bits[m] == blk[b]->lo) lo[b] = m;
                if (ps.bits[m] == blk[b]->hi) hi[b] = m;
            }
        if (lo[0] < 0 || hi[0] < 0 || lo[1] < 0 || hi[1] < 0) return false;
        auto lidx = [&](int b, int j) { return 2 * ((j >> hi[b]) & 1) + ((j >> lo[b]) & 1); };
        uint64_t pre_off[16], post_off[16];
        slot_offsets(ps.bits, ps.pre, pre_off);
        slot_offsets(ps.bits, ps.post, post_off);
        for (int j = 0; j < 16; ++j)        // logical output slot
            for (int c = 0; c < 16; ++c)    // logical input slot
                M16[slot_of(ps.bits, post_off[j])][slot_of(ps.bits, pre_off[c])] =
                    blk[0]->m[lidx(0, j)][lidx(0, c)] * blk[1]->m[lidx(1, j)][lidx(1, c)];
    } else if (ps.pair >= 0) {
        // one block: its two bits and the two lowest other bits form the tile
        const PairBlock& b = plan.pairs[ps.pair];
        int bs[4] = {b.lo, b.hi, -1, -1}, nb = 2;
        for (int q = 0; q < n && nb < 4; ++q)
            if (q != b.lo && q != b.hi) bs[nb++] = q;
        if (nb < 4) return false;
        std::sort(bs, bs + 4);
        for (int m = 0; m < 4; ++m) out->bits[m] = bs[m];
        int lo = 0, hi = 0;
        for (int m = 0; m < 4; ++m) {
            if (bs[m] == b.lo) lo = m;
            if (bs[m] == b.hi) hi = m;
        }
        const int blockmask = (1 << lo) | (1 << hi);
        for (int j = 0; j < 16; ++j)
            for (int c = 0; c < 16; ++c)
                if (((j ^ c) & ~blockmask) == 0)
                    M16[j][c] = b.m[2 * ((j >> hi) & 1) + ((j >> lo) & 1)][2 * ((c >> hi) & 1) + ((c >> lo) & 1)];
    } else {
        return false;
    }
    out->bimg.assign(4096, 0u);
    out->kap.assign(32 * dg::KAP, 0);
    return dg_build_image(M16, out->bimg.data(), reinterpret_cast<int32_t(*)[dg::KAP]>(out->kap.data()));
}

// Frobenius norm of a Custom gate's effective map (None inputs keep their amplitude): a bound on
// how much it can grow the register's largest amplitude.
static double custom_growth(const LocalGate& g) {
    const size_t d = (size_t)1 << g.k;
    double s = 0.0;
    for (size_t l = 0; l < d; ++l) {
        if (g.none[l]) {
            s += 1.0;
            continue;
        }
        for (size_t j = 0; j < d; ++j)
            if (!g.none[j]) s += std::norm(g.M[j * d + l]);
    }
    return std::sqrt(s);
}

static bool is_pair_pass(const Pass& p) {
    return p.custom < 0 && !p.xor_pass && (p.pair2 >= 0 || p.pair >= 0);
}

// Whether a float-pair plan runs on the resident layout: it saves the split and join of every
// arithmetic pass for two extra streaming passes, so it pays once the plan carries several
// arithmetic passes (passes that run as digit passes do not count). Custom blocks read
// complex128 and keep the plan on the plain layout. QGPU_FF_RESIDENT=0/1 forces it off/on.
static bool plan_resident(const qgpu_handle* h, const Plan& plan, const std::vector<char>& dig) {
    if (policy_of(h) != POL_FF || !plan.customs.empty()) return false;
    static const int force = env_int("QGPU_FF_RESIDENT", -1);
    if (force >= 0) return force != 0;
    int arith = 0;
    for (size_t i = 0; i < plan.passes.size(); ++i) {
        const Pass& ps = plan.passes[i];
        arith += (!dig[i] && ps.custom < 0 && !ps.xor_pass && ps.arith);
    }
    return arith >= 8;
}

// One launch of a plan: a pass in a given layout, or a layout conversion.
enum LaunchKind { LK_PASS = 0, LK_FF_TO_PAIRS, LK_FF_TO_C128, LK_DG_FROM_C128, LK_DG_FROM_RES,
                  LK_DG_TO_C128, LK_DG_TO_RES };
constexpr int LAY_DIG = 4;  // the digit layout (digits.cuh), inside runs of pair passes
struct LaunchItem {
    int kind = LK_PASS;
    int pass = -1;
    int lay = LAY_PLAIN;
    int sx = 0;            // digit conversions: the run's scale
};

// pre_resident: the buffer already holds the resident float-pair layout (the adjoint sweep keeps
// its vectors that way); the passes use it as is and no layout conversion is launched.
static int run_plan(qgpu_handle* h, const Plan& plan, bool sync = true, bool pre_resident = false) {
    const int pol = policy_of(h);
    const size_t np = plan.passes.size();
    // Runs of at least QGPU_DIGITS_MIN_RUN pair passes (XOR passes between them allowed: they
    // move whole slots) run as digit passes on the tensor cores when every pass of the run passes
    // the exactness bound; two conversion passes bracket each run.
    std::vector<char> dig(np, 0);
    std::vector<DgPass> dgp(np);
    bool any_dig = false;
    // (QGPU_PAIR2_TC selects the earlier tensor-core pair kernels instead)
    if (!pre_resident && h->active == nullptr && dg_supported(h) && !pair2_tc_enabled()) {
        static const int min_run = std::max(1, env_int("QGPU_DIGITS_MIN_RUN", 6));
        size_t i = 0;
        while (i < np) {
            if (!is_pair_pass(plan.passes[i])) {
                ++i;
                continue;
            }
            size_t j = i, last = i;
            int npair = 0;
            while (j < np && (is_pair_pass(plan.passes[j]) || plan.passes[j].xor_pass)) {
                if (is_pair_pass(plan.passes[j])) {
                    last = j;
                    ++npair;
                }
                ++j;
            }
            bool ok = npair >= min_run;
            for (size_t k = i; ok && k <= last; ++k)
                if (is_pair_pass(plan.passes[k])) ok = dg_pass_image(plan, plan.passes[k], h->n_qubits, &dgp[k]);
            if (ok) {
                for (size_t k = i; k <= last; ++k) dig[k] = 1;
                any_dig = true;
            }
            i = j;
        }
    }
    if (any_dig && !h->norm_valid) {  // the digit scale needs a bound on the amplitudes
        double2 r;
        int st = reduce_state(h, 0, &r);
        if (st != QGPU_OK) return st;
        h->norm_bound = std::sqrt(std::max(0.0, r.x)) * (1.0 + 1e-9);
        h->norm_valid = true;
    }
    const bool resident = pre_resident || plan_resident(h, plan, dig);
    // phase tables for every TABLE step of the plan, uploaded once
    const size_t nent = plan.table_f64.size() / 2;
    const float4* tab_ff = nullptr;
    const double2* tab_f64 = nullptr;
    if (nent) {
        const size_t ffb = align_up(nent * 16, 256);
        int st = h->tables.ensure(ffb + nent * 16);
        if (st != QGPU_OK) return st;
        QGPU_CUDA(copy_async(h, h->tables.ptr, plan.table_ff.data(), nent * 16,
                             cudaMemcpyHostToDevice));
        QGPU_CUDA(copy_async(h, (uint8_t*)h->tables.ptr + ffb, plan.table_f64.data(), nent * 16,
                             cudaMemcpyHostToDevice));
        tab_ff = (const float4*)h->tables.ptr;
        tab_f64 = (const double2*)((uint8_t*)h->tables.ptr + ffb);
    }
    // Custom blocks: upload their tables once
    std::vector<const LocalGate*> blocks;
    for (const LocalGate& g : plan.customs) blocks.push_back(&g);
    std::vector<GroupTables> lay(blocks.size());
    std::vector<GroupArgs> gargs(blocks.size());
    if (!blocks.empty()) {
        size_t at = 0;
        for (size_t i = 0; i < blocks.size(); ++i) {
            lay[i] = group_layout(blocks[i]->k, at);
            at = align_up(lay[i].none_off + ((size_t)1 << blocks[i]->k), 256);
        }
        std::vector<uint8_t> host(at, 0);
        for (size_t i = 0; i < blocks.size(); ++i) {
            std::memset(&gargs[i], 0, sizeof(GroupArgs));
            group_fill(*blocks[i], h->n_qubits, host, 0, lay[i], &gargs[i]);
        }
        int st = h->gates.ensure(at);
        if (st != QGPU_OK) return st;
        QGPU_CUDA(copy_async(h, h->gates.ptr, host.data(), at, cudaMemcpyHostToDevice));
        QGPU_CUDA(cudaStreamSynchronize(h->stream));
    }
    // The launch sequence: layouts follow the passes. Float-pair passes of a resident plan run
    // on the resident layout; the first one that meets complex128 converts it on its loads
    // (LAY_IN) and the plan's last non-XOR pass writes complex128 back (LAY_OUT) where it can;
    // elsewhere a k_ff_layout pass converts. Digit runs are bracketed by k_dg_from / k_dg_to.
    static const int fuse = env_int("QGPU_FUSE_LAYOUT", 1);  // tuning knob: 0 = separate passes
    auto fusable = [](const Pass& p) {
        return p.custom < 0 && !p.xor_pass && (p.pair >= 0 || (p.arith && p.nbits <= MAX_TILE_BITS));
    };
    int last_nonxor = (int)np - 1;
    while (last_nonxor >= 0 && plan.passes[last_nonxor].xor_pass) --last_nonxor;
    std::vector<LaunchItem> items;
    items.reserve(np + 8);
    int cur = pre_resident ? LAY_RES : LAY_PLAIN;
    double bound = h->norm_bound;
    int run_sx = dg::SX_UNIT;
    bool first_arith = true;
    for (size_t pi = 0; pi < np; ++pi) {
        const Pass& p = plan.passes[pi];
        LaunchItem it;
        it.pass = (int)pi;
        if (dig[pi]) {
            if (cur != LAY_DIG) {
                // scale: |x| <= bound <= 2^e, so |X| = |x| 2^sx <= 2^54
                int e = 0;
                if (bound > 0.0) e = (int)std::ceil(std::log2(bound));
                run_sx = std::max(-60, std::min(120, dg::SX_UNIT - e));  // 2^-120: still a normal float
                LaunchItem cv;
                cv.kind = cur == LAY_RES ? LK_DG_FROM_RES : LK_DG_FROM_C128;
                cv.sx = run_sx;
                items.push_back(cv);
                cur = LAY_DIG;
            }
            it.lay = LAY_DIG;
        } else if (p.xor_pass) {
            it.lay = cur;  // slot moves: any layout
        } else if (p.custom >= 0) {
            if (cur == LAY_DIG || cur == LAY_RES) {
                LaunchItem cv;
                cv.kind = cur == LAY_DIG ? LK_DG_TO_C128 : LK_FF_TO_C128;
                cv.sx = run_sx;
                items.push_back(cv);
                cur = LAY_PLAIN;
            }
            it.lay = LAY_PLAIN;
            bound *= custom_growth(plan.customs[p.custom]);
        } else if (resident) {
            if (cur == LAY_DIG) {
                LaunchItem cv;
                cv.kind = LK_DG_TO_RES;
                cv.sx = run_sx;
                items.push_back(cv);
                cur = LAY_RES;
            }
            const bool can_fuse = fuse && fusable(p) && !pre_resident;
            if (cur == LAY_PLAIN && can_fuse && first_arith) {
                it.lay = LAY_IN;
                cur = LAY_RES;
            } else {
                if (cur == LAY_PLAIN) {
                    LaunchItem cv;
                    cv.kind = LK_FF_TO_PAIRS;
                    items.push_back(cv);
                    cur = LAY_RES;
                }
                if ((int)pi == last_nonxor && can_fuse && !first_arith) {
                    it.lay = LAY_OUT;
                    cur = LAY_PLAIN;
                } else {
                    it.lay = LAY_RES;
                }
            }
            first_arith = false;
        } else {
            if (cur == LAY_DIG) {
                LaunchItem cv;
                cv.kind = LK_DG_TO_C128;
                cv.sx = run_sx;
                items.push_back(cv);
                cur = LAY_PLAIN;
            }
            it.lay = LAY_PLAIN;
        }
        items.push_back(it);
    }
    if (!pre_resident && (cur == LAY_DIG || cur == LAY_RES)) {
        LaunchItem cv;
        cv.kind = cur == LAY_DIG ? LK_DG_TO_C128 : LK_FF_TO_C128;
        cv.sx = run_sx;
        items.push_back(cv);
    }
    if (!pre_resident && h->active == nullptr) h->norm_bound = bound;

    const size_t nlaunch = items.size();
    std::vector<std::string> prof_names;
    std::vector<double> prof_bytes;
    size_t ev_base = 0;
    if (h->profile) {
        int st = prof_events(h, nlaunch, &ev_base);
        if (st != QGPU_OK) return st;
    }
    static const char* pol_name[] = {"ff", "f64", "f32"};
    QGPU_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    const double full_bytes = 2.0 * (double)h->amp_bytes * (double)h->dim;
    TileParams tp;
    for (size_t li = 0; li < nlaunch; ++li) {
        const LaunchItem& it = items[li];
        const Pass* ps = it.kind == LK_PASS ? &plan.passes[it.pass] : nullptr;
        const int play = it.lay;
        if (h->profile) {
            QGPU_CUDA(cudaEventRecord(h->events[2 * (ev_base + li)], h->stream));
            if (!ps) {
                prof_names.push_back(it.kind == LK_FF_TO_PAIRS || it.kind == LK_FF_TO_C128 ? "k_ff_layout"
                                     : (it.kind == LK_DG_FROM_C128 || it.kind == LK_DG_FROM_RES) ? "k_dg_from"
                                                                                                 : "k_dg_to");
            } else if (play == LAY_DIG && !ps->xor_pass) {
                prof_names.push_back("k_dg2");
            } else if (ps->pair2 >= 0) {
                prof_names.push_back(h->precision == QGPU_C64 ? "k_pair2<f32>"
                                     : (play == LAY_RES && pair2_tc_enabled() && pair2_tc_supported(h))
                                         ? (pair2_tc_variant() == 2 ? "k_pair2_ws" : "k_pair2_tc")
                                     : resident ? "k_pair2<ffr>"
                                                : "k_pair2<ff>");
            } else if (ps->pair >= 0) {
                prof_names.push_back(h->precision == QGPU_C64 ? "k_pair<f32>"
                                     : resident               ? "k_pair<ffr>"
                                                              : "k_pair<ff>");
            } else if (ps->custom >= 0) {
                prof_names.push_back("k_group");
            } else if (ps->xor_pass) {
                BitPermArgs bp;
                prof_names.push_back(xor_as_bitperm(h, ps->xp, &bp) ? "k_bitperm" : "k_xor_perm");
            } else {
                prof_names.push_back(std::string("k_tile<") + std::to_string(ps->nbits) + "," +
                                     (ps->arith ? (resident ? "ffr" : pol_name[pol]) : "move") + ">");
            }
            prof_bytes.push_back(full_bytes * (ps ? ps->touched : 1.0));
        }
        int st = QGPU_OK;
        if (!ps) {
            switch (it.kind) {
                case LK_FF_TO_PAIRS: st = launch_ff_layout(h, true); break;
                case LK_FF_TO_C128: st = launch_ff_layout(h, false); break;
                case LK_DG_FROM_C128: st = dg_convert(h, true, 0, it.sx); break;
                case LK_DG_FROM_RES: st = dg_convert(h, true, 1, it.sx); break;
                case LK_DG_TO_C128: st = dg_convert(h, false, 0, it.sx); break;
                default: st = dg_convert(h, false, 1, it.sx); break;
            }
        } else if (play == LAY_DIG && !ps->xor_pass) {
            const DgPass& d = dgp[it.pass];
            st = dg_launch_pass(h, d.bits, d.bimg.data(),
                                reinterpret_cast<const int32_t(*)[dg::KAP]>(d.kap.data()));
        } else if (ps->pair2 >= 0) {
            st = launch_pair2(h, plan, *ps, play);
        } else if (ps->pair >= 0) {
            st = launch_pair(h, plan.pairs[ps->pair], play);
        } else if (ps->custom >= 0) {
            st = launch_group(h, gargs[ps->custom], (const uint8_t*)h->gates.ptr, lay[ps->custom]);
        } else if (ps->xor_pass) {
            st = launch_xor(h, ps->xp);
        } else {
            st = launch_pass(h, *ps, pol, play, tab_ff, tab_f64, tp);
        }
        if (st != QGPU_OK) return st;
        if (h->profile) QGPU_CUDA(cudaEventRecord(h->events[2 * (ev_base + li) + 1], h->stream));
    }
    int st = h->profile ? prof_collect(h, prof_names, prof_bytes) : QGPU_OK;
    if (st != QGPU_OK) return st;
    if (!sync && !any_dig) return QGPU_OK;  // queued; later calls on the stream are ordered after it
    int err = 0;
    QGPU_CUDA(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    if (err == 10)
        return fail(QGPU_ERR_INVALID, "an amplitude exceeded the bound the digit passes were scaled for");
    if (err) return fail(QGPU_ERR_TIMEOUT, "a pipelined pass gave up waiting (code " + std::to_string(err) + ")");
    return st;
}

static int launch_pass(qgpu_handle* h, const Pass& ps, int pol, int lay,
                       const float4* tab_ff, const double2* tab_f64, TileParams& tp) {
    const bool resident = lay == LAY_RES;
    {
        std::memset(&tp, 0, sizeof(tp));
        tp.nbits = ps.nbits;
        for (int m = 0; m < ps.nbits; ++m) tp.bits[m] = ps.bits[m];
        tp.ngroups = h->dim >> ps.nbits;
        tp.nsteps = (int)ps.steps.size();
        for (int s = 0; s < tp.nsteps; ++s) tp.steps[s] = ps.steps[s];
        tp.tab_ff = tab_ff;
        tp.tab_f64 = tab_f64;
        // L2 prefetch of the next iteration measured slower on GB300 (0.88 vs 0.94 of HBM peak
        // for the dense pass on the same box): off unless QGPU_PREFETCH=1
        static const int prefetch = env_int("QGPU_PREFETCH", 0);
        tp.prefetch = prefetch;
        // streaming hints for passes that read phase tables (tuning knob QGPU_TILE_STREAMING:
        // 0 never, 1 passes with a TABLE step, 2 every pass)
        static const int streaming = env_int("QGPU_TILE_STREAMING", 1);
        bool has_table = false;
        for (const DevStep& d : ps.steps) has_table = has_table || d.type == ST_TABLE;
        tp.streaming = streaming == 2 || (streaming == 1 && has_table);
        int st;
        if (lay == LAY_IN || lay == LAY_OUT) {
            if (!ps.arith) return fail(QGPU_ERR_UNSUPPORTED, "layout-converting pass without arithmetic");
            st = lay == LAY_IN ? launch_tile_k<PolFFIn>(h, tp) : launch_tile_k<PolFFOut>(h, tp);
        } else if (resident) {
            st = ps.arith ? launch_tile_k<PolFFR>(h, tp) : launch_tile_k<PolRawFFR>(h, tp);
        } else if (!ps.arith) {
            st = (h->precision == QGPU_C64) ? launch_tile_k<PolRaw<float2>>(h, tp)
                                            : launch_tile_k<PolRaw<double2>>(h, tp);
        } else if (pol == POL_F32) {
            st = launch_tile_k<PolF32>(h, tp);
        } else if (pol == POL_F64) {
            st = launch_tile_k<PolF64>(h, tp);
        } else {
            st = launch_tile_k<PolFF>(h, tp);
        }
        return st;
    }
}

PlanOptions plan_options_for(const qgpu_handle* h) {
    PlanOptions o;
    o.policy = policy_of(h);
    // Float-pair budget: 280 admits two fused dense 2x2 steps per 2-bit pass. On the resident
    // layout the 30-qubit brickwork+QFT step measured 2549 ms at 280 against 3625 ms at 140
    // (one dense step per pass) on GB300.
    if (o.policy == POL_FF) o.budget = h->batch_budget > 0 ? h->batch_budget : env_int("QGPU_FF_BUDGET", 280);
    else if (o.policy == POL_F32) o.budget = h->batch_budget > 0 ? h->batch_budget : env_int("QGPU_F32_BUDGET", 48);
    else o.budget = env_int("QGPU_F64_BUDGET", 1 << 20);
    o.max_bits = std::max(2, std::min(env_int("QGPU_TILE_BITS", MAX_TILE_BITS), MAX_TILE_BITS));
    // float-pair arithmetic on 8 amplitudes per thread needs ~120 registers (2 CTAs per SM):
    // keep arithmetic passes at 2 tile bits
    o.max_arith_bits = o.policy == POL_FF ? env_int("QGPU_ARITH_TILE_BITS", 2) : MAX_TILE_BITS;
    // 4x4 pair blocks (k_pair) for the float-pair policy; QGPU_PAIR_FUSION=0 turns them off
    o.pair_fusion = (o.policy == POL_FF || o.policy == POL_F32) && env_int("QGPU_PAIR_FUSION", 1) != 0;
    // two pair blocks per pass with the XOR layers folded in (k_pair2); QGPU_PAIR_GROUP=0: off
    o.group_pairs = env_int("QGPU_PAIR_GROUP", 1) != 0;
    // phase-table field width (tuning knob QGPU_TABLE_BITS): 10 bits measured best on GB300 for
    // the 30-qubit QFT rows (1114 ms per step; 11: 1118, 12: 1156, 9: 1182 ms)
    o.table_bits = env_int("QGPU_TABLE_BITS", 10);
    return o;
}

int apply_blocks(qgpu_handle* h, const qgpu_op* ops, size_t n_ops, const double* mats,
                 size_t n_mats, const uint8_t* none, size_t n_none, int bq, int mg);  // blocks.cu

// Runs non-Custom ops as fused passes on `buffer` (a state-sized device vector of the handle's
// precision) instead of the register.
int run_plan_on(qgpu_handle* h, void* buffer, const Plan& plan, bool sync, bool pre_resident);

int apply_ops_on(qgpu_handle* h, void* buffer, const qgpu_op* ops, size_t n_ops) {
    Plan plan;
    int st = build_plan(ops, n_ops, h->n_qubits, nullptr, 0, nullptr, 0, plan_options_for(h), &plan);
    if (st != QGPU_OK) return st;
    return run_plan_on(h, buffer, plan, true, false);
}

// Runs an already built plan (no Custom gates) on `buffer`; with sync = false the launches are
// only queued on the handle's stream (the plan's tables are copied before this returns). With
// pre_resident the buffer is in the resident float-pair layout and stays in it.
int run_plan_on(qgpu_handle* h, void* buffer, const Plan& plan, bool sync, bool pre_resident) {
    void* saved = h->active;
    h->active = buffer;
    const int st = run_plan(h, plan, sync, pre_resident);
    h->active = saved;
    return st;
}

// Converts a complex128 work vector to the resident float-pair layout or back, in place.
int ff_layout_on(qgpu_handle* h, void* buffer, bool to_pairs) {
    void* saved = h->active;
    h->active = buffer;
    const int st = launch_ff_layout(h, to_pairs);
    h->active = saved;
    return st;
}

}  // namespace qgpu

using namespace qgpu;

extern "C" int qgpu_apply_program(qgpu_handle* h, const qgpu_op* ops, size_t n_ops,
                                  const double* mats, size_t n_mat_doubles,
                                  const uint8_t* none_flags, size_t n_none_flags) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_apply_program: NULL handle");
    if (n_ops && !ops) return fail(QGPU_ERR_INVALID, "qgpu_apply_program: ops is NULL");
    if (n_ops == 0) return QGPU_OK;
    // the exact and dense-block paths do not carry the amplitude bound through Custom gates
    bool has_custom = false;
    for (size_t g = 0; g < n_ops; ++g) has_custom = has_custom || ops[g].kind == QGPU_GATE_CUSTOM;
    if (has_custom && ((h->precision == QGPU_C128 && h->mode == QGPU_MODE_EXACT) || h->block_qubits > 0))
        h->norm_valid = false;
    if (h->precision == QGPU_C128 && h->mode == QGPU_MODE_EXACT) {
        std::vector<LocalGate> gates;
        gates.reserve(n_ops);
        for (size_t g = 0; g < n_ops; ++g) {
            if (ops[g].kind == QGPU_GATE_ID) continue;  // simulation.rs:38-41
            LocalGate lg;
            int st = tabulate(ops[g], h->n_qubits, mats, n_mat_doubles, none_flags, n_none_flags, &lg);
            if (st != QGPU_OK) return st;
            gates.push_back(std::move(lg));
        }
        // tables for a window of gates at a time keeps the device staging bounded
        const size_t window = 512;
        for (size_t i = 0; i < gates.size(); i += window) {
            std::vector<const LocalGate*> part;
            for (size_t j = i; j < gates.size() && j < i + window; ++j) part.push_back(&gates[j]);
            int st = run_groups(h, part);
            if (st != QGPU_OK) return st;
        }
        return QGPU_OK;
    }
    if (h->block_qubits > 0)
        return apply_blocks(h, ops, n_ops, mats, n_mat_doubles, none_flags, n_none_flags,
                            h->block_qubits, h->block_gates);
    Plan plan;
    int st = build_plan(ops, n_ops, h->n_qubits, mats, n_mat_doubles, none_flags, n_none_flags,
                        plan_options_for(h), &plan);
    if (st != QGPU_OK) return st;
    // Fast mode carries f64 values as float pairs, which share the float32 exponent range: a
    // program whose Custom gates could grow the register's amplitudes past 2^100 (the running
    // product of their effective maps' Frobenius norms times the register's bound) runs with
    // native f64 arithmetic instead of overflowing.
    if (h->precision == QGPU_C128 && h->mode == QGPU_MODE_FAST && !plan.customs.empty()) {
        double running = 1.0, peak = 1.0;
        for (const LocalGate& g : plan.customs) {
            running *= custom_growth(g);
            peak = std::max(peak, running);
        }
        if (peak > 1.0 && !h->norm_valid) {
            double2 r;
            st = reduce_state(h, 0, &r);
            if (st != QGPU_OK) return st;
            h->norm_bound = std::sqrt(std::max(0.0, r.x)) * (1.0 + 1e-9);
            h->norm_valid = true;
        }
        if (h->norm_bound * peak > 0x1p100) {
            h->mode = QGPU_MODE_F64;
            Plan wide;
            st = build_plan(ops, n_ops, h->n_qubits, mats, n_mat_doubles, none_flags, n_none_flags,
                            plan_options_for(h), &wide);
            if (st == QGPU_OK) st = run_plan(h, wide, true);
            h->mode = QGPU_MODE_FAST;
            return st;
        }
    }
    // queued without a final synchronisation unless the plan can report a bounded-wait timeout
    return run_plan(h, plan, pipe_enabled() != 0 || pair2_tc_enabled());
}

// One CTA waits, with the pipelined kernels' bounded poll, on an mbarrier phase that nothing
// completes; when the poll limit runs out it records the failure exactly as k_tile1_pipe does.
__global__ void k_wait_selftest(uint32_t polls, int* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);
        fence_proxy_async_shared();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(smem_u32(&bar), 0, polls);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(err, 1);
}

extern "C" int qgpu_selftest_bounded_wait(qgpu_handle* h, uint32_t polls) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_selftest_bounded_wait: NULL handle");
    if (polls == 0 || polls > (1u << 20))
        return fail(QGPU_ERR_INVALID, "qgpu_selftest_bounded_wait: polls must be 1..2^20");
    QGPU_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    k_wait_selftest<<<1, 32, 0, h->stream>>>(polls, h->d_err);
    QGPU_CHECK_LAUNCH("k_wait_selftest");
    h->launches++;
    int err = 0;
    QGPU_CUDA(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    QGPU_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    if (err) return fail(QGPU_ERR_TIMEOUT, "bounded wait gave up after " + std::to_string(polls) + " polls");
    return QGPU_OK;
}

extern "C" int qgpu_set_fusion(qgpu_handle* h, int block_qubits, int max_gates) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_set_fusion: NULL handle");
    if (block_qubits < 0 || block_qubits > 6 || max_gates < 1)
        return fail(QGPU_ERR_INVALID, "qgpu_set_fusion: block_qubits must be 0..6 and max_gates >= 1");
    h->block_qubits = block_qubits;
    h->block_gates = max_gates;
    return QGPU_OK;
}
