// adjoint.cu — energies <psi|H|psi> and adjoint-method gradients (no counterpart in quantr).
//
// H = sum_i a_i Z_i Z_{(i+1) mod n} + sum_i b_i X_i on wires i (wire i = index bit n-1-i).
// Gradient by the adjoint method (Jones & Gacon 2020, arXiv:2009.02823): after the forward pass
// |psi_L> = U_L ... U_1 |psi_0>, set phi = psi_L, lambda = H psi_L and walk the gates backwards.
// For a rotation U_l = exp(-i theta P / 2) (quantr's Rx, Ry, Rz; P = X, Y, Z) the derivative is
// dE/dtheta_l = 2 Re <lambda_l| dU_l |psi_{l-1}> = Im <lambda_l| P |phi_l>, read from the two
// vectors before the gate is undone; Phase(theta) = exp(i theta / 2) I gives -Im <lambda|phi>.
// Then phi <- U_l^dagger phi and lambda <- U_l^dagger lambda. In QGPU_MODE_FAST the runs of
// single-wire gates go through k_adj_tile (all gates of a wire, or of two wires, per pass, float-
// pair arithmetic), or up to 22 qubits k_adj_group (the wires of a tile of up to 11 bits per
// pass); QGPU_MODE_F64 uses k_adj_1q, one gate per pass in f64. Multi-wire gates are
// undone with the fused gate passes of program.cu on each vector.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "plan.h"

namespace qgpu {

int apply_ops_on(qgpu_handle* h, void* buffer, const qgpu_op* ops, size_t n_ops);  // program.cu
int run_plan_on(qgpu_handle* h, void* buffer, const Plan& plan, bool sync,
                bool pre_resident);                                                 // program.cu
int ff_layout_on(qgpu_handle* h, void* buffer, bool to_pairs);                      // program.cu
PlanOptions plan_options_for(const qgpu_handle* h);

constexpr int ADJ_THREADS = 256;
constexpr int MAX_HAM_QUBITS = 40;

struct Ham {
    int n;
    double a[MAX_HAM_QUBITS];
    double b[MAX_HAM_QUBITS];
};

// lambda = H psi, and per-block partial sums of Re(conj(psi) lambda). T = double2 (complex128,
// f64 arithmetic) or float2 (complex64: lambda in f32, the energy sums in f64).
template <class T>
__global__ void __launch_bounds__(ADJ_THREADS)
k_apply_zzx(const T* __restrict__ psi, T* __restrict__ lam, uint64_t dim,
            const __grid_constant__ Ham H, double* __restrict__ partial) {
    using R = decltype(T::x);
    __shared__ double sh[ADJ_THREADS];
    double acc = 0.0;
    const int n = H.n;
    for (uint64_t x = blockIdx.x * (uint64_t)ADJ_THREADS + threadIdx.x; x < dim;
         x += (uint64_t)gridDim.x * ADJ_THREADS) {
        R d = 0;
        for (int i = 0; i < n; ++i) {
            const int j = (i + 1) % n;
            const uint64_t p = ((x >> (n - 1 - i)) ^ (x >> (n - 1 - j))) & 1ull;
            d += p ? -(R)H.a[i] : (R)H.a[i];
        }
        const T v = psi[x];
        R re = d * v.x, im = d * v.y;
        for (int i = 0; i < n; ++i) {
            const T w = psi[x ^ (1ull << (n - 1 - i))];
            re = fma((R)H.b[i], w.x, re);
            im = fma((R)H.b[i], w.y, im);
        }
        T o;
        o.x = re;
        o.y = im;
        lam[x] = o;
        acc = fma((double)v.x, (double)re, fma((double)v.y, (double)im, acc));
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// One single-wire gate of the reverse sweep on bit t: optional gradient term (generator code
// gen: 0 none, 1 X, 2 Y, 3 Z, 4 identity with sign -1), then phi, lambda <- V (phi, lambda)
// with V = U^dagger given row-major as v[0..7] = (v00, v01, v10, v11) complex.
struct AdjStep {
    int t;
    int gen;
    double v[8];
};

__global__ void __launch_bounds__(ADJ_THREADS)
k_adj_1q(double2* __restrict__ phi, double2* __restrict__ lam, uint64_t npairs,
         const AdjStep s, double* __restrict__ partial) {
    __shared__ double sh[ADJ_THREADS];
    double acc = 0.0;
    for (uint64_t p = blockIdx.x * (uint64_t)ADJ_THREADS + threadIdx.x; p < npairs;
         p += (uint64_t)gridDim.x * ADJ_THREADS) {
        const uint64_t i0 = insert_zero(p, s.t), i1 = i0 | (1ull << s.t);
        const double2 f0 = phi[i0], f1 = phi[i1], l0 = lam[i0], l1 = lam[i1];
        // Im(conj(l) * f) = l.x f.y - l.y f.x ; Re(conj(l) * f) = l.x f.x + l.y f.y
        switch (s.gen) {
            case 1:  // X
                acc += (l0.x * f1.y - l0.y * f1.x) + (l1.x * f0.y - l1.y * f0.x);
                break;
            case 2:  // Y: Im(conj(l0)(-i f1) + conj(l1)(i f0)) = -Re(conj(l0) f1) + Re(conj(l1) f0)
                acc += -(l0.x * f1.x + l0.y * f1.y) + (l1.x * f0.x + l1.y * f0.y);
                break;
            case 3:  // Z
                acc += (l0.x * f0.y - l0.y * f0.x) - (l1.x * f1.y - l1.y * f1.x);
                break;
            case 4:  // global phase
                acc -= (l0.x * f0.y - l0.y * f0.x) + (l1.x * f1.y - l1.y * f1.x);
                break;
            default:
                break;
        }
        const double* v = s.v;
        auto mv = [&](double2 a, double2 b, double2& o0, double2& o1) {
            o0 = make_double2(v[0] * a.x - v[1] * a.y + v[2] * b.x - v[3] * b.y,
                              v[0] * a.y + v[1] * a.x + v[2] * b.y + v[3] * b.x);
            o1 = make_double2(v[4] * a.x - v[5] * a.y + v[6] * b.x - v[7] * b.y,
                              v[4] * a.y + v[5] * a.x + v[6] * b.y + v[7] * b.x);
        };
        double2 o0, o1;
        mv(f0, f1, o0, o1);
        phi[i0] = o0;
        phi[i1] = o1;
        mv(l0, l1, o0, o1);
        lam[i0] = o0;
        lam[i1] = o1;
    }
    if (!partial) return;
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// The same sweep step for QGPU_MODE_FAST: the gradient term stays f64 (4 FMAs per pair on the
// loaded doubles) while phi and lambda are updated with float-pair arithmetic (packed Dot2).
struct AdjStepFF {
    int t;
    int gen;
    u64 pk[32];  // ST_DENSE packed constants of V = U^dagger
};

__global__ void __launch_bounds__(ADJ_THREADS)
k_adj_1q_ff(double2* __restrict__ phi, double2* __restrict__ lam, uint64_t npairs,
            const __grid_constant__ AdjStepFF s, double* __restrict__ partial) {
    __shared__ double sh[ADJ_THREADS];
    double acc = 0.0;
    for (uint64_t p = blockIdx.x * (uint64_t)ADJ_THREADS + threadIdx.x; p < npairs;
         p += (uint64_t)gridDim.x * ADJ_THREADS) {
        const uint64_t i0 = insert_zero(p, s.t), i1 = i0 | (1ull << s.t);
        const double2 f0 = phi[i0], f1 = phi[i1], l0 = lam[i0], l1 = lam[i1];
        switch (s.gen) {
            case 1: acc += fma(l0.x, f1.y, -l0.y * f1.x) + fma(l1.x, f0.y, -l1.y * f0.x); break;
            case 2: acc += fma(l1.x, f0.x, l1.y * f0.y) - fma(l0.x, f1.x, l0.y * f1.y); break;
            case 3: acc += fma(l0.x, f0.y, -l0.y * f0.x) - fma(l1.x, f1.y, -l1.y * f1.x); break;
            case 4: acc -= fma(l0.x, f0.y, -l0.y * f0.x) + fma(l1.x, f1.y, -l1.y * f1.x); break;
            default: break;
        }
        ffp a = to_ffp(f0), b = to_ffp(f1);
        ff_dense(a, b, s.pk);
        phi[i0] = from_ffp(a);
        phi[i1] = from_ffp(b);
        a = to_ffp(l0);
        b = to_ffp(l1);
        ff_dense(a, b, s.pk);
        lam[i0] = from_ffp(a);
        lam[i1] = from_ffp(b);
    }
    if (!partial) return;
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = ADJ_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// ---------------------------------------------------------------------------------------------
// k_adj_tile<K>: a run of single-wire gates of the reverse sweep, on up to K wires, in one pass.
// Gates on different wires commute, so the run is regrouped wire by wire (each wire's gates in
// their reverse order); a thread holds the 2^K amplitudes of phi and lambda that differ in the
// pass's K bits (as float pairs) and, step by step, adds the gate's gradient term and applies
// V = U^dagger to both vectors, exactly as the one-gate sweep would. Gradient terms are packed
// float-pair dot products (lane sums of l * x with per-lane signs), accumulated per step with the
// Dot2 error terms and reduced per CTA in f64.
// ---------------------------------------------------------------------------------------------
constexpr int ADJ_TILE_STEPS = 4;   // gates per pass (registers: a Dot2 accumulator each)
constexpr int ADJ_TILE_BITS = 2;    // wires per pass

struct AdjTileStep {
    int lb;      // tile bit
    int gen;     // term summed before the update: 0 none, 1 X, 2 Y, 3 Z, 4 -I (global phase)
    int slot;    // row of partial the term's sums go to, -1 for none
    int apply;   // 1: then apply V to both vectors; 0: the step only sums its term
    u64 pk[32];  // ST_DENSE packed constants of V
};

struct AdjTileParams {
    uint64_t ngroups;
    int nbits;
    int bits[ADJ_TILE_BITS];
    int nsteps;
    int nb;  // CTAs (row length of partial)
    AdjTileStep steps[ADJ_TILE_STEPS];
};

// acc += sum over lanes of (sr * l.re * x.re, si * l.im * x.im), all float pairs
__device__ __forceinline__ void adj_term(PDot2& acc, bool& first, const ffp& l, const ffp& x,
                                         float sr, float si) {
    const u64 sg = p2(sr, si);
    u64 c[4];
    c[0] = pmul(l.h, sg);
    c[1] = pmul(l.l, sg);
    c[2] = pmul(c[0], p2(-1.f, -1.f));
    c[3] = pmul(c[1], p2(-1.f, -1.f));
    if (first) {
        acc.first(c, x.h, x.l);
        first = false;
    } else {
        acc.add(c, x.h, x.l);
    }
}

template <int K, int B>
__device__ __forceinline__ void adj_tile_step(ffp* f, ffp* l, const AdjTileStep& s, PDot2& acc,
                                              bool& first) {
    constexpr int T = 1 << K;
#pragma unroll
    for (int j = 0; j < T; ++j) {
        if ((j >> B) & 1) continue;
        const int j1 = j | (1 << B);
        if (s.gen) {
            const ffp f0 = f[j], f1 = f[j1], l0 = l[j], l1 = l[j1];
            ffp f0s, f1s;  // swapped lanes (im, re)
            f0s.h = pswap(f0.h);
            f0s.l = pswap(f0.l);
            f1s.h = pswap(f1.h);
            f1s.l = pswap(f1.l);
            // Re(conj(l) f) = lanes(l * f) with (+, +); Im(conj(l) f) = lanes(l * swap(f)), (+, -)
            switch (s.gen) {
                case 1:  // X: Im(l0* f1) + Im(l1* f0)
                    adj_term(acc, first, l0, f1s, 1.f, -1.f);
                    adj_term(acc, first, l1, f0s, 1.f, -1.f);
                    break;
                case 2:  // Y: -Re(l0* f1) + Re(l1* f0)
                    adj_term(acc, first, l0, f1, -1.f, -1.f);
                    adj_term(acc, first, l1, f0, 1.f, 1.f);
                    break;
                case 3:  // Z: Im(l0* f0) - Im(l1* f1)
                    adj_term(acc, first, l0, f0s, 1.f, -1.f);
                    adj_term(acc, first, l1, f1s, -1.f, 1.f);
                    break;
                default:  // global phase: -(Im(l0* f0) + Im(l1* f1))
                    adj_term(acc, first, l0, f0s, -1.f, 1.f);
                    adj_term(acc, first, l1, f1s, -1.f, 1.f);
                    break;
            }
        }
        if (s.apply) {
            ff_dense(f[j], f[j1], s.pk);
            ff_dense(l[j], l[j1], s.pk);
        }
    }
}

template <int K, bool FFR>
__global__ void __launch_bounds__(ADJ_THREADS, K == 1 ? 4 : 2)
k_adj_tile(double2* __restrict__ phi, double2* __restrict__ lam,
           const __grid_constant__ AdjTileParams p, double* __restrict__ partial) {
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
    PDot2 acc[ADJ_TILE_STEPS];
    bool first[ADJ_TILE_STEPS];
#pragma unroll
    for (int s = 0; s < ADJ_TILE_STEPS; ++s) {
        first[s] = true;
        acc[s].s = 0;
        acc[s].en = 0;
    }
    for (uint64_t g = blockIdx.x * (uint64_t)ADJ_THREADS + threadIdx.x; g < p.ngroups;
         g += (uint64_t)gridDim.x * ADJ_THREADS) {
        uint64_t b = g;
#pragma unroll
        for (int m = 0; m < K; ++m) b = insert_zero(b, p.bits[m]);
        ffp f[T], l[T];
#pragma unroll
        for (int j = 0; j < T; ++j) {
            f[j] = FFR ? ffr_load(phi[b | off[j]]) : to_ffp(phi[b | off[j]]);
            l[j] = FFR ? ffr_load(lam[b | off[j]]) : to_ffp(lam[b | off[j]]);
        }
#pragma unroll
        for (int s = 0; s < ADJ_TILE_STEPS; ++s) {
            if (s >= p.nsteps) break;
            const AdjTileStep& st = p.steps[s];
            if (st.lb == 0) adj_tile_step<K, 0>(f, l, st, acc[s], first[s]);
            if constexpr (K > 1) if (st.lb == 1) adj_tile_step<K, (K > 1 ? 1 : 0)>(f, l, st, acc[s], first[s]);
            if constexpr (K > 2) if (st.lb == 2) adj_tile_step<K, (K > 2 ? 2 : 0)>(f, l, st, acc[s], first[s]);
        }
#pragma unroll
        for (int j = 0; j < T; ++j) {
            phi[b | off[j]] = FFR ? ffr_store(f[j]) : from_ffp(f[j]);
            lam[b | off[j]] = FFR ? ffr_store(l[j]) : from_ffp(l[j]);
        }
    }
    // per-CTA sums of every step's term: warp shuffles, then one shared-memory stage
    double v[ADJ_TILE_STEPS];
#pragma unroll
    for (int s = 0; s < ADJ_TILE_STEPS; ++s) {
        v[s] = 0.0;
        if (s < p.nsteps && !first[s]) {
            u64 h, lo;
            acc[s].result(h, lo);
            float h0, h1, l0, l1;
            up2(h, h0, h1);
            up2(lo, l0, l1);
            v[s] = ((double)h0 + (double)h1) + ((double)l0 + (double)l1);
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
#pragma unroll
        for (int s = 0; s < ADJ_TILE_STEPS; ++s) v[s] += __shfl_down_sync(0xffffffffu, v[s], d);
    __shared__ double wsum[ADJ_THREADS / 32][ADJ_TILE_STEPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int s = 0; s < ADJ_TILE_STEPS; ++s) wsum[warp][s] = v[s];
    __syncthreads();
    if (threadIdx.x < ADJ_TILE_STEPS && threadIdx.x < p.nsteps && p.steps[threadIdx.x].slot >= 0) {
        double t = 0.0;
        for (int w = 0; w < ADJ_THREADS / 32; ++w) t += wsum[w][threadIdx.x];
        partial[(size_t)p.steps[threadIdx.x].slot * p.nb + blockIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------------------------
// k_adj_group: the runs of single-wire gates of the reverse sweep on up to ADJ_GROUP_MAX_BITS
// wires in one pass over phi and lambda (in place, resident float-pair layout). A CTA stages a
// tile of both vectors in shared memory: the 2^K amplitudes that share every bit outside the
// pass's K tile bits (the wires' bits and the lowest other bits, so that 32 consecutive
// amplitudes load together). Then, wire by wire, each thread takes the wire's Pauli sums over its
// pairs (packed Dot2, reduced per warp in float pairs into shared accumulators) and applies the
// run's undo to its pairs of both vectors. Gates on different wires commute and a wire's sums are
// taken before its own undo, so the results are those of one pass per wire (k_adj_tile with
// Pauli steps), with one read and one write of each vector per pass.
// ---------------------------------------------------------------------------------------------
constexpr int ADJ_GROUP_MAX_BITS = ADJ_GROUP_TILE_BITS;
constexpr int ADJ_GROUP_THREADS = 256;
constexpr int ADJ_GROUP_WARPS = ADJ_GROUP_THREADS / 32;

struct AdjGroupWire {
    int lb;      // tile bit of the wire
    int row[4];  // partial rows of its sums over X, Y, Z, -I (-1: not needed)
    u64 pk[32];  // ST_DENSE packed constants of the run's undo
};
struct AdjGroupParams {
    uint64_t ngroups;
    int nbits;
    int bits[ADJ_GROUP_MAX_BITS];  // ascending
    int nwires;
    int nb;                        // row length of partial (>= the grid)
    AdjGroupWire w[ADJ_GROUP_MAX_BITS];
};

__host__ __device__ constexpr size_t adj_group_smem(int nbits) {
    return (size_t)2 * 16 * ((size_t)1 << nbits) + (size_t)ADJ_GROUP_WARPS * ADJ_GROUP_MAX_BITS * 4 * 8 +
           (32 + 64) * 8;
}

// (h, l) += (bh, bl) in float-pair arithmetic (TwoSum of the heads, then the tails)
__device__ __forceinline__ void ff2_acc(float& h, float& l, float bh, float bl) {
    const float s = __fadd_rn(h, bh);
    const float bb = __fadd_rn(s, -h);
    float e = __fadd_rn(__fadd_rn(h, -__fadd_rn(s, -bb)), __fadd_rn(bh, -bb));
    e = __fadd_rn(e, __fadd_rn(l, bl));
    h = __fadd_rn(s, e);
    l = __fadd_rn(e, -__fadd_rn(h, -s));
}

__global__ void __launch_bounds__(ADJ_GROUP_THREADS, 2)
k_adj_group(double2* __restrict__ phi, double2* __restrict__ lam,
            const __grid_constant__ AdjGroupParams p, double* __restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int T = 1 << p.nbits;
    double2* sf = reinterpret_cast<double2*>(smem);    // phi tile
    double2* sl = sf + T;                               // lambda tile
    float2* sacc = reinterpret_cast<float2*>(sl + T);   // [warp][wire][pauli] float pairs
    uint64_t* lo_tab = reinterpret_cast<uint64_t*>(sacc + ADJ_GROUP_WARPS * ADJ_GROUP_MAX_BITS * 4);
    uint64_t* hi_tab = lo_tab + 32;                     // [T >> nlo] (at most 64)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nlo = p.nbits < 5 ? p.nbits : 5;
    for (int i = tid; i < 32 + (T >> nlo); i += ADJ_GROUP_THREADS) {
        uint64_t o = 0;
        if (i < 32) {
            for (int m = 0; m < nlo; ++m)
                if ((i >> m) & 1) o |= 1ull << p.bits[m];
            lo_tab[i] = o;
        } else {
            const int v = i - 32;
            for (int m = nlo; m < p.nbits; ++m)
                if ((v >> (m - nlo)) & 1) o |= 1ull << p.bits[m];
            hi_tab[v] = o;
        }
    }
    for (int i = tid; i < ADJ_GROUP_WARPS * ADJ_GROUP_MAX_BITS * 4; i += ADJ_GROUP_THREADS)
        sacc[i] = make_float2(0.f, 0.f);
    __syncthreads();
    const int lomask = (1 << nlo) - 1;
    for (uint64_t g = blockIdx.x; g < p.ngroups; g += gridDim.x) {
        uint64_t base = g;
        for (int m = 0; m < p.nbits; ++m) base = insert_zero(base, p.bits[m]);
        for (int i = tid; i < T; i += ADJ_GROUP_THREADS) {
            const uint64_t o = base | lo_tab[i & lomask] | hi_tab[i >> nlo];
            sf[i] = phi[o];
            sl[i] = lam[o];
        }
        __syncthreads();
        for (int w = 0; w < p.nwires; ++w) {
            const int lb = p.w[w].lb;
            const u64* pk = p.w[w].pk;
            PDot2 acc[4];
            bool first[4] = {true, true, true, true};
            const bool need[4] = {p.w[w].row[0] >= 0, p.w[w].row[1] >= 0, p.w[w].row[2] >= 0,
                                  p.w[w].row[3] >= 0};
            for (int q = tid; q < (T >> 1); q += ADJ_GROUP_THREADS) {
                const int i0 = ((q >> lb) << (lb + 1)) | (q & ((1 << lb) - 1));
                const int i1 = i0 | (1 << lb);
                ffp f0 = ffr_load(sf[i0]), f1 = ffr_load(sf[i1]);
                ffp l0 = ffr_load(sl[i0]), l1 = ffr_load(sl[i1]);
                ffp f0s, f1s;  // swapped lanes (im, re)
                f0s.h = pswap(f0.h);
                f0s.l = pswap(f0.l);
                f1s.h = pswap(f1.h);
                f1s.l = pswap(f1.l);
                if (need[0]) {  // X: Im(l0* f1) + Im(l1* f0)
                    adj_term(acc[0], first[0], l0, f1s, 1.f, -1.f);
                    adj_term(acc[0], first[0], l1, f0s, 1.f, -1.f);
                }
                if (need[1]) {  // Y: -Re(l0* f1) + Re(l1* f0)
                    adj_term(acc[1], first[1], l0, f1, -1.f, -1.f);
                    adj_term(acc[1], first[1], l1, f0, 1.f, 1.f);
                }
                if (need[2]) {  // Z: Im(l0* f0) - Im(l1* f1)
                    adj_term(acc[2], first[2], l0, f0s, 1.f, -1.f);
                    adj_term(acc[2], first[2], l1, f1s, -1.f, 1.f);
                }
                if (need[3]) {  // global phase: -(Im(l0* f0) + Im(l1* f1))
                    adj_term(acc[3], first[3], l0, f0s, -1.f, 1.f);
                    adj_term(acc[3], first[3], l1, f1s, -1.f, 1.f);
                }
                ff_dense(f0, f1, pk);
                ff_dense(l0, l1, pk);
                sf[i0] = ffr_store(f0);
                sf[i1] = ffr_store(f1);
                sl[i0] = ffr_store(l0);
                sl[i1] = ffr_store(l1);
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (!need[m]) continue;
                float h = 0.f, l = 0.f;
                if (!first[m]) {
                    u64 rh, rl;
                    acc[m].result(rh, rl);
                    float h1, l1;
                    up2(rh, h, h1);
                    up2(rl, l, l1);
                    ff2_acc(h, l, h1, l1);
                }
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) {
                    const float oh = __shfl_down_sync(0xffffffffu, h, d);
                    const float ol = __shfl_down_sync(0xffffffffu, l, d);
                    ff2_acc(h, l, oh, ol);
                }
                if (lane == 0) {
                    float2& a = sacc[(warp * ADJ_GROUP_MAX_BITS + w) * 4 + m];
                    ff2_acc(a.x, a.y, h, l);
                }
            }
            __syncthreads();
        }
        for (int i = tid; i < T; i += ADJ_GROUP_THREADS) {
            const uint64_t o = base | lo_tab[i & lomask] | hi_tab[i >> nlo];
            phi[o] = sf[i];
            lam[o] = sl[i];
        }
        __syncthreads();
    }
    // per-CTA sums into column blockIdx.x; columns past the grid (partial rows have nb columns) get 0
    for (int k = tid; k < p.nwires * 4; k += ADJ_GROUP_THREADS) {
        const int w = k >> 2, m = k & 3;
        if (p.w[w].row[m] < 0) continue;
        double t = 0.0;
        for (int v = 0; v < ADJ_GROUP_WARPS; ++v) {
            const float2 a = sacc[(v * ADJ_GROUP_MAX_BITS + w) * 4 + m];
            t += (double)a.x + (double)a.y;
        }
        double* row = partial + (size_t)p.w[w].row[m] * p.nb;
        row[blockIdx.x] = t;
        for (int c = blockIdx.x + gridDim.x; c < p.nb; c += gridDim.x) row[c] = 0.0;
    }
}

// Event-timed launch under qgpu_set_profiling (filed under `name`, bytes = reads + writes of both
// vectors); a plain launch otherwise.
template <class F>
static int adj_profiled(qgpu_handle* h, const char* name, double bytes, F&& launch) {
    size_t base = 0;
    if (h->profile) {
        int st = prof_events(h, 1, &base);
        if (st != QGPU_OK) return st;
        QGPU_CUDA(cudaEventRecord(h->events[2 * base], h->stream));
    }
    int st = launch();
    if (st != QGPU_OK) return st;
    if (h->profile) {
        QGPU_CUDA(cudaEventRecord(h->events[2 * base + 1], h->stream));
        return prof_collect(h, {name}, {bytes});
    }
    return QGPU_OK;
}

static int launch_adj_group(qgpu_handle* h, double2* phi, double2* lam, const AdjGroupParams& p,
                            double* partial) {
    const size_t smem = adj_group_smem(p.nbits);
    QGPU_CUDA(smem_opt_in((const void*)k_adj_group, adj_group_smem(ADJ_GROUP_MAX_BITS)));
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_adj_group, ADJ_GROUP_THREADS, smem) != cudaSuccess || occ < 1)
        occ = 1;
    const uint64_t grid = std::max<uint64_t>(
        1, std::min<uint64_t>({p.ngroups, (uint64_t)h->sm_count * occ, (uint64_t)p.nb}));
    return adj_profiled(h, "k_adj_group", 64.0 * (double)h->dim, [&]() -> int {
        k_adj_group<<<(unsigned)grid, ADJ_GROUP_THREADS, smem, h->stream>>>(phi, lam, p, partial);
        QGPU_CHECK_LAUNCH("k_adj_group");
        h->launches++;
        h->h2d_bytes += sizeof(p);
        return QGPU_OK;
    });
}

// k_adj_group_f32: k_adj_group for complex64 vectors. Plain f32 complex arithmetic for the Pauli
// sums and the undo, the sums reduced per warp in f32 and accumulated per CTA in f64.
struct AdjGroupWireF {
    int lb;      // tile bit of the wire
    int row[4];  // partial rows of its sums over X, Y, Z, -I (-1: not needed)
    float u[8];  // the run's undo, row-major complex (u00, u01, u10, u11)
};
struct AdjGroupParamsF {
    uint64_t ngroups;
    int nbits;
    int bits[ADJ_GROUP_MAX_BITS];
    int nwires;
    int nb;
    AdjGroupWireF w[ADJ_GROUP_MAX_BITS];
};

__host__ __device__ constexpr size_t adj_group_f32_smem(int nbits) {
    return (size_t)2 * 8 * ((size_t)1 << nbits) + (size_t)ADJ_GROUP_WARPS * ADJ_GROUP_MAX_BITS * 4 * 8 +
           (32 + 64) * 8;
}

__device__ __forceinline__ float2 cmul_add(float ur, float ui, float2 a, float vr, float vi, float2 b) {
    return make_float2(fmaf(ur, a.x, fmaf(-ui, a.y, fmaf(vr, b.x, -vi * b.y))),
                       fmaf(ur, a.y, fmaf(ui, a.x, fmaf(vr, b.y, vi * b.x))));
}

__global__ void __launch_bounds__(ADJ_GROUP_THREADS)
k_adj_group_f32(float2* __restrict__ phi, float2* __restrict__ lam,
                const __grid_constant__ AdjGroupParamsF p, double* __restrict__ partial) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int T = 1 << p.nbits;
    float2* sf = reinterpret_cast<float2*>(smem);
    float2* sl = sf + T;
    double* sacc = reinterpret_cast<double*>(sl + T);   // [warp][wire][pauli]
    uint64_t* lo_tab = reinterpret_cast<uint64_t*>(sacc + ADJ_GROUP_WARPS * ADJ_GROUP_MAX_BITS * 4);
    uint64_t* hi_tab = lo_tab + 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nlo = p.nbits < 5 ? p.nbits : 5;
    for (int i = tid; i < 32 + (T >> nlo); i += ADJ_GROUP_THREADS) {
        uint64_t o = 0;
        if (i < 32) {
            for (int m = 0; m < nlo; ++m)
                if ((i >> m) & 1) o |= 1ull << p.bits[m];
            lo_tab[i] = o;
        } else {
            const int v = i - 32;
            for (int m = nlo; m < p.nbits; ++m)
                if ((v >> (m - nlo)) & 1) o |= 1ull << p.bits[m];
            hi_tab[v] = o;
        }
    }
    for (int i = tid; i < ADJ_GROUP_WARPS * ADJ_GROUP_MAX_BITS * 4; i += ADJ_GROUP_THREADS) sacc[i] = 0.0;
    __syncthreads();
    const int lomask = (1 << nlo) - 1;
    for (uint64_t g = blockIdx.x; g < p.ngroups; g += gridDim.x) {
        uint64_t base = g;
        for (int m = 0; m < p.nbits; ++m) base = insert_zero(base, p.bits[m]);
        for (int i = tid; i < T; i += ADJ_GROUP_THREADS) {
            const uint64_t o = base | lo_tab[i & lomask] | hi_tab[i >> nlo];
            sf[i] = phi[o];
            sl[i] = lam[o];
        }
        __syncthreads();
        for (int w = 0; w < p.nwires; ++w) {
            const AdjGroupWireF& W = p.w[w];
            const int lb = W.lb;
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            for (int q = tid; q < (T >> 1); q += ADJ_GROUP_THREADS) {
                const int i0 = ((q >> lb) << (lb + 1)) | (q & ((1 << lb) - 1));
                const int i1 = i0 | (1 << lb);
                const float2 f0 = sf[i0], f1 = sf[i1], l0 = sl[i0], l1 = sl[i1];
                // Im(conj(a) b) = a.x b.y - a.y b.x, Re(conj(a) b) = a.x b.x + a.y b.y
                const float i01 = fmaf(l0.x, f1.y, -l0.y * f1.x), i10 = fmaf(l1.x, f0.y, -l1.y * f0.x);
                const float r01 = fmaf(l0.x, f1.x, l0.y * f1.y), r10 = fmaf(l1.x, f0.x, l1.y * f0.y);
                const float i00 = fmaf(l0.x, f0.y, -l0.y * f0.x), i11 = fmaf(l1.x, f1.y, -l1.y * f1.x);
                acc[0] += i01 + i10;     // X
                acc[1] += r10 - r01;     // Y
                acc[2] += i00 - i11;     // Z
                acc[3] -= i00 + i11;     // global phase
                sf[i0] = cmul_add(W.u[0], W.u[1], f0, W.u[2], W.u[3], f1);
                sf[i1] = cmul_add(W.u[4], W.u[5], f0, W.u[6], W.u[7], f1);
                sl[i0] = cmul_add(W.u[0], W.u[1], l0, W.u[2], W.u[3], l1);
                sl[i1] = cmul_add(W.u[4], W.u[5], l0, W.u[6], W.u[7], l1);
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                if (W.row[m] < 0) continue;
                float v = acc[m];
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
                if (lane == 0) sacc[(warp * ADJ_GROUP_MAX_BITS + w) * 4 + m] += (double)v;
            }
            __syncthreads();
        }
        for (int i = tid; i < T; i += ADJ_GROUP_THREADS) {
            const uint64_t o = base | lo_tab[i & lomask] | hi_tab[i >> nlo];
            phi[o] = sf[i];
            lam[o] = sl[i];
        }
        __syncthreads();
    }
    for (int k = tid; k < p.nwires * 4; k += ADJ_GROUP_THREADS) {
        const int w = k >> 2, m = k & 3;
        if (p.w[w].row[m] < 0) continue;
        double t = 0.0;
        for (int v = 0; v < ADJ_GROUP_WARPS; ++v) t += sacc[(v * ADJ_GROUP_MAX_BITS + w) * 4 + m];
        double* row = partial + (size_t)p.w[w].row[m] * p.nb;
        row[blockIdx.x] = t;
        for (int c = blockIdx.x + gridDim.x; c < p.nb; c += gridDim.x) row[c] = 0.0;
    }
}

static int launch_adj_group_f32(qgpu_handle* h, float2* phi, float2* lam, const AdjGroupParamsF& p,
                                double* partial) {
    const size_t smem = adj_group_f32_smem(p.nbits);
    QGPU_CUDA(smem_opt_in((const void*)k_adj_group_f32, adj_group_f32_smem(ADJ_GROUP_MAX_BITS)));
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_adj_group_f32, ADJ_GROUP_THREADS, smem) != cudaSuccess || occ < 1)
        occ = 1;
    const uint64_t grid = std::max<uint64_t>(
        1, std::min<uint64_t>({p.ngroups, (uint64_t)h->sm_count * occ, (uint64_t)p.nb}));
    return adj_profiled(h, "k_adj_group_f32", 32.0 * (double)h->dim, [&]() -> int {
        k_adj_group_f32<<<(unsigned)grid, ADJ_GROUP_THREADS, smem, h->stream>>>(phi, lam, p, partial);
        QGPU_CHECK_LAUNCH("k_adj_group_f32");
        h->launches++;
        h->h2d_bytes += sizeof(p);
        return QGPU_OK;
    });
}

template <int K>
static int launch_adj_tile(qgpu_handle* h, double2* phi, double2* lam, const AdjTileParams& p,
                           double* partial) {
    // phi and lambda stay in the resident float-pair layout for the whole sweep
    return adj_profiled(h, "k_adj_tile", 64.0 * (double)h->dim, [&]() -> int {
        k_adj_tile<K, true><<<p.nb, ADJ_THREADS, 0, h->stream>>>(phi, lam, p, partial);
        QGPU_CHECK_LAUNCH("k_adj_tile");
        h->launches++;
        h->h2d_bytes += sizeof(AdjTileParams);
        return QGPU_OK;
    });
}

// ---------------------------------------------------------------------------------------------
// k_linperm: a run of CNot / X / Swap gates maps basis index y to an affine function of y over
// GF(2). The run is applied out of place as one gather, dst[y] = src[h(y)] with h the inverse
// map (h(y) = d xor the columns of y's set bits, read from 8-bit chunk tables in shared memory):
// writes are coalesced, reads follow the map. A CNot ring (the ansatz's entangler, a chain of
// dependent gates the register-tile passes can only take two at a time) becomes one pass.
// ---------------------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(ADJ_THREADS)
k_linperm(const T* __restrict__ src, T* __restrict__ dst, uint64_t dim,
          const uint64_t* __restrict__ tabs, int nchunks, uint64_t d) {
    extern __shared__ uint64_t tsm[];
    for (int i = threadIdx.x; i < nchunks * 256; i += ADJ_THREADS) tsm[i] = tabs[i];
    __syncthreads();
    for (uint64_t y = blockIdx.x * (uint64_t)ADJ_THREADS + threadIdx.x; y < dim;
         y += (uint64_t)gridDim.x * ADJ_THREADS) {
        uint64_t x = d;
        for (int c = 0; c < nchunks; ++c) x ^= tsm[c * 256 + (int)((y >> (8 * c)) & 255u)];
        dst[y] = src[x];
    }
}

// out[g] = sum over blocks of partial[g * nb + b], for g in [0, ng): one warp per row (lanes
// stride over the blocks, then a fixed shuffle tree; the order is the same on every run)
__global__ void k_sum_partials(const double* __restrict__ partial, int nb, int ng,
                               double* __restrict__ out) {
    const int g = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (g >= ng) return;  // whole warps leave together
    double s = 0.0;
    for (int b = lane; b < nb; b += 32) s += partial[(size_t)g * nb + b];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
    if (lane == 0) out[g] = s;
}

static int adj_blocks(const qgpu_handle* h, uint64_t work) {
    uint64_t b = (work + ADJ_THREADS - 1) / ADJ_THREADS;
    const uint64_t cap = (uint64_t)h->sm_count * 4;
    if (b > cap) b = cap;
    return (int)std::max<uint64_t>(1, b);
}

// Energy of the vector at `psi` into *energy; lambda = H psi left at `lam`.
template <class T>
static int energy_into(qgpu_handle* h, const T* psi, T* lam, const Ham& H, double* partial,
                       double* energy) {
    const int nb = adj_blocks(h, h->dim);
    k_apply_zzx<T><<<nb, ADJ_THREADS, 0, h->stream>>>(psi, lam, h->dim, H, partial);
    QGPU_CHECK_LAUNCH("k_apply_zzx");
    h->launches++;
    k_sum_partials<<<1, 32, 0, h->stream>>>(partial, nb, 1, partial + nb);
    QGPU_CHECK_LAUNCH("k_sum_partials");
    h->launches++;
    QGPU_CUDA(copy_async(h, energy, partial + nb, sizeof(double), cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

static int ham_from(const qgpu_handle* h, const double* a, const double* b, Ham* H) {
    if (!a || !b) return fail(QGPU_ERR_INVALID, "observable coefficients are NULL");
    if (h->n_qubits > MAX_HAM_QUBITS)
        return fail(QGPU_ERR_UNSUPPORTED, "observable supports at most 40 qubits");
    std::memset(H, 0, sizeof(Ham));
    H->n = h->n_qubits;
    for (int i = 0; i < H->n; ++i) {
        H->a[i] = a[i];
        H->b[i] = b[i];
    }
    return QGPU_OK;
}

// The adjoint sweep of a complex64 handle (the forward pass has run on the register): phi and
// lambda as complex64 work vectors, every run of single-wire gates in grouped passes
// (k_adj_group_f32), runs of multi-wire gates undone as one index gather (k_linperm) or through
// the register-tile passes. The gradients are formed on the host from the Pauli sums, as in the
// complex128 sweep.
static int adjoint_sweep_c64(qgpu_handle* h, const qgpu_op* ops, size_t n_ops, const Ham& H,
                             double* energy, double* grads) {
    size_t nrot = 0;
    for (size_t g = 0; g < n_ops; ++g) nrot += is_rotation(ops[g].kind) ? 1 : 0;
    const int nb = adj_blocks(h, h->dim);  // row length of the partial sums (covers every grid)
    const size_t vec = h->dim * 8;
    const size_t nrow_cap = 4 * nrot + 4;
    const size_t part_doubles = (nrow_cap + 1) * (size_t)nb + nrow_cap + 64;
    int st = h->work2.ensure(2 * vec + part_doubles * 8 + 512);
    if (st != QGPU_OK) return st;
    float2* phi = (float2*)h->work2.ptr;
    float2* lam = (float2*)((uint8_t*)h->work2.ptr + vec);
    double* partial = (double*)((uint8_t*)h->work2.ptr + 2 * vec);
    double* gsum = partial + (nrow_cap + 1) * (size_t)nb;
    QGPU_CUDA(cudaMemcpyAsync(phi, h->state, vec, cudaMemcpyDeviceToDevice, h->stream));
    st = energy_into(h, (const float2*)phi, lam, H, partial + nrow_cap * (size_t)nb, energy);
    if (st != QGPU_OK) return st;
    std::vector<std::vector<std::pair<int, double>>> terms(n_ops);
    int nrows = 0;
    std::vector<qgpu_op> seg;  // consecutive multi-wire gates, undone together
    float2* spare = nullptr;   // third vector for out-of-place index permutations
    auto flush_seg = [&]() -> int {
        if (seg.empty()) return QGPU_OK;
        std::vector<uint64_t> tabs;
        uint64_t d = 0;
        if (h->n_qubits >= 10 && seg.size() >= 3 &&
            affine_tables(seg.data(), seg.size(), h->n_qubits, &tabs, &d)) {
            if (!spare && h->work3.ensure(vec) == QGPU_OK) spare = (float2*)h->work3.ptr;
            if (spare && h->tables.ensure(tabs.size() * 8) == QGPU_OK) {
                QGPU_CUDA(copy_async(h, h->tables.ptr, tabs.data(), tabs.size() * 8,
                                     cudaMemcpyHostToDevice));
                const int nch = (h->n_qubits + 7) / 8;
                const int blocks = adj_blocks(h, h->dim);
                for (float2** v : {&phi, &lam}) {
                    k_linperm<float2><<<blocks, ADJ_THREADS, nch * 256 * 8, h->stream>>>(
                        *v, spare, h->dim, (const uint64_t*)h->tables.ptr, nch, d);
                    QGPU_CHECK_LAUNCH("k_linperm");
                    h->launches++;
                    std::swap(*v, spare);
                }
                seg.clear();
                return QGPU_OK;
            }
        }
        Plan plan;
        int s2 = build_plan(seg.data(), seg.size(), h->n_qubits, nullptr, 0, nullptr, 0,
                            plan_options_for(h), &plan);
        if (s2 == QGPU_OK) s2 = run_plan_on(h, phi, plan, false, false);
        if (s2 == QGPU_OK) s2 = run_plan_on(h, lam, plan, false, false);
        seg.clear();
        return s2;
    };
    std::vector<size_t> run;  // op indices of the current single-wire run, in reverse order
    auto flush_run = [&]() -> int {
        if (run.empty()) return QGPU_OK;
        std::vector<int> wires;                  // bit of each wire, in first-seen order
        std::vector<std::vector<size_t>> gates;  // per wire, its ops in reverse order
        for (size_t gi : run) {
            const int bit = h->n_qubits - 1 - ops[gi].target;
            size_t w = std::find(wires.begin(), wires.end(), bit) - wires.begin();
            if (w == wires.size()) {
                wires.push_back(bit);
                gates.emplace_back();
            }
            gates[w].push_back(gi);
        }
        run.clear();
        std::vector<PauliRun> prs(wires.size());
        for (size_t w = 0; w < wires.size(); ++w) {
            int s3 = pauli_run(ops, gates[w], h->n_qubits, &prs[w]);
            if (s3 != QGPU_OK) return s3;
        }
        for (const auto& pass : adj_group_passes(wires, h->n_qubits, ADJ_GROUP_MAX_BITS)) {
            AdjGroupParamsF p;
            std::memset(&p, 0, sizeof(p));
            for (int b = 0; b < 64; ++b)
                if ((pass.first >> b) & 1ull) p.bits[p.nbits++] = b;
            p.ngroups = h->dim >> p.nbits;
            p.nb = nb;
            p.nwires = (int)pass.second.size();
            for (int c = 0; c < p.nwires; ++c) {
                const size_t w = pass.second[c];
                AdjGroupWireF& gw = p.w[c];
                gw.lb = (int)(std::find(p.bits, p.bits + p.nbits, wires[w]) - p.bits);
                int kind_row[5] = {-1, -1, -1, -1, -1};
                for (int m = 1; m <= 4; ++m) {
                    gw.row[m - 1] = -1;
                    if (prs[w].need[m]) gw.row[m - 1] = kind_row[m] = nrows++;
                }
                for (int e = 0; e < 4; ++e) {
                    gw.u[2 * e] = (float)prs[w].undo[e].real();
                    gw.u[2 * e + 1] = (float)prs[w].undo[e].imag();
                }
                for (const auto& r : prs[w].rots)
                    for (int m = 1; m <= 4; ++m)
                        if (r.second[m] != 0.0) terms[r.first].emplace_back(kind_row[m], r.second[m]);
            }
            int s2 = launch_adj_group_f32(h, phi, lam, p, partial);
            if (s2 != QGPU_OK) return s2;
        }
        return QGPU_OK;
    };
    for (size_t gi = n_ops; gi-- > 0;) {
        const qgpu_op& op = ops[gi];
        if (op.kind == QGPU_GATE_ID) continue;
        int k = 1;
        op_arity(op, h->n_qubits, &k);
        if (k > 1) {
            st = flush_run();
            if (st != QGPU_OK) return st;
            seg.push_back(inverse_op(op));
            continue;
        }
        st = flush_seg();
        if (st != QGPU_OK) return st;
        run.push_back(gi);
    }
    st = flush_run();
    if (st != QGPU_OK) return st;
    st = flush_seg();
    if (st != QGPU_OK) return st;
    if (nrows > (int)nrow_cap) return fail(QGPU_ERR_UNSUPPORTED, "adjoint: partial-sum rows overflow");
    if (nrows) {
        k_sum_partials<<<(unsigned)((nrows + 3) / 4), 128, 0, h->stream>>>(partial, nb, nrows, gsum);
        QGPU_CHECK_LAUNCH("k_sum_partials");
        h->launches++;
    }
    std::vector<double> gr(nrows);
    if (nrows) QGPU_CUDA(copy_async(h, gr.data(), gsum, (size_t)nrows * 8, cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t g = 0; g < n_ops; ++g) {
        double v = 0.0;
        for (const auto& t : terms[g]) v += t.second * gr[t.first];
        grads[g] = v;
    }
    return QGPU_OK;
}

}  // namespace qgpu

using namespace qgpu;

extern "C" {

int qgpu_expectation_zzx(qgpu_handle* h, const double* a, const double* b, double* energy) {
    if (!h || !energy) return fail(QGPU_ERR_INVALID, "qgpu_expectation_zzx: NULL argument");
    Ham H;
    int st = ham_from(h, a, b, &H);
    if (st != QGPU_OK) return st;
    const int nb = adj_blocks(h, h->dim);
    const size_t vec = h->dim * h->amp_bytes;
    st = h->work2.ensure(vec + (size_t)(nb + 8) * 8 + 256);
    if (st != QGPU_OK) return st;
    double* partial = (double*)((uint8_t*)h->work2.ptr + vec);
    if (h->precision == QGPU_C64)
        return energy_into(h, (const float2*)h->state, (float2*)h->work2.ptr, H, partial, energy);
    return energy_into(h, (const double2*)h->state, (double2*)h->work2.ptr, H, partial, energy);
}

int qgpu_adjoint_grad(qgpu_handle* h, const qgpu_op* ops, size_t n_ops, const double* mats,
                      size_t n_mat_doubles, const uint8_t* none_flags, size_t n_none_flags,
                      const double* a, const double* b, double* energy, double* grads) {
    if (!h || !energy || !grads || (n_ops && !ops))
        return fail(QGPU_ERR_INVALID, "qgpu_adjoint_grad: NULL argument");
    Ham H;
    int st = ham_from(h, a, b, &H);
    if (st != QGPU_OK) return st;
    for (size_t g = 0; g < n_ops; ++g) {
        if (ops[g].kind == QGPU_GATE_CUSTOM)
            return fail(QGPU_ERR_NONUNITARY, "adjoint gradients need invertible gates; the circuit "
                                             "contains a Custom gate");
        int k;
        st = op_arity(ops[g], h->n_qubits, &k);
        if (ops[g].kind != QGPU_GATE_ID && st != QGPU_OK) return st;
    }
    // forward pass on the register
    st = qgpu_apply_program(h, ops, n_ops, mats, n_mat_doubles, none_flags, n_none_flags);
    if (st != QGPU_OK) return st;
    if (h->precision == QGPU_C64) return adjoint_sweep_c64(h, ops, n_ops, H, energy, grads);
    // work vectors: phi (copy of psi_L), lambda, block partials per rotation
    size_t nrot = 0;
    for (size_t g = 0; g < n_ops; ++g) nrot += is_rotation(ops[g].kind) ? 1 : 0;
    // CTAs of the sweep kernels: one wave at k_adj_tile's occupancy (a second, partial wave
    // would leave most SMs idle at the end of every pass)
    static thread_local int adj_occ = 0;
    if (!adj_occ) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&adj_occ, k_adj_tile<1, true>, ADJ_THREADS,
                                                          0) != cudaSuccess || adj_occ < 1)
            adj_occ = 1;
    }
    int nb = (int)std::min<uint64_t>((h->dim / 2 + ADJ_THREADS - 1) / ADJ_THREADS,
                                     (uint64_t)h->sm_count * adj_occ);
    nb = std::max(nb, 1);
    const size_t vec = h->dim * 16;
    // rows of per-CTA partial sums: one per summed term. A rotation undone alone takes one row;
    // a wire's run of gates takes at most four (its Pauli sums), so 4 per rotation bounds them.
    const size_t nrow_cap = 4 * nrot + 4;
    const size_t part_doubles = (nrow_cap + 1) * (size_t)nb + nrow_cap + 64;
    st = h->work2.ensure(2 * vec + part_doubles * 8 + 512);
    if (st != QGPU_OK) return st;
    double2* phi = (double2*)h->work2.ptr;
    double2* lam = (double2*)((uint8_t*)h->work2.ptr + vec);
    double* partial = (double*)((uint8_t*)h->work2.ptr + 2 * vec);
    double* gsum = partial + (nrow_cap + 1) * (size_t)nb;
    QGPU_CUDA(cudaMemcpyAsync(phi, h->state, vec, cudaMemcpyDeviceToDevice, h->stream));
    st = energy_into(h, phi, lam, H, partial + nrow_cap * (size_t)nb, energy);
    if (st != QGPU_OK) return st;
    // QGPU_MODE_FAST: the sweep works on phi and lambda in the resident float-pair layout (one
    // conversion each here; the vectors are scratch, nothing converts them back)
    const bool tiles = h->mode == QGPU_MODE_FAST;
    if (tiles) {
        st = ff_layout_on(h, phi, true);
        if (st == QGPU_OK) st = ff_layout_on(h, lam, true);
        if (st != QGPU_OK) return st;
    }

    // gradient of op g = sum over terms[g] of coefficient x (row sum)
    std::vector<std::vector<std::pair<int, double>>> terms(n_ops);
    int nrows = 0;
    // reverse sweep
    std::vector<qgpu_op> seg;  // consecutive multi-wire gates, undone together
    double2* spare = nullptr;  // third vector for out-of-place index permutations
    auto flush_seg = [&]() -> int {  // one plan for both vectors, launches queued without a sync
        if (seg.empty()) return QGPU_OK;
        std::vector<uint64_t> tabs;
        uint64_t d = 0;
        if (h->n_qubits >= 10 && seg.size() >= 3 &&
            affine_tables(seg.data(), seg.size(), h->n_qubits, &tabs, &d)) {
            if (!spare && h->work3.ensure(vec) == QGPU_OK) spare = (double2*)h->work3.ptr;
            if (spare && h->tables.ensure(tabs.size() * 8) == QGPU_OK) {
                QGPU_CUDA(copy_async(h, h->tables.ptr, tabs.data(), tabs.size() * 8,
                                     cudaMemcpyHostToDevice));
                const int nch = (h->n_qubits + 7) / 8;
                const int blocks = adj_blocks(h, h->dim);
                for (double2** v : {&phi, &lam}) {
                    k_linperm<double2><<<blocks, ADJ_THREADS, nch * 256 * 8, h->stream>>>(
                        *v, spare, h->dim, (const uint64_t*)h->tables.ptr, nch, d);
                    QGPU_CHECK_LAUNCH("k_linperm");
                    h->launches++;
                    std::swap(*v, spare);
                }
                seg.clear();
                return QGPU_OK;
            }
        }
        Plan plan;
        int s2 = build_plan(seg.data(), seg.size(), h->n_qubits, nullptr, 0, nullptr, 0,
                            plan_options_for(h), &plan);
        if (s2 == QGPU_OK) s2 = run_plan_on(h, phi, plan, false, tiles);
        if (s2 == QGPU_OK) s2 = run_plan_on(h, lam, plan, false, tiles);
        seg.clear();
        return s2;
    };
    // QGPU_MODE_FAST: runs of single-wire gates go through k_adj_tile, up to 2 wires and 4 gates
    // per pass; each wire keeps its gates in reverse order (gates on other wires commute).
    // Wires per pass (tuning knob QGPU_ADJ_TILE_BITS: 1 or 2). One wire per pass measured faster
    // on GB300 (20-qubit ansatz: 10.2 ms against 11.2 ms): the 2-wire kernel needs 162 registers,
    // one CTA per SM, and is latency-bound.
    static const int tile_bits = [] {
        const char* e = std::getenv("QGPU_ADJ_TILE_BITS");
        return (e && e[0] == '2') ? 2 : 1;
    }();
    std::vector<size_t> run;  // op indices of the current single-wire run, in reverse order
    auto flush_run = [&]() -> int {
        if (run.empty()) return QGPU_OK;
        std::vector<int> wires;                  // bit of each wire, in first-seen order
        std::vector<std::vector<size_t>> gates;  // per wire, its ops in reverse order
        for (size_t gi : run) {
            const int bit = h->n_qubits - 1 - ops[gi].target;
            size_t w = std::find(wires.begin(), wires.end(), bit) - wires.begin();
            if (w == wires.size()) {
                wires.push_back(bit);
                gates.emplace_back();
            }
            gates[w].push_back(gi);
        }
        run.clear();
        // Pauli-sum passes take less arithmetic (one 2x2 update per vector per wire instead of
        // one per gate) and win once the vectors live in HBM; with the vectors in L2 (up to 21
        // qubits) the per-gate passes measured faster on GB300 (20 qubits: 6.39 against 6.68 ms;
        // 24 qubits: 35.1 against 29.9 ms). Tuning knob QGPU_ADJ_PAULI: 0 / 1 forces either.
        const char* pk = std::getenv("QGPU_ADJ_PAULI");  // read per call (tests force either)
        const int pauli_knob = (pk && pk[0] == '0') ? 0 : (pk && pk[0] == '1') ? 1 : -1;
        // Grouped passes (k_adj_group: the wires of a run in tiles of up to 11 bits, one pass
        // per tile) up to 22 qubits; QGPU_ADJ_GROUP=0 / 1 (read per call) forces them off / on.
        // Measured on GB300 (4-layer ansatz, energy + gradient): 20 qubits 5.23 against 6.34 ms
        // (30 launches instead of 200), 22 qubits 7.72 against 7.76 ms, 24 qubits 31.8 against
        // 29.8 ms: a wire's float-pair sums and undo keep the FMA pipe 64 % busy for about as
        // long as one streaming pass over both vectors takes, so from 23 qubits the per-wire
        // passes (HBM-bound, the arithmetic hidden under the traffic) are kept.
        // The batch autotuner's pick (h->adj_group) comes first.
        const char* gk = std::getenv("QGPU_ADJ_GROUP");
        const int forced = h->adj_group >= 0 ? h->adj_group : gk ? (gk[0] != '0' ? 1 : 0) : -1;
        const bool group = pauli_knob != 0 && (forced >= 0 ? forced == 1 : h->n_qubits <= 22);
        const bool pauli = pauli_knob >= 0 ? pauli_knob == 1 : h->n_qubits >= 22;
        if (group) {
            std::vector<PauliRun> prs(wires.size());
            for (size_t w = 0; w < wires.size(); ++w) {
                int s3 = pauli_run(ops, gates[w], h->n_qubits, &prs[w]);
                if (s3 != QGPU_OK) return s3;
            }
            for (const auto& pass : adj_group_passes(wires, h->n_qubits, ADJ_GROUP_MAX_BITS)) {
                const uint64_t mask = pass.first;
                const std::vector<size_t>& chosen = pass.second;
                AdjGroupParams p;
                std::memset(&p, 0, sizeof(p));
                for (int b = 0; b < 64; ++b)
                    if ((mask >> b) & 1ull) p.bits[p.nbits++] = b;
                p.ngroups = h->dim >> p.nbits;
                p.nb = nb;
                p.nwires = (int)chosen.size();
                for (int c = 0; c < p.nwires; ++c) {
                    const size_t w = chosen[c];
                    AdjGroupWire& gw = p.w[c];
                    gw.lb = (int)(std::find(p.bits, p.bits + p.nbits, wires[w]) - p.bits);
                    int kind_row[5] = {-1, -1, -1, -1, -1};
                    for (int m = 1; m <= 4; ++m) {
                        gw.row[m - 1] = -1;
                        if (prs[w].need[m]) gw.row[m - 1] = kind_row[m] = nrows++;
                    }
                    const std::array<cd, 4>& undo = prs[w].undo;
                    const DevStep ds = dense_step(undo[0], undo[1], undo[2], undo[3]);
                    std::memcpy(gw.pk, ds.pk, sizeof(gw.pk));
                    for (const auto& r : prs[w].rots)
                        for (int m = 1; m <= 4; ++m)
                            if (r.second[m] != 0.0) terms[r.first].emplace_back(kind_row[m], r.second[m]);
                }
                int s2 = launch_adj_group(h, phi, lam, p, partial);
                if (s2 != QGPU_OK) return s2;
            }
            return QGPU_OK;
        }
        if (tile_bits == 1 && pauli) {
            // One pass per wire: the sums <lambda| s |phi> for the Paulis s the run's rotations
            // need, all taken before any of its gates is undone, then the whole run undone as one
            // 2x2. A rotation G_j = exp(-i theta P/2) followed on its wire by V (the run's later
            // gates; gates on other wires commute with P) has gradient Im <lambda| V P V^dag |phi>,
            // and V P V^dag = q0 I + qx X + qy Y + qz Z: its gradient is that combination of the
            // Pauli sums, formed on the host.
            for (size_t w = 0; w < wires.size(); ++w) {
                PauliRun pr;
                int s3 = pauli_run(ops, gates[w], h->n_qubits, &pr);
                if (s3 != QGPU_OK) return s3;
                const std::array<cd, 4>& undo = pr.undo;
                const bool* need = pr.need;
                const auto& rots = pr.rots;
                AdjTileParams p;
                std::memset(&p, 0, sizeof(p));
                p.nbits = 1;
                p.bits[0] = wires[w];
                p.ngroups = h->dim >> 1;
                p.nb = nb;
                int kind_row[5] = {-1, -1, -1, -1, -1};
                int ns = 0;
                for (int m = 1; m <= 4; ++m) {
                    if (!need[m]) continue;
                    AdjTileStep& t = p.steps[ns++];
                    t.lb = 0;
                    t.gen = m;
                    t.slot = kind_row[m] = nrows++;
                    t.apply = 0;
                }
                if (ns == 0) {  // nothing to differentiate: just the update
                    p.steps[0].lb = 0;
                    p.steps[0].gen = 0;
                    p.steps[0].slot = -1;
                    ns = 1;
                }
                AdjTileStep& last = p.steps[ns - 1];
                last.apply = 1;
                const DevStep ds = dense_step(undo[0], undo[1], undo[2], undo[3]);
                std::memcpy(last.pk, ds.pk, sizeof(last.pk));
                p.nsteps = ns;
                for (const auto& r : rots)
                    for (int m = 1; m <= 4; ++m)
                        if (r.second[m] != 0.0) terms[r.first].emplace_back(kind_row[m], r.second[m]);
                int s2 = launch_adj_tile<1>(h, phi, lam, p, partial);
                if (s2 != QGPU_OK) return s2;
            }
            return QGPU_OK;
        }
        AdjTileParams p;
        std::vector<std::pair<int, size_t>> pend;  // (bit, op) of the pass being filled
        std::vector<int> pbits;
        auto launch = [&]() -> int {
            if (pend.empty()) return QGPU_OK;
            std::memset(&p, 0, sizeof(p));
            std::sort(pbits.begin(), pbits.end());
            p.nbits = (int)pbits.size();
            for (int m = 0; m < p.nbits; ++m) p.bits[m] = pbits[m];
            p.ngroups = h->dim >> p.nbits;
            p.nsteps = (int)pend.size();
            p.nb = nb;
            for (size_t q = 0; q < pend.size(); ++q) {
                const qgpu_op& op = ops[pend[q].second];
                AdjTileStep& t = p.steps[q];
                t.lb = (int)(std::find(pbits.begin(), pbits.end(), pend[q].first) - pbits.begin());
                switch (op.kind) {
                    case QGPU_GATE_RX: t.gen = 1; break;
                    case QGPU_GATE_RY: t.gen = 2; break;
                    case QGPU_GATE_RZ: t.gen = 3; break;
                    case QGPU_GATE_PHASE: t.gen = 4; break;
                    default: t.gen = 0; break;
                }
                t.slot = -1;
                if (is_rotation(op.kind)) {
                    t.slot = nrows++;
                    terms[pend[q].second].emplace_back(t.slot, 1.0);
                }
                t.apply = 1;
                LocalGate lg;
                int s3 = tabulate(inverse_op(op), h->n_qubits, nullptr, 0, nullptr, 0, &lg);
                if (s3 != QGPU_OK) return s3;
                // V[l][j] = M[j * 2 + l]
                const DevStep ds = dense_step(lg.M[0], lg.M[2], lg.M[1], lg.M[3]);
                std::memcpy(t.pk, ds.pk, sizeof(t.pk));
            }
            pend.clear();
            pbits.clear();
            return p.nbits == 1 ? launch_adj_tile<1>(h, phi, lam, p, partial)
                                : launch_adj_tile<2>(h, phi, lam, p, partial);
        };
        for (size_t w = 0; w < wires.size(); ++w) {
            for (size_t q = 0; q < gates[w].size(); ++q) {
                const bool have = std::find(pbits.begin(), pbits.end(), wires[w]) != pbits.end();
                if ((!have && (int)pbits.size() == tile_bits) || pend.size() == ADJ_TILE_STEPS) {
                    int s2 = launch();
                    if (s2 != QGPU_OK) return s2;
                }
                if (std::find(pbits.begin(), pbits.end(), wires[w]) == pbits.end())
                    pbits.push_back(wires[w]);
                pend.emplace_back(wires[w], gates[w][q]);
            }
        }
        return launch();
    };
    for (size_t gi = n_ops; gi-- > 0;) {
        const qgpu_op& op = ops[gi];
        if (op.kind == QGPU_GATE_ID) continue;
        int k = 1;
        op_arity(op, h->n_qubits, &k);
        if (k > 1) {
            st = flush_run();
            if (st != QGPU_OK) return st;
            seg.push_back(inverse_op(op));
            continue;
        }
        st = flush_seg();
        if (st != QGPU_OK) return st;
        if (tiles) {
            run.push_back(gi);
            continue;
        }
        LocalGate lg;
        st = tabulate(inverse_op(op), h->n_qubits, nullptr, 0, nullptr, 0, &lg);
        if (st != QGPU_OK) return st;
        AdjStep s;
        s.t = h->n_qubits - 1 - op.target;
        switch (op.kind) {
            case QGPU_GATE_RX: s.gen = 1; break;
            case QGPU_GATE_RY: s.gen = 2; break;
            case QGPU_GATE_RZ: s.gen = 3; break;
            case QGPU_GATE_PHASE: s.gen = 4; break;
            default: s.gen = 0; break;
        }
        // row-major V from the column-major images: V[l][j] = M[j*2 + l]
        for (int l = 0; l < 2; ++l)
            for (int j = 0; j < 2; ++j) {
                s.v[2 * (2 * l + j)] = lg.M[j * 2 + l].real();
                s.v[2 * (2 * l + j) + 1] = lg.M[j * 2 + l].imag();
            }
        double* part = nullptr;
        if (is_rotation(op.kind)) {
            terms[gi].emplace_back(nrows, 1.0);
            part = partial + (size_t)(nrows++) * nb;
        }
        if (h->mode == QGPU_MODE_FAST) {
            AdjStepFF f;
            f.t = s.t;
            f.gen = s.gen;
            const cd v00(s.v[0], s.v[1]), v01(s.v[2], s.v[3]), v10(s.v[4], s.v[5]), v11(s.v[6], s.v[7]);
            const DevStep ds = dense_step(v00, v01, v10, v11);
            std::memcpy(f.pk, ds.pk, sizeof(f.pk));
            k_adj_1q_ff<<<nb, ADJ_THREADS, 0, h->stream>>>(phi, lam, h->dim / 2, f, part);
            QGPU_CHECK_LAUNCH("k_adj_1q_ff");
        } else {
            k_adj_1q<<<nb, ADJ_THREADS, 0, h->stream>>>(phi, lam, h->dim / 2, s, part);
            QGPU_CHECK_LAUNCH("k_adj_1q");
        }
        h->launches++;
    }
    st = flush_run();
    if (st != QGPU_OK) return st;
    st = flush_seg();
    if (st != QGPU_OK) return st;
    if (nrows > (int)nrow_cap) return fail(QGPU_ERR_UNSUPPORTED, "adjoint: partial-sum rows overflow");
    if (nrows) {
        k_sum_partials<<<(unsigned)((nrows + 3) / 4), 128, 0, h->stream>>>(partial, nb, nrows,
                                                                            gsum);
        QGPU_CHECK_LAUNCH("k_sum_partials");
        h->launches++;
    }
    std::vector<double> gr(nrows);
    if (nrows) QGPU_CUDA(copy_async(h, gr.data(), gsum, (size_t)nrows * 8, cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t g = 0; g < n_ops; ++g) {
        double v = 0.0;
        for (const auto& t : terms[g]) v += t.second * gr[t.first];
        grads[g] = v;
    }
    return QGPU_OK;
}

}  // extern "C"
