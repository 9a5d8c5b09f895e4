// internal.cuh — shared definitions of libquantr_gpu (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <utility>
#include <string>
#include <vector>

#include "../../include/qgpu.h"

// ---------------------------------------------------------------------------------------------
// Errors: every entry point returns a status; the message goes to a thread-local string.
// ---------------------------------------------------------------------------------------------
namespace qgpu {

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define QGPU_CUDA(call)                                          \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ::qgpu::cuda_fail(e_, #call); \
    } while (0)

#define QGPU_CHECK_LAUNCH(what)                                     \
    do {                                                            \
        cudaError_t e_ = cudaGetLastError();                        \
        if (e_ != cudaSuccess) return ::qgpu::cuda_fail(e_, what);  \
    } while (0)

// Opts `kernel` into `bytes` of dynamic shared memory on the current device. The attribute
// belongs to the device's context, so it is set once per (kernel, device) and again when a
// larger size is asked for; safe from several host threads.
inline cudaError_t smem_opt_in(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t& have = done[{kernel, dev}];
    if (have >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
}

// Device scratch owned by a handle, grown on demand and reused across calls.
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t need);  // QGPU_OK or QGPU_ERR_OOM
    void release();
};

}  // namespace qgpu

struct qgpu_handle {
    int n_qubits = 0;
    int precision = QGPU_C128;
    int mode = QGPU_MODE_FAST;
    int block_qubits = 0;      // > 0: fuse gates into dense blocks of this many wires
    int block_gates = 12;      // at most this many gates per dense block
    int batch_budget = 0;      // > 0: float-pair fusion budget picked by the batch autotuner
    int adj_group = -1;        // adjoint sweep form picked by the batch autotuner: 1 grouped
                               // tiles (k_adj_group), 0 per-wire passes, -1 by size
    int device = 0;
    int sm_count = 0;
    uint64_t dim = 0;          // 2^n amplitudes
    size_t amp_bytes = 16;     // 16 (c128) or 8 (c64)
    void* state = nullptr;     // device amplitudes: double2[dim] or float2[dim]
    void* active = nullptr;    // when set, gate passes run on this buffer instead of `state`
    int* d_err = nullptr;      // device error word of pipelined kernels (bounded waits)
    cudaStream_t stream = nullptr;
    qgpu::Scratch gates;       // per-program device tables (custom matrices, orders, flags)
    qgpu::Scratch tables;      // per-program phase tables of fused diagonal runs
    qgpu::Scratch work;        // reductions, measurement buffers
    qgpu::Scratch work2;       // second buffer (measurement indices / adjoint vectors)
    qgpu::Scratch work3;       // adjoint: target of out-of-place index permutations
    // An upper bound on the register's largest |amplitude| (its norm, for a normalised state):
    // the digit passes scale their fixed point by it. Exact after set_zero (1), unknown after an
    // upload (computed on the device when a digit pass needs it), carried through plans (Custom
    // gates multiply it by the Frobenius norm of their effective map).
    double norm_bound = 1.0;
    bool norm_valid = true;
    uint64_t launches = 0;     // kernels launched on this handle (for benchmarking claims)
    uint64_t h2d_bytes = 0;    // host->device traffic: copies + kernel parameter blocks
    uint64_t d2h_bytes = 0;    // device->host copies
    // per-pass event profiling (qgpu_set_profiling)
    bool profile = false;
    std::vector<cudaEvent_t> events;
    size_t ev_used = 0;        // event pairs recorded and not yet read back
    std::vector<std::pair<std::string, double>> ev_pending;  // (kernel name, bytes) per pair
    struct ProfEntry {
        uint64_t launches = 0;
        double ms = 0.0;
        double bytes = 0.0;
    };
    std::map<std::string, ProfEntry> prof;
};

namespace qgpu {
// The buffer gate passes operate on (the register, or a work vector of the adjoint sweep).
inline void* cur_state(const qgpu_handle* h) { return h->active ? h->active : h->state; }
// cudaMemcpyAsync on the handle's stream that also counts host<->device bytes.
inline cudaError_t copy_async(qgpu_handle* h, void* dst, const void* src, size_t n,
                              cudaMemcpyKind kind) {
    if (kind == cudaMemcpyHostToDevice) h->h2d_bytes += n;
    if (kind == cudaMemcpyDeviceToHost) h->d2h_bytes += n;
    return cudaMemcpyAsync(dst, src, n, kind, h->stream);
}
// f64 sum over the register of |a|^2 (what = 0) or of a (what = 1); synchronises.
int reduce_state(qgpu_handle* h, int what, double2* host_out);
// Reserves `pairs` event pairs of the handle's pool (grown on demand); *base receives the index
// of the first one (pair i = events[2 (base + i)], events[2 (base + i) + 1]).
int prof_events(qgpu_handle* h, size_t pairs, size_t* base);
// Files the reserved pairs under the given names; they are read back lazily (prof_flush), so
// profiling adds no synchronisation to the calls it measures.
int prof_collect(qgpu_handle* h, const std::vector<std::string>& names,
                 const std::vector<double>& bytes);
// Waits for the stream and accumulates every pending pair into the per-kernel totals.
int prof_flush(qgpu_handle* h);
}  // namespace qgpu

// ---------------------------------------------------------------------------------------------
// Index helpers. Wire w of an n-qubit register is bit (n-1-w) of the amplitude index.
// ---------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ int wire_bit(int n, int wire) { return n - 1 - wire; }

// Insert a zero at bit position q of x (bits >= q move up by one).
__host__ __device__ __forceinline__ uint64_t insert_zero(uint64_t x, int q) {
    uint64_t lo = x & ((1ull << q) - 1ull);
    return ((x >> q) << (q + 1)) | lo;
}

// ---------------------------------------------------------------------------------------------
// Float-pair ("double-float") arithmetic. A value is the unevaluated sum h + l of two floats
// with |l| <= ulp(h)/2: a 48-bit significand carried on the FP32 pipes, which on GB300 issue
// about 67x faster than FP64. Building blocks are the error-free transforms of Dekker (1971)
// and Knuth (TAOCP vol. 2, 4.2.2): TwoProduct via FMA and TwoSum. The __f*_rn intrinsics are
// never contracted or reassociated by the compiler, which the transforms rely on.
// ---------------------------------------------------------------------------------------------
#ifdef __CUDACC__

struct ffc {  // complex value with float-pair real and imaginary parts
    float rh, rl, ih, il;
};

// f64 -> float pair by bit manipulation (the f64<->f32 conversion instructions run on the slow
// FP64 pipe). h takes the sign, exponent and top 23 fraction bits (truncated). The remaining 29
// fraction bits become l, rounded to nearest, so |x - (h + l)| <= 2^-48 |x| without bias.
// Values below 2^-126 in magnitude become 0; the low part is dropped below 2^-75.
__device__ __forceinline__ void split_f64(double x, float& h, float& l) {
    const unsigned lo = (unsigned)__double2loint(x);
    const unsigned hi = (unsigned)__double2hiint(x);
    const unsigned t = hi - (896u << 20);            // rebias 1023 -> 127 (valid when ex > 896)
    unsigned hb = __funnelshift_l(lo, t, 3);          // (t << 3) | (lo >> 29)
    hb = (hb & 0x7FFFFFFFu) | (hi & 0x80000000u);
    // remaining 29 fraction bits: an integer m29 with weight 2^(E-1075); the integer->float
    // conversion rounds it to nearest, the power-of-two scale (carrying x's sign) is exact
    const float m = __uint2float_rn(lo & 0x1FFFFFFFu);
    const float scale = __uint_as_float((hb & 0xFF800000u) - (52u << 23));
    const unsigned ah = hi & 0x7FFFFFFFu;
    h = ah <= (896u << 20) + 0xFFFFFu ? 0.0f : __uint_as_float(hb);  // |x| < 2^-126 -> 0
    l = ah <= (948u << 20) + 0xFFFFFu ? 0.0f : __fmul_rn(m, scale);  // drop below 2^-75
}

// Exact float -> f64 by bit manipulation (zero and subnormal floats give a signed zero).
__device__ __forceinline__ double f32_to_f64_bits(float f) {
    const unsigned b = __float_as_uint(f);
    unsigned hiw = (((b & 0x7FFFFFFFu) >> 3) + (896u << 20)) | (b & 0x80000000u);
    unsigned low = b << 29;
    const bool zero = (b & 0x7F800000u) == 0u;
    hiw = zero ? (b & 0x80000000u) : hiw;
    low = zero ? 0u : low;
    return __hiloint2double((int)hiw, (int)low);
}

// Exact float -> f64 for normal floats only (a zero or subnormal float maps to a value of
// magnitude below 2^-126 instead of 0; join_f64 handles the zero high part).
__device__ __forceinline__ double f32_to_f64_normal(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned hiw = (((b & 0x7FFFFFFFu) >> 3) + (896u << 20)) | (b & 0x80000000u);
    return __hiloint2double((int)hiw, (int)(b << 29));
}

// float pair -> f64: both halves are exact doubles; one f64 add rounds their sum. A high part
// below the float normal range (the pair is then below 2^-126) gives 0.
__device__ __forceinline__ double join_f64(float h, float l) {
    const double d = __dadd_rn(f32_to_f64_normal(h), f32_to_f64_normal(l));
    return (__float_as_uint(h) & 0x7F800000u) ? d : 0.0;
}

__device__ __forceinline__ ffc to_ffc(double2 a) {
    ffc r;
    split_f64(a.x, r.rh, r.rl);
    split_f64(a.y, r.ih, r.il);
    return r;
}
__device__ __forceinline__ double2 from_ffc(const ffc& a) {
    return make_double2(join_f64(a.rh, a.rl), join_f64(a.ih, a.il));
}

// ---- bulk copies (TMA, cp.async.bulk) with mbarrier completion -------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
// Global -> shared bulk copy; both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Bounded wait on an mbarrier phase: false after `limit` unsuccessful polls (each poll already
// suspends the thread for a hardware-chosen interval).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ---- packed f32x2 arithmetic (Blackwell add/sub/mul/fma .rn.f32x2) ---------------------------
// A 64-bit register holds two floats (lane 0, lane 1); each op rounds each lane to nearest,
// exactly as the scalar instruction would, so the error-free transforms hold lane by lane.
typedef uint64_t u64;

__device__ __forceinline__ u64 p2(float x, float y) {
    u64 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ void up2(u64 v, float& x, float& y) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v));
}
__device__ __forceinline__ u64 pmul(u64 a, u64 b) {
    u64 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 pfma(u64 a, u64 b, u64 c) {
    u64 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ u64 padd(u64 a, u64 b) {
    u64 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 psub(u64 a, u64 b) {
    u64 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ u64 pswap(u64 v) {
    float x, y;
    up2(v, x, y);
    return p2(y, x);
}

// Complex value as float pairs, packed by part: h = (re_hi, im_hi), l = (re_lo, im_lo).
struct ffp {
    u64 h, l;
};

__device__ __forceinline__ ffp to_ffp(double2 a) {
    float rh, rl, ih, il;
    split_f64(a.x, rh, rl);
    split_f64(a.y, ih, il);
    return ffp{p2(rh, ih), p2(rl, il)};
}
__device__ __forceinline__ double2 from_ffp(const ffp& v) {
    float rh, ih, rl, il;
    up2(v.h, rh, ih);
    up2(v.l, rl, il);
    return make_double2(join_f64(rh, rl), join_f64(ih, il));
}

// Resident float-pair layout: a 16-byte amplitude slot holds (re_h, im_h | re_l, im_l), read and
// written as the two packed registers of an ffp.
__device__ __forceinline__ ffp ffr_load(double2 a) {
    ffp r;
    r.h = (u64)__double_as_longlong(a.x);
    r.l = (u64)__double_as_longlong(a.y);
    return r;
}
__device__ __forceinline__ double2 ffr_store(const ffp& r) {
    return make_double2(__longlong_as_double((long long)r.h), __longlong_as_double((long long)r.l));
}

// Dot2 on both lanes at once. A term's constants are c[0..3] = (U_hi, U_lo, -U_hi, -U_lo);
// `en` holds the negated error sum so that every update is a single fma/add/sub.
struct PDot2 {
    u64 s, en;
    __device__ __forceinline__ void first(const u64* c, u64 xh, u64 xl) {
        s = pmul(c[0], xh);
        en = pfma(c[2], xh, s);   // s - Uh*xh: minus the product's rounding error
        en = pfma(c[2], xl, en);  // - Uh*xl
        en = pfma(c[3], xh, en);  // - Ul*xh
    }
    __device__ __forceinline__ void add(const u64* c, u64 xh, u64 xl) {
        const u64 p = pmul(c[0], xh);
        u64 rn = pfma(c[2], xh, p);
        rn = pfma(c[2], xl, rn);
        rn = pfma(c[3], xh, rn);
        const u64 t = padd(s, p);  // TwoSum(s, p)
        const u64 bb = psub(t, s);
        const u64 q = padd(psub(s, psub(t, bb)), psub(p, bb));
        s = t;
        en = padd(psub(en, q), rn);
    }
    __device__ __forceinline__ void result(u64& h, u64& l) const {  // FastTwoSum(s, -en)
        h = psub(s, en);
        l = psub(psub(s, h), en);
    }
};

// (a, b) <- (u00 a + u01 b, u10 a + u11 b) with the packed Dot2 terms c[0..31] (DevStep::pk of an
// ST_DENSE step): each output's real and imaginary lanes come from one 4-term Dot2.
__device__ __forceinline__ void ff_dense(ffp& a, ffp& b, const u64* c) {
    const u64 ash = pswap(a.h), asl = pswap(a.l), bsh = pswap(b.h), bsl = pswap(b.l);
    PDot2 d;
    ffp o0, o1;
    d.first(c + 0, a.h, a.l);
    d.add(c + 4, ash, asl);
    d.add(c + 8, b.h, b.l);
    d.add(c + 12, bsh, bsl);
    d.result(o0.h, o0.l);
    d.first(c + 16, a.h, a.l);
    d.add(c + 20, ash, asl);
    d.add(c + 24, b.h, b.l);
    d.add(c + 28, bsh, bsl);
    d.result(o1.h, o1.l);
    a = o0;
    b = o1;
}

// Accurate dot product accumulator (Ogita, Rump & Oishi 2005, "Dot2"): s carries the running
// sum of the leading products, e collects every rounding error plus the small cross products.
struct Dot2 {
    float s, e;
    __device__ __forceinline__ void first(float uh, float ul, float ah, float al) {
        s = __fmul_rn(uh, ah);
        float r = __fmaf_rn(uh, ah, -s);
        r = __fmaf_rn(uh, al, r);
        e = __fmaf_rn(ul, ah, r);
    }
    __device__ __forceinline__ void add(float uh, float ul, float ah, float al) {
        const float p = __fmul_rn(uh, ah);
        float r = __fmaf_rn(uh, ah, -p);
        r = __fmaf_rn(uh, al, r);
        r = __fmaf_rn(ul, ah, r);
        const float t = __fadd_rn(s, p);  // TwoSum(s, p)
        const float bb = __fsub_rn(t, s);
        const float q = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
        s = t;
        e = __fadd_rn(e, __fadd_rn(q, r));
    }
    __device__ __forceinline__ void result(float& h, float& l) const {  // FastTwoSum(s, e)
        h = __fadd_rn(s, e);
        l = __fsub_rn(e, __fsub_rn(h, s));
    }
};

#endif  // __CUDACC__
