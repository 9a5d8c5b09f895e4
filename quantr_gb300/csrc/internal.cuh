// internal.cuh — shared definitions of libquantr_gpu (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
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
    int device = 0;
    int sm_count = 0;
    uint64_t dim = 0;          // 2^n amplitudes
    size_t amp_bytes = 16;     // 16 (c128) or 8 (c64)
    void* state = nullptr;     // device amplitudes: double2[dim] or float2[dim]
    void* active = nullptr;    // when set, gate passes run on this buffer instead of `state`
    cudaStream_t stream = nullptr;
    qgpu::Scratch gates;       // per-program device tables (custom matrices, orders, flags)
    qgpu::Scratch work;        // reductions, measurement buffers
    qgpu::Scratch work2;       // second buffer (measurement indices / adjoint vectors)
    uint64_t launches = 0;     // kernels launched on this handle (for benchmarking claims)
    uint64_t h2d_bytes = 0;    // host->device traffic: copies + kernel parameter blocks
    uint64_t d2h_bytes = 0;    // device->host copies
    // per-pass event profiling (qgpu_set_profiling)
    bool profile = false;
    std::vector<cudaEvent_t> events;
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
// Event pair i of the handle's pool (grown on demand); nullptr when profiling is off.
int prof_events(qgpu_handle* h, size_t pairs);
// Reads back the recorded pairs and accumulates them under the given names.
int prof_collect(qgpu_handle* h, const std::vector<std::string>& names,
                 const std::vector<double>& bytes);
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
// fraction bits are rebuilt as two exact floats with the 2^23 "magic number" subtraction (23
// bits, then 6 bits) whose sum rounds to nearest, so |x - (h + l)| <= 2^-48 |x| without bias.
// Values below 2^-126 in magnitude become 0; the low part is dropped below 2^-97.
__device__ __forceinline__ void split_f64(double x, float& h, float& l) {
    const unsigned lo = (unsigned)__double2loint(x);
    const unsigned hi = (unsigned)__double2hiint(x);
    const unsigned ex = (hi >> 20) & 0x7FFu;
    const unsigned t = hi - (896u << 20);            // rebias 1023 -> 127 (valid when ex > 896)
    unsigned hb = __funnelshift_l(lo, t, 3);          // (t << 3) | (lo >> 29)
    hb = (hb & 0x7FFFFFFFu) | (hi & 0x80000000u);
    const unsigned ea = (hb & 0x7F800000u) - (23u << 23);  // 2^23 * 2^(E-1069): weight of bit 6
    const unsigned eb = ea - (6u << 23);                   // 2^23 * 2^(E-1075): weight of bit 0
    const float ra = __fsub_rn(__uint_as_float(ea | ((lo >> 6) & 0x7FFFFFu)), __uint_as_float(ea));
    const float rb = __fsub_rn(__uint_as_float(eb | (lo & 0x3Fu)), __uint_as_float(eb));
    float lf = __fadd_rn(ra, rb);
    lf = __uint_as_float(__float_as_uint(lf) | (hi & 0x80000000u));
    const bool tiny = ex <= 896u;
    const bool nolo = ex <= 925u;
    h = tiny ? 0.0f : __uint_as_float(hb);
    l = nolo ? 0.0f : lf;
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

// float pair -> f64: both halves are exact doubles; one f64 add rounds their sum.
__device__ __forceinline__ double join_f64(float h, float l) {
    return __dadd_rn(f32_to_f64_bits(h), f32_to_f64_bits(l));
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
