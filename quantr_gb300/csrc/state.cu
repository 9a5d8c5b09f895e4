// state.cu — handle lifecycle, register upload/download, f64 reductions.
//
// Device layout: one contiguous buffer of 2^n amplitudes, index = basis integer with wire 0 as
// the most significant bit (quantr's `binary_basis`, product_states.rs:205-215). complex128 is
// double2 {re, im} (16 B); complex64 is float2 (8 B). cudaMalloc gives 256-byte alignment, so
// every 16/32-byte vector access used by the kernels is aligned.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.cuh"

namespace qgpu {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? QGPU_ERR_OOM : QGPU_ERR_CUDA;
}

int Scratch::ensure(size_t need) {
    if (need <= bytes) return QGPU_OK;
    // Host-side fault injection: with QGPU_INJECT_SCRATCH_OOM=1 in the environment every scratch
    // allocation fails as on a full device (the buffer held so far is kept), so that the error
    // paths of the callers can be tested without any device fault. Read only when an allocation
    // is due.
    const char* inject = std::getenv("QGPU_INJECT_SCRATCH_OOM");
    if (inject && inject[0] == '1')
        return fail(QGPU_ERR_OOM, "device scratch allocation of " + std::to_string(need) +
                                      " bytes failed (injected by QGPU_INJECT_SCRATCH_OOM)");
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t grow = need + need / 4;
    cudaError_t e = cudaMalloc(&ptr, grow);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        e = cudaMalloc(&ptr, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ptr = nullptr;
            return fail(QGPU_ERR_OOM, "device scratch allocation of " + std::to_string(need) +
                                          " bytes failed");
        }
        grow = need;
    }
    bytes = grow;
    return QGPU_OK;
}

void Scratch::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

// ---------------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------------
template <class T>
__global__ void k_set_basis(T* __restrict__ s, uint64_t dim, uint64_t basis) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (; i < dim; i += stride) {
        T v;
        v.x = (i == basis) ? 1 : 0;
        v.y = 0;
        s[i] = v;
    }
}

__global__ void k_d2f(const double2* __restrict__ in, float2* __restrict__ out, uint64_t n) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

__global__ void k_f2d(const float2* __restrict__ in, double2* __restrict__ out, uint64_t n) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) out[i] = make_double2((double)in[i].x, (double)in[i].y);
}

// Deterministic reductions: block b sums a fixed contiguous range with a fixed tree.
constexpr int RED_THREADS = 256;

// what = 0 keeps |re|^2 and |im|^2 in two fused multiply-add chains (two FP64 operations per
// amplitude; the FP64 pipe, not HBM, bounded the separate multiply/add form) and folds them
// together once per thread; what = 1 sums re and im.
template <class T>
__global__ void k_reduce_partial(const T* __restrict__ s, uint64_t dim, uint64_t per_block,
                                 int what, double2* __restrict__ partial) {
    __shared__ double2 sh[RED_THREADS];
    const uint64_t begin = blockIdx.x * per_block;
    uint64_t end = begin + per_block;
    if (end > dim) end = dim;
    double ax = 0.0, ay = 0.0;
    if (what == 0) {
        for (uint64_t i = begin + threadIdx.x; i < end; i += RED_THREADS) {
            const double re = (double)s[i].x, im = (double)s[i].y;
            ax = fma(re, re, ax);
            ay = fma(im, im, ay);
        }
        ax += ay;
        ay = 0.0;
    } else {
        for (uint64_t i = begin + threadIdx.x; i < end; i += RED_THREADS) {
            ax += (double)s[i].x;
            ay += (double)s[i].y;
        }
    }
    sh[threadIdx.x] = make_double2(ax, ay);
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[threadIdx.x].x += sh[threadIdx.x + w].x;
            sh[threadIdx.x].y += sh[threadIdx.x + w].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_reduce_final(const double2* __restrict__ partial, int nb, double2* out) {
    __shared__ double2 sh[RED_THREADS];
    double ax = 0.0, ay = 0.0;
    for (int i = threadIdx.x; i < nb; i += RED_THREADS) {
        ax += partial[i].x;
        ay += partial[i].y;
    }
    sh[threadIdx.x] = make_double2(ax, ay);
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[threadIdx.x].x += sh[threadIdx.x + w].x;
            sh[threadIdx.x].y += sh[threadIdx.x + w].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// Comparison of two registers of one size (qgpu_compare): per block the largest |a_i - b_i| and
// the partial inner product sum conj(a_i) b_i over a fixed contiguous range, then one block
// folds the partials (max, and fixed-tree sums), so the result is deterministic.
template <class TA, class TB>
__global__ void k_compare_partial(const TA* __restrict__ a, const TB* __restrict__ b,
                                  uint64_t dim, uint64_t per_block, double4* __restrict__ partial) {
    __shared__ double4 sh[RED_THREADS];
    const uint64_t begin = blockIdx.x * per_block;
    uint64_t end = begin + per_block;
    if (end > dim) end = dim;
    double mx = 0.0, re = 0.0, im = 0.0;
    for (uint64_t i = begin + threadIdx.x; i < end; i += RED_THREADS) {
        const double ar = (double)a[i].x, ai = (double)a[i].y;
        const double br = (double)b[i].x, bi = (double)b[i].y;
        const double dr = ar - br, di = ai - bi;
        mx = fmax(mx, sqrt(dr * dr + di * di));
        re = fma(ar, br, fma(ai, bi, re));
        im = fma(ar, bi, fma(-ai, br, im));
    }
    sh[threadIdx.x] = make_double4(mx, re, im, 0.0);
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[threadIdx.x].x = fmax(sh[threadIdx.x].x, sh[threadIdx.x + w].x);
            sh[threadIdx.x].y += sh[threadIdx.x + w].y;
            sh[threadIdx.x].z += sh[threadIdx.x + w].z;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_compare_final(const double4* __restrict__ partial, int nb, double4* out) {
    __shared__ double4 sh[RED_THREADS];
    double mx = 0.0, re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < nb; i += RED_THREADS) {
        mx = fmax(mx, partial[i].x);
        re += partial[i].y;
        im += partial[i].z;
    }
    sh[threadIdx.x] = make_double4(mx, re, im, 0.0);
    __syncthreads();
    for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sh[threadIdx.x].x = fmax(sh[threadIdx.x].x, sh[threadIdx.x + w].x);
            sh[threadIdx.x].y += sh[threadIdx.x + w].y;
            sh[threadIdx.x].z += sh[threadIdx.x + w].z;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

int grid_for(const qgpu_handle* h, uint64_t work, int threads) {
    uint64_t blocks = (work + threads - 1) / threads;
    uint64_t cap = (uint64_t)h->sm_count * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

// Sum over the state of |a|^2 (what = 0) or of a (what = 1), in f64.
int reduce_state(qgpu_handle* h, int what, double2* host_out) {
    const uint64_t dim = h->dim;
    int nb = h->sm_count * 8;
    if ((uint64_t)nb > dim) nb = (int)dim;
    const uint64_t per_block = (dim + nb - 1) / nb;
    int st = h->work.ensure(sizeof(double2) * (nb + 1));
    if (st != QGPU_OK) return st;
    double2* partial = (double2*)h->work.ptr;
    if (h->precision == QGPU_C128)
        k_reduce_partial<double2><<<nb, RED_THREADS, 0, h->stream>>>((const double2*)h->state, dim,
                                                                    per_block, what, partial);
    else
        k_reduce_partial<float2><<<nb, RED_THREADS, 0, h->stream>>>((const float2*)h->state, dim,
                                                                   per_block, what, partial);
    QGPU_CHECK_LAUNCH("k_reduce_partial");
    k_reduce_final<<<1, RED_THREADS, 0, h->stream>>>(partial, nb, partial + nb);
    QGPU_CHECK_LAUNCH("k_reduce_final");
    h->launches += 2;
    QGPU_CUDA(copy_async(h, host_out, partial + nb, sizeof(double2), cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

int prof_flush(qgpu_handle* h) {
    if (h->ev_pending.empty()) return QGPU_OK;
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < h->ev_pending.size(); ++i) {
        float ms = 0.f;
        QGPU_CUDA(cudaEventElapsedTime(&ms, h->events[2 * i], h->events[2 * i + 1]));
        qgpu_handle::ProfEntry& e = h->prof[h->ev_pending[i].first];
        e.launches += 1;
        e.ms += ms;
        e.bytes += h->ev_pending[i].second;
    }
    h->ev_pending.clear();
    h->ev_used = 0;
    return QGPU_OK;
}

int prof_events(qgpu_handle* h, size_t pairs, size_t* base) {
    constexpr size_t MAX_PENDING_PAIRS = 16384;  // read back before the pool grows past this
    if (h->ev_used + pairs > MAX_PENDING_PAIRS) {
        int st = prof_flush(h);
        if (st != QGPU_OK) return st;
    }
    while (h->events.size() < 2 * (h->ev_used + pairs)) {
        cudaEvent_t e;
        QGPU_CUDA(cudaEventCreate(&e));
        h->events.push_back(e);
    }
    *base = h->ev_used;
    return QGPU_OK;
}

int prof_collect(qgpu_handle* h, const std::vector<std::string>& names,
                 const std::vector<double>& bytes) {
    for (size_t i = 0; i < names.size(); ++i) h->ev_pending.emplace_back(names[i], bytes[i]);
    h->ev_used += names.size();
    return QGPU_OK;
}

}  // namespace qgpu

using namespace qgpu;

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
extern "C" {

void* qgpu_stream(qgpu_handle* h) { return h ? (void*)h->stream : nullptr; }

uint64_t qgpu_launch_count(const qgpu_handle* h) { return h ? h->launches : 0; }

int qgpu_io_bytes(const qgpu_handle* h, uint64_t* h2d, uint64_t* d2h) {
    if (!h || !h2d || !d2h) return fail(QGPU_ERR_INVALID, "qgpu_io_bytes: NULL argument");
    *h2d = h->h2d_bytes;
    *d2h = h->d2h_bytes;
    return QGPU_OK;
}

int qgpu_synchronize(qgpu_handle* h) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_synchronize: NULL handle");
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

int qgpu_set_profiling(qgpu_handle* h, int on) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_set_profiling: NULL handle");
    h->profile = on != 0;
    return QGPU_OK;
}

int qgpu_profile_json(qgpu_handle* h, char* buf, size_t cap, int reset) {
    if (!h || (!buf && cap)) return fail(QGPU_ERR_INVALID, "qgpu_profile_json: NULL argument");
    int st = prof_flush(h);
    if (st != QGPU_OK) return st;
    std::string s = "{";
    bool first = true;
    for (const auto& kv : h->prof) {
        char tmp[256];
        snprintf(tmp, sizeof(tmp), "%s\"%s\": [%llu, %.6f, %.1f]", first ? "" : ", ",
                 kv.first.c_str(), (unsigned long long)kv.second.launches, kv.second.ms,
                 kv.second.bytes);
        s += tmp;
        first = false;
    }
    s += "}";
    if (cap) {
        const size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
        memcpy(buf, s.data(), n);
        buf[n] = 0;
    }
    if (reset) h->prof.clear();
    return QGPU_OK;
}

}  // extern "C"
extern "C" {

const char* qgpu_last_error(void) { return g_last_error.c_str(); }

int qgpu_create(int n_qubits, int precision, qgpu_handle** out) {
    if (!out) return fail(QGPU_ERR_INVALID, "qgpu_create: out is NULL");
    *out = nullptr;
    if (n_qubits < 1 || n_qubits > 40)
        return fail(QGPU_ERR_INVALID, "qgpu_create: the register must have 1..40 qubits (got " +
                                          std::to_string(n_qubits) + ")");
    if (precision != QGPU_C128 && precision != QGPU_C64)
        return fail(QGPU_ERR_INVALID, "qgpu_create: precision must be QGPU_C128 or QGPU_C64");
    int dev = 0;
    QGPU_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    QGPU_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (prop.major < 10)
        return fail(QGPU_ERR_UNSUPPORTED, std::string("libquantr_gpu needs a Blackwell GPU; ") +
                                              prop.name + " is not one");
    qgpu_handle* h = new qgpu_handle();
    h->n_qubits = n_qubits;
    h->precision = precision;
    h->device = dev;
    h->sm_count = prop.multiProcessorCount;
    h->dim = 1ull << n_qubits;
    h->amp_bytes = precision == QGPU_C128 ? 16 : 8;
    const size_t bytes = (size_t)h->dim * h->amp_bytes;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    if (bytes > free_b) {
        delete h;
        return fail(QGPU_ERR_OOM, "qgpu_create: " + std::to_string(n_qubits) + " qubits need " +
                                      std::to_string(bytes) + " bytes; " + std::to_string(free_b) +
                                      " are free on the device");
    }
    cudaError_t e = cudaMalloc(&h->state, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return fail(QGPU_ERR_OOM, "qgpu_create: cudaMalloc of " + std::to_string(bytes) +
                                      " bytes failed: " + cudaGetErrorString(e));
    }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaFree(h->state);
        delete h;
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    e = cudaMalloc(&h->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->d_err, 0, sizeof(int));
    if (e != cudaSuccess) {
        qgpu_destroy(h);
        return cuda_fail(e, "cudaMalloc(error word)");
    }
    int st = qgpu_set_zero(h);
    if (st != QGPU_OK) {
        qgpu_destroy(h);
        return st;
    }
    *out = h;
    return QGPU_OK;
}

int qgpu_destroy(qgpu_handle* h) {
    if (!h) return QGPU_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->gates.release();
    h->tables.release();
    h->work.release();
    h->work2.release();
    h->work3.release();
    for (cudaEvent_t e : h->events) cudaEventDestroy(e);
    if (h->d_err) cudaFree(h->d_err);
    if (h->state) cudaFree(h->state);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return QGPU_OK;
}

int qgpu_num_qubits(const qgpu_handle* h) {
    return h ? h->n_qubits : fail(QGPU_ERR_INVALID, "qgpu_num_qubits: NULL handle");
}

int qgpu_set_mode(qgpu_handle* h, int mode) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_set_mode: NULL handle");
    if (mode != QGPU_MODE_FAST && mode != QGPU_MODE_EXACT && mode != QGPU_MODE_F64)
        return fail(QGPU_ERR_INVALID, "qgpu_set_mode: unknown mode " + std::to_string(mode));
    h->mode = mode;
    return QGPU_OK;
}

int qgpu_set_zero(qgpu_handle* h) {
    if (!h) return fail(QGPU_ERR_INVALID, "qgpu_set_zero: NULL handle");
    const int threads = 256;
    const int grid = grid_for(h, h->dim, threads);
    if (h->precision == QGPU_C128)
        k_set_basis<double2><<<grid, threads, 0, h->stream>>>((double2*)h->state, h->dim, 0);
    else
        k_set_basis<float2><<<grid, threads, 0, h->stream>>>((float2*)h->state, h->dim, 0);
    QGPU_CHECK_LAUNCH("k_set_basis");
    h->launches++;
    h->norm_bound = 1.0;
    h->norm_valid = true;
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

int qgpu_upload(qgpu_handle* h, const double* interleaved, size_t n_amplitudes) {
    if (!h || !interleaved) return fail(QGPU_ERR_INVALID, "qgpu_upload: NULL argument");
    if (n_amplitudes != h->dim)
        return fail(QGPU_ERR_INVALID,
                    "qgpu_upload: the register has " + std::to_string(n_amplitudes) +
                        " amplitudes but the circuit has " + std::to_string(h->dim) +
                        " (2^" + std::to_string(h->n_qubits) + ")");
    h->norm_valid = false;
    if (h->precision == QGPU_C128) {
        QGPU_CUDA(copy_async(h, h->state, interleaved, h->dim * 16, cudaMemcpyHostToDevice));
        QGPU_CUDA(cudaStreamSynchronize(h->stream));
        return QGPU_OK;
    }
    const uint64_t chunk = 1ull << 24;  // 256 MiB of f64 staging per step
    const uint64_t stage = h->dim < chunk ? h->dim : chunk;
    int st = h->work.ensure(stage * 16);
    if (st != QGPU_OK) return st;
    for (uint64_t off = 0; off < h->dim; off += stage) {
        const uint64_t cnt = (h->dim - off) < stage ? (h->dim - off) : stage;
        QGPU_CUDA(copy_async(h, h->work.ptr, interleaved + 2 * off, cnt * 16,
                             cudaMemcpyHostToDevice));
        k_d2f<<<grid_for(h, cnt, 256), 256, 0, h->stream>>>((const double2*)h->work.ptr,
                                                            (float2*)h->state + off, cnt);
        QGPU_CHECK_LAUNCH("k_d2f");
        h->launches++;
    }
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

int qgpu_download(qgpu_handle* h, double* out, size_t n_amplitudes) {
    if (!h || !out) return fail(QGPU_ERR_INVALID, "qgpu_download: NULL argument");
    if (n_amplitudes != h->dim)
        return fail(QGPU_ERR_INVALID, "qgpu_download: buffer holds " +
                                          std::to_string(n_amplitudes) + " amplitudes, need " +
                                          std::to_string(h->dim));
    if (h->precision == QGPU_C128) {
        QGPU_CUDA(copy_async(h, out, h->state, h->dim * 16, cudaMemcpyDeviceToHost));
        QGPU_CUDA(cudaStreamSynchronize(h->stream));
        return QGPU_OK;
    }
    const uint64_t chunk = 1ull << 24;
    const uint64_t stage = h->dim < chunk ? h->dim : chunk;
    int st = h->work.ensure(stage * 16);
    if (st != QGPU_OK) return st;
    for (uint64_t off = 0; off < h->dim; off += stage) {
        const uint64_t cnt = (h->dim - off) < stage ? (h->dim - off) : stage;
        k_f2d<<<grid_for(h, cnt, 256), 256, 0, h->stream>>>((const float2*)h->state + off,
                                                            (double2*)h->work.ptr, cnt);
        QGPU_CHECK_LAUNCH("k_f2d");
        h->launches++;
        QGPU_CUDA(copy_async(h, out + 2 * off, h->work.ptr, cnt * 16, cudaMemcpyDeviceToHost));
    }
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

int qgpu_norm(qgpu_handle* h, double* out) {
    if (!h || !out) return fail(QGPU_ERR_INVALID, "qgpu_norm: NULL argument");
    double2 r;
    int st = reduce_state(h, 0, &r);
    if (st == QGPU_OK) *out = r.x;
    return st;
}

int qgpu_checksum(qgpu_handle* h, double* re_out, double* im_out) {
    if (!h || !re_out || !im_out) return fail(QGPU_ERR_INVALID, "qgpu_checksum: NULL argument");
    double2 r;
    int st = reduce_state(h, 1, &r);
    if (st == QGPU_OK) {
        *re_out = r.x;
        *im_out = r.y;
    }
    return st;
}

int qgpu_compare(qgpu_handle* a, qgpu_handle* b, double* max_abs_diff, double* inner_re,
                 double* inner_im) {
    if (!a || !b || !max_abs_diff || !inner_re || !inner_im)
        return fail(QGPU_ERR_INVALID, "qgpu_compare: NULL argument");
    if (a->n_qubits != b->n_qubits)
        return fail(QGPU_ERR_INVALID, "qgpu_compare: registers of " + std::to_string(a->n_qubits) +
                                          " and " + std::to_string(b->n_qubits) + " qubits");
    if (a->device != b->device)
        return fail(QGPU_ERR_INVALID, "qgpu_compare: the registers live on different devices");
    // b's queued passes finish before a's stream reads b.
    QGPU_CUDA(cudaStreamSynchronize(b->stream));
    const uint64_t dim = a->dim;
    int nb = a->sm_count * 8;
    if ((uint64_t)nb > dim) nb = (int)dim;
    const uint64_t per_block = (dim + nb - 1) / nb;
    int st = a->work.ensure(sizeof(double4) * (nb + 1));
    if (st != QGPU_OK) return st;
    double4* partial = (double4*)a->work.ptr;
    const bool a64 = a->precision == QGPU_C128, b64 = b->precision == QGPU_C128;
    if (a64 && b64)
        k_compare_partial<double2, double2><<<nb, RED_THREADS, 0, a->stream>>>(
            (const double2*)a->state, (const double2*)b->state, dim, per_block, partial);
    else if (a64)
        k_compare_partial<double2, float2><<<nb, RED_THREADS, 0, a->stream>>>(
            (const double2*)a->state, (const float2*)b->state, dim, per_block, partial);
    else if (b64)
        k_compare_partial<float2, double2><<<nb, RED_THREADS, 0, a->stream>>>(
            (const float2*)a->state, (const double2*)b->state, dim, per_block, partial);
    else
        k_compare_partial<float2, float2><<<nb, RED_THREADS, 0, a->stream>>>(
            (const float2*)a->state, (const float2*)b->state, dim, per_block, partial);
    QGPU_CHECK_LAUNCH("k_compare_partial");
    k_compare_final<<<1, RED_THREADS, 0, a->stream>>>(partial, nb, partial + nb);
    QGPU_CHECK_LAUNCH("k_compare_final");
    a->launches += 2;
    double4 r;
    QGPU_CUDA(copy_async(a, &r, partial + nb, sizeof(double4), cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(a->stream));
    *max_abs_diff = r.x;
    *inner_re = r.y;
    *inner_im = r.z;
    return QGPU_OK;
}

}  // extern "C"
