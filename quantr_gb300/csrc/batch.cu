// batch.cu — many independent circuits: energies and adjoint gradients (no counterpart in quantr).
//
// Circuits whose two work vectors fit in one SM's shared memory (complex128 up to 12 qubits,
// complex64 up to 13) run in one persistent launch, replayed from a CUDA graph: one CTA per SM
// takes circuit after circuit from an atomic work counter (no CTA ever waits on another) and runs
// the forward pass, lambda = H psi, the energy and the adjoint reverse sweep entirely in shared
// memory. Larger circuits run one after another through the register-tile passes and
// qgpu_adjoint_grad on a handle per register size in the batch's precision, with the fusion
// budget (and, for complex128, the adjoint sweep form) picked per size bucket by timing the
// candidates on the bucket's first circuit.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.cuh"
#include "plan.h"

namespace qgpu {

constexpr int BATCH_THREADS = 1024;
constexpr int BATCH_MAX_Q = 40;

// One gate of a batched circuit in controlled-2x2 form (or a swap of two bits).
struct BOp {
    uint8_t swap, t, b2, gen;  // gen: gradient generator 0 none, 1 X, 2 Y, 3 Z, 4 identity(-)
    uint32_t cm;               // control bits that must be 1
    double u[8];               // U row-major (complex)
    double v[8];               // U^dagger row-major
};

struct BCirc {
    int n, nops;
    int64_t op0;    // first BOp
    int64_t obs0;   // a[n] then b[n] in the observable array
    int64_t grad0;  // first gradient slot (one per op)
};

template <class T>
struct BMath;
template <>
struct BMath<double2> {
    using R = double;
};
template <>
struct BMath<float2> {
    using R = float;
};

template <class T>
__device__ __forceinline__ void apply2(T* v, const BOp& o, const double* m, int dim) {
    using R = typename BMath<T>::R;
    const R m0 = (R)m[0], m1 = (R)m[1], m2 = (R)m[2], m3 = (R)m[3], m4 = (R)m[4], m5 = (R)m[5],
            m6 = (R)m[6], m7 = (R)m[7];
    for (int p = threadIdx.x; p < dim / 2; p += blockDim.x) {
        const int i0 = (int)insert_zero((uint64_t)p, o.t), i1 = i0 | (1 << o.t);
        if (o.swap) {
            // exchange (bit t, bit b2) = (1, 0) with (0, 1): visit each exchanged pair once
            if (((i0 >> o.b2) & 1) == 1) {
                const int j = i0 ^ (1 << o.b2) ^ (1 << o.t);
                const T x = v[i0];
                v[i0] = v[j];
                v[j] = x;
            }
            continue;
        }
        if (((uint32_t)i0 & o.cm) != o.cm) continue;
        const T a = v[i0], b = v[i1];
        T r0, r1;
        r0.x = m0 * a.x - m1 * a.y + m2 * b.x - m3 * b.y;
        r0.y = m0 * a.y + m1 * a.x + m2 * b.y + m3 * b.x;
        r1.x = m4 * a.x - m5 * a.y + m6 * b.x - m7 * b.y;
        r1.y = m4 * a.y + m5 * a.x + m6 * b.y + m7 * b.x;
        v[i0] = r0;
        v[i1] = r1;
    }
}

// deterministic block sum of one double per thread
__device__ __forceinline__ double block_sum(double x, double* sh) {
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int w = BATCH_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

template <class T>
__global__ void __launch_bounds__(BATCH_THREADS)
k_batch_small(const BCirc* __restrict__ circs, int ncirc, const BOp* __restrict__ ops,
              const double* __restrict__ obs, double* __restrict__ energy, double* __restrict__ grads,
              unsigned* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[BATCH_THREADS];
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int c = cur;
        __syncthreads();
        if (c >= ncirc) return;
        const BCirc C = circs[c];
        const int dim = 1 << C.n;
        T* phi = reinterpret_cast<T*>(smem);
        T* lam = phi + dim;
        for (int x = threadIdx.x; x < dim; x += blockDim.x) {
            phi[x].x = x == 0 ? 1 : 0;
            phi[x].y = 0;
        }
        __syncthreads();
        const BOp* op = ops + C.op0;
        for (int g = 0; g < C.nops; ++g) {
            apply2(phi, op[g], op[g].u, dim);
            __syncthreads();
        }
        // lambda = H phi, energy = Re <phi|lambda>
        const double* a = obs + C.obs0;
        const double* b = a + C.n;
        double e = 0.0;
        for (int x = threadIdx.x; x < dim; x += blockDim.x) {
            double d = 0.0;
            for (int i = 0; i < C.n; ++i) {
                const int j = (i + 1) % C.n;
                const int par = ((x >> (C.n - 1 - i)) ^ (x >> (C.n - 1 - j))) & 1;
                d += par ? -a[i] : a[i];
            }
            double re = d * (double)phi[x].x, im = d * (double)phi[x].y;
            for (int i = 0; i < C.n; ++i) {
                const T w = phi[x ^ (1 << (C.n - 1 - i))];
                re = fma(b[i], (double)w.x, re);
                im = fma(b[i], (double)w.y, im);
            }
            lam[x].x = re;
            lam[x].y = im;
            e = fma((double)phi[x].x, re, fma((double)phi[x].y, im, e));
        }
        __syncthreads();
        e = block_sum(e, red);
        if (threadIdx.x == 0) energy[c] = e;
        // reverse sweep
        for (int g = C.nops - 1; g >= 0; --g) {
            const BOp& o = op[g];
            if (o.gen) {
                double acc = 0.0;
                for (int p = threadIdx.x; p < dim / 2; p += blockDim.x) {
                    const int i0 = (int)insert_zero((uint64_t)p, o.t), i1 = i0 | (1 << o.t);
                    const double f0x = phi[i0].x, f0y = phi[i0].y, f1x = phi[i1].x, f1y = phi[i1].y;
                    const double l0x = lam[i0].x, l0y = lam[i0].y, l1x = lam[i1].x, l1y = lam[i1].y;
                    switch (o.gen) {
                        case 1: acc += (l0x * f1y - l0y * f1x) + (l1x * f0y - l1y * f0x); break;
                        case 2: acc += -(l0x * f1x + l0y * f1y) + (l1x * f0x + l1y * f0y); break;
                        case 3: acc += (l0x * f0y - l0y * f0x) - (l1x * f1y - l1y * f1x); break;
                        default: acc -= (l0x * f0y - l0y * f0x) + (l1x * f1y - l1y * f1x); break;
                    }
                }
                acc = block_sum(acc, red);
                if (threadIdx.x == 0) grads[C.grad0 + g] = acc;
            } else if (threadIdx.x == 0) {
                grads[C.grad0 + g] = 0.0;
            }
            apply2(phi, o, o.v, dim);
            apply2(lam, o, o.v, dim);
            __syncthreads();
        }
    }
}

static int bgen(int kind) {
    switch (kind) {
        case QGPU_GATE_RX: return 1;
        case QGPU_GATE_RY: return 2;
        case QGPU_GATE_RZ: return 3;
        case QGPU_GATE_PHASE: return 4;
        default: return 0;
    }
}

// Host tabulation of one op into controlled-2x2 / swap form.
static int to_bop(const qgpu_op& op, int n, BOp* out) {
    if (op.kind == QGPU_GATE_CUSTOM)
        return fail(QGPU_ERR_NONUNITARY, "batched gradients need invertible gates; found a Custom gate");
    LocalGate lg;
    int st = tabulate(op, n, nullptr, 0, nullptr, 0, &lg);
    if (st != QGPU_OK) return st;
    std::memset(out, 0, sizeof(BOp));
    out->gen = (uint8_t)bgen(op.kind);
    if (op.kind == QGPU_GATE_SWAP) {
        out->swap = 1;
        out->t = (uint8_t)(n - 1 - op.target);
        out->b2 = (uint8_t)(n - 1 - op.controls[0]);
        return QGPU_OK;
    }
    const int k = lg.k;
    const size_t d = (size_t)1 << k, call = (d - 1) & ~(size_t)1;
    out->t = (uint8_t)(n - 1 - op.target);
    for (int m = 0; m < k - 1; ++m) out->cm |= 1u << (n - 1 - lg.wires[m]);
    cd U[2][2];
    for (int lo = 0; lo < 2; ++lo)
        for (int in = 0; in < 2; ++in) U[lo][in] = lg.M[(call | in) * d + (call | lo)];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            out->u[2 * (2 * r + c)] = U[r][c].real();
            out->u[2 * (2 * r + c) + 1] = U[r][c].imag();
            out->v[2 * (2 * r + c)] = U[c][r].real();   // conjugate transpose
            out->v[2 * (2 * r + c) + 1] = -U[c][r].imag();
        }
    return QGPU_OK;
}

int apply_ops_on(qgpu_handle* h, void* buffer, const qgpu_op* ops, size_t n_ops);

}  // namespace qgpu

using namespace qgpu;

extern "C" int qgpu_batch_run(const qgpu_batch_item* items, size_t n_items, const qgpu_op* ops,
                              size_t n_ops_total, const double* obs, size_t n_obs, int precision,
                              double* energies, double* grads, int* tuned_budget) {
    if (!items || !ops || !obs || !energies || !grads)
        return fail(QGPU_ERR_INVALID, "qgpu_batch_run: NULL argument");
    if (precision != QGPU_C128 && precision != QGPU_C64)
        return fail(QGPU_ERR_INVALID, "qgpu_batch_run: precision must be QGPU_C128 or QGPU_C64");
    const int small_max = precision == QGPU_C128 ? 12 : 13;
    if (tuned_budget)
        for (int q = 0; q <= BATCH_MAX_Q; ++q) tuned_budget[q] = 0;
    // ---- validate and split
    std::vector<size_t> small, large;
    for (size_t i = 0; i < n_items; ++i) {
        const qgpu_batch_item& it = items[i];
        if (it.n_qubits < 1 || it.n_qubits > BATCH_MAX_Q || it.n_ops < 0 || it.op_offset < 0 ||
            (size_t)(it.op_offset + it.n_ops) > n_ops_total || it.obs_offset < 0 ||
            (size_t)(it.obs_offset + 2 * it.n_qubits) > n_obs || it.grad_offset < 0)
            return fail(QGPU_ERR_INVALID, "qgpu_batch_run: item " + std::to_string(i) + " out of range");
        (it.n_qubits <= small_max ? small : large).push_back(i);
    }
    int dev = 0;
    QGPU_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    QGPU_CUDA(cudaGetDeviceProperties(&prop, dev));
    // ---- small circuits: one persistent launch from a CUDA graph
    if (!small.empty()) {
        std::vector<BCirc> circs;
        std::vector<BOp> bops;
        for (size_t i : small) {
            const qgpu_batch_item& it = items[i];
            BCirc c;
            c.n = it.n_qubits;
            c.nops = it.n_ops;
            c.op0 = (int64_t)bops.size();
            c.obs0 = it.obs_offset;
            c.grad0 = it.grad_offset;
            for (int g = 0; g < it.n_ops; ++g) {
                BOp b;
                int st = to_bop(ops[it.op_offset + g], it.n_qubits, &b);
                if (st != QGPU_OK) return st;
                bops.push_back(b);
            }
            circs.push_back(c);
        }
        size_t ngrad = 0;
        for (size_t i = 0; i < n_items; ++i)
            ngrad = std::max(ngrad, (size_t)(items[i].grad_offset + items[i].n_ops));
        const size_t esz = precision == QGPU_C128 ? 16 : 8;
        const size_t smem = 2 * ((size_t)1 << small_max) * esz;
        void *d_c = nullptr, *d_o = nullptr, *d_obs = nullptr, *d_e = nullptr, *d_g = nullptr, *d_cnt = nullptr;
        cudaStream_t s = nullptr;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        int st = QGPU_OK;
        auto cleanup = [&]() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            if (s) cudaStreamDestroy(s);
            for (void* p : {d_c, d_o, d_obs, d_e, d_g, d_cnt})
                if (p) cudaFree(p);
        };
#define BATCH_TRY(call)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) {                          \
            st = cuda_fail(e_, #call);                    \
            cleanup();                                    \
            return st;                                    \
        }                                                 \
    } while (0)
        BATCH_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        BATCH_TRY(cudaMalloc(&d_c, circs.size() * sizeof(BCirc)));
        BATCH_TRY(cudaMalloc(&d_o, std::max<size_t>(1, bops.size()) * sizeof(BOp)));
        BATCH_TRY(cudaMalloc(&d_obs, n_obs * sizeof(double)));
        BATCH_TRY(cudaMalloc(&d_e, n_items * sizeof(double)));
        BATCH_TRY(cudaMalloc(&d_g, std::max<size_t>(1, ngrad) * sizeof(double)));
        BATCH_TRY(cudaMalloc(&d_cnt, sizeof(unsigned)));
        BATCH_TRY(cudaMemcpyAsync(d_c, circs.data(), circs.size() * sizeof(BCirc), cudaMemcpyHostToDevice, s));
        if (!bops.empty())
            BATCH_TRY(cudaMemcpyAsync(d_o, bops.data(), bops.size() * sizeof(BOp), cudaMemcpyHostToDevice, s));
        BATCH_TRY(cudaMemcpyAsync(d_obs, obs, n_obs * sizeof(double), cudaMemcpyHostToDevice, s));
        BATCH_TRY(cudaStreamSynchronize(s));
        if (precision == QGPU_C128)
            BATCH_TRY(smem_opt_in((const void*)k_batch_small<double2>, smem));
        else
            BATCH_TRY(smem_opt_in((const void*)k_batch_small<float2>, smem));
        // capture: counter reset + persistent kernel, replayed as one graph
        BATCH_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(d_cnt, 0, sizeof(unsigned), s);
        if (precision == QGPU_C128)
            k_batch_small<double2><<<prop.multiProcessorCount, BATCH_THREADS, smem, s>>>(
                (const BCirc*)d_c, (int)circs.size(), (const BOp*)d_o, (const double*)d_obs,
                (double*)d_e, (double*)d_g, (unsigned*)d_cnt);
        else
            k_batch_small<float2><<<prop.multiProcessorCount, BATCH_THREADS, smem, s>>>(
                (const BCirc*)d_c, (int)circs.size(), (const BOp*)d_o, (const double*)d_obs,
                (double*)d_e, (double*)d_g, (unsigned*)d_cnt);
        BATCH_TRY(cudaStreamEndCapture(s, &graph));
        BATCH_TRY(cudaGraphInstantiate(&exec, graph, 0));
        BATCH_TRY(cudaGraphLaunch(exec, s));
        BATCH_TRY(cudaStreamSynchronize(s));
        // energies are indexed by position in the small list on the device
        std::vector<double> e_small(circs.size());
        BATCH_TRY(cudaMemcpy(e_small.data(), d_e, circs.size() * sizeof(double), cudaMemcpyDeviceToHost));
        std::vector<double> g_all(std::max<size_t>(1, ngrad));
        BATCH_TRY(cudaMemcpy(g_all.data(), d_g, g_all.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t q = 0; q < small.size(); ++q) {
            const qgpu_batch_item& it = items[small[q]];
            energies[small[q]] = e_small[q];
            for (int g = 0; g < it.n_ops; ++g) grads[it.grad_offset + g] = g_all[it.grad_offset + g];
        }
        cleanup();
#undef BATCH_TRY
    }
    // ---- large circuits: register-tile passes. The fusion budget is tuned once per size (the
    // forward pass timed per candidate), and so is the adjoint sweep's width (one energy +
    // gradient timed with the runs of single-wire gates grouped in tiles of up to 11 wires per
    // pass, and with one pass per wire); then W host threads, each with its own handles (and so
    // its own stream), take circuits largest first from a shared counter, so that the launch and
    // synchronisation overhead of medium circuits overlaps with other circuits' kernels.
    if (large.empty()) return QGPU_OK;
    std::stable_sort(large.begin(), large.end(), [&](size_t x, size_t y) {
        return items[x].n_qubits > items[y].n_qubits;
    });
    std::map<int, int> budget, sweep;
    {
        std::map<int, qgpu_handle*> tune;
        int st = QGPU_OK;
        for (size_t i : large) {
            const qgpu_batch_item& it = items[i];
            if (budget.count(it.n_qubits)) continue;
            qgpu_handle* h = nullptr;
            st = qgpu_create(it.n_qubits, precision, &h);
            if (st != QGPU_OK) break;
            tune[it.n_qubits] = h;
            const qgpu_op* po = ops + it.op_offset;
            // candidates of the float-pair (complex128) or f32 (complex64) fusion budget
            static const int cand128[] = {100, 140, 200, 280}, cand64[] = {24, 48, 96, 160};
            const int* cand = precision == QGPU_C128 ? cand128 : cand64;
            double best = 1e30;
            int pick = cand[3];
            for (int ci = 0; ci < 4; ++ci) {
                const int b = cand[ci];
                h->batch_budget = b;
                qgpu_set_zero(h);
                auto t0 = std::chrono::steady_clock::now();
                st = qgpu_apply_program(h, po, (size_t)it.n_ops, nullptr, 0, nullptr, 0);
                const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                if (st != QGPU_OK) break;
                if (dt < best) {
                    best = dt;
                    pick = b;
                }
            }
            if (st != QGPU_OK) break;
            budget[it.n_qubits] = pick;
            h->batch_budget = pick;
            // the sweep form (complex128; complex64 sweeps are always grouped): a first (untimed)
            // gradient allocates the work vectors
            std::vector<double> g((size_t)std::max(1, it.n_ops));
            double e = 0.0, tsweep[2] = {0.0, 0.0};
            const std::vector<int> forms = precision == QGPU_C128 ? std::vector<int>{1, 1, 0} : std::vector<int>{};
            for (int form : forms) {
                h->adj_group = form;
                qgpu_set_zero(h);
                auto t0 = std::chrono::steady_clock::now();
                st = qgpu_adjoint_grad(h, po, (size_t)it.n_ops, nullptr, 0, nullptr, 0, obs + it.obs_offset,
                                       obs + it.obs_offset + it.n_qubits, &e, g.data());
                if (st != QGPU_OK) break;
                tsweep[form] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            }
            if (st != QGPU_OK) break;
            sweep[it.n_qubits] = precision == QGPU_C128 ? (tsweep[1] <= tsweep[0] ? 1 : 0) : 1;
            if (tuned_budget) tuned_budget[it.n_qubits] = pick + (sweep[it.n_qubits] ? 65536 : 0);
        }
        for (auto& kv : tune) qgpu_destroy(kv.second);
        if (st != QGPU_OK) return st;
    }
    const char* env = std::getenv("QGPU_BATCH_WORKERS");
    const int workers = std::max(1, std::min(16, env ? std::atoi(env) : 4));
    std::atomic<size_t> next{0};
    std::atomic<int> first_err{QGPU_OK};
    std::string err_msg;
    std::mutex err_mu;
    auto work = [&]() {
        std::map<int, qgpu_handle*> handles;
        for (;;) {
            if (first_err.load() != QGPU_OK) break;
            const size_t q = next.fetch_add(1);
            if (q >= large.size()) break;
            const size_t i = large[q];
            const qgpu_batch_item& it = items[i];
            qgpu_handle*& h = handles[it.n_qubits];
            int st = QGPU_OK;
            if (!h) st = qgpu_create(it.n_qubits, precision, &h);
            if (st == QGPU_OK) {
                h->batch_budget = budget[it.n_qubits];
                h->adj_group = sweep[it.n_qubits];
                st = qgpu_set_zero(h);
            }
            if (st == QGPU_OK)
                st = qgpu_adjoint_grad(h, ops + it.op_offset, (size_t)it.n_ops, nullptr, 0, nullptr, 0,
                                       obs + it.obs_offset, obs + it.obs_offset + it.n_qubits,
                                       &energies[i], grads + it.grad_offset);
            if (st != QGPU_OK) {
                int expect = QGPU_OK;
                if (first_err.compare_exchange_strong(expect, st)) {
                    std::lock_guard<std::mutex> lk(err_mu);
                    err_msg = qgpu_last_error();
                }
                break;
            }
        }
        for (auto& kv : handles)
            if (kv.second) qgpu_destroy(kv.second);
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < workers; ++w) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    if (first_err.load() != QGPU_OK) return fail(first_err.load(), err_msg);
    return QGPU_OK;
}
