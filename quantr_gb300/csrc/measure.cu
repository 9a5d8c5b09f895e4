// measure.cu — `SimulatedCircuit::measure_all` (src/simulated_circuit.rs:63-73, 116-130) on the
// device.
//
// The reference draws u = fastrand::f64() per shot and scans the register linearly, returning
// the first index i with u < sum_{j<=i} |a_j|^2, or None when u reaches the total
// (super_positions.rs:332-342): O(2^n) per shot. Here:
//   1. k_chunk_sums: |a|^2 summed over chunks of CHUNK amplitudes, one warp per chunk: each lane
//      sums 16 consecutive probabilities in order, then a fixed warp scan combines the lanes.
//   2. scan_exclusive: deterministic multi-level scan of the chunk sums -> chunk offsets.
//   3. the shot uniforms are generated already sorted (exponential spacings: if e_0..e_N are
//      i.i.d. Exp(1) and S_k their prefix sums, (S_0, ..., S_{N-1}) / S_N is distributed as the
//      order statistics of N i.i.d. U(0, 1); Devroye, "Non-Uniform Random Variate Generation",
//      1986, V.2), so the sampled indices come out sorted and the histogram is a run-length pass.
//   4. k_sample: one warp per shot: binary search over chunk offsets, then the same lane/warp
//      cumulative sums as step 1 locate the first index whose cumulative probability exceeds u.
// All sums are f64.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // CUcontext / CUresult types only; the driver is reached through the runtime

#include "internal.cuh"

namespace qgpu {

constexpr int CHUNK_BITS = 9;   // 512 amplitudes per chunk: 32 lanes x 16
constexpr int SCAN_TILE = 1024;

template <class S>
__device__ __forceinline__ double prob(const S* st, uint64_t i) {
    const double re = (double)st[i].x, im = (double)st[i].y;
    return __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));  // num-complex norm_sqr
}

// inclusive warp scan in a fixed order
__device__ __forceinline__ double warp_incl_scan(double v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const double o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v = __dadd_rn(v, o);
    }
    return v;
}

// Lane sum of the lane's run of a chunk (sequential, like the reference's running sum).
template <class S>
__device__ __forceinline__ double lane_run_sum(const S* st, uint64_t first, int count) {
    double s = 0.0;
    for (int q = 0; q < count; ++q) s = __dadd_rn(s, prob(st, first + q));
    return s;
}

template <class S>
__global__ void k_chunk_sums(const S* __restrict__ st, uint64_t nchunks, int chunk_len,
                             double* __restrict__ sums) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int per_lane = chunk_len >> 5 ? chunk_len >> 5 : 1;
    for (uint64_t c = warp; c < nchunks; c += nwarps) {
        const uint64_t first = c * (uint64_t)chunk_len + (uint64_t)lane * per_lane;
        const double s = (lane * per_lane < chunk_len) ? lane_run_sum(st, first, per_lane) : 0.0;
        const double inc = warp_incl_scan(s);
        if (lane == 31) sums[c] = inc;
    }
}

// Block-level exclusive scan of SCAN_TILE doubles, writing tile totals.
__global__ void k_scan_tiles(double* __restrict__ data, uint64_t n, double* __restrict__ tile_sums) {
    __shared__ double sh[SCAN_TILE];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    const int t = threadIdx.x;  // SCAN_TILE threads
    const double x = (base + t < n) ? data[base + t] : 0.0;
    sh[t] = x;
    __syncthreads();
    // Hillis-Steele inclusive scan (fixed order)
    for (int d = 1; d < SCAN_TILE; d <<= 1) {
        const double o = (t >= d) ? sh[t - d] : 0.0;
        __syncthreads();
        if (t >= d) sh[t] = __dadd_rn(sh[t], o);
        __syncthreads();
    }
    if (base + t < n) data[base + t] = (t == 0) ? 0.0 : sh[t - 1];
    if (t == SCAN_TILE - 1 && tile_sums) tile_sums[blockIdx.x] = sh[t];
}

__global__ void k_scan_add(double* __restrict__ data, uint64_t n, const double* __restrict__ offs) {
    const uint64_t i = (uint64_t)blockIdx.x * SCAN_TILE + threadIdx.x;
    if (i < n) data[i] = __dadd_rn(data[i], offs[blockIdx.x]);
}

// Exclusive scan of data[0..n) in place; tmp must hold scan_tmp_len(n) doubles. Writes the
// grand total to *total (device).
static size_t scan_tmp_len(uint64_t n) {
    size_t len = 0;
    while (n > 1) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        len += n + 1;
    }
    return len + 2;
}

static int scan_exclusive(qgpu_handle* h, double* data, uint64_t n, double* tmp, double* total) {
    const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    double* ts = tmp;
    k_scan_tiles<<<(unsigned)tiles, SCAN_TILE, 0, h->stream>>>(data, n, ts);
    QGPU_CHECK_LAUNCH("k_scan_tiles");
    h->launches++;
    if (tiles == 1) {
        QGPU_CUDA(cudaMemcpyAsync(total, ts, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
        return QGPU_OK;
    }
    int st = scan_exclusive(h, ts, tiles, tmp + tiles + 1, total);
    if (st != QGPU_OK) return st;
    k_scan_add<<<(unsigned)tiles, SCAN_TILE, 0, h->stream>>>(data, n, ts);
    QGPU_CHECK_LAUNCH("k_scan_add");
    h->launches++;
    return QGPU_OK;
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// e_k = -log(v_k), v_k in (0, 1], counter-based from (seed, k)
__global__ void k_exponentials(double* __restrict__ e, uint64_t count, uint64_t seed) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t x = splitmix64(seed ^ splitmix64(i + 0x5851F42D4C957F2Dull));
    const double v = 1.0 - (double)(x >> 11) * 0x1.0p-53;  // (0, 1]
    e[i] = -log(v);
}

// After the exclusive scan, e holds S_{k-1}; u_k = (S_{k-1} + e_k) / S_N. The scan is exclusive,
// so the inclusive value is recomputed from the saved exponentials.
__global__ void k_normalise(const double* __restrict__ ex_scan, const double* __restrict__ e,
                            uint64_t count, const double* __restrict__ total, double* __restrict__ u) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    u[i] = __ddiv_rn(__dadd_rn(ex_scan[i], e[i]), *total);
}

template <class S>
__global__ void k_sample(const S* __restrict__ st, uint64_t dim, const double* __restrict__ offs,
                         const double* __restrict__ sums, uint64_t nchunks, int chunk_len,
                         const double* __restrict__ u, uint64_t nshots, int64_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const int per_lane = chunk_len >> 5 ? chunk_len >> 5 : 1;
    for (uint64_t s = warp; s < nshots; s += nwarps) {
        const double x = u[s];
        // first chunk c with x < offs[c] + sums[c]
        uint64_t lo = 0, hi = nchunks;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (x < __dadd_rn(offs[mid], sums[mid])) hi = mid;
            else lo = mid + 1;
        }
        if (lo == nchunks) {
            if (lane == 0) out[s] = -1;  // `measure` returns None: u reached the total
            continue;
        }
        const uint64_t c = lo;
        const uint64_t first = c * (uint64_t)chunk_len + (uint64_t)lane * per_lane;
        const bool active = lane * per_lane < chunk_len;
        const double ls = active ? lane_run_sum(st, first, per_lane) : 0.0;
        const double inc = warp_incl_scan(ls);
        const double start = __dadd_rn(offs[c], inc - ls);  // lane's exclusive offset
        const double excl = __shfl_up_sync(0xffffffffu, inc, 1);
        const double lane_start = __dadd_rn(offs[c], lane == 0 ? 0.0 : excl);
        (void)start;
        const double lane_end = __dadd_rn(offs[c], inc);
        const unsigned hit = __ballot_sync(0xffffffffu, active && x < lane_end);
        int64_t result;
        if (hit) {
            const int L = __ffs(hit) - 1;
            // lane L walks its run sequentially
            int64_t idx = -1;
            if (lane == L) {
                double cum = lane_start;
                const uint64_t f = c * (uint64_t)chunk_len + (uint64_t)L * per_lane;
                int64_t last_nz = (int64_t)f + per_lane - 1;
                for (int q = 0; q < per_lane; ++q) {
                    const double p = prob(st, f + q);
                    cum = __dadd_rn(cum, p);
                    if (x < cum) { idx = (int64_t)(f + q); break; }
                    if (p > 0.0) last_nz = (int64_t)(f + q);
                }
                if (idx < 0) idx = last_nz;  // rounding edge between the two sum orders
            }
            result = __shfl_sync(0xffffffffu, idx, L);
        } else {
            // x lies below the chunk's end by the chunk-sum ordering but above every lane end
            // by the lane ordering (last-bit disagreement): take the chunk's last index.
            result = (int64_t)((c + 1) * (uint64_t)chunk_len - 1);
        }
        if (lane == 0) out[s] = result;
    }
}

// Shared front half: chunk sums + offsets in h->work. Returns pointers into the scratch.
struct Cdf {
    double* sums;
    double* offs;
    double* total;
    uint64_t nchunks;
    int chunk_len;
    size_t used;
};

static int build_cdf(qgpu_handle* h, size_t extra_doubles, Cdf* c) {
    const int cb = h->n_qubits < CHUNK_BITS ? h->n_qubits : CHUNK_BITS;
    c->chunk_len = 1 << cb;
    c->nchunks = h->dim >> cb;
    const size_t tmp = scan_tmp_len(c->nchunks);
    const size_t need = (2 * c->nchunks + tmp + 2 + extra_doubles) * sizeof(double) + 1024;
    int st = h->work.ensure(need);
    if (st != QGPU_OK) return st;
    double* w = (double*)h->work.ptr;
    c->sums = w;
    c->offs = w + c->nchunks;
    c->total = w + 2 * c->nchunks;
    double* scan_tmp = c->total + 2;
    c->used = 2 * c->nchunks + 2 + tmp;
    const int threads = 256;
    uint64_t blocks = (c->nchunks * 32 + threads - 1) / threads;
    if (blocks > (uint64_t)h->sm_count * 16) blocks = (uint64_t)h->sm_count * 16;
    if (h->precision == QGPU_C128)
        k_chunk_sums<double2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const double2*)h->state, c->nchunks, c->chunk_len, c->sums);
    else
        k_chunk_sums<float2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const float2*)h->state, c->nchunks, c->chunk_len, c->sums);
    QGPU_CHECK_LAUNCH("k_chunk_sums");
    h->launches++;
    QGPU_CUDA(cudaMemcpyAsync(c->offs, c->sums, c->nchunks * sizeof(double),
                              cudaMemcpyDeviceToDevice, h->stream));
    return scan_exclusive(h, c->offs, c->nchunks, scan_tmp, c->total);
}

static int run_sample(qgpu_handle* h, const Cdf& c, const double* u, uint64_t n, int64_t* out) {
    const int threads = 256;
    uint64_t blocks = (n * 32 + threads - 1) / threads;
    if (blocks > (uint64_t)h->sm_count * 32) blocks = (uint64_t)h->sm_count * 32;
    if (blocks < 1) blocks = 1;
    if (h->precision == QGPU_C128)
        k_sample<double2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const double2*)h->state, h->dim, c.offs, c.sums, c.nchunks, c.chunk_len, u, n, out);
    else
        k_sample<float2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const float2*)h->state, h->dim, c.offs, c.sums, c.nchunks, c.chunk_len, u, n, out);
    QGPU_CHECK_LAUNCH("k_sample");
    h->launches++;
    return QGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Sparse extraction (`SuperPosition::to_hash_map`, super_positions.rs:315-323): amplitudes whose
// |a|^2 is not within `margin` of zero, in increasing index order. Per 512-amplitude chunk:
// count (k_nz_count), exclusive scan of the counts (scan_exclusive), then each chunk writes its
// survivors at its offset with a warp ballot + popcount order (k_nz_write).
// ---------------------------------------------------------------------------------------------
template <class S>
__global__ void k_nz_count(const S* __restrict__ st, uint64_t nchunks, int chunk_len, double margin,
                           double* __restrict__ counts) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t c = warp; c < nchunks; c += nwarps) {
        unsigned cnt = 0;
        for (int q = lane; q < chunk_len; q += 32) {
            const double p = prob(st, c * (uint64_t)chunk_len + q);
            cnt += !(p > -margin && p < margin);
        }
        for (int d = 16; d > 0; d >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, d);
        if (lane == 0) counts[c] = (double)cnt;
    }
}

template <class S>
__global__ void k_nz_write(const S* __restrict__ st, uint64_t nchunks, int chunk_len, double margin,
                           const double* __restrict__ offs, uint64_t cap,
                           uint64_t* __restrict__ idx, double2* __restrict__ amp) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t c = warp; c < nchunks; c += nwarps) {
        uint64_t at = (uint64_t)offs[c];
        for (int q0 = 0; q0 < chunk_len; q0 += 32) {
            const int q = q0 + lane;
            bool keep = false;
            double2 a = make_double2(0, 0);
            const uint64_t i = c * (uint64_t)chunk_len + q;
            if (q < chunk_len) {
                a = make_double2((double)st[i].x, (double)st[i].y);
                const double p = __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y));
                keep = !(p > -margin && p < margin);
            }
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            const uint64_t pos = at + __popc(m & ((1u << lane) - 1u));
            if (keep && pos < cap) {
                idx[pos] = i;
                amp[pos] = a;
            }
            at += __popc(m);
        }
    }
}

}  // namespace qgpu

using namespace qgpu;

extern "C" {

int qgpu_extract_nonzero(qgpu_handle* h, double margin, uint64_t* idx_out, double* amp_out,
                         size_t cap, size_t* count) {
    if (!h || !count || (cap && (!idx_out || !amp_out)))
        return fail(QGPU_ERR_INVALID, "qgpu_extract_nonzero: NULL argument");
    Cdf c;  // chunk geometry and scratch of the sampler; sums hold survivor counts here
    const int cb = h->n_qubits < CHUNK_BITS ? h->n_qubits : CHUNK_BITS;
    c.chunk_len = 1 << cb;
    c.nchunks = h->dim >> cb;
    const size_t tmp = scan_tmp_len(c.nchunks);
    int st = h->work.ensure((c.nchunks + tmp + 4) * sizeof(double) + 256);
    if (st != QGPU_OK) return st;
    double* counts = (double*)h->work.ptr;
    double* total = counts + c.nchunks;
    double* scan_tmp = total + 2;
    const int threads = 256;
    uint64_t blocks = (c.nchunks * 32 + threads - 1) / threads;
    if (blocks > (uint64_t)h->sm_count * 16) blocks = (uint64_t)h->sm_count * 16;
    if (h->precision == QGPU_C128)
        k_nz_count<double2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const double2*)h->state, c.nchunks, c.chunk_len, margin, counts);
    else
        k_nz_count<float2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const float2*)h->state, c.nchunks, c.chunk_len, margin, counts);
    QGPU_CHECK_LAUNCH("k_nz_count");
    h->launches++;
    st = scan_exclusive(h, counts, c.nchunks, scan_tmp, total);  // counts -> offsets (exact:
    if (st != QGPU_OK) return st;                                 // integers below 2^53)
    double tot = 0.0;
    QGPU_CUDA(copy_async(h, &tot, total, sizeof(double), cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    const uint64_t n = (uint64_t)tot;
    *count = (size_t)n;
    const uint64_t keep = n < cap ? n : cap;
    if (keep) {
        st = h->work2.ensure(keep * 24 + 512);
        if (st != QGPU_OK) return st;
        uint64_t* d_idx = (uint64_t*)h->work2.ptr;
        double2* d_amp = (double2*)((uint8_t*)h->work2.ptr + ((keep * 8 + 255) / 256) * 256);
        if (h->precision == QGPU_C128)
            k_nz_write<double2><<<(unsigned)blocks, threads, 0, h->stream>>>(
                (const double2*)h->state, c.nchunks, c.chunk_len, margin, counts, keep, d_idx, d_amp);
        else
            k_nz_write<float2><<<(unsigned)blocks, threads, 0, h->stream>>>(
                (const float2*)h->state, c.nchunks, c.chunk_len, margin, counts, keep, d_idx, d_amp);
        QGPU_CHECK_LAUNCH("k_nz_write");
        h->launches++;
        QGPU_CUDA(copy_async(h, idx_out, d_idx, keep * 8, cudaMemcpyDeviceToHost));
        QGPU_CUDA(copy_async(h, amp_out, d_amp, keep * 16, cudaMemcpyDeviceToHost));
        QGPU_CUDA(cudaStreamSynchronize(h->stream));
    }
    if (n > cap)
        return fail(QGPU_ERR_INVALID, "qgpu_extract_nonzero: " + std::to_string(n) +
                                          " amplitudes survive, cap is " + std::to_string(cap));
    return QGPU_OK;
}

int qgpu_measure_uniforms(qgpu_handle* h, const double* u, size_t n, int64_t* out) {
    if (!h || (n && (!u || !out))) return fail(QGPU_ERR_INVALID, "qgpu_measure_uniforms: NULL argument");
    if (n == 0) return QGPU_OK;
    Cdf c;
    int st = build_cdf(h, 0, &c);
    if (st != QGPU_OK) return st;
    st = h->work2.ensure(n * 16 + 256);
    if (st != QGPU_OK) return st;
    double* du = (double*)h->work2.ptr;
    int64_t* dout = (int64_t*)((uint8_t*)h->work2.ptr + ((n * 8 + 255) / 256) * 256);
    QGPU_CUDA(copy_async(h, du, u, n * sizeof(double), cudaMemcpyHostToDevice));
    st = run_sample(h, c, du, n, dout);
    if (st != QGPU_OK) return st;
    QGPU_CUDA(copy_async(h, out, dout, n * sizeof(int64_t), cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}

int qgpu_measure(qgpu_handle* h, uint64_t shots, uint64_t seed, uint64_t* idx_out,
                 uint64_t* cnt_out, size_t cap, size_t* n_unique, uint64_t* n_failed) {
    if (!h || !n_unique || !n_failed) return fail(QGPU_ERR_INVALID, "qgpu_measure: NULL argument");
    *n_unique = 0;
    *n_failed = 0;
    if (shots == 0) return QGPU_OK;
    if (shots > (1ull << 31))
        return fail(QGPU_ERR_INVALID, "qgpu_measure: at most 2^31 shots per call");
    Cdf c;
    int st = build_cdf(h, 0, &c);
    if (st != QGPU_OK) return st;
    const uint64_t ne = shots + 1;
    const size_t ebytes = ((ne * 8 + 255) / 256) * 256;
    // work2: exponentials | their exclusive scan | uniforms | indices | scan tmp
    const size_t tmp = scan_tmp_len(ne);
    st = h->work2.ensure(3 * ebytes + shots * 8 + 256 + (tmp + 2) * 8);
    if (st != QGPU_OK) return st;
    uint8_t* w = (uint8_t*)h->work2.ptr;
    double* e = (double*)w;
    double* es = (double*)(w + ebytes);
    double* du = (double*)(w + 2 * ebytes);
    int64_t* dout = (int64_t*)(w + 3 * ebytes);
    double* stmp = (double*)(w + 3 * ebytes + ((shots * 8 + 255) / 256) * 256);
    const int threads = 256;
    k_exponentials<<<(unsigned)((ne + threads - 1) / threads), threads, 0, h->stream>>>(e, ne, seed);
    QGPU_CHECK_LAUNCH("k_exponentials");
    h->launches++;
    QGPU_CUDA(cudaMemcpyAsync(es, e, ne * 8, cudaMemcpyDeviceToDevice, h->stream));
    double* total = stmp;
    st = scan_exclusive(h, es, ne, stmp + 2, total);
    if (st != QGPU_OK) return st;
    k_normalise<<<(unsigned)((shots + threads - 1) / threads), threads, 0, h->stream>>>(es, e, shots,
                                                                                      total, du);
    QGPU_CHECK_LAUNCH("k_normalise");
    h->launches++;
    st = run_sample(h, c, du, shots, dout);
    if (st != QGPU_OK) return st;
    std::vector<int64_t> idx(shots);
    QGPU_CUDA(copy_async(h, idx.data(), dout, shots * 8, cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    // indices are non-decreasing (sorted uniforms, monotone search); None (-1) shots come last
    size_t nu = 0;
    uint64_t failed = 0;
    for (uint64_t s = 0; s < shots;) {
        if (idx[s] < 0) {
            ++failed;
            ++s;
            continue;
        }
        uint64_t e2 = s + 1;
        while (e2 < shots && idx[e2] == idx[s]) ++e2;
        if (nu < cap && idx_out && cnt_out) {
            idx_out[nu] = (uint64_t)idx[s];
            cnt_out[nu] = e2 - s;
        }
        ++nu;
        s = e2;
    }
    *n_unique = nu;
    *n_failed = failed;
    if (nu > cap)
        return fail(QGPU_ERR_INVALID, "qgpu_measure: " + std::to_string(nu) +
                                          " distinct outcomes exceed cap " + std::to_string(cap));
    return QGPU_OK;
}

}  // extern "C"

// =============================================================================================
// Allocation-free sampler: qgpu_measure_uniforms_noalloc
//
// Some callers cannot let this library allocate device memory: a host framework that already
// owns all of the GPU's memory through its own caching pool, or a latency-critical loop that
// must not enter the CUDA allocator. For them the uniform sampler has a variant whose scratch
// (chunk sums, chunk offsets, scan workspace, uniform and index staging) lives in the
// file-scope array below instead of the handle's cudaMalloc'ed buffers. The array is part of
// this library's device image: every GPU that loads the library holds its
// NOALLOC_SCRATCH_BYTES until the process exits.
// =============================================================================================
namespace qgpu {

constexpr int NOALLOC_MAX_QUBITS = 24;            // register size served (2^15 chunks)
constexpr uint64_t NOALLOC_MAX_UNIFORMS = 65536;  // uniforms per call
constexpr uint64_t NOALLOC_MAX_CHUNKS = 1ull << (NOALLOC_MAX_QUBITS - CHUNK_BITS);
constexpr size_t NOALLOC_SCAN_DOUBLES = 64;       // >= scan_tmp_len(NOALLOC_MAX_CHUNKS)
constexpr size_t NOALLOC_SCRATCH_BYTES =
    (2 * NOALLOC_MAX_CHUNKS + 2 + NOALLOC_SCAN_DOUBLES) * sizeof(double) +
    NOALLOC_MAX_UNIFORMS * (sizeof(double) + sizeof(int64_t));

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch. In host code the array's name is only a host-side
// stand-in, so the address is looked up with the device current. A device's address belongs to
// the CUDA context the library's module was loaded into: after a cudaDeviceReset (or any
// teardown of the primary context) the next context loads the module again, possibly at another
// address. So the cache is keyed on the device AND the current context's unique ID
// (cuCtxGetId, fetched through the runtime's driver entry point so the library does not link
// libcuda); a new context repeats the lookup. The lookup allocates nothing.
constexpr int NOALLOC_MAX_DEVICES = 64;
struct NoallocSlot {
    unsigned long long ctx_id = 0;  // 0: not looked up yet (context IDs start above 0)
    void* ptr = nullptr;
};
static NoallocSlot g_noalloc_slot[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mutex;

using CtxGetCurrentFn = CUresult(CUDAAPI*)(CUcontext*);
using CtxGetIdFn = CUresult(CUDAAPI*)(CUcontext, unsigned long long*);

// ID of the context current on the calling thread (the device's primary context unless the
// caller made another one current).
static int current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        QGPU_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1));
        QGPU_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return fail(QGPU_ERR_UNSUPPORTED,
                        "qgpu_measure_uniforms_noalloc: driver has no cuCtxGetCurrent/cuCtxGetId");
        get_current = (CtxGetCurrentFn)f1;
        get_id = (CtxGetIdFn)f2;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx)
        return fail(QGPU_ERR_CUDA, "qgpu_measure_uniforms_noalloc: no current CUDA context");
    if (get_id(ctx, id) != CUDA_SUCCESS)
        return fail(QGPU_ERR_CUDA, "qgpu_measure_uniforms_noalloc: cuCtxGetId failed");
    return QGPU_OK;
}

static int noalloc_scratch(int device, unsigned char** out) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return fail(QGPU_ERR_UNSUPPORTED, "qgpu_measure_uniforms_noalloc: device index " +
                                              std::to_string(device) + " out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    int cur = 0;
    QGPU_CUDA(cudaGetDevice(&cur));
    if (cur != device) QGPU_CUDA(cudaSetDevice(device));
    // The handle's creation initialised the device's context, so the query below finds it.
    unsigned long long id = 0;
    int st = current_context_id(&id);
    void* p = nullptr;
    if (st == QGPU_OK) {
        NoallocSlot& slot = g_noalloc_slot[device];
        if (slot.ptr && slot.ctx_id == id) {
            p = slot.ptr;
        } else {
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                st = cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            } else {
                slot.ctx_id = id;
                slot.ptr = p;
            }
        }
    }
    if (cur != device) cudaSetDevice(cur);
    if (st != QGPU_OK) return st;
    *out = (unsigned char*)p;
    return QGPU_OK;
}

}  // namespace qgpu

extern "C" int qgpu_measure_uniforms_noalloc(qgpu_handle* h, const double* u, size_t n,
                                             int64_t* out) {
    if (!h || (n && (!u || !out)))
        return fail(QGPU_ERR_INVALID, "qgpu_measure_uniforms_noalloc: NULL argument");
    if (h->n_qubits > NOALLOC_MAX_QUBITS)
        return fail(QGPU_ERR_INVALID, "qgpu_measure_uniforms_noalloc: the register has " +
                                          std::to_string(h->n_qubits) + " qubits; at most " +
                                          std::to_string(NOALLOC_MAX_QUBITS) + " are supported");
    if (n > NOALLOC_MAX_UNIFORMS)
        return fail(QGPU_ERR_INVALID, "qgpu_measure_uniforms_noalloc: " + std::to_string(n) +
                                          " uniforms requested; at most " +
                                          std::to_string(NOALLOC_MAX_UNIFORMS) + " per call");
    if (n == 0) return QGPU_OK;
    unsigned char* base = nullptr;
    int st = noalloc_scratch(h->device, &base);
    if (st != QGPU_OK) return st;
    // Layout of the shared array. Every word this call reads is written earlier in the same
    // call (sums, offsets, scan tiles, staged uniforms), so nothing needs clearing between calls.
    Cdf c;
    const int cb = h->n_qubits < CHUNK_BITS ? h->n_qubits : CHUNK_BITS;
    c.chunk_len = 1 << cb;
    c.nchunks = h->dim >> cb;
    if (scan_tmp_len(c.nchunks) > NOALLOC_SCAN_DOUBLES)
        return fail(QGPU_ERR_INVALID, "qgpu_measure_uniforms_noalloc: scan workspace too small");
    double* w = (double*)base;
    c.sums = w;
    c.offs = w + NOALLOC_MAX_CHUNKS;
    c.total = w + 2 * NOALLOC_MAX_CHUNKS;
    double* scan_tmp = c.total + 2;
    double* du = scan_tmp + NOALLOC_SCAN_DOUBLES;
    int64_t* dout = (int64_t*)(du + NOALLOC_MAX_UNIFORMS);
    const int threads = 256;
    uint64_t blocks = (c.nchunks * 32 + threads - 1) / threads;
    if (blocks > (uint64_t)h->sm_count * 16) blocks = (uint64_t)h->sm_count * 16;
    if (h->precision == QGPU_C128)
        k_chunk_sums<double2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const double2*)h->state, c.nchunks, c.chunk_len, c.sums);
    else
        k_chunk_sums<float2><<<(unsigned)blocks, threads, 0, h->stream>>>(
            (const float2*)h->state, c.nchunks, c.chunk_len, c.sums);
    QGPU_CHECK_LAUNCH("k_chunk_sums");
    h->launches++;
    QGPU_CUDA(cudaMemcpyAsync(c.offs, c.sums, c.nchunks * sizeof(double), cudaMemcpyDeviceToDevice,
                              h->stream));
    st = scan_exclusive(h, c.offs, c.nchunks, scan_tmp, c.total);
    if (st != QGPU_OK) return st;
    QGPU_CUDA(copy_async(h, du, u, n * sizeof(double), cudaMemcpyHostToDevice));
    st = run_sample(h, c, du, n, dout);
    if (st != QGPU_OK) return st;
    QGPU_CUDA(copy_async(h, out, dout, n * sizeof(int64_t), cudaMemcpyDeviceToHost));
    QGPU_CUDA(cudaStreamSynchronize(h->stream));
    return QGPU_OK;
}
