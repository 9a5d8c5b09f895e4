// tc_probe.cu — checks the tensor-core helpers of quantr_gb300/csrc/tc.cuh on one CTA: a
// 128 x 128 x 16 TF32 product (two K=8 MMAs, the second accumulating) and a 128 x 128 x 16 BF16
// product (one MMA), operands in the K-major no-swizzle layout, accumulators read back from
// tensor memory. Inputs are small dyadic values, so every product and sum is exact in F32 and
// the result must equal the host product bit for bit. A third case multiplies 8-bit integer
// slices (BF16 holds them exactly) over K = 192 in 12 accumulating MMAs, with sums up to
// 192 x 255 x 255 < 2^24: whether the tensor cores' F32 accumulation is exact on such integers,
// which a fixed-point (Ozaki) splitting of float-pair operands relies on. Exit code 0 when all
// three match.
//
// Every wait is bounded; on a timeout the kernel records it and still frees its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "tc.cuh"

using namespace qgpu;

constexpr int M = 128, N = 128;

template <int MODE>  // 0: TF32 K=16; 1: BF16 K=16; 2: BF16 K=192 (integer slices)
__global__ void __launch_bounds__(128) k_probe(const float* __restrict__ A, const float* __restrict__ Bt,
                                               float* __restrict__ D, int* __restrict__ err) {
    constexpr bool BF16 = MODE != 0;
    constexpr int K = MODE == 2 ? 192 : 16;
    constexpr uint32_t OPB = MODE == 2 ? 49152 : 8192;  // bytes reserved per operand
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;
    uint8_t* sB = sm + OPB;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * OPB);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + 2 * OPB + 64);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int ES = BF16 ? 2 : 4;          // element bytes
    constexpr int T = 16 / ES;                // elements per core-matrix row
    constexpr uint32_t LBO = 128;             // core matrices adjacent along K
    constexpr uint32_t SBO = (K / T) * 128;   // 8-row groups
    for (int e = tid; e < M * K; e += 128) {
        const int r = e / K, k = e % K;
        const uint32_t off = (r % 8) * 16 + (k % T) * ES + (k / T) * LBO + (r / 8) * SBO;
        if (BF16) {
            *reinterpret_cast<__nv_bfloat16*>(sA + off) = __float2bfloat16_rn(A[e]);
            *reinterpret_cast<__nv_bfloat16*>(sB + off) = __float2bfloat16_rn(Bt[e]);
        } else {
            *reinterpret_cast<float*>(sA + off) = A[e];
            *reinterpret_cast<float*>(sB + off) = Bt[e];
        }
    }
    if (tid == 0) {
        mbar_init(smem_u32(bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::alloc(smem_u32(slot), 512);
    fence_proxy_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        if (BF16) {
            const uint32_t id = tc::idesc_bf16(M, N);
            for (int kk = 0; kk < K / 16; ++kk) {  // 16 BF16 elements = 2 core matrices along K
                const uint32_t adv = kk * 2 * LBO;
                tc::mma_bf16(tmem, tc::smem_desc(smem_u32(sA) + adv, LBO, SBO),
                             tc::smem_desc(smem_u32(sB) + adv, LBO, SBO), id, kk > 0);
            }
        } else {
            const uint32_t id = tc::idesc_tf32(M, N);
            for (int kk = 0; kk < K / 8; ++kk) {  // 8 TF32 elements = 32 bytes = 2 core matrices
                const uint32_t adv = kk * 2 * LBO;
                tc::mma_tf32(tmem, tc::smem_desc(smem_u32(sA) + adv, LBO, SBO),
                             tc::smem_desc(smem_u32(sB) + adv, LBO, SBO), id, kk > 0);
            }
        }
        tc::commit(smem_u32(bar));
    }
    const bool ok = mbar_wait_bounded(smem_u32(bar), 0, 1u << 22);
    tc::fence_after_sync();
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
    } else {
        const int row = warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) D[row * N + c0 + i] = v[i];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::dealloc(tmem, 512);
}

template <int MODE>
static int run(const char* name) {
    constexpr int K = MODE == 2 ? 192 : 16;
    std::vector<float> A(M * K), Bt(N * K), D(M * N, -7.0f), ref(M * N, 0.0f);
    if (MODE == 2) {
        // 8-bit slices: unsigned bytes, signed top slices (-128..127), and extreme rows (every
        // product 255 x 255, sums near 12.5 million; alternating signs; sparse rows)
        uint64_t x = 12345;
        auto next = [&]() {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            return z ^ (z >> 31);
        };
        for (int m = 0; m < M; ++m)
            for (int k = 0; k < K; ++k) {
                int v = (int)(next() % 256);
                if (m % 8 == 1) v -= 128;
                if (m == 0) v = 255;
                if (m == 2) v = (k & 1) ? 255 : -128;
                if (m == 3) v = (k % 37 == 0) ? 1 : 0;
                A[m * K + k] = (float)v;
            }
        for (int n = 0; n < N; ++n)
            for (int k = 0; k < K; ++k) {
                int v = (int)(next() % 256);
                if (n % 8 == 5) v -= 128;
                if (n == 0) v = 255;
                Bt[n * K + k] = (float)v;
            }
    } else {
        for (int m = 0; m < M; ++m)
            for (int k = 0; k < K; ++k) A[m * K + k] = (float)((m * 7 + k * 3) % 17 - 8) / 4.0f;
        for (int n = 0; n < N; ++n)
            for (int k = 0; k < K; ++k) Bt[n * K + k] = (float)((n * 5 + k * 11) % 13 - 6) / 2.0f;
    }
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            double s = 0;  // exact: integers below 2^24 / small dyadic values
            for (int k = 0; k < K; ++k) s += (double)A[m * K + k] * Bt[n * K + k];
            ref[m * N + n] = (float)s;
        }
    float *dA, *dB, *dD;
    int* dErr;
    cudaMalloc(&dA, A.size() * 4);
    cudaMalloc(&dB, Bt.size() * 4);
    cudaMalloc(&dD, D.size() * 4);
    cudaMalloc(&dErr, 4);
    cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, Bt.data(), Bt.size() * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dD, D.data(), D.size() * 4, cudaMemcpyHostToDevice);
    cudaMemset(dErr, 0, 4);
    const int smem = MODE == 2 ? 2 * 49152 + 1024 : 64 * 1024;
    cudaFuncSetAttribute(k_probe<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_probe<MODE><<<1, 128, smem>>>(dA, dB, dD, dErr);
    cudaError_t e = cudaDeviceSynchronize();
    int err = 0;
    cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&err, dErr, 4, cudaMemcpyDeviceToHost);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dErr);
    if (e != cudaSuccess) {
        std::printf("FAIL %s: %s\n", name, cudaGetErrorString(e));
        return 1;
    }
    if (err) {
        std::printf("FAIL %s: mbarrier wait timed out\n", name);
        return 1;
    }
    int bad = 0;
    double maxd = 0;
    for (int i = 0; i < M * N; ++i) {
        const double d = std::fabs((double)D[i] - ref[i]);
        if (d > maxd) maxd = d;
        if (D[i] != ref[i] && bad < 5) {
            std::printf("  %s mismatch at (%d, %d): got %g want %g\n", name, i / N, i % N, D[i], ref[i]);
        }
        bad += D[i] != ref[i];
    }
    std::printf("%s %s: %d mismatches, max |diff| %g\n", bad ? "FAIL" : "PASS", name, bad, maxd);
    return bad ? 1 : 0;
}

int main() {
    int rc = run<0>("tf32 128x128x16");
    rc |= run<1>("bf16 128x128x16");
    rc |= run<2>("bf16 integer slices 128x128x192");
    return rc;
}
