// tc_probe.cu — checks the tensor-core helpers of quantr_gb300/csrc/tc.cuh on one CTA: a
// 128 x 128 x 16 TF32 product (two K=8 MMAs, the second accumulating) and a 128 x 128 x 16 BF16
// product (one MMA), operands in the K-major no-swizzle layout, accumulators read back from
// tensor memory. Inputs are small dyadic values, so every product and sum is exact in F32 and
// the result must equal the host product bit for bit. Exit code 0 when both match.
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

constexpr int M = 128, N = 128, K = 16;

template <bool BF16>
__global__ void __launch_bounds__(128) k_probe(const float* __restrict__ A, const float* __restrict__ Bt,
                                               float* __restrict__ D, int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* sA = sm;                 // 8 KB (tf32) / 4 KB (bf16)
    uint8_t* sB = sm + 8192;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 16384);
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + 16384 + 64);
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
            tc::mma_bf16(tmem, tc::smem_desc(smem_u32(sA), LBO, SBO), tc::smem_desc(smem_u32(sB), LBO, SBO),
                         id, 0);
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

template <bool BF16>
static int run(const char* name) {
    std::vector<float> A(M * K), Bt(N * K), D(M * N, -7.0f), ref(M * N, 0.0f);
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k) A[m * K + k] = (float)((m * 7 + k * 3) % 17 - 8) / 4.0f;
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < K; ++k) Bt[n * K + k] = (float)((n * 5 + k * 11) % 13 - 6) / 2.0f;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            double s = 0;
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
    const int smem = 64 * 1024;
    cudaFuncSetAttribute(k_probe<BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_probe<BF16><<<1, 128, smem>>>(dA, dB, dD, dErr);
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
    int rc = run<false>("tf32 128x128x16");
    rc |= run<true>("bf16 128x128x16");
    return rc;
}
