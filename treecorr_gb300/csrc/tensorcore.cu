// tensorcore.cu -- a self-check of the tcgen05 building blocks (tc_mma.cuh): one CTA
// computes C[128 x N] = A[128 x K] * B[N x K]^T through TMEM.  It backs a test of the
// descriptors, the instruction descriptor and the accumulator layout before they are used
// by the multipole contraction.
#include <cstdint>
#include <cstring>

#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "tc_mma.cuh"

namespace tc {

// K <= 64, N in {16, 32, 48, 64}; 128 threads.
__global__ void __launch_bounds__(128) k_tcgen05_selftest(const float* A, const float* B,
                                                          float* C, int N, int K, int* status)
{
    extern __shared__ __align__(1024) unsigned char tsm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t taddr_sh;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nsteps = K / 8;
    unsigned char* sA = tsm;                               // nsteps x 4096 B
    unsigned char* sB = tsm + (size_t)nsteps * 4096;       // nsteps x N*32 B
    for (int idx = tid; idx < 128 * K; idx += 128) {
        const int r = idx / K, k = idx % K;
        *reinterpret_cast<float*>(sA + (k >> 3) * 4096 + umma_tile_off(r, k & 7)) = A[idx];
    }
    for (int idx = tid; idx < N * K; idx += 128) {
        const int r = idx / K, k = idx % K;
        *reinterpret_cast<float*>(sB + (k >> 3) * (N * 32) + umma_tile_off(r, k & 7)) = B[idx];
    }
    if (tid == 0) mbar_init(&mbar, 1);
    fence_async_smem();
    __syncthreads();
    if (wid == 0) tmem_alloc(&taddr_sh, 64);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = taddr_sh;
    if (tid == 0) {
        const uint32_t idesc = umma_idesc_tf32(128, N);
        for (int s = 0; s < nsteps; ++s) {
            const uint64_t ad = umma_desc(smem_u32(sA + s * 4096), 128, 256);
            const uint64_t bd = umma_desc(smem_u32(sB + s * N * 32), 128, 256);
            umma_tf32(taddr, ad, bd, idesc, s > 0 ? 1u : 0u);
        }
        umma_commit(&mbar);
    }
    const bool ok = mbar_wait(&mbar, 0, 1 << 22);
    tc_fence_after();
    if (ok) {
        const int row = 32 * wid + lane;
        for (int c0 = 0; c0 < N; c0 += 8) {
            float v[8];
            tmem_ld8(taddr + ((uint32_t)(32 * wid) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int q = 0; q < 8; ++q) C[row * N + c0 + q] = v[q];
        }
    } else if (tid == 0) {
        *status = 1;
    }
    tc_fence_before();
    __syncthreads();
    if (wid == 0) tmem_dealloc(taddr, 64);
}

int tcgen05_selftest(const float* A, const float* B, float* C, int N, int K, cudaStream_t st)
{
    if (K < 8 || K > 64 || (K & 7) || N < 16 || N > 64 || (N & 15)) {
        set_last_error("selftest shape: K in 8..64 (multiple of 8), N in 16..64 (multiple of 16)");
        return 1;
    }
    float *dA = nullptr, *dB = nullptr, *dC = nullptr;
    int* dst = nullptr;
    int rc = 0;
    do {
        if ((rc = dalloc(&dA, (size_t)128 * K))) break;
        if ((rc = dalloc(&dB, (size_t)N * K))) break;
        if ((rc = dalloc(&dC, (size_t)128 * N))) break;
        if ((rc = dalloc(&dst, 1))) break;
        cudaMemcpyAsync(dA, A, sizeof(float) * 128 * K, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dB, B, sizeof(float) * N * K, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(dst, 0, sizeof(int), st);
        const size_t sm = (size_t)(K / 8) * (4096 + N * 32);
        if (cudaFuncSetAttribute(k_tcgen05_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 64 * 1024) != cudaSuccess) {
            set_last_error("selftest attribute failed"); rc = 2; break;
        }
        count_launch();
        k_tcgen05_selftest<<<1, 128, sm, st>>>(dA, dB, dC, N, K, dst);
        if (cudaGetLastError() != cudaSuccess) { set_last_error("selftest launch failed"); rc = 2; break; }
        int hs = 0;
        cudaMemcpyAsync(C, dC, sizeof(float) * 128 * N, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&hs, dst, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { set_last_error("selftest failed"); rc = 2; break; }
        if (hs) { set_last_error("selftest: the MMA did not complete in time"); rc = 4; }
    } while (0);
    dfree(dA); dfree(dB); dfree(dC); dfree(dst);
    return rc;
}

}  // namespace tc
