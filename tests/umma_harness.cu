// Test-only driver of the tcgen05 building blocks (isce2_gb300/csrc/umma.cuh):
// one CTA computes D = A * B^T (A: 128 x K, B: N x K, fp32 in global memory)
// with bf16 operands in shared memory, either one pass (hi*hi) or the 3-pass
// split (hi*hi + hi*lo + lo*hi), and writes D (128 x N) back.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "umma.cuh"

using namespace ampcor;

__global__ void umma_gemm_kernel(const float* A, const float* B, float* D, int N, int K, int split, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int M = 128;
    __nv_bfloat16* Ah = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* Al = Ah + M * K;
    __nv_bfloat16* Bh = Al + M * K;
    __nv_bfloat16* Bl = Bh + N * K;
    uint64_t* bar = reinterpret_cast<uint64_t*>(Bl + N * K);
    uint32_t* tbase = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    uint32_t ncols = 32;
    while ((int)ncols < N) ncols <<= 1;
    if (warp == 0) umma::tmem_alloc(tbase, ncols);
    for (int t = tid; t < M * K; t += blockDim.x) {
        const int r = t / K, k = t - (t / K) * K;
        __nv_bfloat16 h, l;
        umma::split_bf16(A[t], h, l);
        const size_t o = umma::core_offset(r, k, K) / 2;
        Ah[o] = h;
        Al[o] = l;
    }
    for (int t = tid; t < N * K; t += blockDim.x) {
        const int r = t / K, k = t - (t / K) * K;
        __nv_bfloat16 h, l;
        umma::split_bf16(B[t], h, l);
        const size_t o = umma::core_offset(r, k, K) / 2;
        Bh[o] = h;
        Bl[o] = l;
    }
    if (tid == 0) umma::mbar_init(bar, 1);
    umma::fence_smem_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tbase;
    if (tid == 0) {
        const uint32_t idesc = umma::idesc_bf16(M, N);
        const uint32_t sbo = 16 * K;
        for (int k0 = 0; k0 < K; k0 += 16) {
            const uint32_t koff = (uint32_t)(k0 / 8) * 128;
            const uint64_t ah = umma::make_desc(umma::smem_addr(Ah) + koff, 128, sbo);
            const uint64_t bh = umma::make_desc(umma::smem_addr(Bh) + koff, 128, sbo);
            umma::mma_bf16(tmem, ah, bh, idesc, k0 > 0);
            if (split) {
                const uint64_t al = umma::make_desc(umma::smem_addr(Al) + koff, 128, sbo);
                const uint64_t bl = umma::make_desc(umma::smem_addr(Bl) + koff, 128, sbo);
                umma::mma_bf16(tmem, ah, bl, idesc, true);
                umma::mma_bf16(tmem, al, bh, idesc, true);
            }
        }
        umma::commit(bar);
    }
    const bool ok = umma::mbar_wait(bar, 0);
    if (!ok && (tid & 31) == 0) atomicExch(err, 1);
    umma::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + (tid & 31);
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
            for (int i = 0; i < 16 && c0 + i < N; ++i) D[row * N + c0 + i] = v[i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, ncols);
}

extern "C" int umma_gemm_test(const float* hA, const float* hB, float* hD, int N, int K, int split) {
    const int M = 128;
    if (N % 16 || N < 16 || N > 256 || K % 16 || K <= 0) return -1;
    float *A, *B, *D;
    int* err;
    if (cudaMalloc(&A, sizeof(float) * M * K) || cudaMalloc(&B, sizeof(float) * N * K) ||
        cudaMalloc(&D, sizeof(float) * M * N) || cudaMalloc(&err, sizeof(int)))
        return -2;
    cudaMemcpy(A, hA, sizeof(float) * M * K, cudaMemcpyHostToDevice);
    cudaMemcpy(B, hB, sizeof(float) * N * K, cudaMemcpyHostToDevice);
    cudaMemset(D, 0, sizeof(float) * M * N);
    cudaMemset(err, 0, sizeof(int));
    const size_t sm = (size_t)2 * (M + N) * K * 2 + 64;
    cudaFuncSetAttribute(umma_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    umma_gemm_kernel<<<1, 128, sm>>>(A, B, D, N, K, split, err);
    cudaError_t e = cudaDeviceSynchronize();
    int herr = 0;
    cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(hD, D, sizeof(float) * M * N, cudaMemcpyDeviceToHost);
    cudaFree(A); cudaFree(B); cudaFree(D); cudaFree(err);
    if (e != cudaSuccess) return 100 + (int)e;
    return herr ? -3 : 0;
}
