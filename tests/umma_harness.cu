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

// The lag-shifted operand form of a 2-D correlation on the tensor cores:
// one CTA computes, for every 8-row group g of the template T (tH x tW,
// tH a multiple of 8), D[(q, p), n] += sum_c T[8g+p][c-(15-q)] S[8g+n][c]
// over c in [0, sWp) with A = T read MN-major through a descriptor whose
// 8-row groups step by one 16-byte column (so the 16 lag shifts cost no
// copies), B = S rows K-major, M = 128, N = 32.  D (128 x 32) is written out
// and the caller sums its diagonals: C[u][v] = sum_p D[(15-v)*8+p][p+u].
__global__ void umma_corr_kernel(const float* T, const float* S, float* D, int tH, int tW, int sH, int sW, int split,
                                 int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int sWp = (sW + 15) / 16 * 16, nC = sWp + 15, sHp = tH + 24, G = tH / 8;
    const size_t ttB = (size_t)G * nC * 16, ssB = (size_t)(sWp / 8) * sHp * 16;
    unsigned char* TTh = smem;
    unsigned char* TTl = TTh + ttB;
    unsigned char* SSh = TTl + ttB;
    unsigned char* SSl = SSh + ssB;
    uint64_t* bar = reinterpret_cast<uint64_t*>(SSl + ssB + 2048);  // slack past the operands
    uint32_t* tbase = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) umma::tmem_alloc(tbase, 32);
    for (int t = tid; t < G * nC * 8; t += blockDim.x) {
        const int p = t & 7, c1 = (t >> 3) % nC, g = (t >> 3) / nC, c = c1 - 15;
        const float x = (c >= 0 && c < tW) ? T[(8 * g + p) * tW + c] : 0.f;
        __nv_bfloat16 h, l;
        umma::split_bf16(x, h, l);
        reinterpret_cast<__nv_bfloat16*>(TTh)[t] = h;
        reinterpret_cast<__nv_bfloat16*>(TTl)[t] = l;
    }
    for (int t = tid; t < (sWp / 8) * sHp * 8; t += blockDim.x) {
        const int e = t & 7, r = (t >> 3) % sHp, cg = (t >> 3) / sHp, c = cg * 8 + e;
        const float x = (r < sH && c < sW) ? S[r * sW + c] : 0.f;
        __nv_bfloat16 h, l;
        umma::split_bf16(x, h, l);
        reinterpret_cast<__nv_bfloat16*>(SSh)[t] = h;
        reinterpret_cast<__nv_bfloat16*>(SSl)[t] = l;
    }
    if (tid == 0) umma::mbar_init(bar, 1);
    umma::fence_smem_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tbase;
    if (tid == 0) {
        const uint32_t idesc = umma::idesc_bf16(128, 32) | umma::kIdescAMnMajor;
        bool first = true;
        for (int g = 0; g < G; ++g)
            for (int c0 = 0; c0 < sWp; c0 += 16) {
                const uint32_t ao = (uint32_t)(g * nC * 16 + c0 * 16);
                const uint32_t bo = (uint32_t)((c0 / 8) * sHp * 16 + 8 * g * 16);
                const uint64_t ah = umma::make_desc(umma::smem_addr(TTh) + ao, 128, 16);
                const uint64_t bh = umma::make_desc(umma::smem_addr(SSh) + bo, sHp * 16, 128);
                umma::mma_bf16(tmem, ah, bh, idesc, !first);
                first = false;
                if (split) {
                    const uint64_t al = umma::make_desc(umma::smem_addr(TTl) + ao, 128, 16);
                    const uint64_t bl = umma::make_desc(umma::smem_addr(SSl) + bo, sHp * 16, 128);
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
        for (int c0 = 0; c0 < 32; c0 += 16) {
            float v[16];
            umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
            for (int i = 0; i < 16; ++i) D[row * 32 + c0 + i] = v[i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tmem, 32);
}

extern "C" int umma_corr_test(const float* hT, const float* hS, float* hD, int tH, int tW, int split) {
    if (tH % 8 || tH <= 0 || tH > 64 || tW <= 0 || tW > 96) return -1;
    const int sH = tH + 16, sW = tW + 16;
    const int sWp = (sW + 15) / 16 * 16, nC = sWp + 15, sHp = tH + 24;
    const size_t sm = 2 * ((size_t)(tH / 8) * nC * 16 + (size_t)(sWp / 8) * sHp * 16) + 2048 + 64;
    float *T, *S, *D;
    int* err;
    if (cudaMalloc(&T, sizeof(float) * tH * tW) || cudaMalloc(&S, sizeof(float) * sH * sW) ||
        cudaMalloc(&D, sizeof(float) * 128 * 32) || cudaMalloc(&err, sizeof(int)))
        return -2;
    cudaMemcpy(T, hT, sizeof(float) * tH * tW, cudaMemcpyHostToDevice);
    cudaMemcpy(S, hS, sizeof(float) * sH * sW, cudaMemcpyHostToDevice);
    cudaMemset(D, 0, sizeof(float) * 128 * 32);
    cudaMemset(err, 0, sizeof(int));
    cudaFuncSetAttribute(umma_corr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    umma_corr_kernel<<<1, 128, sm>>>(T, S, D, tH, tW, sH, sW, split, err);
    cudaError_t e = cudaDeviceSynchronize();
    int herr = 0;
    cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(hD, D, sizeof(float) * 128 * 32, cudaMemcpyDeviceToHost);
    cudaFree(T); cudaFree(S); cudaFree(D); cudaFree(err);
    if (e != cudaSuccess) return 100 + (int)e;
    return herr ? -3 : 0;
}

// Issue rate of tcgen05.mma (kind::f16, bf16, M = 128, K = 16): one thread
// issues `n` MMAs back to back over zero operands in shared memory (A
// K-major, or MN-major with the 16-byte M-group stride of the correlation),
// rotating over `nacc` accumulators of N columns; returns the cycles from
// the first issue to the last issue and to completion.
__global__ void umma_rate_kernel(int N, int mode, int n, int nacc, long long* out, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int kOps = 128 * 1024;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kOps);
    uint32_t* tb = reinterpret_cast<uint32_t*>(bar + 1);
    for (int i = threadIdx.x; i < kOps / 16; i += blockDim.x) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
    if (threadIdx.x < 32) umma::tmem_alloc(tb, 512);
    if (threadIdx.x == 0) {
        umma::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    umma::fence_smem_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tb;
    if (threadIdx.x == 0) {
        const uint32_t a = umma::smem_addr(smem), b = a + kOps / 2;
        uint32_t idesc = umma::idesc_bf16(128, N);
        const uint64_t bd = umma::make_desc(b, 128 * (N / 8), 128);  // B K-major, N rows
        uint64_t ad;
        if (mode == 0) {
            ad = umma::make_desc(a, 128, 128 * 16);  // A K-major, 128 rows
        } else {
            ad = umma::make_desc(a, 128, 16);  // A MN-major, M groups 16 bytes apart
            idesc |= umma::kIdescAMnMajor;
        }
        const long long t0 = clock64();
        for (int i = 0; i < n; ++i)
            umma::mma_bf16(tmem + (uint32_t)((i % nacc) * N), ad + (uint64_t)((i & 7) * 16),
                           bd + (uint64_t)((i & 7) * 2), idesc, i >= nacc);
        const long long t1 = clock64();
        umma::commit(bar);
        const bool ok = umma::mbar_wait(bar, 0);
        const long long t2 = clock64();
        out[0] = t1 - t0;
        out[1] = t2 - t0;
        if (!ok) atomicExch(err, 1);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) umma::tmem_free(tmem, 512);
}

extern "C" int umma_rate_test(int N, int mode, int n, int nacc, long long* cycles) {
    if (N % 16 || N < 16 || N > 256 || nacc < 1 || nacc * N > 512 || n < 1 || (mode != 0 && mode != 1)) return -1;
    long long* d;
    int* err;
    if (cudaMalloc(&d, 2 * sizeof(long long)) || cudaMalloc(&err, sizeof(int))) return -2;
    cudaMemset(err, 0, sizeof(int));
    const size_t sm = 128 * 1024 + 64;
    cudaFuncSetAttribute(umma_rate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    umma_rate_kernel<<<1, 128, sm>>>(N, mode, n, nacc, d, err);
    cudaError_t e = cudaDeviceSynchronize();
    int herr = 0;
    cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(cycles, d, 2 * sizeof(long long), cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaFree(err);
    if (e != cudaSuccess) return 100 + (int)e;
    return herr ? -3 : 0;
}

// The same MMAs issued by `per_sm` CTAs on every SM at once (64 KB of
// shared memory each, so several fit): `ms` gets the kernel time of `n`
// MMAs (M = 128, N = 32, K = 16, A MN-major as in the correlation) per CTA.
__global__ void umma_conc_kernel(int n, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 60 * 1024);
    uint32_t* tb = reinterpret_cast<uint32_t*>(bar + 1);
    for (int i = threadIdx.x; i < 60 * 1024 / 16; i += blockDim.x) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
    if (threadIdx.x < 32) umma::tmem_alloc(tb, 32);
    if (threadIdx.x == 0) {
        umma::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    umma::fence_smem_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tb;
    if (threadIdx.x == 0) {
        const uint32_t a = umma::smem_addr(smem), b = a + 32 * 1024;
        const uint32_t idesc = umma::idesc_bf16(128, 32) | umma::kIdescAMnMajor;
        const uint64_t ad = umma::make_desc(a, 128, 16), bd = umma::make_desc(b, 128 * 4, 128);
        for (int i = 0; i < n; ++i)
            umma::mma_bf16(tmem, ad + (uint64_t)((i & 7) * 16), bd + (uint64_t)((i & 7) * 2), idesc, i > 0);
        umma::commit(bar);
        if (!umma::mbar_wait(bar, 0)) atomicExch(err, 1);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) umma::tmem_free(tmem, 32);
}

extern "C" int umma_conc_test(int per_sm, int n, float* ms) {
    if (per_sm < 1 || per_sm > 3 || n < 1) return -1;
    int sms = 0, *err;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    if (cudaMalloc(&err, sizeof(int))) return -2;
    cudaMemset(err, 0, sizeof(int));
    cudaFuncSetAttribute(umma_conc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    umma_conc_kernel<<<sms * per_sm, 128, 64 * 1024>>>(n, err);  // warm-up
    cudaEventRecord(e0);
    umma_conc_kernel<<<sms * per_sm, 128, 64 * 1024>>>(n, err);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    int herr = 0;
    cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(err);
    if (e != cudaSuccess) return 100 + (int)e;
    return herr ? -3 : 0;
}
