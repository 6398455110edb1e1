// Minimal 5th-generation tensor-core (tcgen05) building blocks for sm_103a:
// tensor-memory allocation, shared-memory matrix descriptors for the
// no-swizzle K-major layout, one-thread MMA issue with an mbarrier commit,
// bounded waits, and accumulator loads.  Used for the dense contractions of
// the oversampler and the oversampled correlation.
//
// Operand layout in shared memory ("core matrix" layout, no swizzle): an
// R x K bf16 operand is stored as 8-row groups; inside a group, core matrices
// of 8 rows x 8 bf16 (16 bytes per row, 128 bytes per core matrix) follow
// each other along K.  Element (r, k) sits at byte
//   (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// with SBO = 16 * K bytes (K padded to a multiple of 16).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ampcor {
namespace umma {

// Bounded mbarrier waits: after this many polls a wait gives up and the
// caller reports an error instead of hanging the GPU.
constexpr uint32_t kMaxPolls = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__host__ __device__ __forceinline__ size_t core_offset(int r, int k, int K) {
    return (size_t)(r >> 3) * (16 * K) + (size_t)(k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, leading (K-direction core
// matrix) byte offset, stride (8-row group) byte offset, descriptor version 1,
// no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor for kind::f16 with bf16 A and B (K-major), f32 D.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4)                       // D format f32
           | (1u << 7)                     // A format bf16
           | (1u << 10)                    // B format bf16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// Instruction-descriptor bits that read A (bit 15) or B (bit 16) MN-major:
// the 8 rows of a core matrix are then 8 consecutive K indices (16 bytes
// each) holding 8 consecutive M (N) elements, the descriptor's stride byte
// offset steps between 8-element M (N) groups and its leading byte offset
// between 8-row K groups.
constexpr uint32_t kIdescAMnMajor = 1u << 15;
constexpr uint32_t kIdescBMnMajor = 1u << 16;

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

// Waits for the phase with parity `parity` to complete; false after `polls`
// polls (kMaxPolls in the kernels).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t polls = kMaxPolls) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// The same wait with a suspend-time hint: a thread whose phase is not yet
// complete sleeps up to `hint_ns` per poll instead of spinning, so waiting
// warps leave the issue slots to the working ones.  Bounded by `polls`.
constexpr uint32_t kSleepPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t hint_ns = 1000,
                                                uint32_t polls = kSleepPolls) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t i = 0; i < polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(hint_ns)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Allocate `ncols` (power of two >= 32) TMEM columns; whole warp calls.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the tensor core
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A * B^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate));
}

// Arrive on `bar` once all previously issued MMAs of this thread complete.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_addr(bar)));
}

// 32 lanes x 16 consecutive 32-bit columns: thread i of the warp gets lane
// (base lane + i), columns col .. col+15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Split x into bf16 hi + lo with hi + lo == x to about 16 significant bits.
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

}  // namespace umma
}  // namespace ampcor

namespace ampcor {
namespace tma {

// Tensor-memory-access bulk copies (cp.async.bulk.tensor) into shared memory,
// completing on an mbarrier with a transaction count.
__device__ __forceinline__ void arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(umma::smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// 3-D tiled load of one box at coordinates (x, y, z) of the tensor map.
__device__ __forceinline__ void load_3d(void* dst, const void* tmap, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(umma::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(umma::smem_addr(bar))
        : "memory");
}

// Contiguous bulk copy global -> shared (non-tensor): both addresses 16-byte
// aligned, size a multiple of 16 bytes.
__device__ __forceinline__ void load_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            umma::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(umma::smem_addr(bar))
        : "memory");
}

// Order this thread's earlier generic-proxy global writes before later
// async-proxy (bulk copy) reads.
__device__ __forceinline__ void fence_global_async() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

}  // namespace tma
}  // namespace ampcor
