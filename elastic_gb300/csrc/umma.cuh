// Fifth-generation tensor-core (tcgen05) building blocks for sm_103a:
// descriptor encoders (host and device), tensor-memory allocation, the MMA
// issue, its commit to an mbarrier, and accumulator loads.
//
// Instruction descriptor, .kind::f16 (32 bits; PTX ISA, tcgen05 instruction
// descriptor table):
//   [0,2) sparsity selector   [2] sparsity   [3] saturate
//   [4,6) D type: 0 F16, 1 F32               [6] reserved
//   [7,10) A type: 0 F16, 1 BF16             [10,13) B type
//   [13] negate A   [14] negate B
//   [15] A major: 0 K-major, 1 M-major       [16] B major: 0 K-major, 1 N-major
//   [17,23) N >> 3   [23] reserved   [24,29) M >> 4   [29] reserved
//   [30,32) maximum shift (.ws only)
// Shared-memory matrix descriptor (64 bits):
//   [0,14) start address >> 4 (shared window, 16-byte units)
//   [16,30) leading-dimension byte offset >> 4
//   [32,46) stride-dimension byte offset >> 4
//   [46,48) fixed 0b01   [49,52) base offset   [52] LBO mode (0 relative)
//   [61,64) swizzle: 0 none, 1 128B with 32B atoms, 2 128B, 4 64B, 6 32B
// Canonical K-major layout without swizzle: the matrix is tiled by core
// matrices of 8 rows x 16 bytes (8 bf16 of K), each stored as 128
// contiguous bytes (row r of the core matrix at byte 16 r); the leading
// offset is the distance between core matrices adjacent along K, the stride
// offset between core matrices adjacent along M (or N).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace eg {

__host__ __device__ constexpr uint32_t umma_idesc_f16(int M, int N, bool ab_bf16, bool d_f32)
{
    return (d_f32 ? 1u : 0u) << 4 | (ab_bf16 ? 1u : 0u) << 7 | (ab_bf16 ? 1u : 0u) << 10 |
           (uint32_t)(N >> 3) << 17 | (uint32_t)(M >> 4) << 24;
}

__host__ __device__ constexpr uint64_t umma_sdesc(uint32_t smem_addr, uint32_t lbo, uint32_t sbo, uint32_t swizzle)
{
    return (uint64_t)((smem_addr & 0x3FFFFu) >> 4) | (uint64_t)((lbo >> 4) & 0x3FFFu) << 16 |
           (uint64_t)((sbo >> 4) & 0x3FFFu) << 32 | (uint64_t)1 << 46 | (uint64_t)(swizzle & 7u) << 61;
}

#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Tensor-memory allocation by one whole warp: the allocated base address is
// written to *dst (shared memory).  ncols: a power of two, 32 .. 512.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Shared-memory writes of the generic proxy (st.shared, cp.async) visible to
// the tensor core's (async proxy) reads.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}
// Arrive once on the mbarrier when every MMA issued so far by this thread
// has completed.
__device__ __forceinline__ void umma_commit(void *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_u32(mbar))
                 : "memory");
}
// 16 consecutive FP32 columns of this thread's tensor-memory lane (a warp
// reads lanes 32 (warp % 4) .. + 31 of the address's lane field).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
#endif

}  // namespace eg
