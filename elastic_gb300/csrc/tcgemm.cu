// Checks of the tcgen05 building blocks (umma.cuh) used by the learned
// preconditioner's tensor-core GEMMs: the descriptor encoders, exported for a
// CPU test against the PTX ISA field layout, and a one-instruction probe --
// one 128 x N x 16 BF16 MMA with FP32 accumulation in tensor memory -- that
// a GPU test compares with a host matrix product.
#include <cuda_bf16.h>

#include <cstring>

#include "../../include/elastic_rtm.h"
#include "common.cuh"
#include "elastic2d_v2.cuh"
#include "engine.h"
#include "umma.cuh"

using namespace eg;

namespace {

// The probe's operands are stored K-major without swizzle, core matrices
// adjacent along K 128 bytes apart and along M (N) 256 bytes apart.  Every
// descriptor offset the probe accepts (16 .. 256 bytes) keeps every read
// inside the operand arrays, whatever the hardware makes of the fields.
constexpr int PROBE_K = 16;

__global__ void __launch_bounds__(128) k_umma_probe(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D, int N,
                                                     uint32_t lbo, uint32_t sbo, int *status)
{
    __shared__ __align__(1024) __nv_bfloat16 sA[2 * 128 * PROBE_K];  // twice the operand: 8 KB
    __shared__ __align__(1024) __nv_bfloat16 sB[2 * 256 * PROBE_K];  // 16 KB
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;
    for (int i = tid; i < 2 * 128 * PROBE_K; i += 128) sA[i] = __float2bfloat16(0.f);
    for (int i = tid; i < 2 * 256 * PROBE_K; i += 128) sB[i] = __float2bfloat16(0.f);
    __syncthreads();
    auto place = [](int r, int k) { return (r >> 3) * 128 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7); };  // in bf16
    for (int i = tid; i < 128 * PROBE_K; i += 128) sA[place(i / PROBE_K, i % PROBE_K)] = A[i];
    for (int i = tid; i < N * PROBE_K; i += 128) sB[place(i / PROBE_K, i % PROBE_K)] = B[i];
    if (warp == 0) tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        mbar_init(&bar);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t d = tbase;
    if (tid == 0) {
        const uint64_t ad = umma_sdesc(smem_u32(sA), lbo, sbo, 0), bd = umma_sdesc(smem_u32(sB), lbo, sbo, 0);
        umma_f16(d, ad, bd, umma_idesc_f16(128, N, true, true), false);
        umma_commit(&bar);
    }
    bool ok = mbar_wait(&bar, 0);
    if (!ok) ok = mbar_wait(&bar, 0);  // the MMA may still be running: give it a second limit
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(d + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) D[(32 * warp + lane) * N + c + j] = v[j];
        }
    } else if (tid == 0) {
        *status = 1;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tmem_dealloc(d, ncols);
        tmem_relinquish();
    }
}

// Swizzled K-major operands, as bulk tensor copies with a 128-byte (64-byte)
// swizzle leave them: rows of 128 (64) bytes, 8-row atoms of 1024 (512)
// bytes, the 16-byte chunk c of row r stored at chunk c ^ (r % 8) (c ^ (r % 8
// / 2)).  The probe places A (128 x K) and B (N x K) that way, K = 64 (32),
// and accumulates K / 16 MMAs whose descriptors advance by 32 bytes along K
// inside the atom -- the form the convolution kernels issue.  Both arrays
// are whole atoms on a 1024-byte boundary, so every address a descriptor
// can form lies inside them.
__device__ __forceinline__ uint32_t swz_off(int r, int k, int row_bytes)
{
    const int rr = r & 7, byte = 2 * k, chunk = byte >> 4;
    const int phys = row_bytes == 128 ? (chunk ^ rr) : (chunk ^ (rr >> 1));
    return (uint32_t)((r >> 3) * 8 * row_bytes + rr * row_bytes + phys * 16 + (byte & 15));
}

__global__ void __launch_bounds__(128) k_umma_probe_sw(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D, int N,
                                                        int K, int *status)
{
    extern __shared__ __align__(16) unsigned char pr_raw[];
    unsigned char *base = pr_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(pr_raw) & 1023u)) & 1023u);
    unsigned char *sA = base, *sB = base + 128 * 128;  // A: up to 16 KB
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(sB + 256 * 128);
    uint32_t *tbase = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rb = 2 * K;  // row bytes: 128 (K = 64) or 64 (K = 32)
    const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;
    for (int i = tid; i < 128 * K; i += 128)
        *reinterpret_cast<__nv_bfloat16 *>(sA + swz_off(i / K, i % K, rb)) = A[i];
    for (int i = tid; i < N * K; i += 128)
        *reinterpret_cast<__nv_bfloat16 *>(sB + swz_off(i / K, i % K, rb)) = B[i];
    if (warp == 0) tmem_alloc(tbase, ncols);
    if (tid == 0) {
        mbar_init(bar);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t d = *tbase;
    if (tid == 0) {
        const uint32_t sw = rb == 128 ? 2u : 4u, sbo = 8u * rb;
        for (int k = 0; k < K / 16; k++) {
            const uint64_t ad = umma_sdesc(smem_u32(sA) + 32 * k, 16, sbo, sw);
            const uint64_t bd = umma_sdesc(smem_u32(sB) + 32 * k, 16, sbo, sw);
            umma_f16(d, ad, bd, umma_idesc_f16(128, N, true, true), k > 0);
        }
        umma_commit(bar);
    }
    bool ok = mbar_wait(bar, 0);
    if (!ok) ok = mbar_wait(bar, 0);
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(d + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) D[(32 * warp + lane) * N + c + j] = v[j];
        }
    } else if (tid == 0) {
        *status = 1;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tmem_dealloc(d, ncols);
        tmem_relinquish();
    }
}
constexpr size_t PROBE_SW_SMEM = 1024 + 128 * 128 + 256 * 128 + 16;

// Layout variants of the second probe (one MMA group, K = 16 x K/16):
//   mode 0: A K-major swizzled as above but stored with `shift` extra rows
//           in front; the descriptor starts `shift` rows in, with the base
//           offset field set to (start >> 7) & 7 (boff = 1) or left 0;
//   mode 1: A and B MN-major (M / N contiguous), 128-byte swizzle: atoms of
//           8 K-rows x 64 MN elements; lbo/sbo as given (bytes); K = 32,
//           N a multiple of 64;
//   mode 2: the same with the 64-byte swizzle (atoms of 8 K-rows x 32 MN
//           elements), N a multiple of 32.
// Both arrays are whole atoms inside their regions; every address a
// descriptor can form lies inside them.
__device__ __forceinline__ uint32_t mn_off(int mn, int k, int row_bytes, int atom_stride_mn, int atom_stride_k)
{
    const int per = row_bytes / 2;  // MN elements per row
    const int am = mn / per, mm = mn % per, ak = k / 8, kr = k & 7;
    const int byte = 2 * mm, chunk = byte >> 4;
    const int phys = row_bytes == 128 ? (chunk ^ kr) : (chunk ^ (kr >> 1));
    return (uint32_t)(am * atom_stride_mn + ak * atom_stride_k + kr * row_bytes + phys * 16 + (byte & 15));
}

__global__ void __launch_bounds__(128) k_umma_probe2(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D, int N,
                                                      int K, int mode, int shift, int boff, uint32_t lbo, uint32_t sbo,
                                                      int *status)
{
    extern __shared__ __align__(16) unsigned char pr_raw[];
    unsigned char *base = pr_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(pr_raw) & 1023u)) & 1023u);
    unsigned char *sA = base, *sB = base + 40960;  // A region 40 KB, B region 32 KB
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(sB + 32768);
    uint32_t *tbase = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // row bytes: K-major (mode 0) 128 (K = 64) or 64 (K = 32); MN-major 128
    // (mode 1) or 64 (mode 2)
    const int rb = mode == 0 ? 2 * K : mode == 1 ? 128 : 64;
    const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;
    for (int i = tid; i < 40960 + 32768; i += 128) base[i] = 0;
    __syncthreads();
    if (mode == 0) {
        for (int i = tid; i < (128 + shift) * K; i += 128)
            *reinterpret_cast<__nv_bfloat16 *>(sA + swz_off(i / K, i % K, rb)) = A[i];
        for (int i = tid; i < N * K; i += 128)
            *reinterpret_cast<__nv_bfloat16 *>(sB + swz_off(i / K, i % K, rb)) = B[i];
    } else {
        // MN-major: row = 8 K-rows atoms, MN contiguous in rows of rb bytes;
        // atoms along MN `lbo` apart, along K `sbo` apart (the assignment
        // under test), so the placement below mirrors the descriptor
        for (int i = tid; i < 128 * K; i += 128)
            *reinterpret_cast<__nv_bfloat16 *>(sA + mn_off(i / K, i % K, rb, (int)lbo, (int)sbo)) = A[i];
        for (int i = tid; i < N * K; i += 128)
            *reinterpret_cast<__nv_bfloat16 *>(sB + mn_off(i / K, i % K, rb, (int)lbo, (int)sbo)) = B[i];
    }
    if (warp == 0) tmem_alloc(tbase, ncols);
    if (tid == 0) {
        mbar_init(bar);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t d = *tbase;
    if (tid == 0) {
        const uint32_t sw = rb == 128 ? 2u : 4u;
        if (mode == 0) {
            const uint32_t a0 = smem_u32(sA) + (uint32_t)(shift * rb), b0 = smem_u32(sB);
            for (int k = 0; k < K / 16; k++) {
                uint64_t ad = umma_sdesc(a0 + 32 * k, 16, 8u * rb, sw);
                if (boff) ad |= (uint64_t)(((a0 + 32 * k) >> 7) & 7u) << 49;
                const uint64_t bd = umma_sdesc(b0 + 32 * k, 16, 8u * rb, sw);
                umma_f16(d, ad, bd, umma_idesc_f16(128, N, true, true), k > 0);
            }
        } else {
            // MN-major operands: transpose bits of the instruction descriptor;
            // K advances by whole 8-row atoms (2 per 16-wide step)
            const uint32_t idesc = umma_idesc_f16(128, N, true, true) | (1u << 15) | (1u << 16);
            for (int k = 0; k < K / 16; k++) {
                const uint64_t ad = umma_sdesc(smem_u32(sA) + 2 * k * sbo, lbo, sbo, sw);
                const uint64_t bd = umma_sdesc(smem_u32(sB) + 2 * k * sbo, lbo, sbo, sw);
                umma_f16(d, ad, bd, idesc, k > 0);
            }
        }
        umma_commit(bar);
    }
    bool ok = mbar_wait(bar, 0);
    if (!ok) ok = mbar_wait(bar, 0);
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(d + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int j = 0; j < 16; j++) D[(32 * warp + lane) * N + c + j] = v[j];
        }
    } else if (tid == 0) {
        *status = 1;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tmem_dealloc(d, ncols);
        tmem_relinquish();
    }
}
constexpr size_t PROBE2_SMEM = 1024 + 40960 + 32768 + 16;

}  // namespace

extern "C" int rtm_debug_umma_probe_sw(int N, int K, const unsigned short *A, const unsigned short *B, float *D)
{
    RTM_CHECK_ARG(N >= 16 && N <= 256 && N % 16 == 0, "N must be a multiple of 16 in 16 .. 256");
    RTM_CHECK_ARG(K == 32 || K == 64, "K must be 32 (64-byte swizzle) or 64 (128-byte swizzle)");
    RTM_CHECK_ARG(A && B && D, "null argument");
    TRY(ensure_device());
    DevBuf<__nv_bfloat16> a, b;
    DevBuf<float> d;
    DevBuf<int> st;
    TRY(a.alloc((size_t)128 * K));
    TRY(b.alloc((size_t)N * K));
    TRY(d.alloc((size_t)128 * N));
    TRY(st.alloc(1));
    RTM_CUDA(cudaMemcpy(a.p, A, (size_t)128 * K * 2, cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(b.p, B, (size_t)N * K * 2, cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemset(d.p, 0, (size_t)128 * N * 4));
    RTM_CUDA(cudaMemset(st.p, 0, 4));
    RTM_CUDA(cudaFuncSetAttribute(k_umma_probe_sw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PROBE_SW_SMEM));
    k_umma_probe_sw<<<1, 128, PROBE_SW_SMEM>>>(a.p, b.p, d.p, N, K, st.p);
    RTM_CUDA(cudaGetLastError());
    RTM_CUDA(cudaDeviceSynchronize());
    int s = 0;
    RTM_CUDA(cudaMemcpy(&s, st.p, 4, cudaMemcpyDeviceToHost));
    RTM_CUDA(cudaMemcpy(D, d.p, (size_t)128 * N * 4, cudaMemcpyDeviceToHost));
    if (s) {
        rtm_set_error("the probe's MMA did not complete within its time limit");
        return RTM_ERR_TIMEOUT;
    }
    return RTM_OK;
}

extern "C" int rtm_debug_umma_probe2(int N, int K, int mode, int shift, int boff, unsigned lbo, unsigned sbo,
                                     const unsigned short *A, const unsigned short *B, float *D)
{
    RTM_CHECK_ARG(mode >= 0 && mode <= 2, "mode must be 0, 1 or 2");
    if (mode == 0) {
        RTM_CHECK_ARG(K == 32 || K == 64, "mode 0: K must be 32 or 64");
        RTM_CHECK_ARG(N >= 16 && N <= 256 && N % 16 == 0, "mode 0: N a multiple of 16 in 16 .. 256");
        RTM_CHECK_ARG(shift >= 0 && shift <= 8, "mode 0: shift 0 .. 8");
    } else if (mode == 1) {
        RTM_CHECK_ARG(K == 32, "mode 1: K must be 32");
        RTM_CHECK_ARG(N == 64 || N == 128, "mode 1: N must be 64 or 128");
        RTM_CHECK_ARG((lbo == 4096 && sbo == 1024) || (lbo == 1024 && sbo == 2048),
                      "mode 1: (lbo, sbo) must be (4096, 1024) or (1024, 2048)");
        shift = 0;
    } else {
        RTM_CHECK_ARG(K == 32, "mode 2: K must be 32");
        RTM_CHECK_ARG(N == 32 || N == 64 || N == 96 || N == 128, "mode 2: N must be 32, 64, 96 or 128");
        RTM_CHECK_ARG((lbo == 2048 && sbo == 512) || (lbo == 512 && sbo == 2048),
                      "mode 2: (lbo, sbo) must be (2048, 512) or (512, 2048)");
        shift = 0;
    }
    RTM_CHECK_ARG(A && B && D, "null argument");
    TRY(ensure_device());
    const int arows = mode == 0 ? 128 + shift : 128;
    DevBuf<__nv_bfloat16> a, b;
    DevBuf<float> d;
    DevBuf<int> st;
    TRY(a.alloc((size_t)arows * K));
    TRY(b.alloc((size_t)N * K));
    TRY(d.alloc((size_t)128 * N));
    TRY(st.alloc(1));
    RTM_CUDA(cudaMemcpy(a.p, A, (size_t)arows * K * 2, cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(b.p, B, (size_t)N * K * 2, cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemset(d.p, 0, (size_t)128 * N * 4));
    RTM_CUDA(cudaMemset(st.p, 0, 4));
    RTM_CUDA(cudaFuncSetAttribute(k_umma_probe2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PROBE2_SMEM));
    k_umma_probe2<<<1, 128, PROBE2_SMEM>>>(a.p, b.p, d.p, N, K, mode, shift, boff, lbo, sbo, st.p);
    RTM_CUDA(cudaGetLastError());
    RTM_CUDA(cudaDeviceSynchronize());
    int s = 0;
    RTM_CUDA(cudaMemcpy(&s, st.p, 4, cudaMemcpyDeviceToHost));
    RTM_CUDA(cudaMemcpy(D, d.p, (size_t)128 * N * 4, cudaMemcpyDeviceToHost));
    if (s) {
        rtm_set_error("the probe's MMA did not complete within its time limit");
        return RTM_ERR_TIMEOUT;
    }
    return RTM_OK;
}

extern "C" int rtm_debug_umma_desc(int M, int N, int bf16, int f32, unsigned addr, unsigned lbo, unsigned sbo,
                                   unsigned swizzle, unsigned long long *out)
{
    RTM_CHECK_ARG(out, "null argument");
    out[0] = umma_idesc_f16(M, N, bf16 != 0, f32 != 0);
    out[1] = umma_sdesc(addr, lbo, sbo, swizzle);
    return RTM_OK;
}

extern "C" int rtm_debug_umma_probe(int N, unsigned lbo, unsigned sbo, const unsigned short *A, const unsigned short *B,
                                    float *D)
{
    RTM_CHECK_ARG(N >= 16 && N <= 256 && N % 16 == 0, "N must be a multiple of 16 in 16 .. 256");
    RTM_CHECK_ARG(lbo >= 16 && lbo <= 256 && sbo >= 16 && sbo <= 256 && lbo % 16 == 0 && sbo % 16 == 0,
                  "descriptor offsets must be multiples of 16 in 16 .. 256");
    RTM_CHECK_ARG(A && B && D, "null argument");
    TRY(ensure_device());
    DevBuf<__nv_bfloat16> a, b;
    DevBuf<float> d;
    DevBuf<int> st;
    TRY(a.alloc(128 * PROBE_K));
    TRY(b.alloc((size_t)N * PROBE_K));
    TRY(d.alloc((size_t)128 * N));
    TRY(st.alloc(1));
    RTM_CUDA(cudaMemcpy(a.p, A, 128 * PROBE_K * 2, cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(b.p, B, (size_t)N * PROBE_K * 2, cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemset(d.p, 0, (size_t)128 * N * 4));
    RTM_CUDA(cudaMemset(st.p, 0, 4));
    k_umma_probe<<<1, 128>>>(a.p, b.p, d.p, N, lbo, sbo, st.p);
    RTM_CUDA(cudaGetLastError());
    RTM_CUDA(cudaDeviceSynchronize());
    int s = 0;
    RTM_CUDA(cudaMemcpy(&s, st.p, 4, cudaMemcpyDeviceToHost));
    RTM_CUDA(cudaMemcpy(D, d.p, (size_t)128 * N * 4, cudaMemcpyDeviceToHost));
    if (s) {
        rtm_set_error("the probe's MMA did not complete within its time limit");
        return RTM_ERR_TIMEOUT;
    }
    return RTM_OK;
}
