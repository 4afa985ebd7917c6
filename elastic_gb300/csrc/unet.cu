// Learned image-domain preconditioner: a 4-level 3->3 channel convolutional
// U-Net (about 0.9M parameters) with BF16 weights and activations and FP32
// accumulation, trained with Adam.  Every convolution pass -- forward,
// backward-data and backward-weights -- is one tensor-core GEMM of this file
// on im2col operands in NHWC layout: the forward and backward-data passes on
// the fifth-generation tensor cores (tcgen05 MMAs, accumulators in tensor
// memory, k_gemm_tc), the backward-weights pass (both operands transposed,
// split over K with FP32 atomics) with mma.sync m16n8k16 (k_gemm, cp.async
// 3-stage pipeline), which also serves every pass when unet_set_gemm(0).
//
// Network (channels c = 32, 64, 96, 128; 3x3 convolutions with leaky ReLU,
// slope LEAK for negative inputs, which keeps units from dying without any
// normalisation layer):
//   e1: 3->32->32    (H)      skip s1
//   e2: 32->64->64   (H/2)    skip s2    (2x2 average pool between levels)
//   e3: 64->96->96   (H/4)    skip s3
//   b : 96->128->128 (H/8)
//   d3: [up(b) 128 | s3 96] -> 96 -> 96    (nearest 2x upsampling)
//   d2: [up(d3) 96 | s2 64] -> 64 -> 64
//   d1: [up(d2) 64 | s1 32] -> 32 -> 32
//   out: 1x1 convolution 32->3, no activation; loss = mean squared error.
//
// There is no counterpart in the reference (lgan/elastic only intends an
// iterative solver, 2d_rtm_restart/Src_working/rtm-mod-adj.f90:5-7).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/elastic_rtm.h"
#include "common.cuh"
#include "elastic2d_v2.cuh"
#include "engine.h"
#include "umma.cuh"

namespace {

using bf16 = __nv_bfloat16;
using eg::DevBuf;
using eg::fence_async_smem;
using eg::make_map_nd;
using eg::mbar_expect_tx;
using eg::mbar_init;
using eg::mbar_wait;
using eg::smem_u32;
using eg::tensor_maps_available;
using eg::tma_load_2d;
using eg::tma_load_4d;
using eg::tc_fence_after;
using eg::tc_fence_before;
using eg::tmem_alloc;
using eg::tmem_dealloc;
using eg::tmem_ld16;
using eg::tmem_relinquish;
using eg::umma_commit;
using eg::umma_f16;
using eg::umma_idesc_f16;
using eg::umma_sdesc;

// ----------------------------------------------------------------- GEMM
// C[M,N] = A[M,K] * B[N,K]^T with BF16 operands and FP32 accumulation.
// A_T=false: A[m*lda + k] (K contiguous); A_T=true: A[k*lda + m].
// B_T=false: B[n*ldb + k];                 B_T=true: B[k*ldb + n].
// K is a multiple of 32; split-K over blockIdx.z in chunks of kchunk.
enum Epi { EPI_BF16 = 0, EPI_F32 = 1, EPI_F32_ATOMIC_T = 2 };

struct GemmArgs {
    const bf16 *A;
    long long lda;
    const bf16 *B;
    long long ldb;
    int M, N, K, kchunk;
    const float *bias;  // EPI_BF16 / EPI_F32: per-n bias (or null)
    int relu;           // EPI_BF16: leaky ReLU after the bias
    bf16 *Cb;           // EPI_BF16: Cb[m*ldc + coff + n]
    float *Cf;          // EPI_F32: Cf[m*ldc + n]; EPI_F32_ATOMIC_T: Cf[n*ldc + m] += acc
    long long ldc;
    int coff;
    // implicit 3x3 (pad 1) im2col operand: with conv set, A is not read; the
    // A element of (pixel p, k) is X[p's neighbour at tap k / C][xoff + k % C]
    // of an NHWC tensor (channel stride ldx, H x W images); C % 8 == 0
    int conv;
    const bf16 *X;
    int ldx, xoff, C, H, W;
    int *err;  // tensor-core GEMM: set when a bounded wait ran out (nullable)
};

constexpr int GBM = 128, GBK = 32, GSTAGES = 3, GTHREADS = 256;
constexpr float LEAK = 0.1f;  // negative-side slope of the activation

template <bool A_T, bool B_T, int BM, int BN>
struct GemmSmem {
    static constexpr int A_ELEMS = A_T ? GBK * (BM + 8) : BM * (GBK + 8);
    static constexpr int B_ELEMS = B_T ? GBK * (BN + 8) : BN * (GBK + 8);
    static constexpr int STAGE = A_ELEMS + B_ELEMS;
    static constexpr size_t BYTES = (size_t)GSTAGES * STAGE * sizeof(bf16);
};

__device__ __forceinline__ void cpa16(void *smem, const void *gmem, bool ok)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(ok ? 16 : 0));
}
__device__ __forceinline__ void ldsm_x4(unsigned r[4], const void *p)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(s));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned r[4], const void *p)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(s));
}
__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], unsigned b0, unsigned b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Block tile (32*WM) x BN, 8 warps as WM (along M) x 8/WM (along N), warp
// tile 32 x BN*WM/8.
template <bool A_T, bool B_T, int BN, int WM, int EPI>
__global__ void __launch_bounds__(GTHREADS) k_gemm(const GemmArgs g)
{
    constexpr int BM = 32 * WM, WN = 8 / WM, WNT = BN / WN;
    using S = GemmSmem<A_T, B_T, BM, BN>;
    extern __shared__ __align__(16) unsigned char gsm_raw[];
    bf16 *sm = reinterpret_cast<bf16 *>(gsm_raw);
    constexpr int NT = WNT / 8;  // n8 tiles per warp
    static_assert(NT % 2 == 0 && WM * WN == 8, "warp layout");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp % WM, wn = warp / WM;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * g.kchunk;
    const int kend = min(g.K, kbeg + g.kchunk);
    const int ktiles = kend > kbeg ? (kend - kbeg) / GBK : 0;

    // implicit im2col: address of the 8 channels at (pixel p, column kk)
    auto conv_src = [&](long long p, int kk, bool &ok) -> const bf16 * {
        const int tap = kk / g.C, c = kk - tap * g.C;
        const int ky = tap / 3, kx = tap - 3 * ky;
        const int x = (int)(p % g.W);
        const long long t = p / g.W;
        const int y = (int)(t % g.H);
        const long long b = t / g.H;
        const int yy = y + ky - 1, xx = x + kx - 1;
        ok = ok && tap < 9 && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W;
        return ok ? g.X + ((b * g.H + yy) * g.W + xx) * g.ldx + g.xoff + c : g.X;
    };
    auto load = [&](int kt, int stage) {
        bf16 *sa = sm + stage * S::STAGE, *sb = sa + S::A_ELEMS;
        const int k0 = kbeg + kt * GBK;
        if (!A_T) {
            for (int c = tid; c < BM * 4; c += GTHREADS) {
                const int r = c >> 2, q = c & 3;
                bool ok = m0 + r < g.M;
                const bf16 *src;
                if (g.conv)
                    src = conv_src(m0 + r, k0 + q * 8, ok);
                else
                    src = g.A + (ok ? (long long)(m0 + r) * g.lda + k0 + q * 8 : 0);
                cpa16(sa + r * (GBK + 8) + q * 8, src, ok);
            }
        } else {
            for (int c = tid; c < GBK * (BM / 8); c += GTHREADS) {
                const int r = c / (BM / 8), q = c % (BM / 8);
                bool ok = m0 + q * 8 < g.M;
                const bf16 *src;
                if (g.conv)
                    src = conv_src(k0 + r, m0 + q * 8, ok);
                else
                    src = g.A + (ok ? (long long)(k0 + r) * g.lda + m0 + q * 8 : 0);
                cpa16(sa + r * (BM + 8) + q * 8, src, ok);
            }
        }
        if (!B_T) {
            for (int c = tid; c < BN * 4; c += GTHREADS) {
                const int r = c >> 2, q = c & 3;
                const bool ok = n0 + r < g.N;
                const bf16 *src = g.B + (ok ? (long long)(n0 + r) * g.ldb + k0 + q * 8 : 0);
                cpa16(sb + r * (GBK + 8) + q * 8, src, ok);
            }
        } else {
            for (int c = tid; c < GBK * (BN / 8); c += GTHREADS) {
                const int r = c / (BN / 8), q = c % (BN / 8);
                const bool ok = n0 + q * 8 < g.N;
                const bf16 *src = g.B + (ok ? (long long)(k0 + r) * g.ldb + n0 + q * 8 : 0);
                cpa16(sb + r * (BN + 8) + q * 8, src, ok);
            }
        }
    };

    float acc[2][NT][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < NT; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;

#pragma unroll
    for (int s = 0; s < GSTAGES - 1; s++) {
        if (s < ktiles) load(s, s);
        asm volatile("cp.async.commit_group;\n" ::);
    }
    for (int kt = 0; kt < ktiles; kt++) {
        asm volatile("cp.async.wait_group %0;\n" ::"n"(GSTAGES - 2));
        __syncthreads();
        if (kt + GSTAGES - 1 < ktiles) load(kt + GSTAGES - 1, (kt + GSTAGES - 1) % GSTAGES);
        asm volatile("cp.async.commit_group;\n" ::);
        const bf16 *sa = sm + (kt % GSTAGES) * S::STAGE, *sb = sa + S::A_ELEMS;
#pragma unroll
        for (int ks = 0; ks < GBK; ks += 16) {
            unsigned af[2][4];
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                const int mb = wm * 32 + mt * 16;
                if (!A_T) {
                    ldsm_x4(af[mt], sa + (mb + (lane & 15)) * (GBK + 8) + ks + (lane >> 4) * 8);
                } else {
                    const int k = ks + (lane & 7) + (lane >> 4) * 8, m = mb + ((lane >> 3) & 1) * 8;
                    ldsm_x4_t(af[mt], sa + k * (BM + 8) + m);
                }
            }
#pragma unroll
            for (int np = 0; np < NT / 2; np++) {
                const int nb = wn * WNT + np * 16;
                unsigned bfr[4];
                if (!B_T) {
                    const int n = nb + (lane & 7) + (lane >> 4) * 8, k = ks + ((lane >> 3) & 1) * 8;
                    ldsm_x4(bfr, sb + n * (GBK + 8) + k);
                } else {
                    const int k = ks + (lane & 7) + ((lane >> 3) & 1) * 8, n = nb + (lane >> 4) * 8;
                    ldsm_x4_t(bfr, sb + k * (BN + 8) + n);
                }
#pragma unroll
                for (int mt = 0; mt < 2; mt++) {
                    mma_bf16(acc[mt][2 * np], af[mt], bfr[0], bfr[1]);
                    mma_bf16(acc[mt][2 * np + 1], af[mt], bfr[2], bfr[3]);
                }
            }
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::);

    // epilogue
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int m = m0 + wm * 32 + mt * 16 + (lane >> 2) + h * 8;
                const int n = n0 + wn * WNT + nt * 8 + (lane & 3) * 2;
                if (m >= g.M) continue;
                float v0 = acc[mt][nt][2 * h], v1 = acc[mt][nt][2 * h + 1];
                if (EPI == EPI_F32_ATOMIC_T) {
                    if (n < g.N) atomicAdd(g.Cf + (long long)n * g.ldc + m, v0);
                    if (n + 1 < g.N) atomicAdd(g.Cf + (long long)(n + 1) * g.ldc + m, v1);
                    continue;
                }
                if (g.bias) {
                    if (n < g.N) v0 += g.bias[n];
                    if (n + 1 < g.N) v1 += g.bias[n + 1];
                }
                if (EPI == EPI_F32) {
                    if (n < g.N) g.Cf[(long long)m * g.ldc + n] = v0;
                    if (n + 1 < g.N) g.Cf[(long long)m * g.ldc + n + 1] = v1;
                } else {
                    if (g.relu) {
                        v0 = v0 > 0.f ? v0 : LEAK * v0;
                        v1 = v1 > 0.f ? v1 : LEAK * v1;
                    }
                    bf16 *dst = g.Cb + (long long)m * g.ldc + g.coff + n;
                    if (n + 1 < g.N) {
                        *reinterpret_cast<__nv_bfloat162 *>(dst) = __floats2bfloat162_rn(v0, v1);
                    } else if (n < g.N) {
                        *dst = __float2bfloat16_rn(v0);
                    }
                }
            }
}

// ------------------------------------------------- tensor-core (tcgen05)
// C[M,N] = A[M,K] * B[N,K]^T for K-major A (plain or implicit 3x3 im2col) and
// B, one 128 x BN output tile per CTA (BN >= N, a multiple of 16), FP32
// accumulation in tensor memory.  Per 64-wide K tile the 128 threads stage A
// (128 x 64) and B (BN x 64) with cp.async into the canonical K-major layout
// without swizzle -- 8-row x 16-byte core matrices, 128 bytes apart along K
// and 1024 along M/N -- zero-filling rows past M or N and columns past K;
// one thread issues four 128 x BN x 16 MMAs (tcgen05.mma .kind::f16, BF16
// operands) and commits them to the stage's mbarrier.  Loads run S-2 tiles
// ahead and refill the stage of the tile two back, so the tensor core always
// has the next tiles queued while a stage is being refilled.  Each thread
// loads the same 16-byte K column (8 K values) of the same 8 rows of every
// tile: the rows' pixel coordinates are worked out once.  After the last
// tile the four warps read the accumulator rows from tensor memory (warp w:
// rows 32 w .. 32 w + 31) and apply the epilogue: bias, leaky ReLU, BF16 or
// FP32 store.  Every wait is bounded; one that runs out sets g.err and the
// tile's output is not written.
constexpr int TC_BM = 128, TC_BK = 64, TC_THREADS = 128;
constexpr int TC_ROWS = TC_THREADS / (TC_BK / 8);  // rows a thread pass covers (16)

template <int BN>
struct TcCfg {
    static constexpr int A_BYTES = TC_BM * TC_BK * 2;
    static constexpr int B_BYTES = BN * TC_BK * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int STAGES = (200 * 1024 / STAGE) < 6 ? (200 * 1024 / STAGE) : 6;
    static constexpr uint32_t NCOLS = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE + 1024 + 8 * (STAGES + 2);
    static_assert(STAGES >= 4, "stages");
};

// Epilogue of a 128 x BN tensor-memory accumulator: warp w reads rows
// 32 w .. 32 w + 31 (output pixels m0 + row), adds the bias, applies the
// leaky ReLU (BF16 output) and stores BF16 or FP32.
template <int BN, int EPI>
__device__ __forceinline__ void tc_epilogue(const GemmArgs &g, uint32_t tmem, int m0, int warp, int lane)
{
    const int m = m0 + 32 * warp + lane;
#pragma unroll
    for (int c = 0; c < BN; c += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
        if (m >= g.M) continue;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int n = c + j;
            if (n < g.N && g.bias) v[j] += g.bias[n];
            if (EPI == EPI_BF16 && g.relu) v[j] = v[j] > 0.f ? v[j] : LEAK * v[j];
        }
        if (EPI == EPI_F32) {
            float *dst = g.Cf + (long long)m * g.ldc + c;
            if (c + 16 <= g.N && (g.ldc & 3) == 0) {
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *reinterpret_cast<float4 *>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c + j < g.N) dst[j] = v[j];
            }
        } else {
            bf16 *dst = g.Cb + (long long)m * g.ldc + g.coff + c;
            if (c + 16 <= g.N && ((g.ldc | g.coff) & 7) == 0) {
                uint4 w[2];
                __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(w);
#pragma unroll
                for (int j = 0; j < 8; j++) h[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                reinterpret_cast<uint4 *>(dst)[0] = w[0];
                reinterpret_cast<uint4 *>(dst)[1] = w[1];
            } else {
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c + j < g.N) dst[j] = __float2bfloat16_rn(v[j]);
            }
        }
    }
}

template <int BN, int EPI>
__global__ void __launch_bounds__(TC_THREADS) k_gemm_tc(const __grid_constant__ GemmArgs g)
{
    using T = TcCfg<BN>;
    constexpr int S = T::STAGES, D = S - 2;  // load-ahead distance
    constexpr int AR_ = TC_BM / TC_ROWS, BR_ = BN / TC_ROWS;  // row passes of A and B (8, BN/16)
    extern __shared__ __align__(16) unsigned char tc_raw[];
    unsigned char *base = tc_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(tc_raw) & 1023u)) & 1023u);
    unsigned long long *freeb = reinterpret_cast<unsigned long long *>(base + S * T::STAGE);
    unsigned long long *done = freeb + S;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_BM;
    const int ktiles = (g.K + TC_BK - 1) / TC_BK;
    if (warp == 0) {
        tmem_alloc(tslot, T::NCOLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < S; i++) mbar_init(&freeb[i]);
        mbar_init(done);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    // this thread's K column (8 values at q*8) and rows r0 + 16 i
    const int q = tid & 7, r0 = tid >> 3;
    // shared-memory byte offset of (row r, K column q) in a tile
    auto dst_of = [&](int r) { return ((r >> 3) << 10) | (q << 7) | ((r & 7) << 4); };
    // pixel coordinates of the A rows (implicit im2col)
    int pix[AR_], py[AR_], px[AR_];
#pragma unroll
    for (int i = 0; i < AR_; i++) {
        const int m = m0 + r0 + TC_ROWS * i;
        pix[i] = m < g.M ? m : -1;
        if (g.conv && m < g.M) {
            px[i] = m % g.W;
            py[i] = (m / g.W) % g.H;
        } else {
            px[i] = py[i] = 0;
        }
    }
    auto load = [&](int kt, int stage) {
        unsigned char *sa = base + stage * T::STAGE, *sb = sa + T::A_BYTES;
        const int kk = kt * TC_BK + q * 8;
        const bool kok = kk < g.K;
        if (g.conv) {
            const int tap = kk / g.C, c = kk - tap * g.C;
            const int ky = tap / 3, kx = tap - 3 * ky;
            const bool tok = kok && tap < 9;
            const long long dpix = (long long)(ky - 1) * g.W + (kx - 1);
#pragma unroll
            for (int i = 0; i < AR_; i++) {
                const int yy = py[i] + ky - 1, xx = px[i] + kx - 1;
                const bool ok = tok && pix[i] >= 0 && yy >= 0 && yy < g.H && xx >= 0 && xx < g.W;
                const bf16 *src = ok ? g.X + ((long long)pix[i] + dpix) * g.ldx + g.xoff + c : g.X;
                cpa16(sa + dst_of(r0 + TC_ROWS * i), src, ok);
            }
        } else {
#pragma unroll
            for (int i = 0; i < AR_; i++) {
                const bool ok = kok && pix[i] >= 0;
                cpa16(sa + dst_of(r0 + TC_ROWS * i), g.A + (ok ? (long long)pix[i] * g.lda + kk : 0), ok);
            }
        }
#pragma unroll
        for (int i = 0; i < BR_; i++) {
            const int r = r0 + TC_ROWS * i;
            const bool ok = kok && r < g.N;
            cpa16(sb + dst_of(r), g.B + (ok ? (long long)r * g.ldb + kk : 0), ok);
        }
    };
    constexpr uint32_t IDESC = umma_idesc_f16(TC_BM, BN, true, true);
#pragma unroll
    for (int t = 0; t < D; t++) {
        if (t < ktiles) load(t, t);
        asm volatile("cp.async.commit_group;\n" ::);
    }
    bool fail = false;
    for (int kt = 0; kt < ktiles; kt++) {
        asm volatile("cp.async.wait_group %0;\n" ::"n"(D - 1));
        fence_async_smem();
        __syncthreads();
        const int stage = kt % S;
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a_addr = smem_u32(base + stage * T::STAGE), b_addr = a_addr + T::A_BYTES;
#pragma unroll
            for (int k = 0; k < TC_BK / 16; k++)
                umma_f16(tmem, umma_sdesc(a_addr + 256 * k, 128, 1024, 0), umma_sdesc(b_addr + 256 * k, 128, 1024, 0),
                         IDESC, kt > 0 || k > 0);
            umma_commit(&freeb[stage]);
        }
        const int nt = kt + D;
        if (nt < ktiles && !fail) {
            // tile nt goes into the stage of tile nt - S = kt - 2, once that
            // tile's MMAs (committed two iterations ago) are done
            if (nt >= S && !mbar_wait(&freeb[(nt - S) % S], (unsigned)(((nt - S) / S) & 1))) fail = true;
            if (!fail) load(nt, nt % S);
        }
        asm volatile("cp.async.commit_group;\n" ::);
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
    if (tid == 0) umma_commit(done);
    bool ok = mbar_wait(done, 0);
    if (!ok) ok = mbar_wait(done, 0);  // the MMAs may still be running: a second limit
    tc_fence_after();
    if (__syncthreads_or(fail || !ok)) {
        if (tid == 0 && g.err) atomicExch(g.err, 1);
    } else {
        tc_epilogue<BN, EPI>(g, tmem, m0, warp, lane);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, T::NCOLS);
}

template <int BN, int EPI>
int gemm_tc_launch(const GemmArgs &g, cudaStream_t st)
{
    using T = TcCfg<BN>;
    auto kern = k_gemm_tc<BN, EPI>;
    static bool attr[RTM_MAX_DEVICES] = {};
    {
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!attr[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::SMEM));
            attr[dev] = true;
        }
    }
    kern<<<(g.M + TC_BM - 1) / TC_BM, TC_THREADS, T::SMEM, st>>>(g);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

template <int EPI>
int gemm_tc(const GemmArgs &g, cudaStream_t st)
{
    if (g.N <= 16) return gemm_tc_launch<16, EPI>(g, st);
    if (g.N <= 32) return gemm_tc_launch<32, EPI>(g, st);
    if (g.N <= 64) return gemm_tc_launch<64, EPI>(g, st);
    if (g.N <= 96) return gemm_tc_launch<96, EPI>(g, st);
    if (g.N <= 128) return gemm_tc_launch<128, EPI>(g, st);
    return gemm_tc_launch<256, EPI>(g, st);
}

// ------------------------------------ 3x3 convolution by bulk tensor copies
// The implicit-im2col GEMM of a 3x3 (pad 1) convolution of an NHWC tensor
// X (C channels, C % 32 == 0) for image widths W with W % 128 == 0 or
// 128 % W == 0: a 128-pixel output tile is a segment of one image row
// (W >= 128) or 128 / W whole rows, so its A operand for tap (dy, dx) and
// channel chunk c is ONE box of the activation tensor -- KC channels x the
// tile's pixels shifted by (dy - 1, dx - 1) -- that a bulk tensor copy
// fetches with the zero padding supplied by the copy's out-of-range fill.
// The K loop runs over 9 taps x C / KC chunks (KC = 64 with a 128-byte
// swizzle, 32 with a 64-byte swizzle); B (the weights, K-major [N][9 C]) is
// a box of KC x BN.
// Persistent: one CTA per SM walks tiles blockIdx.x, + gridDim.x, ...
// Warp 4 (one thread) issues the copies of every tile's K steps into an
// S-stage ring (full/empty mbarriers); warp 5 (one thread) issues the MMAs
// (tcgen05.mma, FP32 accumulator in tensor memory), committing each stage
// back to its empty barrier and each finished tile to tfull[buffer]; warps
// 0-3 drain the accumulator buffer of the tile before (two buffers of BN
// columns, released through tempty), so a tile's epilogue -- the epilogue
// of k_gemm_tc -- runs under the next tile's MMAs and copies.  Every wait
// is bounded; a run-out stops every role, sets g.err (outputs then
// incomplete), and the copies in flight are let land before the CTA exits.
struct ConvTcArgs {
    GemmArgs g;
    CUtensorMap tma;  // X + xoff: {C, W, H, images}, box {KC, min(W,128), 128/min(W,128), 1}
    CUtensorMap tmb;  // B: {9 C, N}, box {KC, BN}
    int nk;           // K steps: 9 * C / KC
    int cchunks;      // C / KC
    int ntiles;       // M / 128
};

constexpr int CV_THREADS = 192;  // warps 0-3 epilogue, 4 copies, 5 MMAs

// SH (image rows of at least 128 pixels): a K step is a row of taps dy and a
// channel chunk; its A operand is ONE box of 136 pixels (the tile's 128 and
// its 1-pixel halo, rounded to whole 8-row atoms) and the three taps dx are
// MMAs whose descriptors start dx rows into it (the swizzle follows the
// absolute shared-memory address, so a row-shifted start needs no base
// offset); B is the three taps' weight boxes.
constexpr int CV_SH_ROWS = 136;

template <int BN, int KC, bool SH>
struct ConvCfg {
    static constexpr int A_BYTES = SH ? (CV_SH_ROWS * KC * 2 + 1023) / 1024 * 1024 : TC_BM * KC * 2;
    static constexpr int B_TAP = BN * KC * 2;
    static constexpr int B_BYTES = (SH ? 3 : 1) * B_TAP;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int STAGES = (192 * 1024 / STAGE) > 8 ? 8 : (192 * 1024 / STAGE);
    static constexpr uint32_t NCOLS = 2 * BN <= 64 ? 64 : 2 * BN <= 128 ? 128 : 2 * BN <= 256 ? 256 : 512;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE + 1024 + 8 * (2 * STAGES + 5) + 16;
    static_assert(STAGES >= 4, "stages");
};

template <int BN, int EPI, int KC, bool SH>
__global__ void __launch_bounds__(CV_THREADS, 1) k_conv_tc(const __grid_constant__ ConvTcArgs A)
{
    using T = ConvCfg<BN, KC, SH>;
    constexpr int S = T::STAGES;
    const GemmArgs &g = A.g;
    extern __shared__ __align__(16) unsigned char cv_raw[];
    unsigned char *base = cv_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(cv_raw) & 1023u)) & 1023u);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(base + S * T::STAGE);
    unsigned long long *empty = full + S, *tfull = empty + S, *tempty = tfull + 2, *done = tempty + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    int *fail = reinterpret_cast<int *>(tslot + 1);
    int *issued = fail + 1;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nk = A.nk, HW = g.H * g.W;
    if (warp == 0) {
        tmem_alloc(tslot, T::NCOLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < S; i++) {
            mbar_init(&full[i]);
            mbar_init(&empty[i]);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(&tfull[i]);
            eg::mbar_init_n(&tempty[i], 4);
        }
        mbar_init(done);
        *fail = 0;
        *issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    auto failed = [&]() { return *reinterpret_cast<volatile int *>(fail) != 0; };
    if (warp == 4) {
        if (lane == 0) {
            // copies: K step `it` (counted over all of this CTA's tiles) into
            // stage it % S once the MMAs of step it - S have released it
            int it = 0;
            for (int t = blockIdx.x; t < A.ntiles && !failed(); t += gridDim.x) {
                const int m0 = t * TC_BM, img = m0 / HW, rem = m0 - img * HW, y0 = rem / g.W, x0 = rem - y0 * g.W;
                for (int i = 0; i < nk; i++, it++) {
                    const int st = it % S;
                    if (it >= S && !mbar_wait(&empty[st], (unsigned)(((it - S) / S) & 1))) {
                        atomicExch(fail, 1);
                        break;
                    }
                    unsigned char *sa = base + st * T::STAGE;
                    if (SH) {
                        // row of taps dy, channel chunk cc: one 136-pixel box, three weight boxes
                        const int dy = i / A.cchunks, cc = i - dy * A.cchunks;
                        mbar_expect_tx(&full[st], (unsigned)(CV_SH_ROWS * KC * 2 + 3 * T::B_TAP));
                        tma_load_4d(sa, &A.tma, cc * KC, x0 - 1, y0 + dy - 1, img, &full[st]);
                        for (int dx = 0; dx < 3; dx++)
                            tma_load_2d(sa + T::A_BYTES + dx * T::B_TAP, &A.tmb, (3 * dy + dx) * g.C + cc * KC, 0,
                                        &full[st]);
                    } else {
                        const int tap = i / A.cchunks, cc = i - tap * A.cchunks, dy = tap / 3, dx = tap - 3 * dy;
                        mbar_expect_tx(&full[st], (unsigned)T::STAGE);
                        tma_load_4d(sa, &A.tma, cc * KC, x0 + dx - 1, y0 + dy - 1, img, &full[st]);
                        tma_load_2d(sa + T::A_BYTES, &A.tmb, tap * g.C + cc * KC, 0, &full[st]);
                    }
                    *reinterpret_cast<volatile int *>(issued) = it + 1;
                }
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr uint32_t IDESC = umma_idesc_f16(TC_BM, BN, true, true);
            constexpr uint32_t SW = KC == 64 ? 2u : 4u, SBO = 8u * KC * 2u;
            int it = 0, j = 0;
            for (int t = blockIdx.x; t < A.ntiles && !failed(); t += gridDim.x, j++) {
                const int buf = j & 1;
                // the epilogue has drained this buffer (tile j - 2)
                if (j >= 2 && !mbar_wait(&tempty[buf], (unsigned)(((j - 2) >> 1) & 1))) {
                    atomicExch(fail, 1);
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(buf * BN);
                bool ok = true;
                for (int i = 0; i < nk; i++, it++) {
                    const int st = it % S;
                    if (!mbar_wait(&full[st], (unsigned)((it / S) & 1))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_addr = smem_u32(base + st * T::STAGE), b_addr = a_addr + T::A_BYTES;
#pragma unroll
                    for (int dx = 0; dx < (SH ? 3 : 1); dx++)
#pragma unroll
                        for (int k = 0; k < KC / 16; k++)
                            umma_f16(acc, umma_sdesc(a_addr + dx * (KC * 2) + 32 * k, 16, SBO, SW),
                                     umma_sdesc(b_addr + dx * T::B_TAP + 32 * k, 16, SBO, SW), IDESC,
                                     i > 0 || dx > 0 || k > 0);
                    umma_commit(&empty[st]);
                }
                if (!ok) {
                    atomicExch(fail, 1);
                    break;
                }
                umma_commit(&tfull[buf]);
            }
            umma_commit(done);  // tracks every MMA issued, also after a failure
        }
    } else {
        // epilogue warps 0-3: tensor-memory lanes 32 warp .. + 31
        int j = 0;
        for (int t = blockIdx.x; t < A.ntiles; t += gridDim.x, j++) {
            const int buf = j & 1;
            bool ok = mbar_wait(&tfull[buf], (unsigned)((j >> 1) & 1));
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) {
                if (lane == 0) atomicExch(fail, 1);
                break;
            }
            tc_fence_after();
            tc_epilogue<BN, EPI>(g, tmem + (uint32_t)(buf * BN), t * TC_BM, warp, lane);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) eg::mbar_arrive(&tempty[buf]);
            if (failed()) break;
        }
    }
    // every MMA complete before the tensor memory is released
    if (warp == 5 || tid == 0) {
        bool ok = mbar_wait(done, 0);
        if (!ok) ok = mbar_wait(done, 0);
        if (!ok) atomicExch(fail, 1);
    }
    tc_fence_after();
    if (__syncthreads_or(failed())) {
        if (tid == 0) {
            if (g.err) atomicExch(g.err, 1);
            // let issued copies land (bounded): the last S issued steps
            const int n = *reinterpret_cast<volatile int *>(issued);
            for (int i = n - 1; i >= 0 && i >= n - S; i--) mbar_wait(&full[i % S], (unsigned)((i / S) & 1));
        }
        __syncthreads();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, T::NCOLS);
}

// Tensor maps and launch of k_conv_tc; RTM_ERR_ARG when the geometry does
// not fit (the caller then uses k_gemm_tc).
template <int BN, int EPI, int KC, bool SH>
int conv_tc_launch(const GemmArgs &g, cudaStream_t st)
{
    using T = ConvCfg<BN, KC, SH>;
    ConvTcArgs a;
    memset(&a, 0, sizeof a);
    a.g = g;
    a.cchunks = g.C / KC;
    a.nk = (SH ? 3 : 9) * a.cchunks;
    const int bw = SH ? CV_SH_ROWS : g.W < 128 ? g.W : 128, bh = SH ? 1 : 128 / bw;
    const long long imgs = (long long)g.M / ((long long)g.H * g.W);
    {
        const long long dims[4] = {g.C, g.W, g.H, imgs};
        const long long strides[3] = {2LL * g.ldx, 2LL * g.ldx * g.W, 2LL * g.ldx * g.W * g.H};
        const int box[4] = {KC, bw, bh, 1};
        TRY(make_map_nd(&a.tma, g.X + g.xoff, true, 4, dims, strides, box, 2 * KC));
    }
    {
        const long long dims[2] = {9LL * g.C, g.N};
        const long long strides[1] = {2LL * g.ldb};
        const int box[2] = {KC, BN};
        TRY(make_map_nd(&a.tmb, g.B, true, 2, dims, strides, box, 2 * KC));
    }
    a.ntiles = g.M / TC_BM;
    auto kern = k_conv_tc<BN, EPI, KC, SH>;
    static bool attr[RTM_MAX_DEVICES] = {};
    {
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!attr[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::SMEM));
            attr[dev] = true;
        }
    }
    const int grid = std::min(a.ntiles, eg::device_sm_count());
    kern<<<grid, CV_THREADS, T::SMEM, st>>>(a);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

int g_conv_shift = 1;  // 1: the shifted-box form where the image rows allow (W % 128 == 0)

// row-segment tiles (W % 128 == 0) take the shifted-box form where its stage
// (one 136-pixel box and three weight boxes) leaves at least four stages
template <int BN, int EPI, int KC>
int conv_tc_bn(const GemmArgs &g, cudaStream_t st)
{
    if constexpr (KC == 32 || BN <= 64) {
        if (g_conv_shift && g.W % 128 == 0) return conv_tc_launch<BN, EPI, KC, true>(g, st);
    }
    return conv_tc_launch<BN, EPI, KC, false>(g, st);
}

template <int EPI, int KC>
int conv_tc_kc(const GemmArgs &g, cudaStream_t st)
{
    if (g.N <= 32) return conv_tc_bn<32, EPI, KC>(g, st);
    if (g.N <= 64) return conv_tc_bn<64, EPI, KC>(g, st);
    if (g.N <= 96) return conv_tc_bn<96, EPI, KC>(g, st);
    if (g.N <= 128) return conv_tc_bn<128, EPI, KC>(g, st);
    return conv_tc_launch<256, EPI, KC, false>(g, st);
}

// True when k_conv_tc covers this GEMM.
bool conv_tc_fits(const GemmArgs &g)
{
    if (!g.conv || g.C % 32 || g.N > 256 || g.K != 9 * g.C || g.M % TC_BM) return false;
    if (!(g.W % 128 == 0 || 128 % g.W == 0) || ((long long)g.H * g.W) % TC_BM) return false;
    if (((uintptr_t)(g.X + g.xoff) & 15) || ((uintptr_t)g.B & 15) || g.ldx % 8 || g.ldb % 8) return false;
    return tensor_maps_available();
}

template <int EPI>
int conv_tc(const GemmArgs &g, cudaStream_t st)
{
    return g.C % 64 == 0 ? conv_tc_kc<EPI, 64>(g, st) : conv_tc_kc<EPI, 32>(g, st);
}

// ------------------------------- 3x3 weight gradients by bulk tensor copies
// dW[co][kw] += sum over pixels p of dY[p][co] X[p + shift(tap(kw))][ci(kw)],
// kw = tap * Cin + ci: a GEMM with M = kw (128 per CTA), N = Cout, K =
// pixels, both operands MN-major (channels contiguous in the NHWC tensors):
// per 64-pixel K step the A tile is four boxes of 32 channels x 64 pixels of
// X shifted by the tap of each 32-channel chunk of kw (zero padding from the
// copies' out-of-range fill), the B tile Cout/32 boxes of dY; each box lands
// as eight 512-byte atoms of 8 pixels x 32 channels with the 64-byte swizzle
// (MN-major canonical layout: leading offset 4096 bytes between boxes along
// M/N, stride offset 512 bytes between atoms along K).  The pixel range is
// split over CTAs; each adds its 128 x Cout partial sums to dW with FP32
// atomics.  Roles and bounded waits as in k_conv_tc.
struct WgradArgs {
    float *dw;        // dW[n * ldc + m]
    long long ldc;
    int M, N;         // 9 Cin, Cout
    int Cin, H, W;
    int ksteps;       // 64-pixel steps in all
    int steps_per_cta;
    int *err;
    CUtensorMap tmx;  // X + xoff: {Cin, W, H, images}, box {32, min(W,64), 64/min(W,64), 1}
    CUtensorMap tmy;  // dY: {Cout, W, H, images}, same box
};

constexpr int WG_K = 64;                           // pixels per K step
constexpr int WG_BOX = 32 * WG_K * 2;              // bytes of one 32-channel box (4 KB)

template <int BN>
struct WgCfg {
    static constexpr int A_BYTES = 4 * WG_BOX;             // 128 kw
    static constexpr int B_BYTES = (BN / 32) * WG_BOX;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int STAGES = (192 * 1024 / STAGE) > 8 ? 8 : (192 * 1024 / STAGE);
    static constexpr uint32_t NCOLS = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE + 1024 + 8 * (2 * STAGES + 1) + 16;
    static_assert(STAGES >= 4, "stages");
};

template <int BN>
__global__ void __launch_bounds__(TC_THREADS) k_wgrad_tc(const __grid_constant__ WgradArgs A)
{
    using T = WgCfg<BN>;
    constexpr int S = T::STAGES;
    extern __shared__ __align__(16) unsigned char wg_raw[];
    unsigned char *base = wg_raw + ((1024u - ((unsigned)__cvta_generic_to_shared(wg_raw) & 1023u)) & 1023u);
    unsigned long long *full = reinterpret_cast<unsigned long long *>(base + S * T::STAGE);
    unsigned long long *empty = full + S, *done = empty + S;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    int *fail = reinterpret_cast<int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_BM;
    const int k0 = blockIdx.y * A.steps_per_cta, k1 = min(A.ksteps, k0 + A.steps_per_cta);
    if (k0 >= k1) return;
    const int nk = k1 - k0;
    if (warp == 0) {
        tmem_alloc(tslot, T::NCOLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < S; i++) {
            mbar_init(&full[i]);
            mbar_init(&empty[i]);
        }
        mbar_init(done);
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int HW = A.H * A.W, bw = A.W < WG_K ? A.W : WG_K;
    if (tid == 0) {
        // the A boxes of this CTA's kw rows: chunk j covers kw m0+32j ..
        int nbox = 0, tapj[4], cj[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int kw = m0 + 32 * j;
            tapj[j] = kw < A.M ? kw / A.Cin : -1;
            cj[j] = kw < A.M ? kw - tapj[j] * A.Cin : 0;
            nbox += kw < A.M;
        }
        const unsigned bytes = (unsigned)((nbox + BN / 32) * WG_BOX);
        for (int i = 0; i < nk; i++) {
            const int st = i % S;
            if (i >= S && !mbar_wait(&empty[st], (unsigned)(((i - S) / S) & 1))) {
                atomicExch(fail, 1);
                break;
            }
            const int p0 = (k0 + i) * WG_K, img = p0 / HW, rem = p0 - img * HW, y0 = rem / A.W, x0 = rem - y0 * A.W;
            unsigned char *sa = base + st * T::STAGE, *sb = sa + T::A_BYTES;
            mbar_expect_tx(&full[st], bytes);
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (tapj[j] >= 0) {
                    const int dy = tapj[j] / 3, dx = tapj[j] - 3 * dy;
                    tma_load_4d(sa + j * WG_BOX, &A.tmx, cj[j], x0 + dx - 1, y0 + dy - 1, img, &full[st]);
                }
#pragma unroll
            for (int j = 0; j < BN / 32; j++) tma_load_4d(sb + j * WG_BOX, &A.tmy, 32 * j, x0, y0, img, &full[st]);
            (void)bw;
        }
    } else if (tid == 32) {
        constexpr uint32_t IDESC = umma_idesc_f16(TC_BM, BN, true, true) | (1u << 15) | (1u << 16);
        for (int i = 0; i < nk; i++) {
            const int st = i % S;
            if (!mbar_wait(&full[st], (unsigned)((i / S) & 1))) {
                atomicExch(fail, 1);
                break;
            }
            tc_fence_after();
            const uint32_t a_addr = smem_u32(base + st * T::STAGE), b_addr = a_addr + T::A_BYTES;
#pragma unroll
            for (int k = 0; k < WG_K / 16; k++)
                umma_f16(tmem, umma_sdesc(a_addr + 1024 * k, WG_BOX, 512, 4), umma_sdesc(b_addr + 1024 * k, WG_BOX, 512, 4),
                         IDESC, i > 0 || k > 0);
            umma_commit(&empty[st]);
        }
        umma_commit(done);
    }
    bool ok = mbar_wait(done, 0);
    if (!ok) ok = mbar_wait(done, 0);
    tc_fence_after();
    if (__syncthreads_or(!ok || *reinterpret_cast<volatile int *>(fail))) {
        if (tid == 0) {
            if (A.err) atomicExch(A.err, 1);
            for (int i = 0; i < nk && i < S; i++) mbar_wait(&full[(nk - 1 - i) % S], (unsigned)(((nk - 1 - i) / S) & 1));
        }
    } else {
        const int m = m0 + 32 * warp + lane;
#pragma unroll
        for (int c = 0; c < BN; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
            if (m < A.M) {
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c + j < A.N) atomicAdd(A.dw + (long long)(c + j) * A.ldc + m, v[j]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, T::NCOLS);
}

template <int BN>
int wgrad_tc_launch(WgradArgs &a, int mtiles, int splits, cudaStream_t st)
{
    using T = WgCfg<BN>;
    auto kern = k_wgrad_tc<BN>;
    static bool attr[RTM_MAX_DEVICES] = {};
    {
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!attr[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::SMEM));
            attr[dev] = true;
        }
    }
    kern<<<dim3(mtiles, splits), TC_THREADS, T::SMEM, st>>>(a);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

// True when k_wgrad_tc covers the weight gradient of a 3x3 layer with input
// X (Cin channels, channel stride ldx, offset xoff) and output gradient dY
// (Cout channels, stride ldy) on n images of H x W.
bool wgrad_tc_fits(int Cin, int ldx, int xoff, const bf16 *X, int Cout, int ldy, const bf16 *dY, int H, int W,
                   long long P)
{
    if (Cin % 32 || Cout % 32 || Cout > 128 || ldx % 8 || xoff % 8 || ldy % 8) return false;
    if (!(W % WG_K == 0 || WG_K % W == 0) || ((long long)H * W) % WG_K || P % WG_K) return false;
    if (((uintptr_t)(X + xoff) & 15) || ((uintptr_t)dY & 15)) return false;
    return tensor_maps_available();
}

int wgrad_tc(float *dw, long long ldc, int Cin, const bf16 *X, int ldx, int xoff, int Cout, const bf16 *dY, int ldy,
             int n, int H, int W, int *err, cudaStream_t st)
{
    WgradArgs a;
    memset(&a, 0, sizeof a);
    a.dw = dw;
    a.ldc = ldc;
    a.M = 9 * Cin;
    a.N = Cout;
    a.Cin = Cin;
    a.H = H;
    a.W = W;
    a.err = err;
    const long long P = (long long)n * H * W;
    a.ksteps = (int)(P / WG_K);
    const int bw = W < WG_K ? W : WG_K, bh = WG_K / bw;
    {
        const long long dims[4] = {Cin, W, H, n};
        const long long strides[3] = {2LL * ldx, 2LL * ldx * W, 2LL * ldx * W * H};
        const int box[4] = {32, bw, bh, 1};
        TRY(make_map_nd(&a.tmx, X + xoff, true, 4, dims, strides, box, 64));
    }
    {
        const long long dims[4] = {Cout, W, H, n};
        const long long strides[3] = {2LL * ldy, 2LL * ldy * W, 2LL * ldy * W * H};
        const int box[4] = {32, bw, bh, 1};
        TRY(make_map_nd(&a.tmy, dY, true, 4, dims, strides, box, 64));
    }
    const int mtiles = (a.M + TC_BM - 1) / TC_BM;
    // K splits: about three CTAs per SM, at least 16 steps each
    int splits = std::max(1, std::min(a.ksteps / 16, (3 * eg::device_sm_count() + mtiles - 1) / mtiles));
    a.steps_per_cta = (a.ksteps + splits - 1) / splits;
    splits = (a.ksteps + a.steps_per_cta - 1) / a.steps_per_cta;
    switch ((Cout + 31) / 32) {
    case 1: return wgrad_tc_launch<32>(a, mtiles, splits, st);
    case 2: return wgrad_tc_launch<64>(a, mtiles, splits, st);
    case 3: return wgrad_tc_launch<96>(a, mtiles, splits, st);
    default: return wgrad_tc_launch<128>(a, mtiles, splits, st);
    }
}

int g_gemm_tc = 2;  // 2: 3x3 convolutions by bulk-copied tap boxes, other non-transposed GEMMs on k_gemm_tc;
                    // 1: k_gemm_tc for every non-transposed pass; 0: mma.sync only

template <bool A_T, bool B_T, int BN, int WM, int EPI>
int gemm_launch(const GemmArgs &g, int splits, cudaStream_t st)
{
    constexpr int BM = 32 * WM;
    using S = GemmSmem<A_T, B_T, BM, BN>;
    auto kern = k_gemm<A_T, B_T, BN, WM, EPI>;
    static bool attr[RTM_MAX_DEVICES] = {};
    {
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!attr[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::BYTES));
            attr[dev] = true;
        }
    }
    dim3 grid((g.M + BM - 1) / BM, (g.N + BN - 1) / BN, splits);
    kern<<<grid, GTHREADS, S::BYTES, st>>>(g);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

// Dispatch on operand layouts, epilogue and the tile shape: 128 x N for
// N = 64, 96 and multiples of 128 (warp tile 32 x N/2); otherwise 256 x 32
// tiles with all eight warps along M (warp tile 32 x 32).
template <bool A_T, bool B_T, int EPI>
int gemm_bn(const GemmArgs &g, int splits, cudaStream_t st)
{
    if (g.N == 64) return gemm_launch<A_T, B_T, 64, 4, EPI>(g, splits, st);
    if (g.N == 96) return gemm_launch<A_T, B_T, 96, 4, EPI>(g, splits, st);
    if (g.N % 128 == 0) return gemm_launch<A_T, B_T, 128, 4, EPI>(g, splits, st);
    return gemm_launch<A_T, B_T, 32, 8, EPI>(g, splits, st);
}

int gemm(const GemmArgs &g, bool a_t, bool b_t, int epi, int splits, cudaStream_t st)
{
    RTM_CHECK_ARG(g.K % GBK == 0 && g.kchunk % GBK == 0 && g.kchunk > 0, "GEMM K=%d (chunk %d) not a multiple of 32",
                  g.K, g.kchunk);
    RTM_CHECK_ARG(!a_t || g.M % 8 == 0, "GEMM with M-major A needs M %% 8 == 0 (M=%d)", g.M);
    RTM_CHECK_ARG(!b_t || g.N % 8 == 0, "GEMM with N-major B needs N %% 8 == 0 (N=%d)", g.N);
    RTM_CHECK_ARG(epi != EPI_BF16 || ((g.ldc | g.coff) & 1) == 0, "BF16 GEMM output needs even ldc and offset");
    RTM_CHECK_ARG(!g.conv || (g.C % 32 == 0 && (g.ldx | g.xoff) % 8 == 0 && g.X && g.H > 0 && g.W > 0),
                  "implicit im2col needs C %% 32 == 0 and 16-byte aligned channel runs");
    const bool tc = g_gemm_tc && !a_t && !b_t && splits == 1 && g.kchunk >= g.K && g.N <= 256 &&
                    (g.conv || (g.lda % 8 == 0 && g.A)) && g.ldb % 8 == 0;
    if (tc && g_gemm_tc == 2 && conv_tc_fits(g)) {
        if (epi == EPI_BF16) return conv_tc<EPI_BF16>(g, st);
        if (epi == EPI_F32) return conv_tc<EPI_F32>(g, st);
    }
    if (tc && epi == EPI_BF16) return gemm_tc<EPI_BF16>(g, st);
    if (tc && epi == EPI_F32) return gemm_tc<EPI_F32>(g, st);
    if (epi == EPI_BF16 && !a_t && !b_t) return gemm_bn<false, false, EPI_BF16>(g, splits, st);
    if (epi == EPI_F32 && !a_t && !b_t) return gemm_bn<false, false, EPI_F32>(g, splits, st);
    if (epi == EPI_F32_ATOMIC_T && a_t && b_t) return gemm_bn<true, true, EPI_F32_ATOMIC_T>(g, splits, st);
    rtm_set_error("GEMM variant not instantiated (a_t=%d b_t=%d epi=%d)", a_t, b_t, epi);
    return RTM_ERR_ARG;
}

// ------------------------------------------------------- layout kernels
// im2col of a 3x3, pad-1 convolution in NHWC: col[p][(ky*3+kx)*C + c],
// columns [9C, Kp) zero.  x: channels [coff, coff+C) of pixels with stride ldx.
__global__ void k_im2col3(int n, int H, int W, int C, const bf16 *x, int ldx, int coff, bf16 *col, int Kp)
{
    const long long P = (long long)n * H * W;
    const long long total = P * Kp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / Kp;
        const int k = (int)(i - p * Kp);
        bf16 v = __float2bfloat16_rn(0.f);
        if (k < 9 * C) {
            const int tap = k / C, c = k - tap * C, ky = tap / 3, kx = tap - ky * 3;
            const int xw = (int)(p % W), yh = (int)((p / W) % H);
            const long long b = p / ((long long)W * H);
            const int yy = yh + ky - 1, xx = xw + kx - 1;
            if (yy >= 0 && yy < H && xx >= 0 && xx < W)
                v = x[((b * H + yy) * W + xx) * ldx + coff + c];
        }
        col[i] = v;
    }
}
// Vector im2col for C % 8 == 0 (16-byte chunks of 8 channels).
__global__ void k_im2col3_v8(int n, int H, int W, int C, const bf16 *x, int ldx, int coff, bf16 *col, int Kp)
{
    const long long P = (long long)n * H * W;
    const int kc = Kp / 8;
    const long long total = P * kc;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / kc;
        const int k = (int)(i - p * kc) * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (k < 9 * C) {
            const int tap = k / C, c = k - tap * C, ky = tap / 3, kx = tap - ky * 3;
            const int xw = (int)(p % W), yh = (int)((p / W) % H);
            const long long b = p / ((long long)W * H);
            const int yy = yh + ky - 1, xx = xw + kx - 1;
            if (yy >= 0 && yy < H && xx >= 0 && xx < W)
                v = *reinterpret_cast<const uint4 *>(x + ((b * H + yy) * W + xx) * ldx + coff + c);
        }
        *reinterpret_cast<uint4 *>(col + p * Kp + k) = v;
    }
}

// 8 BF16 values <-> floats
__device__ __forceinline__ void unpack8(const uint4 &u, float f[8])
{
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}
__device__ __forceinline__ uint4 pack8(const float f[8])
{
    uint4 u;
    __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    return u;
}

// Vector forms of the layout kernels below, 8 channels per thread (C, the
// strides and offsets multiples of 8).
__global__ void k_relu_mask8(long long P, int C, int ld, const bf16 *y, bf16 *g)
{
    const int c8 = C / 8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P * c8; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / c8;
        const long long o = p * ld + (i - p * c8) * 8;
        float yv[8], gv[8];
        unpack8(*reinterpret_cast<const uint4 *>(y + o), yv);
        unpack8(*reinterpret_cast<const uint4 *>(g + o), gv);
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (!(yv[k] > 0.f)) gv[k] *= LEAK;
        *reinterpret_cast<uint4 *>(g + o) = pack8(gv);
    }
}
__global__ void k_up_fwd8(int n, int Hi, int Wi, int C, const bf16 *in, int ldi, bf16 *out, int ldo)
{
    const int Ho = 2 * Hi, Wo = 2 * Wi, c8 = C / 8;
    const long long total = (long long)n * Ho * Wo * c8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % c8) * 8;
        const long long p = i / c8;
        const int x = (int)(p % Wo), y = (int)((p / Wo) % Ho);
        const long long b = p / ((long long)Wo * Ho);
        *reinterpret_cast<uint4 *>(out + p * ldo + c) =
            *reinterpret_cast<const uint4 *>(in + ((b * Hi + y / 2) * Wi + x / 2) * ldi + c);
    }
}
__global__ void k_up_bwd8(int n, int Hi, int Wi, int C, const bf16 *gout, int ldo, bf16 *gin, int ldi)
{
    const int Wo = 2 * Wi, Ho = 2 * Hi, c8 = C / 8;
    const long long total = (long long)n * Hi * Wi * c8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % c8) * 8;
        const long long p = i / c8;
        const int x = (int)(p % Wi), y = (int)((p / Wi) % Hi);
        const long long b = p / ((long long)Wi * Hi);
        const long long q = (b * Ho + 2 * y) * Wo + 2 * x;
        const long long qs[4] = {q, q + 1, q + Wo, q + Wo + 1};
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, v[8];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            unpack8(*reinterpret_cast<const uint4 *>(gout + qs[k] * ldo + c), v);
#pragma unroll
            for (int j = 0; j < 8; j++) s[j] += v[j];
        }
        *reinterpret_cast<uint4 *>(gin + p * ldi + c) = pack8(s);
    }
}
__global__ void k_pool_fwd8(int n, int Ho, int Wo, int C, const bf16 *in, int ldi, bf16 *out, int ldo)
{
    const int Wi = 2 * Wo, Hi = 2 * Ho, c8 = C / 8;
    const long long total = (long long)n * Ho * Wo * c8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % c8) * 8;
        const long long p = i / c8;
        const int x = (int)(p % Wo), y = (int)((p / Wo) % Ho);
        const long long b = p / ((long long)Wo * Ho);
        const long long q = (b * Hi + 2 * y) * Wi + 2 * x;
        const long long qs[4] = {q, q + 1, q + Wi, q + Wi + 1};
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, v[8];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            unpack8(*reinterpret_cast<const uint4 *>(in + qs[k] * ldi + c), v);
#pragma unroll
            for (int j = 0; j < 8; j++) s[j] += v[j];
        }
#pragma unroll
        for (int j = 0; j < 8; j++) s[j] *= 0.25f;
        *reinterpret_cast<uint4 *>(out + p * ldo + c) = pack8(s);
    }
}
__global__ void k_pool_bwd_add8(int n, int Ho, int Wo, int C, const bf16 *gout, int ldo, bf16 *gin, int ldi)
{
    const int Wi = 2 * Wo, Hi = 2 * Ho, c8 = C / 8;
    const long long total = (long long)n * Ho * Wo * c8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % c8) * 8;
        const long long p = i / c8;
        const int x = (int)(p % Wo), y = (int)((p / Wo) % Ho);
        const long long b = p / ((long long)Wo * Ho);
        const long long q = (b * Hi + 2 * y) * Wi + 2 * x;
        float g[8], v[8];
        unpack8(*reinterpret_cast<const uint4 *>(gout + p * ldo + c), g);
        const long long qs[4] = {q, q + 1, q + Wi, q + Wi + 1};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint4 *d = reinterpret_cast<uint4 *>(gin + qs[k] * ldi + c);
            unpack8(*d, v);
#pragma unroll
            for (int j = 0; j < 8; j++) v[j] += 0.25f * g[j];
            *d = pack8(v);
        }
    }
}
__global__ void k_copy_ch8(long long P, int C, const bf16 *src, int lds, int soff, bf16 *dst, int ldd, int doff)
{
    const int c8 = C / 8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P * c8; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / c8;
        const int c = (int)(i - p * c8) * 8;
        *reinterpret_cast<uint4 *>(dst + p * ldd + doff + c) = *reinterpret_cast<const uint4 *>(src + p * lds + soff + c);
    }
}


// db[c] += sum_p g[p][c] (channels on threads, pixels split over blocks)
__global__ void k_bias_grad(long long P, int C, int ld, const bf16 *g, float *db)
{
    const int c = threadIdx.x;
    if (c >= C) return;
    const long long per = (P + gridDim.x - 1) / gridDim.x;
    const long long p0 = blockIdx.x * per, p1 = min(P, p0 + per);
    float s = 0.f;
    for (long long p = p0; p < p1; p++) s += __bfloat162float(g[p * ld + c]);
    atomicAdd(db + c, s);
}

// db[c] += sum_p g[p][c] for C % 8 == 0 and 16-byte aligned rows: a thread
// reads 8 channels of a pixel as one 16-byte word (G = C/8 channel groups,
// blockDim/G pixels per pass), sums in shared memory, and one atomic per
// channel and block goes to global memory.
__global__ void k_bias_grad8(long long P, int C, int ld, const bf16 *g, float *db)
{
    __shared__ float red[256];
    const int G = C >> 3, R = blockDim.x / G, t = threadIdx.x, cg = t % G, r = t / G;
    for (int i = t; i < C; i += blockDim.x) red[i] = 0.f;
    __syncthreads();
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (r < R)
        for (long long p = (long long)blockIdx.x * R + r; p < P; p += (long long)gridDim.x * R) {
            const uint4 v = *reinterpret_cast<const uint4 *>(g + p * ld + 8 * cg);
            const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&v);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float2 f = __bfloat1622float2(h[j]);
                s[2 * j] += f.x;
                s[2 * j + 1] += f.y;
            }
        }
    if (r < R)
#pragma unroll
        for (int j = 0; j < 8; j++) atomicAdd(&red[8 * cg + j], s[j]);
    __syncthreads();
    for (int i = t; i < C; i += blockDim.x) atomicAdd(db + i, red[i]);
}

// The activation derivative (g *= LEAK where y <= 0, in place) fused with
// the bias gradient of the masked g (db[c] += sum_p g[p][c]); layout as
// k_bias_grad8.
__global__ void k_relu_bias8(long long P, int C, int ld, const bf16 *y, bf16 *g, float *db)
{
    __shared__ float red[256];
    const int G = C >> 3, R = blockDim.x / G, t = threadIdx.x, cg = t % G, r = t / G;
    for (int i = t; i < C; i += blockDim.x) red[i] = 0.f;
    __syncthreads();
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (r < R)
        for (long long p = (long long)blockIdx.x * R + r; p < P; p += (long long)gridDim.x * R) {
            const long long o = p * ld + 8 * cg;
            float yv[8], gv[8];
            unpack8(*reinterpret_cast<const uint4 *>(y + o), yv);
            unpack8(*reinterpret_cast<const uint4 *>(g + o), gv);
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (!(yv[k] > 0.f)) gv[k] *= LEAK;
            const uint4 w = pack8(gv);
            *reinterpret_cast<uint4 *>(g + o) = w;
            unpack8(w, gv);  // the bias gradient sums the stored (BF16) values
#pragma unroll
            for (int k = 0; k < 8; k++) s[k] += gv[k];
        }
    if (r < R)
#pragma unroll
        for (int j = 0; j < 8; j++) atomicAdd(&red[8 * cg + j], s[j]);
    __syncthreads();
    for (int i = t; i < C; i += blockDim.x) atomicAdd(db + i, red[i]);
}

// The first layer (CIN input channels, 3x3, pad 1) on the CUDA cores: its
// K = 9 CIN is too small for a tensor-core GEMM to pay for an im2col.
// Forward: a thread per pixel gathers its 9 CIN inputs once and forms all
// COUT outputs from the weights in shared memory (BF16 values, exact FP32
// products, FP32 sums), bias and leaky ReLU fused, BF16 stores.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv_first(int n, int H, int W, const bf16 *x, int ldx, const bf16 *w,
                                                    int kp, const float *bias, bf16 *y, int ldy)
{
    __shared__ float sw[COUT][9 * CIN];
    __shared__ float sb[COUT];
    for (int i = threadIdx.x; i < COUT * 9 * CIN; i += blockDim.x)
        sw[i / (9 * CIN)][i % (9 * CIN)] = __bfloat162float(w[(i / (9 * CIN)) * kp + i % (9 * CIN)]);
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) sb[i] = bias ? bias[i] : 0.f;
    __syncthreads();
    const long long P = (long long)n * H * W;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const int xw = (int)(p % W), yh = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
        float acc[COUT];
#pragma unroll
        for (int j = 0; j < COUT; j++) acc[j] = sb[j];
#pragma unroll 1
        for (int tap = 0; tap < 9; tap++) {
            const int yy = yh + tap / 3 - 1, xx = xw + tap % 3 - 1;
            const bool ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
            float in[CIN];
#pragma unroll
            for (int c = 0; c < CIN; c++) in[c] = ok ? __bfloat162float(x[((b * H + yy) * W + xx) * ldx + c]) : 0.f;
#pragma unroll
            for (int j = 0; j < COUT; j++)
#pragma unroll
                for (int c = 0; c < CIN; c++) acc[j] = fmaf(sw[j][tap * CIN + c], in[c], acc[j]);
        }
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 8) {
            uint4 v;
            __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&v);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float a0 = acc[c0 + 2 * j], a1 = acc[c0 + 2 * j + 1];
                h[j] = __floats2bfloat162_rn(a0 > 0.f ? a0 : LEAK * a0, a1 > 0.f ? a1 : LEAK * a1);
            }
            *reinterpret_cast<uint4 *>(y + p * ldy + c0) = v;
        }
    }
}

// Weight gradient of the first layer: dW[co][k] += sum_p g[p][co] x_k(p)
// (k = tap * CIN + c).  A block stages 128 pixels' inputs and output
// gradients in shared memory; thread t < 3 * 8 * 9 owns the 4 x CIN block
// (co 4b .. 4b+3, tap, c = 0 .. CIN-1) over the pixels pi = t / 72 (mod 3)
// of each tile, keeping its sums in registers; at the end the three pixel
// groups are summed in shared memory and added to dW with one atomic each.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_wgrad_first(int n, int H, int W, const bf16 *x, int ldx, const bf16 *g, int ldg,
                                                     float *dw, int ldw)
{
    constexpr int K = 9 * CIN, NP = 128, NB = (COUT / 4) * 9, NG = 3;
    static_assert(NB * NG <= 256 && COUT % 4 == 0, "blocking");
    __shared__ float sx[NP][K + 1];
    __shared__ float sg[NP][COUT + 1];
    const long long P = (long long)n * H * W;
    const long long per = (P + gridDim.x - 1) / gridDim.x;
    const long long q0 = blockIdx.x * per, q1 = min(P, q0 + per);
    const int t = threadIdx.x, pg = t / NB, ob = t % NB, co0 = 4 * (ob / 9), tap = ob % 9;
    float acc[4][CIN];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < CIN; c++) acc[i][c] = 0.f;
    for (long long p0 = q0; p0 < q1; p0 += NP) {
        __syncthreads();
        // threads 0 .. NP-1 stage the inputs of pixel p0 + t (its coordinates
        // worked out once), threads NP .. 2 NP-1 its output gradients
        if (t < NP) {
            const long long p = p0 + t;
            const bool in = p < q1;
            const int xw = in ? (int)(p % W) : 0, yh = in ? (int)((p / W) % H) : 0;
            const long long b = in ? p / ((long long)W * H) : 0;
#pragma unroll
            for (int tp = 0; tp < 9; tp++) {
                const int yy = yh + tp / 3 - 1, xx = xw + tp % 3 - 1;
                const bool ok = in && yy >= 0 && yy < H && xx >= 0 && xx < W;
                const bf16 *src = x + ((b * H + yy) * W + xx) * ldx;
#pragma unroll
                for (int c = 0; c < CIN; c++) sx[t][tp * CIN + c] = ok ? __bfloat162float(src[c]) : 0.f;
            }
        } else if (t < 2 * NP) {
            const int pi = t - NP;
            const long long p = p0 + pi;
#pragma unroll
            for (int co = 0; co < COUT; co++) sg[pi][co] = p < q1 ? __bfloat162float(g[p * ldg + co]) : 0.f;
        }
        __syncthreads();
        if (pg < NG)
            for (int pi = pg; pi < NP; pi += NG) {
                float gv[4], xv[CIN];
#pragma unroll
                for (int i = 0; i < 4; i++) gv[i] = sg[pi][co0 + i];
#pragma unroll
                for (int c = 0; c < CIN; c++) xv[c] = sx[pi][tap * CIN + c];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int c = 0; c < CIN; c++) acc[i][c] = fmaf(gv[i], xv[c], acc[i][c]);
            }
    }
    // sum the pixel groups (the tiles' shared memory is free now)
    __syncthreads();
    float *part = &sx[0][0];  // NG x NB x 4 x CIN floats
    if (pg < NG)
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int c = 0; c < CIN; c++) part[((pg * NB + ob) * 4 + i) * CIN + c] = acc[i][c];
    __syncthreads();
    if (t < NB)
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int c = 0; c < CIN; c++) {
                float v = 0.f;
                for (int q = 0; q < NG; q++) v += part[((q * NB + ob) * 4 + i) * CIN + c];
                atomicAdd(dw + (co0 + i) * ldw + tap * CIN + c, v);
            }
}

// FP32 NHWC (C channels) -> BF16
__global__ void k_to_bf16(long long n, const float *x, bf16 *y)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}
// loss partials and output gradient: out (P x ldo FP32, channels [0,C)),
// target (P x C); g (P x ldg BF16, channels [0,C) = 2(out-t)/(P*C), rest 0)
__global__ void k_mse(long long P, int C, const float *out, int ldo, const float *t, bf16 *g, int ldg, double *part)
{
    double acc = 0.0;
    const float scale = (float)(2.0 / ((double)P * C));
    const long long total = P * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / C;
        const int c = (int)(i - p * C);
        const float d = out[p * ldo + c] - t[i];
        acc += (double)d * (double)d;
        g[p * ldg + c] = __float2bfloat16_rn(scale * d);
    }
    __shared__ double red[32];
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        part[blockIdx.x] = s;
    }
}
// out (P x ldo FP32) channels [0,C) -> y (P x C)
__global__ void k_take(long long P, int C, const float *out, int ldo, float *y)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P * C; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i / C;
        y[i] = out[p * ldo + (int)(i - p * C)];
    }
}
// Adam on a flat FP32 parameter vector (bias-corrected step sizes given)
__global__ void k_adam(long long n, float *w, const float *g, float *m, float *v, float lr_t, float b1, float b2,
                       float eps_t)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr_t * mi / (sqrtf(vi) + eps_t);
    }
}
// BF16 weights of a layer: W [coutp][kp] and the backward-data weights
// Wt [cin][9*coutp'] (3x3: flipped taps, cout/cin swapped; 1x1: transpose
// into [cin][32]).
__global__ void k_weights(int ks, int cin, int cout, int coutp, int kp, int ktp, const float *w, bf16 *wb, bf16 *wt)
{
    const int nw = coutp * kp;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) wb[i] = __float2bfloat16_rn(w[i]);
    if (!wt) return;
    const int nt = cin * ktp;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        const int ci = i / ktp, k = i - ci * ktp;
        float v = 0.f;
        if (ks == 3) {
            const int tap = k / coutp, co = k - tap * coutp;  // tap = ky'*3+kx'
            if (co < cout) v = w[co * kp + (8 - tap) * cin + ci];
        } else {
            if (k < cout) v = w[k * kp + ci];
        }
        wt[i] = __float2bfloat16_rn(v);
    }
}

int grid_for(long long n, int per = 256)
{
    long long g = (n + per - 1) / per;
    const long long cap = 16LL * eg::device_sm_count() * 8;
    return (int)std::max(1LL, std::min(g, cap));
}

// ------------------------------------------------------------- network
struct Layer {
    int ks, cin, cout, coutp, kp, ktp;  // ktp: K of the backward-data GEMM
    long long woff, boff;              // offsets in the flat parameter vector
    int H, W;                          // spatial size of this layer's output
    DevBuf<bf16> wb, wt;
    bool relu;
};

constexpr int NCONV = 15;

}  // namespace

struct unet {
    int H = 0, W = 0, nmax = 0, cin = 3, cout = 3;
    int ch[4] = {32, 64, 96, 128};
    Layer L[NCONV];
    long long nparam = 0;
    DevBuf<float> w, gw, m, v;       // FP32 master weights, gradients, Adam moments
    long long step = 0;
    // activations (BF16 NHWC)
    DevBuf<bf16> xin, a[NCONV], pool[3], cat[3];
    DevBuf<bf16> ga[NCONV], gpool[3], gcat[3];
    DevBuf<bf16> col, gout;
    DevBuf<float> out, tgt;
    DevBuf<double> part;
    DevBuf<int> err;  // set by a tensor-core GEMM whose bounded wait ran out
    cudaStream_t st = nullptr;
    int n_last = 0;

    ~unet()
    {
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

// layer order: e1a e1b e2a e2b e3a e3b ba bb d3a d3b d2a d2b d1a d1b out
int setup(unet *u)
{
    const int *c = u->ch;
    struct Spec { int ks, cin, cout, lvl; } spec[NCONV] = {
        {3, u->cin, c[0], 0}, {3, c[0], c[0], 0}, {3, c[0], c[1], 1}, {3, c[1], c[1], 1},
        {3, c[1], c[2], 2},   {3, c[2], c[2], 2}, {3, c[2], c[3], 3}, {3, c[3], c[3], 3},
        {3, c[3] + c[2], c[2], 2}, {3, c[2], c[2], 2}, {3, c[2] + c[1], c[1], 1}, {3, c[1], c[1], 1},
        {3, c[1] + c[0], c[0], 0}, {3, c[0], c[0], 0}, {1, c[0], u->cout, 0}};
    long long off = 0;
    for (int i = 0; i < NCONV; i++) {
        Layer &l = u->L[i];
        l.ks = spec[i].ks;
        l.cin = spec[i].cin;
        l.cout = spec[i].cout;
        l.coutp = l.ks == 1 ? 8 : l.cout;
        l.kp = l.ks == 3 ? (9 * l.cin + 31) / 32 * 32 : (l.cin + 31) / 32 * 32;
        l.ktp = l.ks == 3 ? 9 * l.coutp : 32;
        l.H = u->H >> spec[i].lvl;
        l.W = u->W >> spec[i].lvl;
        l.relu = i != NCONV - 1;
        l.woff = off;
        off += (long long)l.coutp * l.kp;
        l.boff = off;
        off += l.coutp;
        TRY(l.wb.alloc((size_t)l.coutp * l.kp));
        TRY(l.wt.alloc((size_t)l.cin * l.ktp));
    }
    u->nparam = off;
    TRY(u->w.alloc(off));
    TRY(u->gw.alloc(off));
    TRY(u->m.alloc(off));
    TRY(u->v.alloc(off));
    RTM_CUDA(cudaMemset(u->w.p, 0, off * sizeof(float)));
    RTM_CUDA(cudaMemset(u->m.p, 0, off * sizeof(float)));
    RTM_CUDA(cudaMemset(u->v.p, 0, off * sizeof(float)));
    // activations for nmax images
    const long long P0 = (long long)u->nmax * u->H * u->W;
    long long maxcol = 0;
    for (int i = 0; i < NCONV; i++) {
        const Layer &l = u->L[i];
        const long long P = (long long)u->nmax * l.H * l.W;
        TRY(u->a[i].alloc((size_t)P * l.coutp));
        TRY(u->ga[i].alloc((size_t)P * std::max(l.coutp, 32)));
        maxcol = std::max(maxcol, P * (long long)std::max(l.kp, l.ktp));
    }
    for (int k = 0; k < 3; k++) {
        const long long Pp = (long long)u->nmax * (u->H >> (k + 1)) * (u->W >> (k + 1));
        TRY(u->pool[k].alloc((size_t)Pp * c[k]));
        TRY(u->gpool[k].alloc((size_t)Pp * c[k]));
        const long long Pc = (long long)u->nmax * (u->H >> k) * (u->W >> k);
        const int cc = c[k + 1] + c[k];
        TRY(u->cat[k].alloc((size_t)Pc * cc));
        TRY(u->gcat[k].alloc((size_t)Pc * cc));
    }
    TRY(u->col.alloc((size_t)maxcol));
    TRY(u->xin.alloc((size_t)P0 * u->cin));
    TRY(u->gout.alloc((size_t)P0 * 32));
    // channels >= cout of the output gradient are never written: zero once
    RTM_CUDA(cudaMemset(u->gout.p, 0, (size_t)P0 * 32 * sizeof(bf16)));
    TRY(u->out.alloc((size_t)P0 * 8));
    TRY(u->tgt.alloc((size_t)P0 * u->cout));
    TRY(u->part.alloc(4096));
    TRY(u->err.alloc(1));
    RTM_CUDA(cudaMemset(u->err.p, 0, sizeof(int)));
    return RTM_OK;
}

int refresh_weights(unet *u)
{
    for (int i = 0; i < NCONV; i++) {
        Layer &l = u->L[i];
        k_weights<<<64, 256, 0, u->st>>>(l.ks, l.cin, l.cout, l.coutp, l.kp, l.ktp, u->w.p + l.woff, l.wb.p, l.wt.p);
        RTM_CUDA(cudaGetLastError());
    }
    return RTM_OK;
}

int im2col(unet *u, int n, int H, int W, int C, const bf16 *x, int ldx, int coff, int Kp)
{
    const long long P = (long long)n * H * W;
    if (C % 8 == 0 && ldx % 8 == 0 && coff % 8 == 0)
        k_im2col3_v8<<<grid_for(P * (Kp / 8)), 256, 0, u->st>>>(n, H, W, C, x, ldx, coff, u->col.p, Kp);
    else
        k_im2col3<<<grid_for(P * Kp), 256, 0, u->st>>>(n, H, W, C, x, ldx, coff, u->col.p, Kp);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

// GEMM A operand as the implicit im2col of an NHWC tensor (C % 32 == 0, so
// K = 9*C needs no padding and a 32-column chunk stays within one tap)
void set_implicit(GemmArgs &g, const bf16 *x, int ldx, int xoff, int C, int H, int W)
{
    g.conv = 1;
    g.X = x;
    g.ldx = ldx;
    g.xoff = xoff;
    g.C = C;
    g.H = H;
    g.W = W;
    g.A = x;
    g.lda = 0;
}

// input of conv i: (buffer, channel stride, channel offset, channels)
struct In {
    const bf16 *p;
    int ld, off, c;
};

In layer_input(unet *u, int i)
{
    const int *c = u->ch;
    switch (i) {
    case 0: return {u->xin.p, u->cin, 0, u->cin};
    case 2: return {u->pool[0].p, c[0], 0, c[0]};
    case 4: return {u->pool[1].p, c[1], 0, c[1]};
    case 6: return {u->pool[2].p, c[2], 0, c[2]};
    case 8: return {u->cat[2].p, c[3] + c[2], 0, c[3] + c[2]};
    case 10: return {u->cat[1].p, c[2] + c[1], 0, c[2] + c[1]};
    case 12: return {u->cat[0].p, c[1] + c[0], 0, c[1] + c[0]};
    default: return {u->a[i - 1].p, u->L[i - 1].coutp, 0, u->L[i].cin};
    }
}

int conv_fwd(unet *u, int i, int n)
{
    Layer &l = u->L[i];
    const In in = layer_input(u, i);
    const long long P = (long long)n * l.H * l.W;
    if (g_gemm_tc == 2 && l.ks == 3 && in.c == 3 && in.off == 0 && l.coutp == 32 && l.relu && i != NCONV - 1) {
        const int ctas = (int)std::min<long long>((P + 255) / 256, 8LL * eg::device_sm_count());
        k_conv_first<3, 32><<<ctas, 256, 0, u->st>>>(n, l.H, l.W, in.p, in.ld, l.wb.p, l.kp, u->w.p + l.boff, u->a[i].p,
                                                     l.coutp);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    }
    GemmArgs g;
    memset(&g, 0, sizeof g);
    g.err = u->err.p;
    if (l.ks == 3 && in.c % 32 == 0) {
        set_implicit(g, in.p, in.ld, in.off, in.c, l.H, l.W);
    } else if (l.ks == 3) {
        TRY(im2col(u, n, l.H, l.W, in.c, in.p, in.ld, in.off, l.kp));
        g.A = u->col.p;
        g.lda = l.kp;
    } else {
        g.A = in.p;  // 1x1: the activation is the operand (cin = 32 = kp)
        g.lda = in.ld;
    }
    g.B = l.wb.p;
    g.ldb = l.kp;
    g.M = (int)P;
    g.N = l.coutp;
    g.K = l.kp;
    g.kchunk = l.kp;
    g.bias = u->w.p + l.boff;
    if (i == NCONV - 1) {
        g.Cf = u->out.p;
        g.ldc = 8;
        return gemm(g, false, false, EPI_F32, 1, u->st);
    }
    g.relu = 1;
    g.Cb = u->a[i].p;
    g.ldc = l.coutp;
    return gemm(g, false, false, EPI_BF16, 1, u->st);
}

int forward(unet *u, int n)
{
    const int *c = u->ch;
    auto pool = [&](int k, const bf16 *src, int ld) {
        const int Ho = u->H >> (k + 1), Wo = u->W >> (k + 1);
        k_pool_fwd8<<<grid_for((long long)n * Ho * Wo * c[k] / 8), 256, 0, u->st>>>(n, Ho, Wo, c[k], src, ld, u->pool[k].p,
                                                                                   c[k]);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    };
    auto concat = [&](int k, const bf16 *low, int clow, const bf16 *skip) {
        // cat[k] = [up(low) (clow ch) | skip (c[k] ch)] at level k
        const int Hl = u->H >> (k + 1), Wl = u->W >> (k + 1), cc = clow + c[k];
        const long long P = (long long)n * (u->H >> k) * (u->W >> k);
        k_up_fwd8<<<grid_for(P * clow / 8), 256, 0, u->st>>>(n, Hl, Wl, clow, low, clow, u->cat[k].p, cc);
        RTM_CUDA(cudaGetLastError());
        k_copy_ch8<<<grid_for(P * c[k] / 8), 256, 0, u->st>>>(P, c[k], skip, c[k], 0, u->cat[k].p, cc, clow);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    };
    TRY(conv_fwd(u, 0, n));
    TRY(conv_fwd(u, 1, n));
    TRY(pool(0, u->a[1].p, c[0]));
    TRY(conv_fwd(u, 2, n));
    TRY(conv_fwd(u, 3, n));
    TRY(pool(1, u->a[3].p, c[1]));
    TRY(conv_fwd(u, 4, n));
    TRY(conv_fwd(u, 5, n));
    TRY(pool(2, u->a[5].p, c[2]));
    TRY(conv_fwd(u, 6, n));
    TRY(conv_fwd(u, 7, n));
    TRY(concat(2, u->a[7].p, c[3], u->a[5].p));
    TRY(conv_fwd(u, 8, n));
    TRY(conv_fwd(u, 9, n));
    TRY(concat(1, u->a[9].p, c[2], u->a[3].p));
    TRY(conv_fwd(u, 10, n));
    TRY(conv_fwd(u, 11, n));
    TRY(concat(0, u->a[11].p, c[1], u->a[1].p));
    TRY(conv_fwd(u, 12, n));
    TRY(conv_fwd(u, 13, n));
    TRY(conv_fwd(u, 14, n));
    return RTM_OK;
}

// gradient buffer of the input of conv i (where dX goes), channel stride
struct GIn {
    bf16 *p;
    int ld;
};
GIn layer_ginput(unet *u, int i)
{
    const int *c = u->ch;
    switch (i) {
    case 2: return {u->gpool[0].p, c[0]};
    case 4: return {u->gpool[1].p, c[1]};
    case 6: return {u->gpool[2].p, c[2]};
    case 8: return {u->gcat[2].p, c[3] + c[2]};
    case 10: return {u->gcat[1].p, c[2] + c[1]};
    case 12: return {u->gcat[0].p, c[1] + c[0]};
    default: return {u->ga[i - 1].p, u->L[i - 1].coutp};
    }
}

// backward of conv i given the gradient of its output in ga[i] (or gout for
// the last layer): relu mask, bias and weight gradients, input gradient
int conv_bwd(unet *u, int i, int n, bool need_dx)
{
    Layer &l = u->L[i];
    const long long P = (long long)n * l.H * l.W;
    const bool last = i == NCONV - 1;
    bf16 *gy = last ? u->gout.p : u->ga[i].p;
    const int ldg = last ? 32 : l.coutp;
    const bool vec = l.coutp % 8 == 0 && ldg % 8 == 0 && l.coutp <= 256;
    const int rb_ctas = (int)std::min<long long>(4LL * eg::device_sm_count(), std::max<long long>(1, P / 64));
    if (l.relu && vec) {
        k_relu_bias8<<<rb_ctas, 256, 0, u->st>>>(P, l.coutp, ldg, u->a[i].p, gy, u->gw.p + l.boff);
    } else {
        if (l.relu) {
            k_relu_mask8<<<grid_for(P * l.coutp / 8), 256, 0, u->st>>>(P, l.coutp, ldg, u->a[i].p, gy);
            RTM_CUDA(cudaGetLastError());
        }
        if (vec)
            k_bias_grad8<<<rb_ctas, 256, 0, u->st>>>(P, l.coutp, ldg, gy, u->gw.p + l.boff);
        else
            k_bias_grad<<<std::min<long long>(1024, std::max<long long>(1, P / 64)), 128, 0, u->st>>>(
                P, l.coutp, ldg, gy, u->gw.p + l.boff);
    }
    RTM_CUDA(cudaGetLastError());
    // weight gradient: dW^T[kp][coutp] = col^T[kp][P] * gy[P][coutp]
    const In in = layer_input(u, i);
    GemmArgs g;
    if (g_gemm_tc == 2 && l.ks == 3 && in.c % 32 == 0 && l.kp == 9 * in.c &&
        wgrad_tc_fits(in.c, in.ld, in.off, in.p, l.coutp, ldg, gy, l.H, l.W, P)) {
        TRY(wgrad_tc(u->gw.p + l.woff, l.kp, in.c, in.p, in.ld, in.off, l.coutp, gy, ldg, n, l.H, l.W, u->err.p,
                     u->st));
    } else if (g_gemm_tc == 2 && l.ks == 3 && in.c == 3 && in.off == 0 && l.coutp == 32) {
        k_wgrad_first<3, 32><<<4 * eg::device_sm_count(), 256, 0, u->st>>>(n, l.H, l.W, in.p, in.ld, gy, ldg,
                                                                          u->gw.p + l.woff, l.kp);
        RTM_CUDA(cudaGetLastError());
    } else {
        memset(&g, 0, sizeof g);
        g.err = u->err.p;
        if (l.ks == 3 && in.c % 32 == 0) {
            set_implicit(g, in.p, in.ld, in.off, in.c, l.H, l.W);
        } else if (l.ks == 3) {
            TRY(im2col(u, n, l.H, l.W, in.c, in.p, in.ld, in.off, l.kp));
            g.A = u->col.p;
            g.lda = l.kp;
        } else {
            g.A = in.p;
            g.lda = in.ld;
        }
        g.B = gy;
        g.ldb = ldg;
        g.M = l.kp;
        g.N = l.coutp;
        const long long Kfull = (P + 31) / 32 * 32;
        RTM_CHECK_ARG(P % 32 == 0, "pixel count %lld of a U-Net layer is not a multiple of 32", P);
        g.K = (int)Kfull;
        // split the pixel reduction so that the grid covers the SMs
        const int tiles = ((g.M + 255) / 256) * ((g.N + 31) / 32);
        int splits = (int)std::max(1LL, std::min<long long>(Kfull / 256, (4LL * eg::device_sm_count() + tiles - 1) / tiles));
        long long kc = (Kfull + splits - 1) / splits;
        kc = (kc + 31) / 32 * 32;
        splits = (int)((Kfull + kc - 1) / kc);
        g.kchunk = (int)kc;
        g.Cf = u->gw.p + l.woff;
        g.ldc = l.kp;
        TRY(gemm(g, true, true, EPI_F32_ATOMIC_T, splits, u->st));
    }
    if (!need_dx) return RTM_OK;
    // input gradient: dX[P][cin] = im2col(gy)[P][ktp] * Wt[cin][ktp]^T
    const GIn gin = layer_ginput(u, i);
    memset(&g, 0, sizeof g);
    g.err = u->err.p;
    if (l.ks == 3) {
        set_implicit(g, gy, ldg, 0, l.coutp, l.H, l.W);
    } else {
        g.A = gy;
        g.lda = ldg;
    }
    g.B = l.wt.p;
    g.ldb = l.ktp;
    g.M = (int)P;
    g.N = l.cin;
    g.K = l.ktp;
    g.kchunk = l.ktp;
    g.Cb = gin.p;
    g.ldc = gin.ld;
    return gemm(g, false, false, EPI_BF16, 1, u->st);
}

int backward(unet *u, int n)
{
    const int *c = u->ch;
    RTM_CUDA(cudaMemsetAsync(u->gw.p, 0, u->nparam * sizeof(float), u->st));
    auto split = [&](int k, int clow, bf16 *glow, bf16 *gskip) {
        // gcat[k] -> grad of the upsampled low level (into glow) and of the skip
        const int Hl = u->H >> (k + 1), Wl = u->W >> (k + 1), cc = clow + c[k];
        const long long P = (long long)n * (u->H >> k) * (u->W >> k);
        k_up_bwd8<<<grid_for((long long)n * Hl * Wl * clow / 8), 256, 0, u->st>>>(n, Hl, Wl, clow, u->gcat[k].p, cc, glow,
                                                                           clow);
        RTM_CUDA(cudaGetLastError());
        k_copy_ch8<<<grid_for(P * c[k] / 8), 256, 0, u->st>>>(P, c[k], u->gcat[k].p, cc, clow, gskip, c[k], 0);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    };
    auto pool_bwd = [&](int k, bf16 *gdst) {
        const int Ho = u->H >> (k + 1), Wo = u->W >> (k + 1);
        k_pool_bwd_add8<<<grid_for((long long)n * Ho * Wo * c[k] / 8), 256, 0, u->st>>>(n, Ho, Wo, c[k], u->gpool[k].p,
                                                                                  c[k], gdst, c[k]);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    };
    TRY(conv_bwd(u, 14, n, true));
    TRY(conv_bwd(u, 13, n, true));
    TRY(conv_bwd(u, 12, n, true));
    TRY(split(0, c[1], u->ga[11].p, u->ga[1].p));
    TRY(conv_bwd(u, 11, n, true));
    TRY(conv_bwd(u, 10, n, true));
    TRY(split(1, c[2], u->ga[9].p, u->ga[3].p));
    TRY(conv_bwd(u, 9, n, true));
    TRY(conv_bwd(u, 8, n, true));
    TRY(split(2, c[3], u->ga[7].p, u->ga[5].p));
    TRY(conv_bwd(u, 7, n, true));
    TRY(conv_bwd(u, 6, n, true));
    TRY(pool_bwd(2, u->ga[5].p));
    TRY(conv_bwd(u, 5, n, true));
    TRY(conv_bwd(u, 4, n, true));
    TRY(pool_bwd(1, u->ga[3].p));
    TRY(conv_bwd(u, 3, n, true));
    TRY(conv_bwd(u, 2, n, true));
    TRY(pool_bwd(0, u->ga[1].p));
    TRY(conv_bwd(u, 1, n, true));
    TRY(conv_bwd(u, 0, n, false));
    return RTM_OK;
}

int load_input(unet *u, const float *x, int n, int on_device)
{
    RTM_CHECK_ARG(n >= 1 && n <= u->nmax, "batch %d outside 1..%d", n, u->nmax);
    const long long cnt = (long long)n * u->H * u->W * u->cin;
    const float *src = x;
    if (!on_device) {
        RTM_CUDA(cudaMemcpyAsync(u->tgt.p, x, cnt * sizeof(float), cudaMemcpyHostToDevice, u->st));
        src = u->tgt.p;
    }
    k_to_bf16<<<grid_for(cnt), 256, 0, u->st>>>(cnt, src, u->xin.p);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

int loss_and_grad(unet *u, const float *t, int n, int on_device, double *loss)
{
    const long long P = (long long)n * u->H * u->W;
    const float *tp = t;
    if (!on_device) {
        RTM_CUDA(cudaMemcpyAsync(u->tgt.p, t, P * u->cout * sizeof(float), cudaMemcpyHostToDevice, u->st));
        tp = u->tgt.p;
    }
    const int blocks = std::min(grid_for(P * 32), 4096);
    k_mse<<<blocks, 256, 0, u->st>>>(P, u->cout, u->out.p, 8, tp, u->gout.p, 32, u->part.p);
    RTM_CUDA(cudaGetLastError());
    std::vector<double> hp(blocks);
    RTM_CUDA(cudaMemcpyAsync(hp.data(), u->part.p, blocks * sizeof(double), cudaMemcpyDeviceToHost, u->st));
    RTM_CUDA(cudaStreamSynchronize(u->st));
    double s = 0;
    for (double x : hp) s += x;
    *loss = s / ((double)P * u->cout);
    return RTM_OK;
}

}  // namespace

// ================================================================== C-ABI
extern "C" unet *unet_create(int H, int W, int max_batch, unsigned seed)
{
    if (H < 8 || W < 8 || H % 8 || W % 8 || max_batch < 1) {
        rtm_set_error("unet_create: H, W must be multiples of 8 (got %d x %d), batch >= 1", H, W);
        return nullptr;
    }
    if (eg::ensure_device()) return nullptr;
    unet *u = new unet();
    u->H = H;
    u->W = W;
    u->nmax = max_batch;
    if (setup(u) || cudaStreamCreateWithFlags(&u->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete u;
        return nullptr;
    }
    // He-normal initial weights, zero biases (host RNG, then upload)
    std::vector<float> w(u->nparam, 0.f);
    std::mt19937 rng(seed);
    for (int i = 0; i < NCONV; i++) {
        const Layer &l = u->L[i];
        const int fan_in = l.ks * l.ks * l.cin;
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / fan_in));
        for (int co = 0; co < l.cout; co++)
            for (int k = 0; k < l.ks * l.ks * l.cin; k++) w[l.woff + (long long)co * l.kp + k] = nd(rng);
    }
    if (cudaMemcpy(u->w.p, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        refresh_weights(u) || cudaStreamSynchronize(u->st) != cudaSuccess) {
        rtm_set_error("unet_create: weight upload failed");
        delete u;
        return nullptr;
    }
    return u;
}

extern "C" void unet_destroy(unet *u) { delete u; }

extern "C" long long unet_num_params(const unet *u) { return u ? u->nparam : -1; }

// info[0..8]: ks, cin, cout, coutp, kp, woff, boff, H, W of conv layer i
extern "C" int unet_layer_info(const unet *u, int i, long long *info)
{
    RTM_CHECK_ARG(u && info && i >= 0 && i < NCONV, "unet_layer_info: bad arguments");
    const Layer &l = u->L[i];
    const long long v[9] = {l.ks, l.cin, l.cout, l.coutp, l.kp, l.woff, l.boff, l.H, l.W};
    for (int k = 0; k < 9; k++) info[k] = v[k];
    return RTM_OK;
}

extern "C" int unet_get_params(const unet *u, float *w)
{
    RTM_CHECK_ARG(u && w, "null argument");
    RTM_CUDA(cudaMemcpy(w, u->w.p, u->nparam * sizeof(float), cudaMemcpyDeviceToHost));
    return RTM_OK;
}

extern "C" int unet_set_params(unet *u, const float *w)
{
    RTM_CHECK_ARG(u && w, "null argument");
    RTM_CUDA(cudaMemcpy(u->w.p, w, u->nparam * sizeof(float), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemset(u->m.p, 0, u->nparam * sizeof(float)));
    RTM_CUDA(cudaMemset(u->v.p, 0, u->nparam * sizeof(float)));
    u->step = 0;
    TRY(refresh_weights(u));
    RTM_CUDA(cudaStreamSynchronize(u->st));
    return RTM_OK;
}

namespace {
// status 4 when a tensor-core GEMM's bounded wait ran out during the call
int check_gemm_waits(unet *u)
{
    int e = 0;
    RTM_CUDA(cudaMemcpy(&e, u->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        RTM_CUDA(cudaMemset(u->err.p, 0, sizeof(int)));
        rtm_set_error("a tensor-core GEMM's wait did not complete within its time limit");
        return RTM_ERR_TIMEOUT;
    }
    return RTM_OK;
}
}  // namespace

extern "C" int unet_set_gemm(int tensor_core)
{
    RTM_CHECK_ARG(tensor_core >= 0 && tensor_core <= 2, "tensor_core must be 0, 1 or 2");
    g_gemm_tc = tensor_core;
    return RTM_OK;
}

extern "C" int unet_forward(unet *u, const float *x, int n, float *y, int on_device)
{
    RTM_CHECK_ARG(u && x && y, "null argument");
    TRY(eg::ensure_device());
    TRY(load_input(u, x, n, on_device));
    TRY(forward(u, n));
    const long long P = (long long)n * u->H * u->W;
    float *dst = y;
    if (!on_device) dst = u->tgt.p;
    k_take<<<grid_for(P * u->cout), 256, 0, u->st>>>(P, u->cout, u->out.p, 8, dst);
    RTM_CUDA(cudaGetLastError());
    if (!on_device)
        RTM_CUDA(cudaMemcpyAsync(y, u->tgt.p, P * u->cout * sizeof(float), cudaMemcpyDeviceToHost, u->st));
    RTM_CUDA(cudaStreamSynchronize(u->st));
    return check_gemm_waits(u);
}

extern "C" int unet_loss_grad(unet *u, const float *x, const float *t, int n, int on_device, double *loss, float *grad)
{
    RTM_CHECK_ARG(u && x && t && loss, "null argument");
    TRY(eg::ensure_device());
    TRY(load_input(u, x, n, on_device));
    TRY(forward(u, n));
    TRY(loss_and_grad(u, t, n, on_device, loss));
    TRY(backward(u, n));
    if (grad) RTM_CUDA(cudaMemcpyAsync(grad, u->gw.p, u->nparam * sizeof(float), cudaMemcpyDeviceToHost, u->st));
    RTM_CUDA(cudaStreamSynchronize(u->st));
    return check_gemm_waits(u);
}

extern "C" int unet_train_step(unet *u, const float *x, const float *t, int n, int on_device, float lr, float beta1,
                               float beta2, float eps, double *loss)
{
    RTM_CHECK_ARG(u && x && t && loss, "null argument");
    TRY(eg::ensure_device());
    TRY(load_input(u, x, n, on_device));
    TRY(forward(u, n));
    TRY(loss_and_grad(u, t, n, on_device, loss));
    TRY(backward(u, n));
    u->step++;
    const double bc1 = 1.0 - std::pow((double)beta1, (double)u->step);
    const double bc2 = 1.0 - std::pow((double)beta2, (double)u->step);
    // w -= lr * mhat / (sqrt(vhat) + eps)  ==  lr*sqrt(bc2)/bc1 * m / (sqrt(v) + eps*sqrt(bc2))
    const float lr_t = (float)(lr * std::sqrt(bc2) / bc1), eps_t = (float)(eps * std::sqrt(bc2));
    k_adam<<<grid_for(u->nparam), 256, 0, u->st>>>(u->nparam, u->w.p, u->gw.p, u->m.p, u->v.p, lr_t, beta1, beta2,
                                                    eps_t);
    RTM_CUDA(cudaGetLastError());
    TRY(refresh_weights(u));
    RTM_CUDA(cudaStreamSynchronize(u->st));
    return check_gemm_waits(u);
}
