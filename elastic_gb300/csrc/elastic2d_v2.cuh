// Fused 2D elastic step, version 2 (float, 16-byte aligned layouts).
//
// Same per-cell arithmetic as k_step2d (elastic2d.cuh) -- in EXACT mode the
// results are bit-identical -- with a staging and compute layout built for
// sm_103a's memory system:
//  * a tile is 128 z-rows x TX columns; its neighbour level (and, for the
//    adjoint, the coefficients and the FP16 source snapshots) is staged with
//    an 8-row aligned z halo and a 5-column x halo by cp.async (16-byte
//    chunks, hardware zero-fill outside the shot), so every byte of the tile
//    is in flight at once instead of being loaded through registers;
//  * each thread owns 4 consecutive z cells of TX/8 columns: x-stencils read
//    one 128-bit shared word per tap, z-stencils read a 20-value window in
//    five 128-bit words, own/coefficient/output traffic is float4;
//  * with twice the stage size of dynamic shared memory the CTA stages its
//    next work item while it computes the current one (two stages);
//  * fused imaging reads the FP16 snapshots as 4-half words and adds the
//    level's image terms either with per-level Kahan compensation (imgc set)
//    or into FP32 partial planes that the caller folds into compensated
//    totals every few levels (imgc null).
// Requirements (checked by the launcher): ldz % 4 == 0, 16-byte aligned
// planes, rows [nz, ldz) of staged planes zero.
#pragma once
#include "elastic2d.cuh"

namespace eg {

constexpr int V2_TZ = 128;              // tile rows (32 lanes x 4)
constexpr int V2_ZH = 8;                // aligned z halo
constexpr int V2_LZ = V2_TZ + 2 * V2_ZH;  // staged rows per column (144)

template <int TX>
struct V2 {
    static constexpr int LX = TX + 2 * HALO;        // staged columns
    static constexpr int SIZE = V2_LZ * LX;         // floats per staged array
    static constexpr int SIZEH = (SIZE + 63) / 64 * 64;  // halves per FP16 array (128-byte multiple)
    static constexpr int CHUNKS = (V2_LZ / 4) * LX; // 16-byte chunks per array
};

// Dynamic shared memory beyond the stages: 128 bytes of alignment slack (TMA
// destinations are 128-byte aligned) and two mbarriers.
constexpr int V2_SMEM_EXTRA = 128 + 16;

__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"((unsigned)__cvta_generic_to_shared(bar)));
}
// mbarrier expecting `count` arrivals per phase
__device__ __forceinline__ void mbar_init_n(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"((unsigned)__cvta_generic_to_shared(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"((unsigned)__cvta_generic_to_shared(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(bar)),
                 "r"(bytes)
                 : "memory");
}
// Wait for phase `parity` of the barrier, giving up after about a second.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    const long long t0 = clock64();
    while (true) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done) return true;
        if (clock64() - t0 > 2000000000LL) return false;
    }
}
// One 3D tile load (coordinates c0 innermost) completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int c0, int c1, int c2,
                                            unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::
            "r"((unsigned)__cvta_generic_to_shared(dst)),
        "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"((unsigned)__cvta_generic_to_shared(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int c0, int c1, unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            (unsigned)__cvta_generic_to_shared(dst)),
        "l"(tm), "r"(c0), "r"(c1), "r"((unsigned)__cvta_generic_to_shared(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *tm, int c0, int c1, int c2, int c3,
                                            unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
        "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"((unsigned)__cvta_generic_to_shared(bar))
        : "memory");
}

// Prefetch of one 3D tile box into L2 (no shared memory written).
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap *tm, int c0, int c1, int c2)
{
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];\n" ::"l"(tm), "r"(c0), "r"(c1),
                 "r"(c2)
                 : "memory");
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem, bool valid)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 8 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
// L2 eviction-priority policy for the coefficient planes, which every time
// level reads again: evict_last.
__device__ __forceinline__ unsigned long long l2_evict_last()
{
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}
__device__ __forceinline__ float4 ldg4_pol(const float *p, unsigned long long pol)
{
    float4 v;
    asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;\n"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
}

// 4 consecutive floats of array `arr` at local column x (tile coords, may be
// -5..TX+4) and local row z (multiple of 4, may be -8..V2_TZ+4).
template <int TX>
__device__ __forceinline__ float4 lds4(const float *sm, int arr, int x, int z)
{
    return *reinterpret_cast<const float4 *>(sm + arr * V2<TX>::SIZE + (x + HALO) * V2_LZ + (z + V2_ZH));
}
__device__ __forceinline__ float f4(const float4 &v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

// 20-value z window rows z-8 .. z+11 of array `arr` at column x.
template <int TX>
__device__ __forceinline__ void zwin(const float *sm, int arr, int x, int z, float w[20])
{
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const float4 v = lds4<TX>(sm, arr, x, z - 8 + 4 * q);
        w[4 * q] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
    }
}

// Forward staggered difference for 4 outputs (rows z..z+3) at column x.
// Along x: taps are float4 reads at columns x+hi / x+lo.  Along z: from the
// window w (w[8+j+o] is the value at row z+j+o).
template <bool EXACT, int TX, bool PTYPE>
__device__ __forceinline__ void fwd_poly_x4(const float *sm, int arr, int x, int z, float p[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int hi = PTYPE ? 5 - k : 4 - k, lo = PTYPE ? -4 + k : -5 + k;
        const float4 va = lds4<TX>(sm, arr, x + hi, z), vb = lds4<TX>(sm, arr, x + lo, z);
        const float c = StagCoef<float>::c(k);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float t = Ar<EXACT>::mul(c, Ar<EXACT>::sub(f4(va, j), f4(vb, j)));
            p[j] = k == 0 ? t : Ar<EXACT>::add(p[j], t);
        }
    }
}
template <bool EXACT, bool PTYPE>
__device__ __forceinline__ void fwd_poly_z4(const float w[20], float p[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int hi = PTYPE ? 5 - k : 4 - k, lo = PTYPE ? -4 + k : -5 + k;
        const float c = StagCoef<float>::c(k);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float t = Ar<EXACT>::mul(c, Ar<EXACT>::sub(w[8 + j + hi], w[8 + j + lo]));
            p[j] = k == 0 ? t : Ar<EXACT>::add(p[j], t);
        }
    }
}

// Adjoint gathers for 4 outputs.  Exact: terms (coef*c_k)*field in the
// reference order (M5: +c_k at -5+k for k=0..4, then -c_k at +4-k for
// k=4..0; P5: +c_k at -4+k, then -c_k at +5-k).  Fast: products array.
template <int TX, bool PTYPE>
__device__ __forceinline__ void adj_exact_x4(const float *sm, int ca, int fa, int x, int z, float v[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int o = PTYPE ? -4 + k : -5 + k;
        const float4 c4 = lds4<TX>(sm, ca, x + o, z), f = lds4<TX>(sm, fa, x + o, z);
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = add_rn(v[j], mul_rn(mul_rn(f4(c4, j), StagCoef<float>::c(k)), f4(f, j)));
    }
#pragma unroll
    for (int k = 4; k >= 0; k--) {
        const int o = PTYPE ? 5 - k : 4 - k;
        const float4 c4 = lds4<TX>(sm, ca, x + o, z), f = lds4<TX>(sm, fa, x + o, z);
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = sub_rn(v[j], mul_rn(mul_rn(f4(c4, j), StagCoef<float>::c(k)), f4(f, j)));
    }
}
template <bool PTYPE>
__device__ __forceinline__ void adj_exact_z4(const float cw[20], const float fw[20], float v[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int o = PTYPE ? -4 + k : -5 + k;
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = add_rn(v[j], mul_rn(mul_rn(cw[8 + j + o], StagCoef<float>::c(k)), fw[8 + j + o]));
    }
#pragma unroll
    for (int k = 4; k >= 0; k--) {
        const int o = PTYPE ? 5 - k : 4 - k;
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = sub_rn(v[j], mul_rn(mul_rn(cw[8 + j + o], StagCoef<float>::c(k)), fw[8 + j + o]));
    }
}
template <int TX, bool PTYPE>
__device__ __forceinline__ void adj_fast_x4(const float *sm, int pa, int x, int z, float v[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int op = PTYPE ? -4 + k : -5 + k, om = PTYPE ? 5 - k : 4 - k;
        const float4 a = lds4<TX>(sm, pa, x + op, z), b = lds4<TX>(sm, pa, x + om, z);
        const float c = StagCoef<float>::c(k);
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = v[j] + c * (f4(a, j) - f4(b, j));
    }
}
template <bool PTYPE>
__device__ __forceinline__ void adj_fast_z4(const float w[20], float v[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int op = PTYPE ? -4 + k : -5 + k, om = PTYPE ? 5 - k : 4 - k;
        const float c = StagCoef<float>::c(k);
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = v[j] + c * (w[8 + j + op] - w[8 + j + om]);
    }
}

// Threads per CTA: 256, or 512 for the fast kernels with TX >= 16 (one
// column per warp at TX = 16).
__host__ __device__ constexpr int v2_max_threads(bool exact) { return exact ? 256 : 512; }

template <bool ADJ, bool EXACT>
struct V2Arr {
    static constexpr int NRAW = ADJ ? 10 : 5;  // staged float arrays
};

// Shared memory of one stage of a v2 launch: NRAW float arrays (+ 2 FP16
// snapshot arrays for fused imaging, stored as halves); a multiple of 128
// bytes.
template <bool ADJ, bool EXACT, int TX>
__host__ __device__ constexpr size_t v2_smem(bool img)
{
    return (size_t)V2Arr<ADJ, EXACT>::NRAW * V2<TX>::SIZE * sizeof(float) +
           (ADJ && img ? (size_t)2 * V2<TX>::SIZEH * sizeof(__half) : 0);
}

template <typename V>
__device__ __forceinline__ float4 ld_f4(const V *p) { return *reinterpret_cast<const float4 *>(p); }

// 4 halves at (column x, rows z..z+3) of FP16 array `arr` (z multiple of 4).
template <int TX>
__device__ __forceinline__ float4 ldh4(const __half *smh, int arr, int x, int z)
{
    const uint2 u = *reinterpret_cast<const uint2 *>(smh + arr * V2<TX>::SIZEH + (x + HALO) * V2_LZ + (z + V2_ZH));
    const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

// Issue the cp.async staging of work item t into the stage at `sm`.
template <bool ADJ, int TX>
__device__ __forceinline__ void v2_stage(const Step2DArgs<float> &a, int t, float *sm, bool img, unsigned long long keep,
                                         unsigned long long *bar)
{
    constexpr int NRAW = V2Arr<ADJ, false>::NRAW;
    constexpr int SZ = V2<TX>::SIZE;
    __half *smh = reinterpret_cast<__half *>(sm + NRAW * SZ);
    const int s = find_shot<float>(a.shots, a.nshots, t);
    const ShotGeom &g = a.shots[s];
    const int lt = t - g.tile0;
    const int tz0 = (lt % g.ntz) * V2_TZ, tx0 = (lt / g.ntz) * TX;
    const int nz = g.nz, nx = g.nx, ldz = a.ldz;
    if (a.tma) {
        // one thread stages the whole tile: zeros outside the tensors come
        // from the hardware fill, zeros across shot edges from the engine's
        // guard columns
        if (threadIdx.x == 0) {
            const int c0 = tz0 - V2_ZH, c1 = (int)(g.off / ldz) + tx0 - HALO;
            constexpr unsigned FB = V2_LZ * V2<TX>::LX * 4, HB = V2_LZ * V2<TX>::LX * 2;
            mbar_expect_tx(bar, 5 * FB + (ADJ ? 5 * FB + (img ? 2 * HB : 0) : 0));
#pragma unroll
            for (int f = 0; f < 5; f++) tma_load_3d(sm + f * SZ, &a.tm[0], c0, c1, a.nb_plane[f], bar);
            if (ADJ) {
#pragma unroll
                for (int f = 0; f < 5; f++) tma_load_3d(sm + (5 + f) * SZ, &a.tm[1], c0, c1, f, bar);
                if (img) {
                    tma_load_3d(smh, &a.tm[2], c0, c1, a.snap_plane[0], bar);
                    tma_load_3d(smh + V2<TX>::SIZEH, &a.tm[2], c0, c1, a.snap_plane[1], bar);
                }
            }
        }
        return;
    }
    for (int c = threadIdx.x; c < V2<TX>::CHUNKS; c += blockDim.x) {
        const int col = c / (V2_LZ / 4), zc = c - col * (V2_LZ / 4);
        const int gx = tx0 - HALO + col, gz = tz0 - V2_ZH + 4 * zc;
        const bool ok = (gx >= 0) & (gx < nx) & (gz >= 0) & (gz < ldz);
        const long long o = ok ? g.off + (long long)gx * ldz + gz : 0;
        const int so = col * V2_LZ + 4 * zc;
#pragma unroll
        for (int f = 0; f < 5; f++) cp_async16(sm + f * SZ + so, a.nb[f] + o, ok);
        if (ADJ) {
#pragma unroll
            for (int f = 0; f < 5; f++) cp_async16(sm + (5 + f) * SZ + so, a.coef[f] + o, ok);
            if (img) {
                const bool oks = ok & (gz < nz);
                cp_async8(smh + so, a.isnap0[0] + o, oks);
                cp_async8(smh + V2<TX>::SIZEH + so, a.isnap0[1] + o, oks);
            }
        }
    }
    asm volatile("cp.async.commit_group;\n" ::);
}

template <bool EXACT, bool ADJ, int TX>
__global__ void __launch_bounds__(v2_max_threads(EXACT)) k_step2d_v2(const __grid_constant__ Step2DArgs<float> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NRAW = V2Arr<ADJ, EXACT>::NRAW;
    constexpr int SZ = V2<TX>::SIZE;
    const int cw = TX * 32 / (int)blockDim.x;  // columns per warp (blockDim.x = 32 * TX / cw)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool img = ADJ && a.img[0] != nullptr;
    // one or two stages, depending on the shared memory this launch received;
    // stages start on a 128-byte boundary, the two mbarriers follow them
    unsigned dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const size_t stage_bytes = v2_smem<ADJ, EXACT, TX>(img);
    const unsigned long long keep = l2_evict_last();
    const bool dbuf = dyn >= 2 * stage_bytes + V2_SMEM_EXTRA;
    unsigned char *base = smem_raw + ((128u - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127u)) & 127u);
    auto stage = [&](int k) { return reinterpret_cast<float *>(base + (k ? stage_bytes : 0)); };
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(base + (dbuf ? 2 : 1) * stage_bytes);
    const bool tma = a.tma != 0;
    unsigned phase = 0;  // bit k: parity of the next completion of bars[k]
    if (tma) {
        if (threadIdx.x == 0) {
            mbar_init(&bars[0]);
            mbar_init(&bars[1]);
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        __syncthreads();
    }

    int cur = 0;
    if (blockIdx.x < a.ntiles) v2_stage<ADJ, TX>(a, blockIdx.x, stage(0), img, keep, &bars[0]);
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const int tn = t + gridDim.x;
        float *sm = stage(cur);
        __half *smh = reinterpret_cast<__half *>(sm + NRAW * SZ);
        if (dbuf && tn < a.ntiles) v2_stage<ADJ, TX>(a, tn, stage(cur ^ 1), img, keep, &bars[cur ^ 1]);
        const int s = find_shot<float>(a.shots, a.nshots, t);
        const ShotGeom g = a.shots[s];
        const int lt = t - g.tile0;
        const int tz0 = (lt % g.ntz) * V2_TZ, tx0 = (lt / g.ntz) * TX;
        const long long off = g.off;
        const int nz = g.nz, nx = g.nx, ldz = a.ldz;
        const int z = 4 * lane;  // local row of this thread's 4 cells
        const int gz = tz0 + z;
        // Global operands of one column (own fields; forward: coefficients;
        // imaging: next level's snapshots).  The first column's are issued
        // before the wait for the staged tile, so their latency overlaps it.
        float4 gown[5], gcoef[5];
        uint2 gsn[2];
        auto fetch = [&](int r) {
            const int gx = tx0 + warp * cw + r;
            if (gx >= nx || gz >= nz) return false;
            const long long o = off + (long long)gx * ldz + gz;
#pragma unroll
            for (int f = 0; f < 5; f++) gown[f] = ld_f4(a.own2[f] + o);
            if (!ADJ) {
#pragma unroll
                for (int k = 0; k < 5; k++) gcoef[k] = ldg4_pol(a.coef[k] + o, keep);
            }
            if (ADJ && img && !a.ilast) {
                gsn[0] = *reinterpret_cast<const uint2 *>(a.isnap1[0] + o);
                gsn[1] = *reinterpret_cast<const uint2 *>(a.isnap1[1] + o);
            }
            if (ADJ && img && (lane & 7) == 0) {
                // the image planes are read-modified-written after the
                // column's compute: bring their lines (one per 8 lanes) to L2
#pragma unroll
                for (int i = 0; i < 3; i++) asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.img[i] + o));
            }
            return true;
        };
        bool have = fetch(0);
        if (tma) {
            const bool ok = mbar_wait(&bars[cur], (phase >> cur) & 1u);
            phase ^= 1u << cur;
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0 && a.err) atomicExch(a.err, 1);
                return;
            }
        } else {
            if (dbuf && tn < a.ntiles) {
                asm volatile("cp.async.wait_group 1;\n" ::);
            } else {
                asm volatile("cp.async.wait_group 0;\n" ::);
            }
            __syncthreads();
        }
        if (ADJ && !EXACT) {
            // products coef*field in place (slots 0..6 of the 10 raw arrays),
            // four elements per 128-bit shared access
            float4 *s4 = reinterpret_cast<float4 *>(sm);
            constexpr int SZ4 = SZ / 4;
            auto mul4 = [](float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); };
            for (int e = threadIdx.x; e < SZ4; e += blockDim.x) {
                float4 fv[5], cv[5];
#pragma unroll
                for (int f = 0; f < 5; f++) { fv[f] = s4[f * SZ4 + e]; cv[f] = s4[(5 + f) * SZ4 + e]; }
                s4[P_A23XX * SZ4 + e] = mul4(cv[A23], fv[SXX]);
                s4[P_A2ZZ * SZ4 + e] = mul4(cv[A2], fv[SZZ]);
                s4[P_A3XZ * SZ4 + e] = mul4(cv[A3], fv[SXZ]);
                s4[P_A2XX * SZ4 + e] = mul4(cv[A2], fv[SXX]);
                s4[P_A23ZZ * SZ4 + e] = mul4(cv[A23], fv[SZZ]);
                s4[P_M1XVX * SZ4 + e] = mul4(cv[M1X], fv[VX]);
                s4[P_M1ZVZ * SZ4 + e] = mul4(cv[M1Z], fv[VZ]);
            }
            __syncthreads();
        }

        float wmax0 = 0.f, wmax1 = 0.f;
#pragma unroll 1
        for (int r = 0; r < cw; r++) {
            const int x = warp * cw + r, gx = tx0 + x;
            if (r > 0) have = fetch(r);
            if (!have) continue;
            const long long o = off + (long long)gx * ldz + gz;
            const int nval = min(4, nz - gz);  // rows of this group inside the shot
            float v[5][4];
#pragma unroll
            for (int f = 0; f < 5; f++) {
                const float4 b = gown[f];
                v[f][0] = b.x; v[f][1] = b.y; v[f][2] = b.z; v[f][3] = b.w;
                if (a.inplane[f]) {
                    const float4 q = ld_f4(a.inplane[f] + o);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[f][j] = Ar<EXACT>::add(f4(q, j), v[f][j]);
                }
            }
            if (!ADJ) {
                if (a.has_src && gx == g.src_ix && g.src_iz >= gz && g.src_iz < gz + 4) {
                    const int j = g.src_iz - gz;
#pragma unroll
                    for (int jj = 0; jj < 4; jj++)
                        if (jj == j) {
                            v[SXX][jj] = Ar<EXACT>::add(v[SXX][jj], a.srcval);
                            v[SZZ][jj] = Ar<EXACT>::add(v[SZZ][jj], a.srcval);
                        }
                }
                const float4 cm1x = gcoef[M1X], cm1z = gcoef[M1Z], ca2 = gcoef[A2], ca3 = gcoef[A3], ca23 = gcoef[A23];
                float p[4], w[20];
                // Vx: Ax (x, M, sxx) then Bx (z, P, sxz)
                fwd_poly_x4<EXACT, TX, false>(sm, SXX, x, z, p);
#pragma unroll
                for (int j = 0; j < 4; j++) v[VX][j] = Ar<EXACT>::add(v[VX][j], Ar<EXACT>::mul(f4(cm1x, j), p[j]));
                zwin<TX>(sm, SXZ, x, z, w);
                fwd_poly_z4<EXACT, true>(w, p);
#pragma unroll
                for (int j = 0; j < 4; j++) v[VX][j] = Ar<EXACT>::add(v[VX][j], Ar<EXACT>::mul(f4(cm1x, j), p[j]));
                // Vz: Az (x, P, sxz) then Bz (z, M, szz)
                fwd_poly_x4<EXACT, TX, true>(sm, SXZ, x, z, p);
#pragma unroll
                for (int j = 0; j < 4; j++) v[VZ][j] = Ar<EXACT>::add(v[VZ][j], Ar<EXACT>::mul(f4(cm1z, j), p[j]));
                zwin<TX>(sm, SZZ, x, z, w);
                fwd_poly_z4<EXACT, false>(w, p);
#pragma unroll
                for (int j = 0; j < 4; j++) v[VZ][j] = Ar<EXACT>::add(v[VZ][j], Ar<EXACT>::mul(f4(cm1z, j), p[j]));
                // sxx: D (x, P, vx) with a23, szz: F (same poly) with a2
                fwd_poly_x4<EXACT, TX, true>(sm, VX, x, z, p);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    v[SXX][j] = Ar<EXACT>::add(v[SXX][j], Ar<EXACT>::mul(f4(ca23, j), p[j]));
                    v[SZZ][j] = Ar<EXACT>::add(v[SZZ][j], Ar<EXACT>::mul(f4(ca2, j), p[j]));
                }
                // sxx: E (z, P, vz) with a2, szz: G (same poly) with a23
                zwin<TX>(sm, VZ, x, z, w);
                fwd_poly_z4<EXACT, true>(w, p);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    v[SXX][j] = Ar<EXACT>::add(v[SXX][j], Ar<EXACT>::mul(f4(ca2, j), p[j]));
                    v[SZZ][j] = Ar<EXACT>::add(v[SZZ][j], Ar<EXACT>::mul(f4(ca23, j), p[j]));
                }
                // sxz: H (z, M, vx) then J (x, M, vz), both with a3
                zwin<TX>(sm, VX, x, z, w);
                fwd_poly_z4<EXACT, false>(w, p);
#pragma unroll
                for (int j = 0; j < 4; j++) v[SXZ][j] = Ar<EXACT>::add(v[SXZ][j], Ar<EXACT>::mul(f4(ca3, j), p[j]));
                fwd_poly_x4<EXACT, TX, false>(sm, VZ, x, z, p);
#pragma unroll
                for (int j = 0; j < 4; j++) v[SXZ][j] = Ar<EXACT>::add(v[SXZ][j], Ar<EXACT>::mul(f4(ca3, j), p[j]));
            } else {
                if (a.rec && g.rec_iz >= gz && g.rec_iz < gz + 4) {
                    const int j = g.rec_iz - gz;
                    int slot = 0;
#pragma unroll
                    for (int f = 0; f < 5; f++)
                        if (a.comp_mask & (1 << f)) {
                            const float d = a.rec[g.doff + ((long long)a.it * a.ncomp + slot) * nx + gx];
#pragma unroll
                            for (int jj = 0; jj < 4; jj++)
                                if (jj == j) v[f][jj] = Ar<EXACT>::add(d, v[f][jj]);
                            slot++;
                        }
                }
                if (EXACT) {
                    float cw[20], fw[20];
                    adj_exact_x4<TX, false>(sm, 5 + A23, SXX, x, z, v[VX]);
                    adj_exact_x4<TX, false>(sm, 5 + A2, SZZ, x, z, v[VX]);
                    zwin<TX>(sm, 5 + A3, x, z, cw); zwin<TX>(sm, SXZ, x, z, fw);
                    adj_exact_z4<true>(cw, fw, v[VX]);
                    zwin<TX>(sm, 5 + A2, x, z, cw); zwin<TX>(sm, SXX, x, z, fw);
                    adj_exact_z4<false>(cw, fw, v[VZ]);
                    zwin<TX>(sm, 5 + A23, x, z, cw); zwin<TX>(sm, SZZ, x, z, fw);
                    adj_exact_z4<false>(cw, fw, v[VZ]);
                    adj_exact_x4<TX, true>(sm, 5 + A3, SXZ, x, z, v[VZ]);
                    adj_exact_x4<TX, true>(sm, 5 + M1X, VX, x, z, v[SXX]);
                    zwin<TX>(sm, 5 + M1Z, x, z, cw); zwin<TX>(sm, VZ, x, z, fw);
                    adj_exact_z4<true>(cw, fw, v[SZZ]);
                    zwin<TX>(sm, 5 + M1X, x, z, cw); zwin<TX>(sm, VX, x, z, fw);
                    adj_exact_z4<false>(cw, fw, v[SXZ]);
                    adj_exact_x4<TX, false>(sm, 5 + M1Z, VZ, x, z, v[SXZ]);
                } else {
                    float w[20];
                    adj_fast_x4<TX, false>(sm, P_A23XX, x, z, v[VX]);
                    adj_fast_x4<TX, false>(sm, P_A2ZZ, x, z, v[VX]);
                    zwin<TX>(sm, P_A3XZ, x, z, w);
                    adj_fast_z4<true>(w, v[VX]);
                    adj_fast_x4<TX, true>(sm, P_A3XZ, x, z, v[VZ]);
                    zwin<TX>(sm, P_A2XX, x, z, w);
                    adj_fast_z4<false>(w, v[VZ]);
                    zwin<TX>(sm, P_A23ZZ, x, z, w);
                    adj_fast_z4<false>(w, v[VZ]);
                    adj_fast_x4<TX, true>(sm, P_M1XVX, x, z, v[SXX]);
                    zwin<TX>(sm, P_M1ZVZ, x, z, w);
                    adj_fast_z4<true>(w, v[SZZ]);
                    zwin<TX>(sm, P_M1XVX, x, z, w);
                    adj_fast_z4<false>(w, v[SXZ]);
                    adj_fast_x4<TX, false>(sm, P_M1ZVZ, x, z, v[SXZ]);
                }
            }
            if (a.sponge) {
#pragma unroll
                for (int f = 0; f < 5; f++)
#pragma unroll
                    for (int j = 0; j < 4; j++) v[f][j] = sponge_cell<EXACT>(v[f][j], gz + j, gx, nz, nx, a.filt, a.abc2);
            }
            // ---- stores (rows >= nz are never written)
            if (nval == 4) {
#pragma unroll
                for (int f = 0; f < 5; f++)
                    *reinterpret_cast<float4 *>(a.out[f] + o) = make_float4(v[f][0], v[f][1], v[f][2], v[f][3]);
            } else {
#pragma unroll
                for (int f = 0; f < 5; f++)
                    for (int j = 0; j < nval; j++) a.out[f][o + j] = v[f][j];
            }
            if (!ADJ && a.rec && g.rec_iz >= gz && g.rec_iz < gz + 4) {
                const int j = g.rec_iz - gz;
                int slot = 0;
#pragma unroll
                for (int f = 0; f < 5; f++)
                    if (a.comp_mask & (1 << f)) {
#pragma unroll
                        for (int jj = 0; jj < 4; jj++)
                            if (jj == j) a.rec[g.doff + ((long long)a.it * a.ncomp + slot) * nx + gx] = v[f][jj];
                        slot++;
                    }
            }
            if (!ADJ && a.snap_out[0]) {
                const float m0 = a.snap_max_in[2 * s], m1 = a.snap_max_in[2 * s + 1];
                const float q0 = m0 > 0.f ? SNAP_Q / m0 : 0.f, q1 = m1 > 0.f ? SNAP_Q / m1 : 0.f;
                const float4 c0 = lds4<TX>(sm, VX, x, z), c1 = lds4<TX>(sm, VZ, x, z);
                __half2 h[4];
                h[0] = __floats2half2_rn(c0.x * q0, c0.y * q0);
                h[1] = __floats2half2_rn(c0.z * q0, c0.w * q0);
                h[2] = __floats2half2_rn(c1.x * q1, c1.y * q1);
                h[3] = __floats2half2_rn(c1.z * q1, c1.w * q1);
                if (nval == 4) {
                    *reinterpret_cast<uint2 *>(a.snap_out[0] + o) = make_uint2(*reinterpret_cast<unsigned *>(&h[0]), *reinterpret_cast<unsigned *>(&h[1]));
                    *reinterpret_cast<uint2 *>(a.snap_out[1] + o) = make_uint2(*reinterpret_cast<unsigned *>(&h[2]), *reinterpret_cast<unsigned *>(&h[3]));
                } else {
                    const float cv0[4] = {c0.x, c0.y, c0.z, c0.w}, cv1[4] = {c1.x, c1.y, c1.z, c1.w};
                    for (int j = 0; j < nval; j++) {
                        a.snap_out[0][o + j] = __float2half_rn(cv0[j] * q0);
                        a.snap_out[1][o + j] = __float2half_rn(cv1[j] * q1);
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (j < nval) {
                        wmax0 = fmaxf(wmax0, fabsf(v[VX][j]));
                        wmax1 = fmaxf(wmax1, fabsf(v[VZ][j]));
                    }
            }
            if (img) {
                // imaging condition of level it (W/image-mod-rtm.f90:146-162)
                // on the dequantised source snapshots: x taps are 8-byte
                // reads of 4 halves, z taps come from a 20-row window
                const float d0 = a.imax0[2 * s] * (1.0f / SNAP_Q), d1 = a.imax0[2 * s + 1] * (1.0f / SNAP_Q);
                float wx[20], wz[20];  // z windows of source Vx and Vz, rows z-8..z+11 (raw halves)
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    const float4 tx_ = ldh4<TX>(smh, 0, x, z - 8 + 4 * q), tz_ = ldh4<TX>(smh, 1, x, z - 8 + 4 * q);
                    wx[4 * q] = tx_.x; wx[4 * q + 1] = tx_.y; wx[4 * q + 2] = tx_.z; wx[4 * q + 3] = tx_.w;
                    wz[4 * q] = tz_.x; wz[4 * q + 1] = tz_.y; wz[4 * q + 2] = tz_.z; wz[4 * q + 3] = tz_.w;
                }
                float p4[4] = {0.f, 0.f, 0.f, 0.f}, p7[4] = {0.f, 0.f, 0.f, 0.f};  // x taps: Vx (P), Vz (M)
#pragma unroll
                for (int k = 0; k < 5; k++) {
                    const float c = StagCoef<float>::c(k);
                    const float4 ap = ldh4<TX>(smh, 0, x + 5 - k, z), am = ldh4<TX>(smh, 0, x - 4 + k, z);
                    const float4 bp = ldh4<TX>(smh, 1, x + 4 - k, z), bm = ldh4<TX>(smh, 1, x - 5 + k, z);
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        p4[j] += c * (f4(ap, j) - f4(am, j));
                        p7[j] += c * (f4(bp, j) - f4(bm, j));
                    }
                }
                float s1[4] = {0.f, 0.f, 0.f, 0.f}, s2[4] = {0.f, 0.f, 0.f, 0.f};
                if (!a.ilast) {
                    const float e0 = a.imax1[2 * s] * (1.0f / SNAP_Q), e1 = a.imax1[2 * s + 1] * (1.0f / SNAP_Q);
                    const uint2 u0 = gsn[0], u1 = gsn[1];
                    const float2 a0 = __half22float2(*reinterpret_cast<const __half2 *>(&u0.x));
                    const float2 a1 = __half22float2(*reinterpret_cast<const __half2 *>(&u0.y));
                    const float2 b0 = __half22float2(*reinterpret_cast<const __half2 *>(&u1.x));
                    const float2 b1 = __half22float2(*reinterpret_cast<const __half2 *>(&u1.y));
                    const float nx4[4] = {a0.x, a0.y, a1.x, a1.y}, nz4[4] = {b0.x, b0.y, b1.x, b1.y};
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        s1[j] = a.inv_dt * (nx4[j] * e0 - wx[8 + j] * d0);
                        s2[j] = a.inv_dt * (nz4[j] * e1 - wz[8 + j] * d1);
                    }
                }
                float tt[3][4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int cz = gz + j;
                    float s4 = 0.f, s5 = 0.f, s6 = 0.f;
                    if (cz >= 4 && cz <= nz - 6 && gx >= 4 && gx <= nx - 6) {
                        float p5 = 0.f;
#pragma unroll
                        for (int k = 0; k < 5; k++) p5 += StagCoef<float>::c(k) * (wz[8 + j + 5 - k] - wz[8 + j - 4 + k]);
                        s4 = p4[j] * d0 * a.inv_dx;
                        s5 = p5 * d1 * a.inv_dx;
                    }
                    if (cz >= 5 && cz <= nz - 6 && gx >= 5 && gx <= nx - 6) {
                        float p6 = 0.f;
#pragma unroll
                        for (int k = 0; k < 5; k++) p6 += StagCoef<float>::c(k) * (wx[8 + j + 4 - k] - wx[8 + j - 5 + k]);
                        s6 = (p6 * d0 + p7[j] * d1) * a.inv_dx;
                    }
                    const float s3 = s4 + s5;
                    tt[0][j] = v[VX][j] * s1[j] + v[VZ][j] * s2[j];
                    tt[1][j] = -(v[SXX][j] + v[SZZ][j]) * s3;
                    tt[2][j] = -(2.f * v[SXX][j] * s4 + 2.f * v[SZZ][j] * s5 + v[SXZ][j] * s6);
                }
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    if (a.imgc[i] && nval == 4) {
                        // per-level Kahan compensation
                        float4 sv = ld_f4(a.img[i] + o), cv = ld_f4(a.imgc[i] + o);
                        float sa[4] = {sv.x, sv.y, sv.z, sv.w}, ca[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const float y = tt[i][j] - ca[j];
                            const float tsum = sa[j] + y;
                            ca[j] = (tsum - sa[j]) - y;
                            sa[j] = tsum;
                        }
                        *reinterpret_cast<float4 *>(a.img[i] + o) = make_float4(sa[0], sa[1], sa[2], sa[3]);
                        *reinterpret_cast<float4 *>(a.imgc[i] + o) = make_float4(ca[0], ca[1], ca[2], ca[3]);
                    } else if (a.imgc[i]) {
                        for (int j = 0; j < nval; j++) {
                            float sj = a.img[i][o + j], cj = a.imgc[i][o + j];
                            const float y = tt[i][j] - cj;
                            const float tsum = sj + y;
                            cj = (tsum - sj) - y;
                            a.img[i][o + j] = tsum;
                            a.imgc[i][o + j] = cj;
                        }
                    } else if (nval == 4) {
                        // FP32 partial sums, folded into compensated totals
                        // by the caller every few levels
                        float4 sv = ld_f4(a.img[i] + o);
                        sv.x += tt[i][0]; sv.y += tt[i][1]; sv.z += tt[i][2]; sv.w += tt[i][3];
                        *reinterpret_cast<float4 *>(a.img[i] + o) = sv;
                    } else {
                        for (int j = 0; j < nval; j++) a.img[i][o + j] += tt[i][j];
                    }
                }
            }
        }
        if (!ADJ && a.snap_out[0]) {
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                wmax0 = fmaxf(wmax0, __shfl_xor_sync(0xffffffffu, wmax0, d));
                wmax1 = fmaxf(wmax1, __shfl_xor_sync(0xffffffffu, wmax1, d));
            }
            if (lane == 0) {
                atomic_max_abs(a.snap_max_out + 2 * s, wmax0);
                atomic_max_abs(a.snap_max_out + 2 * s + 1, wmax1);
            }
        }
        // the stage is free for the next tile's loads; the fast adjoint wrote
        // its products into it, and those generic-proxy writes are ordered
        // before the next async-proxy (TMA) writes
        if (tma && ADJ && !EXACT) asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        cur ^= dbuf ? 1 : 0;
        if (!dbuf && tn < a.ntiles) v2_stage<ADJ, TX>(a, tn, stage(0), img, keep, &bars[0]);
    }
}

}  // namespace eg
