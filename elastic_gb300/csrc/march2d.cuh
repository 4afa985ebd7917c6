// Forward step of the batched RTM by marching z-strips (float, fast
// arithmetic; same per-cell arithmetic as k_step2d_v2's forward).
//
// A persistent CTA per SM owns a list of runs: (shot, 128-row strip, range of
// 8-column chunks).  It walks each run left to right with the neighbour level
// held in a ring of 32 staged columns (4 chunks, 8-row aligned z halo), so a
// column is brought on chip once per strip instead of once per tile plus its
// 10-column x halo.  Every operand of a chunk -- the neighbour-level chunk
// one ahead of it, the level's own fields and the five coefficients -- is
// loaded by tensor-memory-access bulk copies that a producer warp issues two
// chunks ahead of the compute; sixteen compute warps read shared memory only
// (eight update the velocities of the chunk's eight columns, eight the
// stresses), and full/empty mbarrier pairs replace block-wide barriers.
//
//   ring  [5 fields][32 columns][144 rows]     92,160 B
//   slots [2][own 5 + coef 5][8 columns][128]  81,920 B
//
// Chunk k reads ring columns 8k-5 .. 8k+12 (chunks k-1, k, k+1).  Once chunk
// k is done the producer issues the group of chunk k+2 (ring chunk k+3 into
// the slot chunk k-1 held, own/coefficients into the slot chunk k held); the
// first group of a run (ring chunks k-1, k, k+1) waits until the previous
// run's last chunk is done.  Zeros beyond the shot come from the engine's
// zero guard columns and the tensor maps' out-of-range fill, exactly as for
// the tile kernel.  Every wait gives up after about a second and reports it
// through the error flag.
#pragma once
#include "elastic2d_v2.cuh"

namespace eg {

constexpr int MC = 8;          // columns per chunk
constexpr int MRING = 32;      // staged neighbour-level columns (power of two)
constexpr int M_CONSUMERS = 16; // compute warps: column (w & 7) of a chunk, lane l rows 4l..4l+3
constexpr int M_THREADS = (M_CONSUMERS + 1) * 32;  // + one producer warp
constexpr int M_RING = 5 * MRING * V2_LZ;   // floats
constexpr int M_SLOT = 10 * MC * V2_TZ;     // floats per own/coefficient slot
constexpr size_t M_SMEM = (size_t)(M_RING + 2 * M_SLOT) * sizeof(float) + 128 + 32;

struct MarchArgs {
    const int4 *runs;   // (shot, first row of the strip, first chunk, end chunk)
    const int *run_lo;  // CTA b walks runs [run_lo[b], run_lo[b + 1])
    int own_plane[5];   // plane (in tm_own) of field f at the level being written
    CUtensorMap tm_nb;  // level planes, box {144 rows, 8 columns, 1}
    CUtensorMap tm_own; // level planes, box {128 rows, 8 columns, 1}
    CUtensorMap tm_coef;  // coefficient planes, box {128 rows, 8 columns, 1}
};

// 4 floats of ring field f at shot column col (any, taken modulo the ring)
// and local row z (multiple of 4, -8 .. 132).
__device__ __forceinline__ float4 rl4(const float *ring, int f, int col, int z)
{
    return *reinterpret_cast<const float4 *>(ring + f * (MRING * V2_LZ) + (col & (MRING - 1)) * V2_LZ + z + V2_ZH);
}

// Forward staggered x difference of 4 outputs (rows z..z+3) at column x: the
// arithmetic of fwd_poly_x4 (fast mode).
template <bool PTYPE>
__device__ __forceinline__ void mfwd_x4(const float *ring, int f, int x, int z, float p[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int hi = PTYPE ? 5 - k : 4 - k, lo = PTYPE ? -4 + k : -5 + k;
        const float4 va = rl4(ring, f, x + hi, z), vb = rl4(ring, f, x + lo, z);
        const float c = StagCoef<float>::c(k);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float t = Ar<false>::mul(c, Ar<false>::sub(f4(va, j), f4(vb, j)));
            p[j] = k == 0 ? t : Ar<false>::add(p[j], t);
        }
    }
}
__device__ __forceinline__ void mzwin(const float *ring, int f, int x, int z, float w[20])
{
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const float4 v = rl4(ring, f, x, z - 8 + 4 * q);
        w[4 * q] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
    }
}

__device__ __forceinline__ void mbar_init_n(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"((unsigned)__cvta_generic_to_shared(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"((unsigned)__cvta_generic_to_shared(bar)) : "memory");
}

// Rank of field f among the recorded components (its trace slot).
__device__ __forceinline__ int rec_slot(int mask, int f) { return __popc(mask & ((1 << f) - 1)); }

// 17 warps put five on one SM sub-partition: at most 96 registers a thread
__global__ void __launch_bounds__(M_THREADS, 1) k_fwd_march(const __grid_constant__ Step2DArgs<float> a, const __grid_constant__ MarchArgs m)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>(smem_raw + ((128u - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127u)) & 127u));
    float *slots = ring + M_RING;
    unsigned long long *full = reinterpret_cast<unsigned long long *>(slots + 2 * M_SLOT);
    unsigned long long *empty = full + 2;
    const int r0 = m.run_lo[blockIdx.x], r1 = m.run_lo[blockIdx.x + 1];
    if (r0 >= r1) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&full[0]);
        mbar_init(&full[1]);
        mbar_init_n(&empty[0], M_CONSUMERS);
        mbar_init_n(&empty[1], M_CONSUMERS);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    if (warp == M_CONSUMERS) {
        // ---- producer: group n holds what chunk n of this CTA's walk reads
        // first (full[n & 1], own/coefficient slot n & 1); it is issued once
        // chunk n - 2 is done (chunk n - 1 for a run's first group)
        if (lane != 0) return;
        constexpr unsigned NB_BYTES = V2_LZ * MC * 4, OWN_BYTES = V2_TZ * MC * 4;
        int n = 0;
        for (int r = r0; r < r1; r++) {
            const int4 R = m.runs[r];
            const int col0 = (int)(a.shots[R.x].off / a.ldz);
            for (int k = R.z; k < R.w; k++, n++) {
                const bool first = k == R.z;
                const int done = first ? n - 1 : n - 2;
                if (done >= 0 && !mbar_wait(&empty[done & 1], (done >> 1) & 1)) {
                    if (a.err) atomicExch(a.err, 1);
                    return;
                }
                unsigned long long *bar = &full[n & 1];
                mbar_expect_tx(bar, (first ? 3u : 1u) * 5u * NB_BYTES + 10u * OWN_BYTES);
                for (int j = first ? k - 1 : k + 1; j <= k + 1; j++) {
                    const int c = col0 + j * MC, dst = ((j * MC) & (MRING - 1)) * V2_LZ;
#pragma unroll
                    for (int f = 0; f < 5; f++)
                        tma_load_3d(ring + f * (MRING * V2_LZ) + dst, &m.tm_nb, R.y - V2_ZH, c, a.nb_plane[f], bar);
                }
                float *sl = slots + (n & 1) * M_SLOT;
#pragma unroll
                for (int f = 0; f < 5; f++)
                    tma_load_3d(sl + f * (MC * V2_TZ), &m.tm_own, R.y, col0 + k * MC, m.own_plane[f], bar);
#pragma unroll
                for (int q = 0; q < 5; q++)
                    tma_load_3d(sl + (5 + q) * (MC * V2_TZ), &m.tm_coef, R.y, col0 + k * MC, q, bar);
            }
        }
        return;
    }

    // ---- consumers: warps 0-7 update Vx, Vz of column (warp & 7) of each
    // chunk, warps 8-15 the three stresses of the same column
    const bool vel = warp < 8;
    const int cl = warp & 7;
    const int z = 4 * lane;
    int i = 0;
    for (int r = r0; r < r1; r++) {
        const int4 R = m.runs[r];
        const int s = R.x;
        const ShotGeom g = a.shots[s];
        const int nz = g.nz, nx = g.nx, ldz = a.ldz;
        const int gz = R.y + z;
        const int nval = min(4, nz - gz);
        float wmax0 = 0.f, wmax1 = 0.f;
        float q0 = 0.f, q1 = 0.f;
        if (vel && a.snap_out[0]) {
            const float m0 = a.snap_max_in[2 * s], m1 = a.snap_max_in[2 * s + 1];
            q0 = m0 > 0.f ? SNAP_Q / m0 : 0.f;
            q1 = m1 > 0.f ? SNAP_Q / m1 : 0.f;
        }
        for (int k = R.z; k < R.w; k++, i++) {
            if (!mbar_wait(&full[i & 1], (i >> 1) & 1)) {
                if (lane == 0 && a.err) atomicExch(a.err, 1);
                return;
            }
            const int gx = k * MC + cl;
            if (gx < nx && gz < nz) {
                const float *sl = slots + (i & 1) * M_SLOT;
                auto sld = [&](int arr) { return *reinterpret_cast<const float4 *>(sl + arr * (MC * V2_TZ) + cl * V2_TZ + z); };
                const long long o = g.off + (long long)gx * ldz + gz;
                float p[4], w[20];
                if (vel) {
                    float v[2][4];
#pragma unroll
                    for (int f = 0; f < 2; f++) {
                        const float4 b = sld(f);
                        v[f][0] = b.x; v[f][1] = b.y; v[f][2] = b.z; v[f][3] = b.w;
                    }
                    const float4 cm1x = sld(5 + M1X), cm1z = sld(5 + M1Z);
                    // Vx: Ax (x, M, sxx) then Bx (z, P, sxz)
                    mfwd_x4<false>(ring, SXX, gx, z, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[VX][j] = Ar<false>::add(v[VX][j], Ar<false>::mul(f4(cm1x, j), p[j]));
                    mzwin(ring, SXZ, gx, z, w);
                    fwd_poly_z4<false, true>(w, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[VX][j] = Ar<false>::add(v[VX][j], Ar<false>::mul(f4(cm1x, j), p[j]));
                    // Vz: Az (x, P, sxz) then Bz (z, M, szz)
                    mfwd_x4<true>(ring, SXZ, gx, z, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[VZ][j] = Ar<false>::add(v[VZ][j], Ar<false>::mul(f4(cm1z, j), p[j]));
                    mzwin(ring, SZZ, gx, z, w);
                    fwd_poly_z4<false, false>(w, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[VZ][j] = Ar<false>::add(v[VZ][j], Ar<false>::mul(f4(cm1z, j), p[j]));
                    if (a.sponge) {
#pragma unroll
                        for (int f = 0; f < 2; f++)
#pragma unroll
                            for (int j = 0; j < 4; j++) v[f][j] = sponge_cell<false>(v[f][j], gz + j, gx, nz, nx, a.filt, a.abc2);
                    }
                    if (nval == 4) {
#pragma unroll
                        for (int f = 0; f < 2; f++)
                            *reinterpret_cast<float4 *>(a.out[f] + o) = make_float4(v[f][0], v[f][1], v[f][2], v[f][3]);
                    } else {
#pragma unroll
                        for (int f = 0; f < 2; f++)
                            for (int j = 0; j < nval; j++) a.out[f][o + j] = v[f][j];
                    }
                    if (a.rec && g.rec_iz >= gz && g.rec_iz < gz + 4) {
                        const int j = g.rec_iz - gz;
#pragma unroll
                        for (int f = 0; f < 2; f++)
                            if (a.comp_mask & (1 << f)) {
#pragma unroll
                                for (int jj = 0; jj < 4; jj++)
                                    if (jj == j)
                                        a.rec[g.doff + ((long long)a.it * a.ncomp + rec_slot(a.comp_mask, f)) * nx + gx] = v[f][jj];
                            }
                    }
                    if (a.snap_out[0]) {
                        // FP16 snapshot of the neighbour level at these cells
                        const float4 c0 = rl4(ring, VX, gx, z), c1 = rl4(ring, VZ, gx, z);
                        __half2 h[4];
                        h[0] = __floats2half2_rn(c0.x * q0, c0.y * q0);
                        h[1] = __floats2half2_rn(c0.z * q0, c0.w * q0);
                        h[2] = __floats2half2_rn(c1.x * q1, c1.y * q1);
                        h[3] = __floats2half2_rn(c1.z * q1, c1.w * q1);
                        if (nval == 4) {
                            *reinterpret_cast<uint2 *>(a.snap_out[0] + o) =
                                make_uint2(*reinterpret_cast<unsigned *>(&h[0]), *reinterpret_cast<unsigned *>(&h[1]));
                            *reinterpret_cast<uint2 *>(a.snap_out[1] + o) =
                                make_uint2(*reinterpret_cast<unsigned *>(&h[2]), *reinterpret_cast<unsigned *>(&h[3]));
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
                } else {
                    float v[3][4];  // sxx, szz, sxz
#pragma unroll
                    for (int f = 0; f < 3; f++) {
                        const float4 b = sld(2 + f);
                        v[f][0] = b.x; v[f][1] = b.y; v[f][2] = b.z; v[f][3] = b.w;
                    }
                    if (a.has_src && gx == g.src_ix && g.src_iz >= gz && g.src_iz < gz + 4) {
                        const int j = g.src_iz - gz;
#pragma unroll
                        for (int jj = 0; jj < 4; jj++)
                            if (jj == j) {
                                v[0][jj] = Ar<false>::add(v[0][jj], a.srcval);
                                v[1][jj] = Ar<false>::add(v[1][jj], a.srcval);
                            }
                    }
                    const float4 ca2 = sld(5 + A2), ca3 = sld(5 + A3), ca23 = sld(5 + A23);
                    // sxx: D (x, P, vx) with a23, szz: F (same poly) with a2
                    mfwd_x4<true>(ring, VX, gx, z, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        v[0][j] = Ar<false>::add(v[0][j], Ar<false>::mul(f4(ca23, j), p[j]));
                        v[1][j] = Ar<false>::add(v[1][j], Ar<false>::mul(f4(ca2, j), p[j]));
                    }
                    // sxx: E (z, P, vz) with a2, szz: G (same poly) with a23
                    mzwin(ring, VZ, gx, z, w);
                    fwd_poly_z4<false, true>(w, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        v[0][j] = Ar<false>::add(v[0][j], Ar<false>::mul(f4(ca2, j), p[j]));
                        v[1][j] = Ar<false>::add(v[1][j], Ar<false>::mul(f4(ca23, j), p[j]));
                    }
                    // sxz: H (z, M, vx) then J (x, M, vz), both with a3
                    mzwin(ring, VX, gx, z, w);
                    fwd_poly_z4<false, false>(w, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[2][j] = Ar<false>::add(v[2][j], Ar<false>::mul(f4(ca3, j), p[j]));
                    mfwd_x4<false>(ring, VZ, gx, z, p);
#pragma unroll
                    for (int j = 0; j < 4; j++) v[2][j] = Ar<false>::add(v[2][j], Ar<false>::mul(f4(ca3, j), p[j]));
                    if (a.sponge) {
#pragma unroll
                        for (int f = 0; f < 3; f++)
#pragma unroll
                            for (int j = 0; j < 4; j++) v[f][j] = sponge_cell<false>(v[f][j], gz + j, gx, nz, nx, a.filt, a.abc2);
                    }
                    if (nval == 4) {
#pragma unroll
                        for (int f = 0; f < 3; f++)
                            *reinterpret_cast<float4 *>(a.out[2 + f] + o) = make_float4(v[f][0], v[f][1], v[f][2], v[f][3]);
                    } else {
#pragma unroll
                        for (int f = 0; f < 3; f++)
                            for (int j = 0; j < nval; j++) a.out[2 + f][o + j] = v[f][j];
                    }
                    if (a.rec && g.rec_iz >= gz && g.rec_iz < gz + 4) {
                        const int j = g.rec_iz - gz;
#pragma unroll
                        for (int f = 0; f < 3; f++)
                            if (a.comp_mask & (1 << (2 + f))) {
#pragma unroll
                                for (int jj = 0; jj < 4; jj++)
                                    if (jj == j)
                                        a.rec[g.doff + ((long long)a.it * a.ncomp + rec_slot(a.comp_mask, 2 + f)) * nx + gx] =
                                            v[f][jj];
                            }
                    }
                }
            }
            // this warp's reads of chunk i's ring columns and slot are done
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[i & 1]);
        }
        if (vel && a.snap_out[0]) {
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
    }
}

}  // namespace eg
