// Steps of the batched RTM by marching z-strips (float, fast arithmetic).
//
// Forward (k_fwd_march, same per-cell arithmetic as k_step2d_v2's forward):
// a persistent CTA per SM owns a list of runs -- (shot, 128-row strip, range
// of 8-column chunks) -- and walks each run left to right with the
// neighbour level held in a ring of 32 staged columns (4 chunks, 8-row
// aligned z halo), so a column is brought on chip once per strip instead of
// once per tile plus its 10-column x halo.  Every operand of a chunk -- the
// neighbour-level chunk one ahead of it, the level's own fields and the five
// coefficients -- is loaded by tensor-memory-access bulk copies that a
// producer warp issues two chunks ahead of the compute (and prefetches to L2
// one chunk further); sixteen compute warps read shared memory only (eight
// update the velocities of the chunk's eight columns, eight the stresses),
// and full/empty mbarrier pairs replace block-wide barriers.
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
constexpr int M_WARPS = 16;  // compute warps: column (w & 7) of a chunk, lane l rows 4l..4l+3
constexpr int M_FWD_THREADS = (M_WARPS + 1) * 32;  // forward: + one producer warp
constexpr int M_THREADS = M_WARPS * 32;            // adjoint: the last warp out issues
constexpr int M_RING = 5 * MRING * V2_LZ;   // floats
constexpr int M_SLOT = 10 * MC * V2_TZ;     // floats per own/coefficient slot
constexpr size_t M_SMEM = (size_t)(M_RING + 2 * M_SLOT) * sizeof(float) + 128 + 64;  // + barriers, cursor

struct MarchArgs {
    const int4 *runs;   // (shot, first row of the strip, first chunk, end chunk)
    const int *run_lo;  // CTA b walks runs [run_lo[b], run_lo[b + 1])
    int own_plane[5];   // plane (in tm_own) of field f at the level being written
    // test hook (null in normal use): a device flag that nothing sets; the
    // producer waits on it before issuing any copy, so the wait runs out,
    // the kernel reports it through the error flag and no copy is in flight
    const int *stall;
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

// Programmatic dependent launch: the next level's launch may start on SMs
// this one has left; it initialises its barriers, then waits here until the
// previous grid has completed and its writes are visible, before any global
// load or store.  It lets its own dependents launch only after that wait, so
// the level two steps back is complete before anyone reads it.
__device__ __forceinline__ void wait_previous_level()
{
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}


// Rank of field f among the recorded components (its trace slot).
__device__ __forceinline__ int rec_slot(int mask, int f) { return __popc(mask & ((1 << f) - 1)); }

// Arrive on a step's barrier (one arrival per warp); true for the warp whose
// arrival completes the phase (the pending count before it was 1), which
// then issues the tensor-map copies that the step released -- no warp waits
// to issue.  Its wait on the completed phase returns at once and orders the
// other warps' work (the issue cursor they advanced) before its own.
__device__ __forceinline__ bool last_arrival(unsigned long long *bar, unsigned parity)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    unsigned pend;
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%1];\n"
                 " mbarrier.pending_count.b64 %0, st;\n}\n"
                 : "=r"(pend)
                 : "r"(a)
                 : "memory");
    if (pend != 1) return false;
    return mbar_wait(bar, parity);
}

// 17 warps put five on one SM sub-partition: at most 96 registers a thread
__global__ void __launch_bounds__(M_FWD_THREADS, 1) k_fwd_march(const __grid_constant__ Step2DArgs<float> a, const __grid_constant__ MarchArgs m)
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
        mbar_init_n(&empty[0], M_WARPS);
        mbar_init_n(&empty[1], M_WARPS);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (warp != M_WARPS) wait_previous_level();

    if (warp == M_WARPS) {
        // ---- producer: group n holds what chunk n of this CTA's walk reads
        // first (full[n & 1], own/coefficient slot n & 1); it is issued once
        // chunk n - 2 is done (chunk n - 1 for a run's first group)
        if (lane != 0) return;
        if (m.stall) {
            const long long t0 = clock64();
            while (*reinterpret_cast<const volatile int *>(m.stall) == 0) {
                if (clock64() - t0 > 2000000000LL) {
                    if (a.err) atomicExch(a.err, 1);
                    return;  // nothing issued: the consumers' waits run out too
                }
            }
        }
        constexpr unsigned NB_BYTES = V2_LZ * MC * 4, OWN_BYTES = V2_TZ * MC * 4;
        {
            // group 0's own fields (written two levels back) and coefficients
            // go out before the wait for the previous level
            const int4 R = m.runs[r0];
            const int col0 = (int)(a.shots[R.x].off / a.ldz);
            mbar_expect_tx(&full[0], 3u * 5u * NB_BYTES + 10u * OWN_BYTES);
#pragma unroll
            for (int f = 0; f < 5; f++) tma_load_3d(slots + f * (MC * V2_TZ), &m.tm_own, R.y, col0 + R.z * MC, m.own_plane[f], &full[0]);
#pragma unroll
            for (int q = 0; q < 5; q++)
                tma_load_3d(slots + (5 + q) * (MC * V2_TZ), &m.tm_coef, R.y, col0 + R.z * MC, q, &full[0]);
        }
        wait_previous_level();
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
                if (n > 0) mbar_expect_tx(bar, (first ? 3u : 1u) * 5u * NB_BYTES + 10u * OWN_BYTES);
                for (int j = first ? k - 1 : k + 1; j <= k + 1; j++) {
                    const int c = col0 + j * MC, dst = ((j * MC) & (MRING - 1)) * V2_LZ;
#pragma unroll
                    for (int f = 0; f < 5; f++)
                        tma_load_3d(ring + f * (MRING * V2_LZ) + dst, &m.tm_nb, R.y - V2_ZH, c, a.nb_plane[f], bar);
                }
                if (n > 0) {
                    float *sl = slots + (n & 1) * M_SLOT;
#pragma unroll
                    for (int f = 0; f < 5; f++)
                        tma_load_3d(sl + f * (MC * V2_TZ), &m.tm_own, R.y, col0 + k * MC, m.own_plane[f], bar);
#pragma unroll
                    for (int q = 0; q < 5; q++)
                        tma_load_3d(sl + (5 + q) * (MC * V2_TZ), &m.tm_coef, R.y, col0 + k * MC, q, bar);
                }
                // the group two chunks further on, to L2: its loads then
                // wait on L2 rather than HBM latency
                if (k + 2 < R.w) {
#pragma unroll
                    for (int f = 0; f < 5; f++) tma_prefetch_3d(&m.tm_nb, R.y - V2_ZH, col0 + (k + 3) * MC, a.nb_plane[f]);
#pragma unroll
                    for (int f = 0; f < 5; f++) tma_prefetch_3d(&m.tm_own, R.y, col0 + (k + 2) * MC, m.own_plane[f]);
#pragma unroll
                    for (int q = 0; q < 5; q++) tma_prefetch_3d(&m.tm_coef, R.y, col0 + (k + 2) * MC, q);
                }
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

// ---------------------------------------------------------------------------
// Adjoint step with the fused imaging condition, by marching z-strips (fast
// arithmetic, FP32 partial image planes; the operator of k_step2d_v2's fast
// adjoint).
//
// The adjoint stencils read coefficient x field products of the level above
// at x and z offsets up to 5, so the CTA keeps those products in a ring of
// 32 columns (4 chunks) and the level's FP16 source snapshots in a second
// ring.  The two pairs of products that share a stencil are summed before
// they are differenced (a23*sxx + a2*szz under the x difference of Vx,
// a2*sxx + a23*szz under the z difference of Vz): the same operator, rounded
// differently from the tile kernel, which differences each product.  Per
// chunk, the raw fields, coefficients and FP16 snapshots (144 rows x 8
// columns each) land in one of two landing slots; the sixteen warps turn a
// slot into the chunk's products and snapshot-ring columns one chunk ahead
// of need, then update the chunk's cells (warps 0-7 the velocities and the
// Vx/Vz image term, warps 8-15 the stresses and the lambda/mu terms).  Own
// fields, next-level snapshots and image partials are read from global
// memory at the end of the previous chunk, their lines prefetched to L2 two
// chunks ahead.
//
//   products ring [5][32 columns][144 rows] floats      92,160 B
//   snapshot ring [2][32 columns][144 rows] halves      18,432 B
//   landing slots 2 x ([10][8][144] floats + [2][8][144] halves)  101,376 B
//
// Order (per run of n chunks k0 .. k0+n-1): product passes of chunks k0-1,
// k0, k0+1, then for each chunk k: wait until every warp has its products
// through chunk k+1 (pd), compute k, signal (cd), and -- once chunk k-1 is
// computed by every warp -- the product pass of chunk k+2 into the ring
// slot of chunk k-2.  The warp whose arrival completes a product pass loads
// the pass two ahead into the landing slot that pass freed (runs follow one
// another: the landing slots are all a load writes).
struct MarchAdjArgs {
    const int4 *runs;
    const int *run_lo;
    CUtensorMap tm_nb;    // adjoint level planes, box {144 rows, 8 columns, 1}
    CUtensorMap tm_coef;  // coefficient planes, box {144 rows, 8 columns, 1}
    CUtensorMap tm_snap;  // FP16 snapshot planes, box {144 rows, 8 columns, 1}
};

// products kept in the ring: the two pairs that share a stencil are summed
enum { Q_X = 0,    // a23*sxx + a2*szz   (Vx, x differences)
       Q_A3 = 1,   // a3*sxz             (Vx z, Vz x)
       Q_Z = 2,    // a2*sxx + a23*szz   (Vz, z differences)
       Q_M1X = 3,  // m1x*vx             (sxx x, sxz z)
       Q_M1Z = 4,  // m1z*vz             (szz z, sxz x)
       MA_NQ = 5 };
constexpr int MA_PROD = MA_NQ * MRING * V2_LZ;  // floats
constexpr int MA_SNAP = 2 * MRING * V2_LZ;      // halves
// one landing slot: 10 float arrays (fields, coefficients) + 2 half arrays
// (snapshots), [8 columns][144 rows] each, in floats
constexpr int MA_LSLOT = 10 * MC * V2_LZ + MC * V2_LZ;
constexpr size_t MA_SMEM = (size_t)MA_PROD * 4 + (size_t)MA_SNAP * 2 + (size_t)2 * MA_LSLOT * 4 + 128 + 96;

// 4 halves of snapshot ring field f at shot column col, rows z..z+3
__device__ __forceinline__ float4 rh4(const __half *ring, int f, int col, int z)
{
    const uint2 u = *reinterpret_cast<const uint2 *>(ring + f * (MRING * V2_LZ) + (col & (MRING - 1)) * V2_LZ + z + V2_ZH);
    const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}
// adj_fast_x4 on the products ring
template <bool PTYPE>
__device__ __forceinline__ void madj_x4(const float *ring, int pa, int x, int z, float v[4])
{
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int op = PTYPE ? -4 + k : -5 + k, om = PTYPE ? 5 - k : 4 - k;
        const float4 a = rl4(ring, pa, x + op, z), b = rl4(ring, pa, x + om, z);
        const float c = StagCoef<float>::c(k);
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = v[j] + c * (f4(a, j) - f4(b, j));
    }
}

__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(n) : "memory"); }

__global__ void __launch_bounds__(M_THREADS, 1)
    k_adj_march(const __grid_constant__ Step2DArgs<float> a, const __grid_constant__ MarchAdjArgs m)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *prod = reinterpret_cast<float *>(smem_raw + ((128u - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127u)) & 127u));
    __half *snap = reinterpret_cast<__half *>(prod + MA_PROD);
    float *land = reinterpret_cast<float *>(snap + MA_SNAP);  // two landing slots
    unsigned long long *lfull = reinterpret_cast<unsigned long long *>(land + 2 * MA_LSLOT);
    unsigned long long *pd = lfull + 2, *cd = lfull + 4;
    // issue cursor: run, pass of the run, passes issued, and the run's first
    // column, first row, first chunk, chunk count
    int *cur = reinterpret_cast<int *>(lfull + 6);
    const int r0 = m.run_lo[blockIdx.x], r1 = m.run_lo[blockIdx.x + 1];
    if (r0 >= r1) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto fail = [&]() {
        if (lane == 0 && a.err) atomicExch(a.err, 1);
    };
    constexpr unsigned NB_BYTES = V2_LZ * MC * 4, SN_BYTES = V2_LZ * MC * 2;
    // landing group of the cursor's product pass P: raw fields,
    // coefficients and FP16 snapshots of its chunk into landing slot P & 1;
    // then the cursor moves to the next pass (runs follow one another: the
    // landing slots are the only thing a group writes)
    auto load_run = [&](int r) {
        const int4 R = m.runs[r];
        cur[0] = r;
        cur[1] = 0;
        cur[3] = (int)(a.shots[R.x].off / a.ldz);
        cur[4] = R.y;
        cur[5] = R.z;
        cur[6] = R.w - R.z;
    };
    auto issue_next = [&]() {
        const int row0 = cur[4] - V2_ZH, col0 = cur[3];
        const int j = cur[5] - 1 + cur[1], c = col0 + j * MC;
        const int slot = cur[2] & 1;
        float *ls = land + slot * MA_LSLOT;
        __half *lh = reinterpret_cast<__half *>(ls + 10 * MC * V2_LZ);
        unsigned long long *bar = &lfull[slot];
        mbar_expect_tx(bar, 10u * NB_BYTES + 2u * SN_BYTES);
#pragma unroll
        for (int f = 0; f < 5; f++) tma_load_3d(ls + f * (MC * V2_LZ), &m.tm_nb, row0, c, a.nb_plane[f], bar);
#pragma unroll
        for (int q = 0; q < 5; q++) tma_load_3d(ls + (5 + q) * (MC * V2_LZ), &m.tm_coef, row0, c, q, bar);
#pragma unroll
        for (int f = 0; f < 2; f++) tma_load_3d(lh + f * (MC * V2_LZ), &m.tm_snap, row0, c, a.snap_plane[f], bar);
        cur[2]++;
        if (++cur[1] > cur[6] + 1) {
            if (cur[0] + 1 < r1) load_run(cur[0] + 1);
            else cur[0] = r1;
        }
    };
    if (threadIdx.x == 0) {
        for (int q = 0; q < 2; q++) {
            mbar_init(&lfull[q]);
            mbar_init_n(&pd[q], M_WARPS);
            mbar_init_n(&cd[q], M_WARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        load_run(r0);
        cur[2] = 0;
    }
    __syncthreads();
    wait_previous_level();
    if (threadIdx.x == 0) {
        issue_next();
        if (cur[0] < r1) issue_next();
    }

    // ---- compute warps
    const bool vel = warp < 8;
    const int cl = warp & 7;
    const int z = 4 * lane;
    int P = 0, C = 0;  // product passes and chunk computes of this CTA so far
    // product pass P (chunk j): landing slot P & 1 -> products ring and
    // snapshot ring
    auto products = [&](int j) -> bool {
        if (!mbar_wait(&lfull[P & 1], (P >> 1) & 1)) return false;
        const int t = threadIdx.x;
        constexpr int NQ = V2_LZ / 4;  // 16-byte row groups per column
        if (t < MC * NQ) {
            const int col = t / NQ, rq = t - col * NQ;
            const float *ls = land + (P & 1) * MA_LSLOT;
            const float4 *L4 = reinterpret_cast<const float4 *>(ls) + col * NQ + rq;
            constexpr int A4 = MC * V2_LZ / 4;  // float4 per landing array
            float4 fv[5], cv[5];
#pragma unroll
            for (int f = 0; f < 5; f++) {
                fv[f] = L4[f * A4];
                cv[f] = L4[(5 + f) * A4];
            }
            auto mul4 = [](float4 x, float4 y) { return make_float4(x.x * y.x, x.y * y.y, x.z * y.z, x.w * y.w); };
            auto add4 = [](float4 x, float4 y) { return make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w); };
            constexpr int R4 = MRING * V2_LZ / 4;  // float4 per ring array
            const int rc = ((j * MC + col) & (MRING - 1)) * NQ + rq;
            float4 *P4 = reinterpret_cast<float4 *>(prod) + rc;
            P4[Q_X * R4] = add4(mul4(cv[A23], fv[SXX]), mul4(cv[A2], fv[SZZ]));
            P4[Q_A3 * R4] = mul4(cv[A3], fv[SXZ]);
            P4[Q_Z * R4] = add4(mul4(cv[A2], fv[SXX]), mul4(cv[A23], fv[SZZ]));
            P4[Q_M1X * R4] = mul4(cv[M1X], fv[VX]);
            P4[Q_M1Z * R4] = mul4(cv[M1Z], fv[VZ]);
            // the chunk's FP16 snapshots into their ring
            const uint2 *LH = reinterpret_cast<const uint2 *>(ls + 10 * MC * V2_LZ) + col * NQ + rq;
            uint2 *S2 = reinterpret_cast<uint2 *>(snap) + rc;
#pragma unroll
            for (int f = 0; f < 2; f++) S2[f * R4] = LH[f * A4];
        }
        __syncwarp();
        // landing slot P & 1 is free once every warp is out: the last one
        // loads pass P + 2 into it
        if (lane == 0 && last_arrival(&pd[P & 1], (P >> 1) & 1) && cur[0] < r1) issue_next();
        P++;
        return true;
    };

    for (int r = r0; r < r1; r++) {
        const int4 R = m.runs[r];
        const int s = R.x, k0 = R.z, n = R.w - R.z;
        const ShotGeom g = a.shots[s];
        const int nz = g.nz, nx = g.nx, ldz = a.ldz;
        const int gz = R.y + z;
        const int nval = min(4, nz - gz);
        if (r > r0) named_sync(1, M_THREADS);  // the previous run's chunks are all computed
        const int P0 = P, C0 = C;
        for (int pl = 0; pl < 3; pl++)
            if (!products(k0 - 1 + pl)) return fail();
        const float d0 = a.imax0[2 * s] * (1.0f / SNAP_Q), d1 = a.imax0[2 * s + 1] * (1.0f / SNAP_Q);
        // global operands of a chunk (own fields, image partials, next-level
        // snapshots): loaded at the end of the previous chunk's iteration,
        // into registers its compute no longer needs
        float4 own[3], im[2];
        uint2 sn1[2];
        auto fetch = [&](int c) {
            const int gx = (k0 + c) * MC + cl;
            if (c >= n || gx >= nx || gz >= nz) return;
            const long long o = g.off + (long long)gx * ldz + gz;
            if (vel) {
                own[0] = ld_f4(a.own2[VX] + o);
                own[1] = ld_f4(a.own2[VZ] + o);
                im[0] = ld_f4(a.img[0] + o);
                if (!a.ilast) {
                    sn1[0] = *reinterpret_cast<const uint2 *>(a.isnap1[0] + o);
                    sn1[1] = *reinterpret_cast<const uint2 *>(a.isnap1[1] + o);
                }
            } else {
#pragma unroll
                for (int f = 0; f < 3; f++) own[f] = ld_f4(a.own2[SXX + f] + o);
                im[0] = ld_f4(a.img[1] + o);
                im[1] = ld_f4(a.img[2] + o);
            }
        };
        fetch(0);
        for (int c = 0; c < n; c++) {
            const int gx = (k0 + c) * MC + cl;
            const bool live = gx < nx && gz < nz;
            const long long o = g.off + (long long)gx * ldz + gz;
            {
                // the global operands of the chunk after next to L2 (one
                // lane per 128-byte line), so their loads are L2 hits
                const int gx1 = gx + 2 * MC;
                if (c + 2 < n && gx1 < nx && gz < nz && (lane & 7) == 0) {
                    const long long o1 = g.off + (long long)gx1 * ldz + gz;
                    if (vel) {
                        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.own2[VX] + o1));
                        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.own2[VZ] + o1));
                        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.img[0] + o1));
                        if (!a.ilast && (lane & 15) == 0) {
                            asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.isnap1[0] + o1));
                            asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.isnap1[1] + o1));
                        }
                    } else {
#pragma unroll
                        for (int f = 0; f < 3; f++) asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.own2[SXX + f] + o1));
                        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.img[1] + o1));
                        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a.img[2] + o1));
                    }
                }
            }
            const int Q = P0 + c + 2;  // product pass of chunk k0 + c + 1
            if (!mbar_wait(&pd[Q & 1], (Q >> 1) & 1)) return fail();
            if (live) {
                float w[20];
                if (vel) {
                    float v[2][4];
#pragma unroll
                    for (int f = 0; f < 2; f++) {
                        v[f][0] = own[f].x; v[f][1] = own[f].y; v[f][2] = own[f].z; v[f][3] = own[f].w;
                    }
                    if (a.rec && g.rec_iz >= gz && g.rec_iz < gz + 4) {
                        const int j = g.rec_iz - gz;
#pragma unroll
                        for (int f = 0; f < 2; f++)
                            if (a.comp_mask & (1 << f)) {
                                const float d = a.rec[g.doff + ((long long)a.it * a.ncomp + rec_slot(a.comp_mask, f)) * nx + gx];
#pragma unroll
                                for (int jj = 0; jj < 4; jj++)
                                    if (jj == j) v[f][jj] = Ar<false>::add(d, v[f][jj]);
                            }
                    }
                    madj_x4<false>(prod, Q_X, gx, z, v[VX]);
                    mzwin(prod, Q_A3, gx, z, w);
                    adj_fast_z4<true>(w, v[VX]);
                    madj_x4<true>(prod, Q_A3, gx, z, v[VZ]);
                    mzwin(prod, Q_Z, gx, z, w);
                    adj_fast_z4<false>(w, v[VZ]);
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
                    // imaging, Vx/Vz term (W/image-mod-rtm.f90:146-162)
                    float s1[4] = {0.f, 0.f, 0.f, 0.f}, s2[4] = {0.f, 0.f, 0.f, 0.f};
                    if (!a.ilast) {
                        const float e0 = a.imax1[2 * s] * (1.0f / SNAP_Q), e1 = a.imax1[2 * s + 1] * (1.0f / SNAP_Q);
                        const float4 wx8 = rh4(snap, 0, gx, z), wz8 = rh4(snap, 1, gx, z);
                        const float2 a0 = __half22float2(*reinterpret_cast<const __half2 *>(&sn1[0].x));
                        const float2 a1 = __half22float2(*reinterpret_cast<const __half2 *>(&sn1[0].y));
                        const float2 b0 = __half22float2(*reinterpret_cast<const __half2 *>(&sn1[1].x));
                        const float2 b1 = __half22float2(*reinterpret_cast<const __half2 *>(&sn1[1].y));
                        const float nx4[4] = {a0.x, a0.y, a1.x, a1.y}, nz4[4] = {b0.x, b0.y, b1.x, b1.y};
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            s1[j] = a.inv_dt * (nx4[j] * e0 - f4(wx8, j) * d0);
                            s2[j] = a.inv_dt * (nz4[j] * e1 - f4(wz8, j) * d1);
                        }
                    }
                    float tt[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) tt[j] = v[VX][j] * s1[j] + v[VZ][j] * s2[j];
                    if (nval == 4) {
                        float4 sv = im[0];
                        sv.x += tt[0]; sv.y += tt[1]; sv.z += tt[2]; sv.w += tt[3];
                        *reinterpret_cast<float4 *>(a.img[0] + o) = sv;
                    } else {
                        for (int j = 0; j < nval; j++) a.img[0][o + j] += tt[j];
                    }
                } else {
                    float v[3][4];  // sxx, szz, sxz
#pragma unroll
                    for (int f = 0; f < 3; f++) {
                        v[f][0] = own[f].x; v[f][1] = own[f].y; v[f][2] = own[f].z; v[f][3] = own[f].w;
                    }
                    if (a.rec && g.rec_iz >= gz && g.rec_iz < gz + 4) {
                        const int j = g.rec_iz - gz;
#pragma unroll
                        for (int f = 0; f < 3; f++)
                            if (a.comp_mask & (1 << (2 + f))) {
                                const float d =
                                    a.rec[g.doff + ((long long)a.it * a.ncomp + rec_slot(a.comp_mask, 2 + f)) * nx + gx];
#pragma unroll
                                for (int jj = 0; jj < 4; jj++)
                                    if (jj == j) v[f][jj] = Ar<false>::add(d, v[f][jj]);
                            }
                    }
                    madj_x4<true>(prod, Q_M1X, gx, z, v[0]);
                    mzwin(prod, Q_M1Z, gx, z, w);
                    adj_fast_z4<true>(w, v[1]);
                    mzwin(prod, Q_M1X, gx, z, w);
                    adj_fast_z4<false>(w, v[2]);
                    madj_x4<false>(prod, Q_M1Z, gx, z, v[2]);
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
                    // imaging, lambda and mu terms: x taps of the snapshots
                    // (8-byte reads of 4 halves), z taps from 20-row windows
                    float p4[4] = {0.f, 0.f, 0.f, 0.f}, p7[4] = {0.f, 0.f, 0.f, 0.f};  // x taps: Vx (P), Vz (M)
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        const float c = StagCoef<float>::c(k);
                        const float4 ap = rh4(snap, 0, gx + 5 - k, z), am = rh4(snap, 0, gx - 4 + k, z);
                        const float4 bp = rh4(snap, 1, gx + 4 - k, z), bm = rh4(snap, 1, gx - 5 + k, z);
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            p4[j] += c * (f4(ap, j) - f4(am, j));
                            p7[j] += c * (f4(bp, j) - f4(bm, j));
                        }
                    }
                    float s4v[4], s5v[4], s6v[4];
                    {
                        float wz[20];  // source Vz, rows z-8 .. z+11
#pragma unroll
                        for (int q = 0; q < 5; q++) {
                            const float4 t_ = rh4(snap, 1, gx, z - 8 + 4 * q);
                            wz[4 * q] = t_.x; wz[4 * q + 1] = t_.y; wz[4 * q + 2] = t_.z; wz[4 * q + 3] = t_.w;
                        }
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int cz = gz + j;
                            float s4 = 0.f, s5 = 0.f;
                            if (cz >= 4 && cz <= nz - 6 && gx >= 4 && gx <= nx - 6) {
                                float p5 = 0.f;
#pragma unroll
                                for (int k = 0; k < 5; k++) p5 += StagCoef<float>::c(k) * (wz[8 + j + 5 - k] - wz[8 + j - 4 + k]);
                                s4 = p4[j] * d0 * a.inv_dx;
                                s5 = p5 * d1 * a.inv_dx;
                            }
                            s4v[j] = s4;
                            s5v[j] = s5;
                        }
                    }
                    {
                        float wx[20];  // source Vx, rows z-8 .. z+11
#pragma unroll
                        for (int q = 0; q < 5; q++) {
                            const float4 t_ = rh4(snap, 0, gx, z - 8 + 4 * q);
                            wx[4 * q] = t_.x; wx[4 * q + 1] = t_.y; wx[4 * q + 2] = t_.z; wx[4 * q + 3] = t_.w;
                        }
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int cz = gz + j;
                            float s6 = 0.f;
                            if (cz >= 5 && cz <= nz - 6 && gx >= 5 && gx <= nx - 6) {
                                float p6 = 0.f;
#pragma unroll
                                for (int k = 0; k < 5; k++) p6 += StagCoef<float>::c(k) * (wx[8 + j + 4 - k] - wx[8 + j - 5 + k]);
                                s6 = (p6 * d0 + p7[j] * d1) * a.inv_dx;
                            }
                            s6v[j] = s6;
                        }
                    }
                    float t1[4], t2[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float s3 = s4v[j] + s5v[j];
                        t1[j] = -(v[0][j] + v[1][j]) * s3;
                        t2[j] = -(2.f * v[0][j] * s4v[j] + 2.f * v[1][j] * s5v[j] + v[2][j] * s6v[j]);
                    }
                    if (nval == 4) {
                        float4 sv = im[0], sw = im[1];
                        sv.x += t1[0]; sv.y += t1[1]; sv.z += t1[2]; sv.w += t1[3];
                        sw.x += t2[0]; sw.y += t2[1]; sw.z += t2[2]; sw.w += t2[3];
                        *reinterpret_cast<float4 *>(a.img[1] + o) = sv;
                        *reinterpret_cast<float4 *>(a.img[2] + o) = sw;
                    } else {
                        for (int j = 0; j < nval; j++) {
                            a.img[1][o + j] += t1[j];
                            a.img[2][o + j] += t2[j];
                        }
                    }
                }
            }
            fetch(c + 1);
            __syncwarp();
            if (lane == 0) mbar_arrive(&cd[C & 1]);
            C++;
            if (c + 3 <= n + 1) {
                // product pass of chunk k0 + c + 2 into the slot of chunk
                // k0 + c - 2, which the compute of chunk k0 + c - 1 read last
                if (c >= 1) {
                    const int D = C0 + c - 1;
                    if (!mbar_wait(&cd[D & 1], (D >> 1) & 1)) return fail();
                }
                if (!products(k0 + c + 2)) return fail();
            }
        }
    }
}

}  // namespace eg
