// Fused 2D elastic velocity-stress step kernels (10th-order staggered grid,
// 2nd order in time) for sm_103a.
//
// One launch advances one time level of every shot in a batch.  Each CTA
// walks a list of (shot, tile) work items; a tile of TZ x TX output cells is
// staged with its 5-cell halo in shared memory, every output cell updates all
// five fields (Vx, Vz, sigma_xx, sigma_zz, sigma_xz) in registers and writes
// them once.  The level written replaces the level two steps back in place
// (each cell reads its own older value only), so a propagation needs two
// buffers per field.
//
// Reference semantics (lgan/elastic, W = 2d_rtm_restart/Src_working):
//  * forward update, W/rtm-mod-adj.f90:225-252 with the operators of
//    W/rtmlib-mod.f90:200-633 (coefficient at the output cell, "P"/"M"
//    staggered stencils), sponge K of W/abc-mod.f90:59-78 afterwards;
//  * adjoint update, the gather recursion of W/rtmlib-modC.c:120-255
//    (coefficient multiplies each neighbour, coefficient planes masked to
//    the forward operators' loop ranges as at W/rtmlib-modC.c:83-93).
// In EXACT mode every product and sum is separately rounded in the
// reference's order (bit-identical to the reference CPU code); otherwise the
// compiler may fuse multiply-adds and the adjoint uses pre-multiplied
// coefficient*field products.
#pragma once
#include <cuda.h>
#include "common.cuh"

namespace eg {

enum Field { VX = 0, VZ = 1, SXX = 2, SZZ = 3, SXZ = 4 };
enum Coef { M1X = 0, M1Z = 1, A2 = 2, A3 = 3, A23 = 4 };

// One shot of a batch: a subgrid of nz x nx cells whose planes start at
// element `off` of every field / coefficient array (column pitch ldz, shared
// by the batch).  Receiver traces of the shot start at `doff`.
struct ShotGeom {
    long long off;
    long long doff;
    int nz, nx;
    int src_iz, src_ix;  // 0-based source cell, -1 = none
    int rec_iz;          // 0-based receiver row, -1 = none
    int tile0;           // first work item of this shot
    int ntz;             // tiles along z
    int pad;
};

template <typename T>
struct Step2DArgs {
    T *out[5];            // level being written
    const T *own2[5];     // the same cells two levels back (forward) or ahead (adjoint)
    const T *nb[5];       // the neighbour level (it-1 forward, it+1 adjoint)
    const T *inplane[5];  // adjoint only: a full input plane at level it, added first (nullable)
    const T *coef[5];     // masked coefficient planes M1X, M1Z, A2, A3, A23
    const ShotGeom *shots;
    int nshots;
    int ntiles;
    int ldz;
    // sponge: filter table of abc2 = abc+5 entries, applied when sponge != 0
    const T *filt;
    int abc2;
    int sponge;
    // forward point source: value added to sigma_xx and sigma_zz at the source cell
    T srcval;
    int has_src;
    // receiver traces, per shot [it][slot][ix] at shots[s].doff; slot = rank of
    // the field in comp_mask.  Forward: record after the update; adjoint:
    // inject before the update.
    T *rec;
    int comp_mask;
    int ncomp;
    int it;  // level index used to address the traces

    // ---- streaming RTM extensions (float only) ----------------------------
    // forward: FP16 snapshot of Vx, Vz of the neighbour level (it-1), each
    // plane scaled by 2^14 / max|.| of that level (snap_max_in[shot][2]); the
    // max-abs of the level being written goes to snap_max_out[shot][2].
    __half *snap_out[2];
    const float *snap_max_in;
    float *snap_max_out;
    // adjoint: fused imaging condition with the source partials S1..S6 taken
    // from the FP16 snapshots of levels it (isnap0, with halo) and it+1
    // (isnap1, centre only); ilast marks the last level (S1 = S2 = 0).
    // Images img[3] accumulate with Kahan compensation imgc[3].
    const __half *isnap0[2];
    const __half *isnap1[2];
    const float *imax0;
    const float *imax1;
    int ilast;
    T *img[3];
    T *imgc[3];
    T inv_dt, inv_dx;

    // ---- TMA tile staging (v2 float kernel, batch engine) ------------------
    // With tma set, the halo tiles of the neighbour level, the coefficients
    // (adjoint) and the level's FP16 snapshots (imaging) are loaded by
    // cp.async.bulk.tensor from 3D tensors (ldz rows x columns x planes):
    // tm[0] the neighbour-level planes (nb_plane[f] selects field f's plane;
    // a plane index past the last reads zeros), tm[1] the five coefficient
    // planes, tm[2] the snapshot planes (snap_plane[f]).  The shot's first
    // column is off / ldz.  err receives 1 if a tile load never completed.
    int tma;
    int nb_plane[5];
    int snap_plane[2];
    int *err;
    CUtensorMap tm[3];  // 128-byte aligned by its type
};

constexpr float SNAP_Q = 16384.0f;  // FP16 snapshot full scale (2^14, headroom to 65504)

template <bool EXACT>
struct Ar {
    template <typename T> static __device__ __forceinline__ T mul(T a, T b) { return mul_rn(a, b); }
    template <typename T> static __device__ __forceinline__ T add(T a, T b) { return add_rn(a, b); }
    template <typename T> static __device__ __forceinline__ T sub(T a, T b) { return sub_rn(a, b); }
};
template <>
struct Ar<false> {
    template <typename T> static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
    template <typename T> static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    template <typename T> static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
};

template <typename T>
__device__ __forceinline__ int find_shot(const ShotGeom *shots, int nshots, int t)
{
    int lo = 0, hi = nshots - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (shots[mid].tile0 <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Sponge K of W/abc-mod.f90:59-78 for one cell (0-based iz, ix).  The
// reference multiplies bottom-strip, top-strip, right-strip and left-strip
// factors in that order where strips overlap.
template <bool EXACT, typename T>
__device__ __forceinline__ T sponge_cell(T v, int iz, int ix, int nz, int nx, const T *filt, int abc2)
{
    const int iz1 = iz + 1, ix1 = ix + 1;
    if (iz1 >= nz - abc2 + 1) v = Ar<EXACT>::mul(v, __ldg(filt + (iz1 - (nz - abc2) - 1)));
    if (iz1 <= abc2) v = Ar<EXACT>::mul(v, __ldg(filt + (abc2 - iz1)));
    if (ix1 >= nx - abc2 + 1) v = Ar<EXACT>::mul(v, __ldg(filt + (ix1 - (nx - abc2) - 1)));
    if (ix1 <= abc2) v = Ar<EXACT>::mul(v, __ldg(filt + (abc2 - ix1)));
    return v;
}

constexpr int HALO = 5;

// Shared-memory tile addressing: array a, local x (may be -5..TX+4), local z.
template <int TZ, int TX>
struct Tile {
    static constexpr int LZ = TZ + 2 * HALO;
    static constexpr int LX = TX + 2 * HALO;
    static constexpr int SIZE = LZ * LX;
    static __device__ __forceinline__ int at(int a, int x, int z) { return a * SIZE + (x + HALO) * LZ + (z + HALO); }
};

// Forward staggered difference of the tile array `a` at (x, z):
// P pairs (i+5,i-4)..(i+1,i); M pairs (i+4,i-5)..(i,i-1).  Sum order c1..c5
// as in the reference's continuation lines.
template <bool EXACT, int TZ, int TX, bool ALONG_X, bool PTYPE, typename T>
__device__ __forceinline__ T fwd_poly(const T *sm, int a, int x, int z)
{
    using TL = Tile<TZ, TX>;
    T p = T(0);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int hi = PTYPE ? 5 - k : 4 - k;
        const int lo = PTYPE ? -4 + k : -5 + k;
        const T va = ALONG_X ? sm[TL::at(a, x + hi, z)] : sm[TL::at(a, x, z + hi)];
        const T vb = ALONG_X ? sm[TL::at(a, x + lo, z)] : sm[TL::at(a, x, z + lo)];
        const T term = Ar<EXACT>::mul(StagCoef<T>::c(k), Ar<EXACT>::sub(va, vb));
        p = (k == 0) ? term : Ar<EXACT>::add(p, term);
    }
    return p;
}

// Adjoint gather of one (coefficient, field) pair in the reference's term
// order.  M5: +c_k at offsets -5+k (k=0..4), then -c_k at +4-k (k=4..0).
// P5: +c_k at -4+k, then -c_k at +5-k.  Each term is (coef*c_k)*field.
template <int TZ, int TX, bool ALONG_X, bool PTYPE, typename T>
__device__ __forceinline__ T adj_gather_exact(T v, const T *sm, int ca, int fa, int x, int z)
{
    using TL = Tile<TZ, TX>;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int o = PTYPE ? -4 + k : -5 + k;
        const int ix = ALONG_X ? x + o : x, iz = ALONG_X ? z : z + o;
        v = add_rn(v, mul_rn(mul_rn(sm[TL::at(ca, ix, iz)], StagCoef<T>::c(k)), sm[TL::at(fa, ix, iz)]));
    }
#pragma unroll
    for (int k = 4; k >= 0; k--) {
        const int o = PTYPE ? 5 - k : 4 - k;
        const int ix = ALONG_X ? x + o : x, iz = ALONG_X ? z : z + o;
        v = sub_rn(v, mul_rn(mul_rn(sm[TL::at(ca, ix, iz)], StagCoef<T>::c(k)), sm[TL::at(fa, ix, iz)]));
    }
    return v;
}

// Same operator on a pre-multiplied product array p = coef*field:
// sum_k c_k * (p(+side) - p(-side)), fused multiply-adds allowed.
template <int TZ, int TX, bool ALONG_X, bool PTYPE, typename T>
__device__ __forceinline__ T adj_gather_fast(T v, const T *sm, int pa, int x, int z)
{
    using TL = Tile<TZ, TX>;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int op = PTYPE ? -4 + k : -5 + k;  // + side
        const int om = PTYPE ? 5 - k : 4 - k;    // - side
        const T pp = ALONG_X ? sm[TL::at(pa, x + op, z)] : sm[TL::at(pa, x, z + op)];
        const T pm = ALONG_X ? sm[TL::at(pa, x + om, z)] : sm[TL::at(pa, x, z + om)];
        v = v + StagCoef<T>::c(k) * (pp - pm);
    }
    return v;
}

// Number of shared-memory tile arrays per kernel flavour.
template <bool ADJ, bool EXACT>
struct NArr { static constexpr int value = ADJ ? (EXACT ? 10 : 7) : 5; };

// Adjoint product arrays in fast mode.
enum { P_A23XX = 0, P_A2ZZ = 1, P_A3XZ = 2, P_A2XX = 3, P_A23ZZ = 4, P_M1XVX = 5, P_M1ZVZ = 6 };

template <typename T, bool EXACT, bool ADJ, int TZ, int TX>
__global__ void __launch_bounds__(256) k_step2d(const __grid_constant__ Step2DArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    using TL = Tile<TZ, TX>;
    constexpr int ROWS = TX / 8;  // x rows per warp (8 warps)
    constexpr int IMG0 = NArr<ADJ, EXACT>::value;  // first imaging array
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
        const int s = find_shot<T>(a.shots, a.nshots, t);
        const ShotGeom g = a.shots[s];
        const int lt = t - g.tile0;
        const int tz0 = (lt % g.ntz) * TZ, tx0 = (lt / g.ntz) * TX;
        const long long off = g.off;
        const int nz = g.nz, nx = g.nx, ldz = a.ldz;

        __syncthreads();  // previous tile fully consumed
        // ---- stage the neighbour level (and coefficients) with halo
        for (int idx = threadIdx.x; idx < TL::SIZE; idx += blockDim.x) {
            const int lx = idx / TL::LZ, lz = idx - lx * TL::LZ;
            const int gx = tx0 + lx - HALO, gz = tz0 + lz - HALO;
            const bool in = (gx >= 0) & (gx < nx) & (gz >= 0) & (gz < nz);
            const long long o = off + (long long)gx * ldz + gz;
            if (!ADJ) {
#pragma unroll
                for (int f = 0; f < 5; f++) sm[f * TL::SIZE + idx] = in ? a.nb[f][o] : T(0);
            } else if (EXACT) {
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    sm[f * TL::SIZE + idx] = in ? a.nb[f][o] : T(0);
                    sm[(5 + f) * TL::SIZE + idx] = in ? __ldg(a.coef[f] + o) : T(0);
                }
            } else {
                T fv[5], cv[5];
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    fv[f] = in ? a.nb[f][o] : T(0);
                    cv[f] = in ? __ldg(a.coef[f] + o) : T(0);
                }
                sm[P_A23XX * TL::SIZE + idx] = cv[A23] * fv[SXX];
                sm[P_A2ZZ * TL::SIZE + idx] = cv[A2] * fv[SZZ];
                sm[P_A3XZ * TL::SIZE + idx] = cv[A3] * fv[SXZ];
                sm[P_A2XX * TL::SIZE + idx] = cv[A2] * fv[SXX];
                sm[P_A23ZZ * TL::SIZE + idx] = cv[A23] * fv[SZZ];
                sm[P_M1XVX * TL::SIZE + idx] = cv[M1X] * fv[VX];
                sm[P_M1ZVZ * TL::SIZE + idx] = cv[M1Z] * fv[VZ];
            }
            if (ADJ && a.img[0]) {
                // dequantised source Vx, Vz of level it for S4..S6
                const float dq0 = a.imax0[2 * s] * (1.0f / SNAP_Q), dq1 = a.imax0[2 * s + 1] * (1.0f / SNAP_Q);
                sm[(IMG0 + 0) * TL::SIZE + idx] = in ? T(__half2float(a.isnap0[0][o]) * dq0) : T(0);
                sm[(IMG0 + 1) * TL::SIZE + idx] = in ? T(__half2float(a.isnap0[1][o]) * dq1) : T(0);
            }
        }
        __syncthreads();

        // ---- update: lane = z, each warp owns ROWS consecutive x rows
        float wmax0 = 0.f, wmax1 = 0.f;  // max-abs of the written Vx, Vz (snapshots)
#pragma unroll 1
        for (int r = 0; r < ROWS; r++) {
            const int x = warp * ROWS + r, z = lane;
            const int gx = tx0 + x, gz = tz0 + z;
            if (gx >= nx || gz >= nz) continue;
            const long long o = off + (long long)gx * ldz + gz;
            T v[5];
            if (!ADJ) {
                // base: level it-2, preceded by the Born secondary source of
                // level it when given (W/rtm-mod-adj.f90:325 "Vx0(it)+Vx0(it-2)")
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    T b = a.own2[f][o];
                    if (a.inplane[f]) b = Ar<EXACT>::add(a.inplane[f][o], b);
                    v[f] = b;
                }
                if (a.has_src && gz == g.src_iz && gx == g.src_ix) {
                    v[SXX] = Ar<EXACT>::add(v[SXX], a.srcval);
                    v[SZZ] = Ar<EXACT>::add(v[SZZ], a.srcval);
                }
                const T cm1x = __ldg(a.coef[M1X] + o), cm1z = __ldg(a.coef[M1Z] + o);
                const T ca2 = __ldg(a.coef[A2] + o), ca3 = __ldg(a.coef[A3] + o), ca23 = __ldg(a.coef[A23] + o);
                // Vx += m1_x*Dx-(sxx) [Ax]; += m1_x*Dz+(sxz) [Bx]
                v[VX] = Ar<EXACT>::add(v[VX], Ar<EXACT>::mul(cm1x, fwd_poly<EXACT, TZ, TX, true, false>(sm, SXX, x, z)));
                v[VX] = Ar<EXACT>::add(v[VX], Ar<EXACT>::mul(cm1x, fwd_poly<EXACT, TZ, TX, false, true>(sm, SXZ, x, z)));
                // Vz += m1_z*Dx+(sxz) [Az]; += m1_z*Dz-(szz) [Bz]
                v[VZ] = Ar<EXACT>::add(v[VZ], Ar<EXACT>::mul(cm1z, fwd_poly<EXACT, TZ, TX, true, true>(sm, SXZ, x, z)));
                v[VZ] = Ar<EXACT>::add(v[VZ], Ar<EXACT>::mul(cm1z, fwd_poly<EXACT, TZ, TX, false, false>(sm, SZZ, x, z)));
                // sxx += a23*Dx+(vx) [D]; += a2*Dz+(vz) [E]
                v[SXX] = Ar<EXACT>::add(v[SXX], Ar<EXACT>::mul(ca23, fwd_poly<EXACT, TZ, TX, true, true>(sm, VX, x, z)));
                v[SXX] = Ar<EXACT>::add(v[SXX], Ar<EXACT>::mul(ca2, fwd_poly<EXACT, TZ, TX, false, true>(sm, VZ, x, z)));
                // szz += a2*Dx+(vx) [F]; += a23*Dz+(vz) [G]
                v[SZZ] = Ar<EXACT>::add(v[SZZ], Ar<EXACT>::mul(ca2, fwd_poly<EXACT, TZ, TX, true, true>(sm, VX, x, z)));
                v[SZZ] = Ar<EXACT>::add(v[SZZ], Ar<EXACT>::mul(ca23, fwd_poly<EXACT, TZ, TX, false, true>(sm, VZ, x, z)));
                // sxz += a3*Dz-(vx) [H]; += a3*Dx-(vz) [J]
                v[SXZ] = Ar<EXACT>::add(v[SXZ], Ar<EXACT>::mul(ca3, fwd_poly<EXACT, TZ, TX, false, false>(sm, VX, x, z)));
                v[SXZ] = Ar<EXACT>::add(v[SXZ], Ar<EXACT>::mul(ca3, fwd_poly<EXACT, TZ, TX, true, false>(sm, VZ, x, z)));
            } else {
                // base value: injected/input level it plus level it+2
#pragma unroll
                for (int f = 0; f < 5; f++) {
                    T b = a.own2[f][o];
                    if (a.inplane[f]) b = Ar<EXACT>::add(a.inplane[f][o], b);
                    v[f] = b;
                }
                if (a.rec && gz == g.rec_iz) {
                    int slot = 0;
#pragma unroll
                    for (int f = 0; f < 5; f++)
                        if (a.comp_mask & (1 << f)) {
                            const T d = a.rec[g.doff + ((long long)a.it * a.ncomp + slot) * nx + gx];
                            v[f] = Ar<EXACT>::add(d, v[f]);
                            slot++;
                        }
                }
                if (EXACT) {
                    // array indices: fields 0..4, coefficients 5..9
                    v[VX] = adj_gather_exact<TZ, TX, true, false>(v[VX], sm, 5 + A23, SXX, x, z);
                    v[VX] = adj_gather_exact<TZ, TX, true, false>(v[VX], sm, 5 + A2, SZZ, x, z);
                    v[VX] = adj_gather_exact<TZ, TX, false, true>(v[VX], sm, 5 + A3, SXZ, x, z);
                    v[VZ] = adj_gather_exact<TZ, TX, false, false>(v[VZ], sm, 5 + A2, SXX, x, z);
                    v[VZ] = adj_gather_exact<TZ, TX, false, false>(v[VZ], sm, 5 + A23, SZZ, x, z);
                    v[VZ] = adj_gather_exact<TZ, TX, true, true>(v[VZ], sm, 5 + A3, SXZ, x, z);
                    v[SXX] = adj_gather_exact<TZ, TX, true, true>(v[SXX], sm, 5 + M1X, VX, x, z);
                    v[SZZ] = adj_gather_exact<TZ, TX, false, true>(v[SZZ], sm, 5 + M1Z, VZ, x, z);
                    v[SXZ] = adj_gather_exact<TZ, TX, false, false>(v[SXZ], sm, 5 + M1X, VX, x, z);
                    v[SXZ] = adj_gather_exact<TZ, TX, true, false>(v[SXZ], sm, 5 + M1Z, VZ, x, z);
                } else {
                    v[VX] = adj_gather_fast<TZ, TX, true, false>(v[VX], sm, P_A23XX, x, z);
                    v[VX] = adj_gather_fast<TZ, TX, true, false>(v[VX], sm, P_A2ZZ, x, z);
                    v[VX] = adj_gather_fast<TZ, TX, false, true>(v[VX], sm, P_A3XZ, x, z);
                    v[VZ] = adj_gather_fast<TZ, TX, false, false>(v[VZ], sm, P_A2XX, x, z);
                    v[VZ] = adj_gather_fast<TZ, TX, false, false>(v[VZ], sm, P_A23ZZ, x, z);
                    v[VZ] = adj_gather_fast<TZ, TX, true, true>(v[VZ], sm, P_A3XZ, x, z);
                    v[SXX] = adj_gather_fast<TZ, TX, true, true>(v[SXX], sm, P_M1XVX, x, z);
                    v[SZZ] = adj_gather_fast<TZ, TX, false, true>(v[SZZ], sm, P_M1ZVZ, x, z);
                    v[SXZ] = adj_gather_fast<TZ, TX, false, false>(v[SXZ], sm, P_M1XVX, x, z);
                    v[SXZ] = adj_gather_fast<TZ, TX, true, false>(v[SXZ], sm, P_M1ZVZ, x, z);
                }
            }
            if (a.sponge) {
#pragma unroll
                for (int f = 0; f < 5; f++) v[f] = sponge_cell<EXACT>(v[f], gz, gx, nz, nx, a.filt, a.abc2);
            }
#pragma unroll
            for (int f = 0; f < 5; f++) a.out[f][o] = v[f];
            if (!ADJ && a.snap_out[0]) {
                // FP16 snapshot of the neighbour level (it-1) at this cell and
                // the max-abs of the level just written
                const float m0 = a.snap_max_in[2 * s], m1 = a.snap_max_in[2 * s + 1];
                const float q0 = m0 > 0.f ? SNAP_Q / m0 : 0.f, q1 = m1 > 0.f ? SNAP_Q / m1 : 0.f;
                a.snap_out[0][o] = __float2half_rn(float(sm[TL::at(VX, x, z)]) * q0);
                a.snap_out[1][o] = __float2half_rn(float(sm[TL::at(VZ, x, z)]) * q1);
                wmax0 = fmaxf(wmax0, fabsf(float(v[VX])));
                wmax1 = fmaxf(wmax1, fabsf(float(v[VZ])));
            }
            if (ADJ && a.img[0]) {
                // imaging condition of level it (W/image-mod-rtm.f90:146-162),
                // accumulated in reverse time order with Kahan compensation
                const T *svx = sm + IMG0 * TL::SIZE, *svz = sm + (IMG0 + 1) * TL::SIZE;
                auto SX = [&](const T *b, int dx_, int dz_) { return b[(x + dx_ + HALO) * TL::LZ + (z + dz_ + HALO)]; };
                T s1 = T(0), s2 = T(0), s4 = T(0), s5 = T(0), s6 = T(0);
                if (!a.ilast) {
                    const float e0 = a.imax1[2 * s] * (1.0f / SNAP_Q), e1 = a.imax1[2 * s + 1] * (1.0f / SNAP_Q);
                    s1 = a.inv_dt * (T(__half2float(a.isnap1[0][o]) * e0) - SX(svx, 0, 0));
                    s2 = a.inv_dt * (T(__half2float(a.isnap1[1][o]) * e1) - SX(svz, 0, 0));
                }
                if (gz >= 4 && gz <= nz - 6 && gx >= 4 && gx <= nx - 6) {
                    T p4 = T(0), p5 = T(0);
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        p4 += StagCoef<T>::c(k) * (SX(svx, 5 - k, 0) - SX(svx, -4 + k, 0));
                        p5 += StagCoef<T>::c(k) * (SX(svz, 0, 5 - k) - SX(svz, 0, -4 + k));
                    }
                    s4 = p4 * a.inv_dx;
                    s5 = p5 * a.inv_dx;
                }
                if (gz >= 5 && gz <= nz - 6 && gx >= 5 && gx <= nx - 6) {
                    T p6 = T(0), p7 = T(0);
#pragma unroll
                    for (int k = 0; k < 5; k++) {
                        p6 += StagCoef<T>::c(k) * (SX(svx, 0, 4 - k) - SX(svx, 0, -5 + k));
                        p7 += StagCoef<T>::c(k) * (SX(svz, 4 - k, 0) - SX(svz, -5 + k, 0));
                    }
                    s6 = (p6 + p7) * a.inv_dx;
                }
                const T s3 = s4 + s5;
                const T t1 = v[VX] * s1 + v[VZ] * s2;
                const T t2 = -(v[SXX] + v[SZZ]) * s3;
                const T t3 = -(T(2) * v[SXX] * s4 + T(2) * v[SZZ] * s5 + v[SXZ] * s6);
                const T tt[3] = {t1, t2, t3};
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    T sum = a.img[i][o], c = a.imgc[i][o];
                    const T y = tt[i] - c;
                    const T tsum = sum + y;
                    c = (tsum - sum) - y;
                    a.img[i][o] = tsum;
                    a.imgc[i][o] = c;
                }
            }
            if (!ADJ && a.rec && gz == g.rec_iz) {
                int slot = 0;
#pragma unroll
                for (int f = 0; f < 5; f++)
                    if (a.comp_mask & (1 << f)) {
                        a.rec[g.doff + ((long long)a.it * a.ncomp + slot) * nx + gx] = v[f];
                        slot++;
                    }
            }
        }
        if (!ADJ && a.snap_out[0]) {  // warp-converged here
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

template <typename T, bool EXACT, bool ADJ, int TZ, int TX>
constexpr size_t step2d_smem(bool img = false)
{
    return (size_t)(NArr<ADJ, EXACT>::value + (ADJ && img ? 2 : 0)) * Tile<TZ, TX>::SIZE * sizeof(T);
}

}  // namespace eg
