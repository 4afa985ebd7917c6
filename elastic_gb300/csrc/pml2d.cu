// Split-field PML Born modelling on the GPU: the program of lgan/elastic
// 2d_rtm_restart/working_Src/born.f90 (born-mod.f90:80-776 with
// bornlib-mod.f90, pml-mod.f90:23-259, source-mod.f90:42-56,
// seis-mod-born.f90:36-98, snap-mod-born.f90:33-68).
//
// The velocities and stresses are split into an x part and a z part (Vx =
// Vx_x + Vx_z, ...), twenty planes per wavefield, each advanced over three
// time levels as
//     new = K1 * ( op(a_x) + op(a_z) + K0 * old [+ source] [+ Born terms] )
// with op a 10-tap staggered difference along x or z scaled by a model
// coefficient, K0 / K1 the PML's pml0 / pml1 factor on that part's axis
// (plain, or averaged over two neighbouring PML columns or rows), and a_x,
// a_z the two parts of the field op differentiates, at the current level.
// The background wavefield carries the Ricker source; the scattered one adds
// the Born terms S1..S8 built from the background's new and current levels.
//
// Layout in HBM: the caller's model planes and outputs are Fortran-ordered
// (nz, nx), z fastest.  The working planes -- 10 coefficient planes
// (rho_Vx, rho_Vz, l, mi, l2mi, dl, dmi, dl2mi, drho_Vx, drho_Vz) and
// 2 wavefields x 3 levels x 10 parts -- are padded: column ix starts 32
// guard rows before row 1 and is ldz (a multiple of 32, >= nz + 44) floats
// long, so that row 1 starts a 128-byte line, every 4-row group starts on a
// 16-byte boundary and the aligned 20-row window of a z-stencil stays inside
// its column; guard rows stay zero.  Then the PML tables (nz x abc per x side, abc x nx per z side;
// pml0 and pml1).  Levels rotate by pointer.
//
// Kernels: each thread owns 4 consecutive rows of one column (blocks of
// 32 x 8 threads: 128 rows x 8 columns), reads a stencil's taps as 16-byte
// words through L1 (10 per x-stencil and 5 per z-stencil for its 4 cells),
// and evaluates each distinct stencil of a field once (D and F share one,
// E and G, S3 and S5, S4 and S6 too).  One launch advances the background,
// one the scattered wavefield (it needs the background's new level at its
// neighbours); receiver lines and snapshots are separate small launches on
// the levels that record.  Every product and sum is a separately rounded
// _rn intrinsic in the reference's order, so the result is bit-identical
// to the reference's CPU execution.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/elastic_rtm.h"
#include "common.cuh"
#include "elastic2d_v2.cuh"
#include "engine.h"

using namespace eg;

namespace {

enum { VXX, VXZ, VZX, VZZ, SXXX, SXXZ, SZZX, SZZZ, SXZX, SXZZ, NF };
enum { C_RVX, C_RVZ, C_L, C_MI, C_L2MI, C_DL, C_DMI, C_DL2MI, C_DRVX, C_DRVZ, NC };

// The four stencil kinds of bornlib-mod.f90.  Pairs (p + (5-k+s) st,
// p - (6-k-s) st), k = 1..5, st the axis stride; the operator runs over rows
// z0..nz-zoff and columns x0..nx-xoff (1-based).
enum { XA, XD, ZB, ZH };
struct StK {
    int axis, s, z0, zoff, x0, xoff;
};
__host__ __device__ constexpr StK stk(int k)
{
    return k == XA ? StK{0, 0, 6, 0, 6, 4}   // Ax, J, S8   (bornlib-mod.f90:62-72, 386-396, 598-608)
         : k == XD ? StK{0, 1, 6, 0, 5, 5}   // Az, D, F, S3, S5 (:143-153, 196-206, 270-280, 494-504, 546-556)
         : k == ZB ? StK{1, 1, 6, 5, 1, 0}   // Bx, E, G, S4, S6 (:96-106, 233-243, 307-317, 520-530, 572-582)
                   : StK{1, 0, 6, 4, 1, 0};  // Bz, H, S7   (:170-180, 344-354, 572-582)
}

// Per part: stencil, coefficient, its two inputs, PML axis (0 x, 1 z),
// averaged PML (O, P, Q, R instead of K, L, M, N), source injection.
struct Part {
    int st, coef, a, b, axis, avg, src;
};
__host__ __device__ constexpr Part part_of(int f)
{
    switch (f) {
    case VXX: return {XA, C_RVX, SXXX, SXXZ, 0, 0, 0};   // born-mod.f90:431-438
    case VXZ: return {ZB, C_RVX, SXZX, SXZZ, 1, 0, 0};   // :440-447
    case VZX: return {XD, C_RVZ, SXZX, SXZZ, 0, 1, 0};   // :449-456
    case VZZ: return {ZH, C_RVZ, SZZX, SZZZ, 1, 1, 0};   // :458-465
    case SXXX: return {XD, C_L2MI, VXX, VXZ, 0, 1, 1};   // :467-472
    case SXXZ: return {ZB, C_L, VZX, VZZ, 1, 1, 1};      // :474-479
    case SZZX: return {XD, C_L, VXX, VXZ, 0, 1, 1};      // :481-486
    case SZZZ: return {ZB, C_L2MI, VZX, VZZ, 1, 1, 1};   // :488-493
    case SXZX: return {ZH, C_MI, VXX, VXZ, 0, 0, 0};     // :495-501
    default: return {XA, C_MI, VZX, VZZ, 1, 0, 0};       // sxz_z :503-509
    }
}

// Born terms of the scattered parts (born-mod.f90:514-600): st < 0 is
// S1 / S2, (bg new - bg cur) * drho on rows 6..nz-5; otherwise S3..S8, a
// stencil of the background's new velocity parts a, b scaled by coef.
struct BornT {
    int st, coef, a, b;
};
__host__ __device__ constexpr BornT born_of(int f)
{
    switch (f) {
    case VXX: return {-1, C_DRVX, VXX, -1};
    case VXZ: return {-1, C_DRVX, VXZ, -1};
    case VZX: return {-1, C_DRVZ, VZX, -1};
    case VZZ: return {-1, C_DRVZ, VZZ, -1};
    case SXXX: return {XD, C_DL2MI, VXX, VXZ};  // S3
    case SXXZ: return {ZB, C_DL, VZX, VZZ};     // S4
    case SZZX: return {XD, C_DL, VXX, VXZ};     // S5
    case SZZZ: return {ZB, C_DL2MI, VZX, VZZ};  // S6
    case SXZX: return {ZH, C_DMI, VXX, VXZ};    // S7
    default: return {XA, C_DMI, VZX, VZZ};      // S8
    }
}

struct PmlTabs {
    const float *x0[2], *x1[2], *z0[2], *z1[2];  // [left/top, right/bottom]
    int abc;
};

constexpr int GZ = 32;  // guard rows above row 1 of a padded column (row 1 starts a 128-byte line)

struct StepArgs {
    int nz, nx, ldz;
    float *nw[NF];
    const float *cur[NF];
    const float *old[NF];
    const float *cf[NC];
    const float *bgn[4];  // scattered step: the background's new and current
    const float *bgc[4];  // velocity parts
    PmlTabs t;
    int zs, xs;
    float src;
    int prefetch;
};

__device__ __forceinline__ float4 ld4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ float at(const float4 &v, int r) { return r == 0 ? v.x : r == 1 ? v.y : r == 2 ? v.z : v.w; }

// x range of a stencil kind for column ix (uniform over a thread's rows)
template <int K>
__device__ __forceinline__ bool x_in(int nx, int ix)
{
    constexpr StK k = stk(K);
    return ix >= k.x0 && ix <= nx - k.xoff;
}
template <int K>
__device__ __forceinline__ bool z_in(int nz, int iz)
{
    constexpr StK k = stk(K);
    return iz >= k.z0 && iz <= nz - k.zoff;
}

// v * PML factor of a part at (iz, ix): the left / top side first, then the
// right / bottom one, as K..R run their two loops (pml-mod.f90:134-257).
// W = 0: pml0 tables (L, N, P, R), W = 1: pml1 tables (K, M, O, Q).
template <int AXIS, int AVG, int W>
__device__ __forceinline__ float pml_apply(const PmlTabs &T, int nz, int nx, int iz, int ix, float v)
{
    const int abc = T.abc;
    if (abc <= 0) return v;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        if (AXIS == 0) {
            const float *t = W ? T.x1[side] : T.x0[side];
            const int i = side == 0 ? ix - 5 : ix - (nx - abc - 5);  // PML column, 1..abc
            if (!AVG && i >= 1 && i <= abc) v = mul_rn(__ldg(t + (long long)(i - 1) * nz + iz - 1), v);
            if (AVG && i >= 1 && i <= abc - 1)
                v = mul_rn(mul_rn(0.5f, add_rn(__ldg(t + (long long)i * nz + iz - 1),
                                               __ldg(t + (long long)(i - 1) * nz + iz - 1))),
                           v);
        } else {
            const float *t = W ? T.z1[side] : T.z0[side];
            const int i = side == 0 ? iz - 5 : iz - (nz - abc - 5);  // PML row, 1..abc
            const long long c = (long long)(ix - 1) * abc;
            if (!AVG && i >= 1 && i <= abc) v = mul_rn(__ldg(t + c + i - 1), v);
            if (AVG && i >= 2 && i <= abc)
                v = mul_rn(mul_rn(0.5f, add_rn(__ldg(t + c + i - 1), __ldg(t + c + i - 2))), v);
        }
    }
    return v;
}

// Stencil sums c1*(m[hi1]-m[lo1]) + ... + c5*(m[hi5]-m[lo5]) (left to right)
// of the 4 rows starting at padded offset q.  x: ten 16-byte words from the
// tap columns; z: the aligned window of rows q-8 .. q+11 (five words).
template <int K>
__device__ __forceinline__ void sten4(const float *__restrict__ m, long long q, long long ld, float out[4])
{
    constexpr StK k = stk(K);
    if constexpr (k.axis == 0) {
#pragma unroll
        for (int j = 1; j <= 5; ++j) {
            const float4 hi = ld4(m + q + (5 - j + k.s) * ld), lo = ld4(m + q - (6 - j - k.s) * ld);
            const float c = StagCoef<float>::c(j - 1);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float t = mul_rn(c, sub_rn(at(hi, r), at(lo, r)));
                out[r] = j == 1 ? t : add_rn(out[r], t);
            }
        }
    } else {
        float w[20];
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            const float4 v = ld4(m + q - 8 + 4 * b);
            w[4 * b] = v.x;
            w[4 * b + 1] = v.y;
            w[4 * b + 2] = v.z;
            w[4 * b + 3] = v.w;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
#pragma unroll
            for (int j = 1; j <= 5; ++j) {
                const float t = mul_rn(StagCoef<float>::c(j - 1), sub_rn(w[8 + r + 5 - j + k.s], w[8 + r - 6 + j + k.s]));
                out[r] = j == 1 ? t : add_rn(out[r], t);
            }
        }
    }
}

// One thread's 4 cells of column ix, rows iz0 .. iz0+3, padded offset q.
struct Cell4 {
    int iz0, ix;
    long long q;
    int nrow;  // rows of the 4 inside the grid
};

// Finishes part F: v = 0 + cf*sa + cf*sb (where the operator runs)
// + K0*old [+ source] [+ Born terms from ba, bb or S1/S2], then K1, stored.
template <int F, bool BORN, bool FAST>
__device__ __forceinline__ void finish(const StepArgs &a, const Cell4 &c, bool op_x, const float sa[4],
                                       const float sb[4], bool born_x, const float ba[4], const float bb[4])
{
    constexpr Part P = part_of(F);
    float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (FAST || op_x) {
        const float4 cf = ld4(a.cf[P.coef] + c.q);
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (FAST || z_in<P.st>(a.nz, c.iz0 + r)) {
                v[r] = add_rn(v[r], mul_rn(at(cf, r), sa[r]));
                v[r] = add_rn(v[r], mul_rn(at(cf, r), sb[r]));
            }
    }
    const float4 o = ld4(a.old[F] + c.q);
#pragma unroll
    for (int r = 0; r < 4; ++r)
        v[r] = add_rn(v[r], FAST ? at(o, r)
                            : r < c.nrow ? pml_apply<P.axis, P.avg, 0>(a.t, a.nz, a.nx, c.iz0 + r, c.ix, at(o, r))
                                         : 0.0f);
    if constexpr (!BORN && P.src) {
        if (c.ix == a.xs && a.zs >= c.iz0 && a.zs < c.iz0 + 4) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (c.iz0 + r == a.zs) v[r] = add_rn(v[r], a.src);
        }
    }
    if constexpr (BORN) {
        constexpr BornT B = born_of(F);
        if constexpr (B.st < 0) {
            const float4 n = ld4(a.bgn[B.a] + c.q), u = ld4(a.bgc[B.a] + c.q), d = ld4(a.cf[B.coef] + c.q);
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (FAST || (c.iz0 + r >= 6 && c.iz0 + r <= a.nz - 5))
                    v[r] = add_rn(v[r], mul_rn(sub_rn(at(n, r), at(u, r)), at(d, r)));
        } else {
            constexpr int KB = B.st < 0 ? 0 : B.st;
            if (FAST || born_x) {
                const float4 cf = ld4(a.cf[B.coef] + c.q);
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (FAST || z_in<KB>(a.nz, c.iz0 + r)) {
                        v[r] = add_rn(v[r], mul_rn(at(cf, r), ba[r]));
                        v[r] = add_rn(v[r], mul_rn(at(cf, r), bb[r]));
                    }
            }
        }
    }
    if (!FAST) {
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < c.nrow) v[r] = pml_apply<P.axis, P.avg, 1>(a.t, a.nz, a.nx, c.iz0 + r, c.ix, v[r]);
    }
    float *dst = a.nw[F] + c.q;
    if (c.nrow == 4) {
        *reinterpret_cast<float4 *>(dst) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int r = 0; r < 4; ++r)
            if (r < c.nrow) dst[r] = v[r];
    }
}

// true when any of the 4 rows lies in the z range of stencil kind K
template <int K>
__device__ __forceinline__ bool any_z(int nz, int iz0)
{
    constexpr StK k = stk(K);
    return iz0 + 3 >= k.z0 && iz0 <= nz - k.zoff;
}

// Parts F (and G, sharing F's stencils when G >= 0): the operator's two
// stencils of cur[a], cur[b] and, for the scattered step, the Born
// stencils of bgn[a], bgn[b] are evaluated once.
template <int F, int G, bool BORN, bool FAST>
__device__ __forceinline__ void part4(const StepArgs &a, const Cell4 &c)
{
    constexpr Part P = part_of(F);
    float sa[4] = {}, sb[4] = {}, ba[4] = {}, bb[4] = {};
    const bool op_x = FAST || (x_in<P.st>(a.nx, c.ix) && any_z<P.st>(a.nz, c.iz0));
    if (op_x) {
        sten4<P.st>(a.cur[P.a], c.q, a.ldz, sa);
        sten4<P.st>(a.cur[P.b], c.q, a.ldz, sb);
    }
    bool born_x = false;
    if constexpr (BORN) {
        constexpr BornT B = born_of(F);
        if constexpr (B.st >= 0) {
            constexpr int KB = B.st < 0 ? 0 : B.st;
            born_x = FAST || (x_in<KB>(a.nx, c.ix) && any_z<KB>(a.nz, c.iz0));
            if (born_x) {
                sten4<KB>(a.bgn[B.a], c.q, a.ldz, ba);
                sten4<KB>(a.bgn[B.b], c.q, a.ldz, bb);
            }
        }
    }
    finish<F, BORN, FAST>(a, c, op_x, sa, sb, born_x, ba, bb);
    if constexpr (G >= 0) finish<G, BORN, FAST>(a, c, op_x, sa, sb, born_x, ba, bb);
}

template <bool BORN, bool FAST>
__device__ __forceinline__ void cell4(const StepArgs &a, const Cell4 &c)
{
    part4<VXX, -1, BORN, FAST>(a, c);
    part4<VXZ, -1, BORN, FAST>(a, c);
    part4<VZX, -1, BORN, FAST>(a, c);
    part4<VZZ, -1, BORN, FAST>(a, c);
    part4<SXXX, SZZX, BORN, FAST>(a, c);  // D, F on Vx (S3, S5 on the background's Vx)
    part4<SXXZ, SZZZ, BORN, FAST>(a, c);  // E, G on Vz (S4, S6)
    part4<SXZX, -1, BORN, FAST>(a, c);
    part4<SXZZ, -1, BORN, FAST>(a, c);
}

constexpr int BZ = 32, BX = 8;  // threads: 32 x 4 = 128 rows, 8 columns

__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// The lines a thread's cells miss on first touch (own cells of the current
// and old levels, the coefficients; for the scattered step the background's
// levels), requested together at the start so that they are in flight at
// once instead of one part after another.
template <bool BORN>
__device__ __forceinline__ void prefetch_cells(const StepArgs &a, long long q)
{
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        prefetch_l2(a.cur[f] + q);
        prefetch_l2(a.old[f] + q);
    }
#pragma unroll
    for (int k = 0; k < (BORN ? NC : C_DL); ++k) prefetch_l2(a.cf[k] + q);
    if (BORN) {
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            prefetch_l2(a.bgn[f] + q);
            prefetch_l2(a.bgc[f] + q);
        }
    }
}

template <bool BORN>
__global__ void __launch_bounds__(BZ * BX) k_pml_step(const StepArgs a)
{
    Cell4 c;
    c.iz0 = (blockIdx.x * BZ + threadIdx.x) * 4 + 1;
    c.ix = blockIdx.y * BX + threadIdx.y + 1;
    if (c.iz0 > a.nz || c.ix > a.nx) return;
    c.q = (long long)(c.ix - 1) * a.ldz + GZ + c.iz0 - 1;
    c.nrow = a.nz - c.iz0 + 1 < 4 ? a.nz - c.iz0 + 1 : 4;
    if (a.prefetch) prefetch_cells<BORN>(a, c.q);
    const int e = a.t.abc + 5;  // interior without PML: rows, columns e+1 .. n-e
    if (c.iz0 > e && c.iz0 + 3 <= a.nz - e && c.ix > e && c.ix <= a.nx - e) cell4<BORN, true>(a, c);
    else cell4<BORN, false>(a, c);
}

// Staged form: a CTA of 128 threads owns a tile of 64 rows x 8 columns; the
// 5760-byte staged arrays (80 x 18 floats) keep 128-byte alignment; the
// planes its stencils read (background: the 10 current parts; scattered:
// its 10 current parts and the background's 4 new velocity parts) arrive as
// one bulk tensor copy each of 80 rows x 18 columns (8-row and 5-column
// halos, zero outside the grid) on one mbarrier, so every staged byte of the
// tile is in flight at once; thread t owns rows 4 (t % 16) .. +3 of column
// t / 16 and reads taps as 16-byte shared words.  The pointwise operands
// (old level, coefficients) are requested into L2 while the copies run.
constexpr int TT_Z = 64, TT_X = 8, TT_LZ = TT_Z + 16, TT_LX = TT_X + 10, TT_SIZE = TT_LZ * TT_LX;
constexpr int TT_THREADS = (TT_Z / 4) * TT_X;

struct TileArgs {
    int plane[14];     // staged planes: index into the field planes of the tensor map
    int *err;          // set when a tile's copies did not arrive in time
    const int *stall;  // test hook (null in normal use): a zeroed flag that nothing sets
};

template <int K>
__device__ __forceinline__ void sten4s(const float *sm, int col, int row, float out[4])
{
    constexpr StK k = stk(K);
    if constexpr (k.axis == 0) {
#pragma unroll
        for (int j = 1; j <= 5; ++j) {
            const float4 hi = *reinterpret_cast<const float4 *>(sm + (col + 5 - j + k.s) * TT_LZ + row);
            const float4 lo = *reinterpret_cast<const float4 *>(sm + (col - (6 - j - k.s)) * TT_LZ + row);
            const float c = StagCoef<float>::c(j - 1);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float t = mul_rn(c, sub_rn(at(hi, r), at(lo, r)));
                out[r] = j == 1 ? t : add_rn(out[r], t);
            }
        }
    } else {
        float w[20];
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            const float4 v = *reinterpret_cast<const float4 *>(sm + col * TT_LZ + row - 8 + 4 * b);
            w[4 * b] = v.x;
            w[4 * b + 1] = v.y;
            w[4 * b + 2] = v.z;
            w[4 * b + 3] = v.w;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
#pragma unroll
            for (int j = 1; j <= 5; ++j) {
                const float t = mul_rn(StagCoef<float>::c(j - 1), sub_rn(w[8 + r + 5 - j + k.s], w[8 + r - 6 + j + k.s]));
                out[r] = j == 1 ? t : add_rn(out[r], t);
            }
        }
    }
}

// staged slot of a current part (0..9) and of a background new velocity
// part (10..13)
template <int F, int G, bool BORN>
__device__ __forceinline__ void part_t(const StepArgs &a, const Cell4 &c, const float *sm, int col, int row)
{
    constexpr Part P = part_of(F);
    float sa[4] = {}, sb[4] = {}, ba[4] = {}, bb[4] = {};
    const bool op_x = x_in<P.st>(a.nx, c.ix) && any_z<P.st>(a.nz, c.iz0);
    if (op_x) {
        sten4s<P.st>(sm + P.a * TT_SIZE, col, row, sa);
        sten4s<P.st>(sm + P.b * TT_SIZE, col, row, sb);
    }
    bool born_x = false;
    if constexpr (BORN) {
        constexpr BornT B = born_of(F);
        if constexpr (B.st >= 0) {
            constexpr int KB = B.st < 0 ? 0 : B.st;
            born_x = x_in<KB>(a.nx, c.ix) && any_z<KB>(a.nz, c.iz0);
            if (born_x) {
                sten4s<KB>(sm + (10 + B.a) * TT_SIZE, col, row, ba);
                sten4s<KB>(sm + (10 + B.b) * TT_SIZE, col, row, bb);
            }
        }
    }
    finish<F, BORN, false>(a, c, op_x, sa, sb, born_x, ba, bb);
    if constexpr (G >= 0) finish<G, BORN, false>(a, c, op_x, sa, sb, born_x, ba, bb);
}

template <bool BORN>
__global__ void __launch_bounds__(TT_THREADS) k_pml_tile(const StepArgs a, const TileArgs ta,
                                                         const __grid_constant__ CUtensorMap tm)
{
    constexpr int NS = BORN ? 14 : 10;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // staged arrays start on a 128-byte boundary (the launch adds 128 bytes)
    float *smem = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    __shared__ __align__(8) unsigned long long bar;
    const int z0 = blockIdx.x * TT_Z + 1, x0 = blockIdx.y * TT_X + 1;  // first row, column (1-based)
    const int t = threadIdx.x;
    if (t == 0) {
        mbar_init(&bar);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (ta.stall) {
        // test hook: wait for a flag that nothing sets, with the same time
        // limit as the copies' wait; no copy has been issued yet
        const long long t0 = clock64();
        while (*(volatile const int *)ta.stall == 0) {
            if (clock64() - t0 > 2000000000LL) {
                if (t == 0) atomicExch(ta.err, 1);
                return;
            }
        }
    }
    if (t == 0) {
        mbar_expect_tx(&bar, NS * TT_SIZE * 4);
        // padded row of z0 - 8 (a multiple of 4), column x0 - 5 (may be < 0:
        // zero fill)
        const int r0 = GZ + z0 - 1 - 8, c0 = x0 - 1 - 5;
#pragma unroll 1
        for (int sl = 0; sl < NS; ++sl) tma_load_3d(smem + sl * TT_SIZE, &tm, r0, c0, ta.plane[sl], &bar);
    }
    Cell4 c;
    const int cx = t / (TT_Z / 4), g = t % (TT_Z / 4);
    c.iz0 = z0 + 4 * g;
    c.ix = x0 + cx;
    const bool live = c.iz0 <= a.nz && c.ix <= a.nx;
    c.q = (long long)(c.ix - 1) * a.ldz + GZ + c.iz0 - 1;
    c.nrow = a.nz - c.iz0 + 1 < 4 ? a.nz - c.iz0 + 1 : 4;
    if (live && a.prefetch) {
#pragma unroll
        for (int f = 0; f < NF; ++f) prefetch_l2(a.old[f] + c.q);
#pragma unroll
        for (int k = 0; k < (BORN ? NC : C_DL); ++k) prefetch_l2(a.cf[k] + c.q);
        if (BORN) {
#pragma unroll
            for (int f = 0; f < 4; ++f) prefetch_l2(a.bgc[f] + c.q);
        }
    }
    if (!mbar_wait(&bar, 0)) {
        if (t == 0) atomicExch(ta.err, 1);
        return;
    }
    if (!live) return;
    const int col = cx + 5, row = 8 + 4 * g;
    part_t<VXX, -1, BORN>(a, c, smem, col, row);
    part_t<VXZ, -1, BORN>(a, c, smem, col, row);
    part_t<VZX, -1, BORN>(a, c, smem, col, row);
    part_t<VZZ, -1, BORN>(a, c, smem, col, row);
    part_t<SXXX, SZZX, BORN>(a, c, smem, col, row);
    part_t<SXXZ, SZZZ, BORN>(a, c, smem, col, row);
    part_t<SXZX, -1, BORN>(a, c, smem, col, row);
    part_t<SXZZ, -1, BORN>(a, c, smem, col, row);
}

// One thread per cell form of the same step (blocks of 32 x 8 cells): every
// tap a 4-byte load through L1, each distinct stencil evaluated once; with
// 40 registers a thread, 64 warps fit on an SM.
template <int K>
__device__ __forceinline__ float sten1(const float *__restrict__ m, long long p, long long ld)
{
    constexpr StK k = stk(K);
    const long long st = k.axis == 0 ? ld : 1;
    float acc = 0.0f;
#pragma unroll
    for (int j = 1; j <= 5; ++j) {
        const float d = sub_rn(__ldg(m + p + (5 - j + k.s) * st), __ldg(m + p - (6 - j - k.s) * st));
        const float t = mul_rn(StagCoef<float>::c(j - 1), d);
        acc = j == 1 ? t : add_rn(acc, t);
    }
    return acc;
}

// Finishes part F of one cell from its operator stencils sa, sb and Born
// stencils ba, bb (evaluated by the caller where they apply).
template <int F, bool BORN, bool FAST>
__device__ __forceinline__ void finish1(const StepArgs &a, int iz, int ix, long long p, bool op, float sa, float sb,
                                        bool born, float ba, float bb)
{
    constexpr Part P = part_of(F);
    float v = 0.0f;
    if (FAST || op) {
        const float cf = __ldg(a.cf[P.coef] + p);
        v = add_rn(v, mul_rn(cf, sa));
        v = add_rn(v, mul_rn(cf, sb));
    }
    const float o = __ldg(a.old[F] + p);
    v = add_rn(v, FAST ? o : pml_apply<P.axis, P.avg, 0>(a.t, a.nz, a.nx, iz, ix, o));
    if constexpr (!BORN && P.src) {
        if (iz == a.zs && ix == a.xs) v = add_rn(v, a.src);
    }
    if constexpr (BORN) {
        constexpr BornT B = born_of(F);
        if constexpr (B.st < 0) {
            if (FAST || (iz >= 6 && iz <= a.nz - 5))
                v = add_rn(v, mul_rn(sub_rn(__ldg(a.bgn[B.a] + p), __ldg(a.bgc[B.a] + p)), __ldg(a.cf[B.coef] + p)));
        } else if (FAST || born) {
            const float cf = __ldg(a.cf[B.coef] + p);
            v = add_rn(v, mul_rn(cf, ba));
            v = add_rn(v, mul_rn(cf, bb));
        }
    }
    a.nw[F][p] = FAST ? v : pml_apply<P.axis, P.avg, 1>(a.t, a.nz, a.nx, iz, ix, v);
}

// Parts F and (G >= 0) G sharing F's stencils, for one cell.  FAST: the
// cell lies where every operator runs and no PML factor applies (the same
// operations without the range checks and the factors of 1).
template <int F, int G, bool BORN, bool FAST>
__device__ __forceinline__ void part1(const StepArgs &a, int iz, int ix, long long p)
{
    constexpr Part P = part_of(F);
    float sa = 0.0f, sb = 0.0f, ba = 0.0f, bb = 0.0f;
    const bool op = FAST || (x_in<P.st>(a.nx, ix) && z_in<P.st>(a.nz, iz));
    if (op) {
        sa = sten1<P.st>(a.cur[P.a], p, a.ldz);
        sb = sten1<P.st>(a.cur[P.b], p, a.ldz);
    }
    bool born = false;
    if constexpr (BORN) {
        constexpr BornT B = born_of(F);
        if constexpr (B.st >= 0) {
            constexpr int KB = B.st < 0 ? 0 : B.st;
            born = FAST || (x_in<KB>(a.nx, ix) && z_in<KB>(a.nz, iz));
            if (born) {
                ba = sten1<KB>(a.bgn[B.a], p, a.ldz);
                bb = sten1<KB>(a.bgn[B.b], p, a.ldz);
            }
        }
    }
    finish1<F, BORN, FAST>(a, iz, ix, p, op, sa, sb, born, ba, bb);
    if constexpr (G >= 0) finish1<G, BORN, FAST>(a, iz, ix, p, op, sa, sb, born, ba, bb);
}

template <bool BORN, bool FAST>
__device__ __forceinline__ void cell1(const StepArgs &a, int iz, int ix, long long p)
{
    part1<VXX, -1, BORN, FAST>(a, iz, ix, p);
    part1<VXZ, -1, BORN, FAST>(a, iz, ix, p);
    part1<VZX, -1, BORN, FAST>(a, iz, ix, p);
    part1<VZZ, -1, BORN, FAST>(a, iz, ix, p);
    part1<SXXX, SZZX, BORN, FAST>(a, iz, ix, p);  // D, F (S3, S5) share their stencils
    part1<SXXZ, SZZZ, BORN, FAST>(a, iz, ix, p);  // E, G (S4, S6)
    part1<SXZX, -1, BORN, FAST>(a, iz, ix, p);
    part1<SXZZ, -1, BORN, FAST>(a, iz, ix, p);
}

template <bool BORN>
__device__ __forceinline__ void step1_body(const StepArgs &a)
{
    const int iz = blockIdx.x * BZ + threadIdx.x + 1;
    const int ix = blockIdx.y * BX + threadIdx.y + 1;
    if (iz > a.nz || ix > a.nx) return;
    const long long p = (long long)(ix - 1) * a.ldz + GZ + iz - 1;
    if (a.prefetch) prefetch_cells<BORN>(a, p);
    // every operator's range and no PML row or column: rows abc+6 ..
    // nz-abc-5, columns abc+6 .. nx-abc-5
    const int e = a.t.abc + 5;
    if (iz > e && iz <= a.nz - e && ix > e && ix <= a.nx - e) cell1<BORN, true>(a, iz, ix, p);
    else cell1<BORN, false>(a, iz, ix, p);
}

template <bool BORN>
__global__ void __launch_bounds__(BZ * BX) k_pml_step1(const StepArgs a)
{
    step1_body<BORN>(a);
}

// the same with a register bound of MINB blocks of 256 threads an SM
template <bool BORN, int MINB>
__global__ void __launch_bounds__(BZ * BX, MINB) k_pml_step1b(const StepArgs a)
{
    step1_body<BORN>(a);
}

// One launch for both wavefields: the background's level t (b) and the
// scattered wavefield's level t-1 (s), whose Born terms read the
// background's levels t-1 and t-2 -- the current and old levels the
// background step of this launch reads at the same cells.  BG / SC drop
// the background step of the launch after the last level or the scattered
// step of the first launch.
template <bool BG, bool SC>
__global__ void __launch_bounds__(BZ * BX, 6) k_pml_fused(const StepArgs b, const StepArgs s)
{
    const int iz = blockIdx.x * BZ + threadIdx.x + 1;
    const int ix = blockIdx.y * BX + threadIdx.y + 1;
    if (iz > b.nz || ix > b.nx) return;
    const long long p = (long long)(ix - 1) * b.ldz + GZ + iz - 1;
    if (b.prefetch) {
        if (BG) prefetch_cells<false>(b, p);
        if (SC) {
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                prefetch_l2(s.cur[f] + p);
                prefetch_l2(s.old[f] + p);
            }
#pragma unroll
            for (int k = C_DL; k < NC; ++k) prefetch_l2(s.cf[k] + p);
            if (!BG) {
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    prefetch_l2(s.bgn[f] + p);
                    prefetch_l2(s.bgc[f] + p);
                }
            }
        }
    }
    const int e = b.t.abc + 5;
    const bool fast = iz > e && iz <= b.nz - e && ix > e && ix <= b.nx - e;
    if (BG) {
        if (fast) cell1<false, true>(b, iz, ix, p);
        else cell1<false, false>(b, iz, ix, p);
    }
    if (SC) {
        if (fast) cell1<true, true>(s, iz, ix, p);
        else cell1<true, false>(s, iz, ix, p);
    }
}

// Model set-up (born-mod.f90:331-389).  The harmonic averages are written in
// place column by column in the reference, but every neighbour it reads
// ((iz+1, ix), (iz, ix+1), (iz+1, ix+1)) is still unaveraged then, so each
// cell here recomputes its neighbours' unaveraged values from the inputs.
struct ModelArgs {
    int nz, nx, ldz, lame;
    float aux1;
    const float *vp0, *vs0, *rho0, *dvp, *dvs, *drho;
    float *cf[NC];
};

struct Raw {
    float l, mi, dl, dmi, l2mi, dl2mi;
};

__device__ __forceinline__ Raw raw_at(const ModelArgs &m, long long q)
{
    Raw r;
    if (m.lame) {
        r.l = m.vp0[q];
        r.mi = m.vs0[q];
        r.dl = m.dvp[q];
        r.dmi = m.dvs[q];
        r.l2mi = 0.0f;
        r.dl2mi = 0.0f;
    } else {
        const float vp = m.vp0[q], vs = m.vs0[q], rho = m.rho0[q];
        const float dvp = m.dvp[q], dvs = m.dvs[q], drho = m.drho[q];
        r.mi = mul_rn(mul_rn(vs, vs), rho);
        r.l = sub_rn(mul_rn(mul_rn(vp, vp), rho), mul_rn(2.0f, r.mi));
        r.l2mi = add_rn(r.l, mul_rn(2.0f, r.mi));
        r.dmi = mul_rn(mul_rn(dvs, dvs), drho);
        r.dl = sub_rn(mul_rn(mul_rn(dvp, dvp), drho), mul_rn(2.0f, r.dmi));
        r.dl2mi = add_rn(r.dl, mul_rn(2.0f, r.dmi));
    }
    return r;
}

__device__ __forceinline__ float harm(float num, float a, float b, float c, float d)
{
    return div_rn(num, add_rn(add_rn(add_rn(div_rn(1.0f, a), div_rn(1.0f, b)), div_rn(1.0f, c)), div_rn(1.0f, d)));
}

__global__ void k_pml_model(const ModelArgs m)
{
    const int iz = blockIdx.x * BZ + threadIdx.x + 1;
    const int ix = blockIdx.y * BX + threadIdx.y + 1;
    if (iz > m.nz || ix > m.nx) return;
    // p: the caller's (nz, nx) planes; w: the padded coefficient planes
    const long long nz = m.nz, p = (ix - 1) * nz + iz - 1, w = (long long)(ix - 1) * m.ldz + GZ + iz - 1;
    const float aux1 = m.aux1;
    // densities on the staggered grids (:360-384)
    if (iz < m.nz) {
        m.cf[C_RVX][w] = div_rn(mul_rn(aux1, 1.0f), mul_rn(0.5f, add_rn(m.rho0[p + 1], m.rho0[p])));
        m.cf[C_DRVX][w] = -add_rn(div_rn(m.drho[p + 1], m.rho0[p + 1]), div_rn(m.drho[p], m.rho0[p]));
    } else {
        m.cf[C_RVX][w] = mul_rn(aux1, div_rn(1.0f, m.rho0[p]));
        m.cf[C_DRVX][w] = -div_rn(m.drho[p], m.rho0[p]);
    }
    if (ix < m.nx) {
        m.cf[C_RVZ][w] = div_rn(mul_rn(aux1, 1.0f), mul_rn(0.5f, add_rn(m.rho0[p + nz], m.rho0[p])));
        m.cf[C_DRVZ][w] = -add_rn(div_rn(m.drho[p + nz], m.rho0[p + nz]), div_rn(m.drho[p], m.rho0[p]));
    } else {
        m.cf[C_RVZ][w] = mul_rn(aux1, div_rn(1.0f, m.rho0[p]));
        m.cf[C_DRVZ][w] = -div_rn(m.drho[p], m.rho0[p]);
    }
    // Lame parameters, harmonic averages inside the outermost ring (:386-407)
    const Raw r = raw_at(m, p);
    float l = r.l, mi = r.mi, dl = r.dl, dmi = r.dmi, l2mi = r.l2mi, dl2mi = r.dl2mi;
    if (iz >= 2 && iz <= m.nz - 1 && ix >= 2 && ix <= m.nx - 1) {
        const Raw b = raw_at(m, p + 1), c = raw_at(m, p + nz), d = raw_at(m, p + nz + 1);
        const float num = mul_rn(aux1, 4.0f);
        l = harm(num, r.l, b.l, c.l, d.l);
        mi = (r.mi == 0.0f || b.mi == 0.0f || c.mi == 0.0f || d.mi == 0.0f) ? 0.0f : harm(num, r.mi, b.mi, c.mi, d.mi);
        dl = (r.dl < 1e-2f || b.dl < 1e-2f || c.dl < 1e-2f || d.dl < 1e-2f) ? 0.0f : harm(num, r.dl, b.dl, c.dl, d.dl);
        dmi = (r.dmi < 1e-2f || b.dmi < 1e-2f || c.dmi < 1e-2f || d.dmi < 1e-2f) ? 0.0f
                                                                                : harm(num, r.dmi, b.dmi, c.dmi, d.dmi);
        l2mi = add_rn(l, mul_rn(2.0f, mi));
        dl2mi = add_rn(dl, mul_rn(2.0f, dmi));
    }
    m.cf[C_L][w] = l;
    m.cf[C_MI][w] = mi;
    m.cf[C_L2MI][w] = l2mi;
    m.cf[C_DL][w] = dl;
    m.cf[C_DMI][w] = dmi;
    m.cf[C_DL2MI][w] = dl2mi;
}

// PML tables (pml-mod.f90:23-89).  d0 = log(1/R) (1.5 vp) / (abc dx) with
// R = 0.001, taken from the first abc columns (x sides) or rows (z sides)
// of vp for both sides; filter(i) = (i/abc)^2.  logL = logf(1/R), rounded
// on the host as the reference's CPU rounds it.
struct TabArgs {
    int nz, nx, abc, free_surface;
    float logL, den, dt;
    const float *vp;
    float *x0[2], *x1[2], *z0[2], *z1[2];
};

__device__ __forceinline__ float pml_filter(int i, int abc)
{
    const float f = div_rn((float)i, mul_rn(1.0f, (float)abc));
    return mul_rn(f, f);
}

__global__ void k_pml_tables(const TabArgs t)
{
    const long long n = (long long)t.nz * t.abc;
    const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 < n) {  // x sides: (iz, i), i = 1..abc
        const int iz = (int)(i0 % t.nz) + 1, i = (int)(i0 / t.nz) + 1;
        const float d0 = div_rn(mul_rn(t.logL, mul_rn(1.5f, t.vp[(long long)(i - 1) * t.nz + iz - 1])), t.den);
        const float dl = mul_rn(d0, pml_filter(t.abc - i + 1, t.abc)), dr = mul_rn(d0, pml_filter(i, t.abc));
        const float hl = div_rn(mul_rn(t.dt, dl), 2.0f), hr = div_rn(mul_rn(t.dt, dr), 2.0f);
        t.x0[0][i0] = sub_rn(1.0f, hl);
        t.x0[1][i0] = sub_rn(1.0f, hr);
        t.x1[0][i0] = div_rn(1.0f, add_rn(1.0f, hl));
        t.x1[1][i0] = div_rn(1.0f, add_rn(1.0f, hr));
    }
    const long long m = (long long)t.abc * t.nx;
    if (i0 < m) {  // z sides: (i, ix), i = 1..abc
        const int i = (int)(i0 % t.abc) + 1, ix = (int)(i0 / t.abc) + 1;
        const float d0 = div_rn(mul_rn(t.logL, mul_rn(1.5f, t.vp[(long long)(ix - 1) * t.nz + i - 1])), t.den);
        const float dtop = mul_rn(d0, pml_filter(t.abc - i + 1, t.abc)), dbot = mul_rn(d0, pml_filter(i, t.abc));
        const float ht = div_rn(mul_rn(t.dt, dtop), 2.0f), hb = div_rn(mul_rn(t.dt, dbot), 2.0f);
        t.z0[0][i0] = t.free_surface ? 1.0f : sub_rn(1.0f, ht);
        t.z0[1][i0] = sub_rn(1.0f, hb);
        t.z1[0][i0] = t.free_surface ? 1.0f : div_rn(1.0f, add_rn(1.0f, ht));
        t.z1[1][i0] = div_rn(1.0f, add_rn(1.0f, hb));
    }
}

// Receiver lines of one recorded level (seis-mod-born.f90:36-98): for
// ix = 1..nx-2a-1 (a = abc, or 1 when abc = 0), column c = ix + a.
struct RecArgs {
    int nz, nx, ldz, a, nseis, zrec, count;
    const float *w[2][NF];  // background, scattered new level
    float *seis[6];         // Vx, Vz, P, Vx_b, Vz_b, P_b: (nseis, nx - 2 abc)
};

__global__ void k_pml_record(const RecArgs r)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (ix > r.nx - 2 * r.a - 1) return;
    const long long nz = r.ldz, c = ix + r.a;  // nz: the padded column stride
    const long long q = (long long)(ix - 1) * r.nseis + r.count - 1;
    const long long pr = (c - 1) * nz + GZ + r.zrec - 1;  // (zrec, c)
#pragma unroll
    for (int w = 0; w < 2; ++w) {
        const float *const *f = r.w[w];
        r.seis[3 * w + 0][q] = mul_rn(0.5f, add_rn(add_rn(add_rn(f[VXX][pr], f[VXZ][pr]), f[VXX][pr - 1]), f[VXZ][pr - 1]));
        r.seis[3 * w + 1][q] =
            mul_rn(0.5f, add_rn(add_rn(add_rn(f[VZX][pr], f[VZZ][pr]), f[VZX][pr - nz]), f[VZZ][pr - nz]));
        r.seis[3 * w + 2][q] =
            mul_rn(0.5f, add_rn(add_rn(add_rn(f[SXXX][pr], f[SXXZ][pr]), f[SZZX][pr - 1]), f[SZZZ][pr - 1]));
    }
}

// Snapshots of one level (snap-mod-born.f90:33-68), rows and columns
// 2..n-2 of the (nz, nx, nsnap) cubes.
struct SnapArgs {
    int nz, nx, ldz;
    long long off;
    const float *w[2][NF];
    float *snap[6];
};

__global__ void k_pml_snap(const SnapArgs s)
{
    const int iz = blockIdx.x * BZ + threadIdx.x + 1;
    const int ix = blockIdx.y * BX + threadIdx.y + 1;
    if (iz < 2 || iz > s.nz - 2 || ix < 2 || ix > s.nx - 2) return;
    const long long p = (long long)(ix - 1) * s.ldz + GZ + iz - 1;
    const long long o = s.off + (long long)(ix - 1) * s.nz + iz - 1;
#pragma unroll
    for (int w = 0; w < 2; ++w) {
        const float *const *f = s.w[w];
        s.snap[3 * w + 0][o] = add_rn(f[VXX][p], f[VXZ][p]);
        s.snap[3 * w + 1][o] = add_rn(f[VZX][p], f[VZZ][p]);
        s.snap[3 * w + 2][o] = mul_rn(0.5f, add_rn(add_rn(add_rn(f[SXXX][p], f[SXXZ][p]), f[SZZX][p]), f[SZZZ][p]));
    }
}

// Ricker sample of level it (source-mod.f90:42-56) with the scaling of
// born-mod.f90:424-428; host arithmetic is built without contraction.
float pml_source(int it, int nsource, float fp, float dt, float dx)
{
    float src = 0.0f;
    if (it < nsource) {
        const float pi = 3.14159265f;
        const float t = ((float)it * dt) - (((float)nsource * dt) / 2.0f);
        const float aux = ((((pi * pi) * fp) * fp) * t) * t;
        src = (1.0f - (2.0f * aux)) * expf(-aux);
        if (it <= nsource / 10) src = 0.0f;
        src = 10.0e7f * src;
    }
    return ((0.7e7f * src) * (dt / (dx * dx))) * 0.25f;
}

// Step kernel form (kind & 15): 0 four rows per thread, 1 one cell per
// thread, 4 the staged tiles; +2 requests each thread's first-touch lines
// into L2 at the start; 8 one launch a level for both wavefields (one cell
// a thread, prefetch, 6 blocks an SM).  kind >> 4: for the one-cell form, a
// register bound of 5, 6 or 8 blocks of 256 threads an SM (0: the
// compiler's choice).
// Default: one cell, prefetch, 6 blocks (40 registers; measured fastest).
int g_pml_kind = 3 + 6 * 16;

struct PmlState {
    DevBuf<float> buf;
    DevBuf<int> err;
    DevBuf<int> stall;  // zeroed flag for the test hook
    bool test_stall = false;
    bool attr_set[RTM_MAX_DEVICES] = {};
    double last_ms = 0.0;
    long long launches = 0;
};
PmlState g_pml;
// the working planes are shared by the calls of a process: one call at a time
std::mutex g_pml_mutex;

struct Geom {
    int nz, nx, nt, nsnap, nseis, abc, zrec, xs, zs, nsource, free_surface, lame;
    float dx, dt, fp;
    long long seis_n() const { return (long long)nseis * (nx - 2 * abc); }
    long long snap_n() const { return (long long)nz * nx * nsnap; }
};

int check_geom(const Geom &g)
{
    RTM_CHECK_ARG(g.nz >= 11 && g.nx >= 11, "grid must be at least 11 x 11 (nz %d, nx %d)", g.nz, g.nx);
    RTM_CHECK_ARG(g.nt >= 1 && g.nsnap >= 1 && g.nsnap <= g.nt, "need 1 <= nsnap <= nt (nsnap %d, nt %d)", g.nsnap,
                  g.nt);
    RTM_CHECK_ARG(g.nseis >= 1, "nseis must be positive");
    RTM_CHECK_ARG(g.abc >= 0 && g.abc <= g.nz && g.abc <= g.nx && g.nx - 2 * g.abc >= 1,
                  "abc %d must be in 0..min(nz, nx) with nx - 2 abc >= 1", g.abc);
    RTM_CHECK_ARG(g.zs >= 1 && g.zs <= g.nz && g.xs >= 1 && g.xs <= g.nx, "source (%d, %d) outside the grid", g.zs,
                  g.xs);
    RTM_CHECK_ARG(g.zrec >= 2 && g.zrec <= g.nz, "zrec %d must be in 2..nz", g.zrec);
    RTM_CHECK_ARG(g.dx > 0.0f && g.dt > 0.0f && g.fp > 0.0f, "dx, dt, fp must be positive");
    // the reference's last recorded level: countseis stays <= nseis when
    // dseis = nt / nseis + 1 (born-mod.f90:372)
    return RTM_OK;
}

// The whole program on device planes: model (6 planes) in, seis[6] and
// snap[6] out (fully written; cells the reference never sets are zero).
int pml_run(const Geom &g, const float *const *model, float *const *seis, float *const *snap, cudaStream_t st)
{
    TRY(check_geom(g));
    TRY(ensure_device());
    // padded working planes: ldz >= nz + GZ + 12 rows (GZ guard rows above,
    // the rest below), a multiple of 32 floats
    const int ldz = (g.nz + GZ + 12 + 31) / 32 * 32;
    const long long n = (long long)ldz * g.nx, nf = (long long)g.nz * g.nx;
    const long long ntab = 4LL * g.nz * g.abc + 4LL * g.abc * g.nx;
    TRY(g_pml.buf.alloc((size_t)(NC * n + 60 * n + ntab + 1)));
    TRY(g_pml.err.alloc(1));
    TRY(g_pml.stall.alloc(1));
    RTM_CUDA(cudaMemsetAsync(g_pml.stall.p, 0, sizeof(int), st));
    float *cf = g_pml.buf.p, *fld = cf + NC * n, *tab = fld + 60 * n;
    RTM_CUDA(cudaMemsetAsync(cf, 0, sizeof(float) * (NC + 60) * n, st));
    RTM_CUDA(cudaMemsetAsync(g_pml.err.p, 0, sizeof(int), st));
    const bool tile = (g_pml_kind & 4) != 0;
    CUtensorMap tm;
    if (tile) {
        RTM_CHECK_ARG(tensor_maps_available(), "bulk tensor copies are not available");
        // all 60 field planes: padded rows x columns x planes
        const long long dims[3] = {ldz, g.nx, 60}, strides[2] = {4LL * ldz, 4LL * n};
        const int box[3] = {TT_LZ, TT_LX, 1};
        TRY(make_map_nd(&tm, fld, false, 3, dims, strides, box, 0));
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!g_pml.attr_set[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(k_pml_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          10 * TT_SIZE * 4 + 128));
            RTM_CUDA(cudaFuncSetAttribute(k_pml_tile<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          14 * TT_SIZE * 4 + 128));
            g_pml.attr_set[dev] = true;
        }
    }
    const dim3 grdt(ceil_div(g.nz, TT_Z), ceil_div(g.nx, TT_X));
    for (int k = 0; k < 6; ++k) {
        RTM_CUDA(cudaMemsetAsync(seis[k], 0, sizeof(float) * g.seis_n(), st));
        RTM_CUDA(cudaMemsetAsync(snap[k], 0, sizeof(float) * g.snap_n(), st));
    }
    long long launches = 0;
    // per-cell kernels: one thread per cell; step kernels: 4 rows per thread
    const dim3 blk(BZ, BX), grd(ceil_div(g.nz, BZ), ceil_div(g.nx, BX)), grd4(ceil_div(g.nz, 4 * BZ), ceil_div(g.nx, BX));
    {
        ModelArgs m;
        m.nz = g.nz;
        m.nx = g.nx;
        m.ldz = ldz;
        m.lame = g.lame;
        m.aux1 = g.dt / g.dx;
        m.vp0 = model[0];
        m.vs0 = model[1];
        m.rho0 = model[2];
        m.dvp = model[3];
        m.dvs = model[4];
        m.drho = model[5];
        for (int k = 0; k < NC; ++k) m.cf[k] = cf + k * n;
        k_pml_model<<<grd, blk, 0, st>>>(m);
        RTM_CUDA(cudaGetLastError());
        ++launches;
    }
    PmlTabs T;
    T.abc = g.abc;
    {
        TabArgs t;
        t.nz = g.nz;
        t.nx = g.nx;
        t.abc = g.abc;
        t.free_surface = g.free_surface;
        const float R = 0.001f;
        t.logL = logf(1.0f / R);
        t.den = (float)g.abc * g.dx;
        t.dt = g.dt;
        t.vp = model[0];
        float *q = tab;
        for (int s = 0; s < 2; ++s) {
            t.x0[s] = q; q += (long long)g.nz * g.abc;
            t.x1[s] = q; q += (long long)g.nz * g.abc;
            t.z0[s] = q; q += (long long)g.abc * g.nx;
            t.z1[s] = q; q += (long long)g.abc * g.nx;
            T.x0[s] = t.x0[s];
            T.x1[s] = t.x1[s];
            T.z0[s] = t.z0[s];
            T.z1[s] = t.z1[s];
        }
        const long long work = (long long)g.abc * (g.nz > g.nx ? g.nz : g.nx);
        if (work > 0) {
            k_pml_tables<<<ceil_div(work, 256), 256, 0, st>>>(t);
            RTM_CUDA(cudaGetLastError());
            ++launches;
        }
    }
    float *lv[2][3][NF];
    for (int w = 0; w < 2; ++w)
        for (int l = 0; l < 3; ++l)
            for (int f = 0; f < NF; ++f) lv[w][l][f] = fld + ((long long)(w * 3 + l) * NF + f) * n;
    int inew = 0, icur = 1, iold = 2;
    const int dseis = g.nt / g.nseis + 1, dsnap = g.nt / g.nsnap;
    const float nsource2 = (float)(2 * (int)lroundf(((sqrtf(6.0f) / 3.14159265f) / g.fp) / g.dt));
    int countseis = 1, countsnap = 1;
    StepArgs a;
    a.nz = g.nz;
    a.nx = g.nx;
    a.ldz = ldz;
    a.prefetch = (g_pml_kind & 2) != 0;
    const bool one = (g_pml_kind & 1) != 0;
    const bool fused = (g_pml_kind & 15) == 8;
    const int minb = g_pml_kind >> 4;
    for (int k = 0; k < NC; ++k) a.cf[k] = cf + k * n;
    a.t = T;
    a.zs = g.zs;
    a.xs = g.xs;
    // receiver lines and snapshots of level it, from its background and
    // scattered parts
    auto record_level = [&](int it, float *const *bgf, float *const *scf) -> int {
        if ((float)it > nsource2 && it % dseis == 0 && countseis <= g.nseis) {
            RecArgs r;
            r.nz = g.nz;
            r.nx = g.nx;
            r.ldz = ldz;
            r.a = g.abc == 0 ? 1 : g.abc;
            r.nseis = g.nseis;
            r.zrec = g.zrec;
            r.count = countseis;
            for (int f = 0; f < NF; ++f) {
                r.w[0][f] = bgf[f];
                r.w[1][f] = scf[f];
            }
            for (int k = 0; k < 6; ++k) r.seis[k] = seis[k];
            const int nrec = g.nx - 2 * r.a - 1;
            if (nrec > 0) {
                k_pml_record<<<ceil_div(nrec, 128), 128, 0, st>>>(r);
                RTM_CUDA(cudaGetLastError());
                ++launches;
            }
            countseis++;
        }
        if (it % dsnap == 0 && countsnap <= g.nsnap) {
            SnapArgs sa;
            sa.nz = g.nz;
            sa.nx = g.nx;
            sa.ldz = ldz;
            sa.off = (long long)(countsnap - 1) * nf;
            for (int f = 0; f < NF; ++f) {
                sa.w[0][f] = bgf[f];
                sa.w[1][f] = scf[f];
            }
            for (int k = 0; k < 6; ++k) sa.snap[k] = snap[k];
            k_pml_snap<<<grd, blk, 0, st>>>(sa);
            RTM_CUDA(cudaGetLastError());
            ++launches;
            countsnap++;
        }
        return RTM_OK;
    };
    if (fused) {
        // launch L: background level L (L <= nt) and scattered level L-1
        // (L >= 2); each wavefield rotates its own three levels
        int bn = 0, bc = 1, bo = 2, sn = 0, sc = 1, so = 2;
        StepArgs b = a, c = a;
        b.prefetch = c.prefetch = 1;
        for (int L = 1; L <= g.nt + 1; ++L) {
            const bool BG = L <= g.nt, SC = L >= 2;
            for (int f = 0; f < NF; ++f) {
                b.nw[f] = lv[0][bn][f];
                b.cur[f] = lv[0][bc][f];
                b.old[f] = lv[0][bo][f];
                c.nw[f] = lv[1][sn][f];
                c.cur[f] = lv[1][sc][f];
                c.old[f] = lv[1][so][f];
            }
            for (int f = 0; f < 4; ++f) {
                c.bgn[f] = lv[0][bc][f];  // background level L-1
                c.bgc[f] = lv[0][bo][f];  // background level L-2
            }
            b.src = BG ? pml_source(L, g.nsource, g.fp, g.dt, g.dx) : 0.0f;
            c.src = 0.0f;
            if (BG && SC) k_pml_fused<true, true><<<grd, blk, 0, st>>>(b, c);
            else if (BG) k_pml_fused<true, false><<<grd, blk, 0, st>>>(b, c);
            else k_pml_fused<false, true><<<grd, blk, 0, st>>>(b, c);
            RTM_CUDA(cudaGetLastError());
            ++launches;
            if (SC) TRY(record_level(L - 1, lv[0][bc], lv[1][sn]));
            if (BG) {
                const int t = bo;
                bo = bc;
                bc = bn;
                bn = t;
            }
            if (SC) {
                const int t = so;
                so = sc;
                sc = sn;
                sn = t;
            }
        }
    }
    for (int it = 1; !fused && it <= g.nt; ++it) {
        for (int w = 0; w < 2; ++w) {
            for (int f = 0; f < NF; ++f) {
                a.nw[f] = lv[w][inew][f];
                a.cur[f] = lv[w][icur][f];
                a.old[f] = lv[w][iold][f];
            }
            for (int f = 0; f < 4; ++f) {
                a.bgn[f] = lv[0][inew][f];
                a.bgc[f] = lv[0][icur][f];
            }
            a.src = w == 0 ? pml_source(it, g.nsource, g.fp, g.dt, g.dx) : 0.0f;
            if (tile) {
                TileArgs ta;
                ta.err = g_pml.err.p;
                ta.stall = g_pml.test_stall && it == 1 && w == 0 ? g_pml.stall.p : nullptr;
                for (int f = 0; f < NF; ++f) ta.plane[f] = (w * 3 + icur) * NF + f;
                for (int f = 0; f < 4; ++f) ta.plane[NF + f] = inew * NF + f;
                if (w == 0) k_pml_tile<false><<<grdt, TT_THREADS, 10 * TT_SIZE * 4 + 128, st>>>(a, ta, tm);
                else k_pml_tile<true><<<grdt, TT_THREADS, 14 * TT_SIZE * 4 + 128, st>>>(a, ta, tm);
            } else if (one) {
                // register bound: at least MINB blocks of 256 threads an SM
                if (minb == 8) {
                    if (w == 0) k_pml_step1b<false, 8><<<grd, blk, 0, st>>>(a);
                    else k_pml_step1b<true, 8><<<grd, blk, 0, st>>>(a);
                } else if (minb == 6) {
                    if (w == 0) k_pml_step1b<false, 6><<<grd, blk, 0, st>>>(a);
                    else k_pml_step1b<true, 6><<<grd, blk, 0, st>>>(a);
                } else if (minb == 5) {
                    if (w == 0) k_pml_step1b<false, 5><<<grd, blk, 0, st>>>(a);
                    else k_pml_step1b<true, 5><<<grd, blk, 0, st>>>(a);
                } else {
                    if (w == 0) k_pml_step1<false><<<grd, blk, 0, st>>>(a);
                    else k_pml_step1<true><<<grd, blk, 0, st>>>(a);
                }
            } else {
                if (w == 0) k_pml_step<false><<<grd4, blk, 0, st>>>(a);
                else k_pml_step<true><<<grd4, blk, 0, st>>>(a);
            }
            RTM_CUDA(cudaGetLastError());
            ++launches;
        }
        TRY(record_level(it, lv[0][inew], lv[1][inew]));
        const int t = iold;
        iold = icur;
        icur = inew;
        inew = t;
    }
    g_pml.launches = launches;
    int err = 0;
    RTM_CUDA(cudaMemcpyAsync(&err, g_pml.err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    RTM_CUDA(cudaStreamSynchronize(st));
    if (err) {
        rtm_set_error("a PML step tile's copies did not arrive within the time limit");
        return RTM_ERR_TIMEOUT;
    }
    return RTM_OK;
}

Geom make_geom(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp, int nsnap,
               int nseis, int abc, int zrec, int free_surface, int lame)
{
    Geom g;
    g.nz = nz;
    g.nx = nx;
    g.nt = nt;
    g.dx = dx;
    g.dt = dt;
    g.xs = xsource;
    g.zs = zsource;
    g.nsource = nsource;
    g.fp = fp;
    g.nsnap = nsnap;
    g.nseis = nseis;
    g.abc = abc;
    g.zrec = zrec;
    g.free_surface = free_surface != 0;
    g.lame = lame != 0;
    return g;
}

}  // namespace

extern "C" int pml_born_dev(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp,
                            int nsnap, int nseis, int abc, int zrec, int free_surface, int lame,
                            const float *const *model, float *const *seis, float *const *snap, void *stream)
{
    RTM_CHECK_ARG(model && seis && snap, "null argument");
    for (int k = 0; k < 6; ++k) RTM_CHECK_ARG(model[k] && seis[k] && snap[k], "null plane");
    const Geom g = make_geom(nz, nx, nt, dx, dt, xsource, zsource, nsource, fp, nsnap, nseis, abc, zrec, free_surface,
                             lame);
    std::lock_guard<std::mutex> lk(g_pml_mutex);
    return pml_run(g, model, seis, snap, (cudaStream_t)stream);
}

// Pinned host staging of the host-array entry, grown on demand: the
// caller's arrays are copied through it (a host copy, then one DMA), which
// on this machine is several times faster than DMA from pageable memory.
struct PinnedBuf {
    float *p = nullptr;
    size_t n = 0;
    ~PinnedBuf()
    {
        if (p) cudaFreeHost(p);
    }
    int alloc(size_t count)
    {
        if (count <= n && p) return RTM_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (cudaHostAlloc(&p, count * sizeof(float), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            rtm_set_error("cudaHostAlloc of %zu bytes failed", count * sizeof(float));
            return RTM_ERR_NOMEM;
        }
        n = count;
        return RTM_OK;
    }
};

extern "C" int pml_born_c_(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp,
                           int nsnap, int nseis, int abc, int zrec, int free_surface, int lame, const float *vp0,
                           const float *vs0, const float *rho0, const float *dvp, const float *dvs, const float *drho,
                           float *const *seis, float *const *snap)
{
    RTM_CHECK_ARG(vp0 && vs0 && rho0 && dvp && dvs && drho && seis && snap, "null argument");
    for (int k = 0; k < 6; ++k) RTM_CHECK_ARG(seis[k] && snap[k], "null output");
    const Geom g = make_geom(nz, nx, nt, dx, dt, xsource, zsource, nsource, fp, nsnap, nseis, abc, zrec, free_surface,
                             lame);
    TRY(check_geom(g));
    TRY(ensure_device());
    std::lock_guard<std::mutex> lk(g_pml_mutex);
    const long long n = (long long)nz * nx;
    const size_t total = (size_t)(6 * n + 6 * g.seis_n() + 6 * g.snap_n());
    static DevBuf<float> io;
    static PinnedBuf pin;
    TRY(io.alloc(total));
    TRY(pin.alloc(total));
    const float *host_in[6] = {vp0, vs0, rho0, dvp, dvs, drho};
    const float *dm[6];
    float *ds[6], *dc[6];
    for (int k = 0; k < 6; ++k) {
        memcpy(pin.p + k * n, host_in[k], sizeof(float) * n);
        dm[k] = io.p + k * n;
        ds[k] = io.p + 6 * n + k * g.seis_n();
        dc[k] = io.p + 6 * n + 6 * g.seis_n() + k * g.snap_n();
    }
    RTM_CUDA(cudaMemcpyAsync(io.p, pin.p, sizeof(float) * 6 * n, cudaMemcpyHostToDevice, 0));
    TRY(pml_run(g, dm, ds, dc, 0));
    // the outputs are contiguous on the device: one copy back
    RTM_CUDA(cudaMemcpyAsync(pin.p + 6 * n, io.p + 6 * n, sizeof(float) * (total - 6 * n), cudaMemcpyDeviceToHost, 0));
    RTM_CUDA(cudaStreamSynchronize(0));
    for (int k = 0; k < 6; ++k) {
        memcpy(seis[k], pin.p + 6 * n + k * g.seis_n(), sizeof(float) * g.seis_n());
        memcpy(snap[k], pin.p + 6 * n + 6 * g.seis_n() + k * g.snap_n(), sizeof(float) * g.snap_n());
    }
    return RTM_OK;
}

extern "C" long long pml_born_launches(void) { return g_pml.launches; }

extern "C" int pml_set_test_stall(int on)
{
    g_pml.test_stall = on != 0;
    return RTM_OK;
}

extern "C" int pml_set_kernel(int kind)
{
    const int base = kind & 15, minb = kind >> 4;
    RTM_CHECK_ARG((base <= 8 && base != 5 && base != 7 && kind >= 0 && (minb == 0 || minb == 5 || minb == 6 || minb == 8)),
                  "kernel kind %d", kind);
    g_pml_kind = kind;
    return RTM_OK;
}
