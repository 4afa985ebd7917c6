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
// Layout in HBM: Fortran-ordered (nz, nx) planes, z fastest, leading
// dimension nz: the 6 model planes, 10 coefficient planes (rho_Vx, rho_Vz,
// l, mi, l2mi, dl, dmi, dl2mi, drho_Vx, drho_Vz), 2 wavefields x 3 levels x
// 10 parts, the PML tables (nz x abc per x side, abc x nx per z side; pml0
// and pml1), the receiver lines and the snapshot cubes.  Levels rotate by
// pointer.
//
// Kernels: one thread per cell, 32 (z) x 8 (x) blocks, every tap a
// read-only load served by L1/L2.  One launch advances the background, one
// the scattered wavefield (it needs the background's new level at its
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

struct StepArgs {
    int nz, nx;
    float *nw[NF];
    const float *cur[NF];
    const float *old[NF];
    const float *cf[NC];
    const float *bgn[4];  // scattered step: the background's new and current
    const float *bgc[4];  // velocity parts
    PmlTabs t;
    int zs, xs;
    float src;
};

template <int K>
__device__ __forceinline__ bool in_range(int nz, int nx, int iz, int ix)
{
    constexpr StK k = stk(K);
    return iz >= k.z0 && iz <= nz - k.zoff && ix >= k.x0 && ix <= nx - k.xoff;
}

// c1*(m[hi1]-m[lo1]) + ... + c5*(m[hi5]-m[lo5]), left to right
template <int K>
__device__ __forceinline__ float sten(const float *__restrict__ m, long long p, long long ld)
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

template <int F, bool BORN>
__device__ __forceinline__ void advance_part(const StepArgs &a, int iz, int ix, long long p)
{
    constexpr Part P = part_of(F);
    float v = 0.0f;
    if (in_range<P.st>(a.nz, a.nx, iz, ix)) {
        const float cf = __ldg(a.cf[P.coef] + p);
        v = add_rn(v, mul_rn(cf, sten<P.st>(a.cur[P.a], p, a.nz)));
        v = add_rn(v, mul_rn(cf, sten<P.st>(a.cur[P.b], p, a.nz)));
    }
    v = add_rn(v, pml_apply<P.axis, P.avg, 0>(a.t, a.nz, a.nx, iz, ix, __ldg(a.old[F] + p)));
    if constexpr (!BORN && P.src) {
        if (iz == a.zs && ix == a.xs) v = add_rn(v, a.src);
    }
    if constexpr (BORN) {
        constexpr BornT B = born_of(F);
        if constexpr (B.st < 0) {
            if (iz >= 6 && iz <= a.nz - 5)
                v = add_rn(v, mul_rn(sub_rn(__ldg(a.bgn[B.a] + p), __ldg(a.bgc[B.a] + p)), __ldg(a.cf[B.coef] + p)));
        } else {
            constexpr int KB = B.st < 0 ? 0 : B.st;
            if (in_range<KB>(a.nz, a.nx, iz, ix)) {
                const float cf = __ldg(a.cf[B.coef] + p);
                v = add_rn(v, mul_rn(cf, sten<KB>(a.bgn[B.a], p, a.nz)));
                v = add_rn(v, mul_rn(cf, sten<KB>(a.bgn[B.b], p, a.nz)));
            }
        }
    }
    a.nw[F][p] = pml_apply<P.axis, P.avg, 1>(a.t, a.nz, a.nx, iz, ix, v);
}

constexpr int BZ = 32, BX = 8;

template <bool BORN>
__global__ void __launch_bounds__(BZ * BX) k_pml_step(const StepArgs a)
{
    const int iz = blockIdx.x * BZ + threadIdx.x + 1;
    const int ix = blockIdx.y * BX + threadIdx.y + 1;
    if (iz > a.nz || ix > a.nx) return;
    const long long p = (long long)(ix - 1) * a.nz + iz - 1;
    advance_part<VXX, BORN>(a, iz, ix, p);
    advance_part<VXZ, BORN>(a, iz, ix, p);
    advance_part<VZX, BORN>(a, iz, ix, p);
    advance_part<VZZ, BORN>(a, iz, ix, p);
    advance_part<SXXX, BORN>(a, iz, ix, p);
    advance_part<SXXZ, BORN>(a, iz, ix, p);
    advance_part<SZZX, BORN>(a, iz, ix, p);
    advance_part<SZZZ, BORN>(a, iz, ix, p);
    advance_part<SXZX, BORN>(a, iz, ix, p);
    advance_part<SXZZ, BORN>(a, iz, ix, p);
}

// Model set-up (born-mod.f90:331-389).  The harmonic averages are written in
// place column by column in the reference, but every neighbour it reads
// ((iz+1, ix), (iz, ix+1), (iz+1, ix+1)) is still unaveraged then, so each
// cell here recomputes its neighbours' unaveraged values from the inputs.
struct ModelArgs {
    int nz, nx, lame;
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
    const long long nz = m.nz, p = (ix - 1) * nz + iz - 1;
    const float aux1 = m.aux1;
    // densities on the staggered grids (:360-384)
    if (iz < m.nz) {
        m.cf[C_RVX][p] = div_rn(mul_rn(aux1, 1.0f), mul_rn(0.5f, add_rn(m.rho0[p + 1], m.rho0[p])));
        m.cf[C_DRVX][p] = -add_rn(div_rn(m.drho[p + 1], m.rho0[p + 1]), div_rn(m.drho[p], m.rho0[p]));
    } else {
        m.cf[C_RVX][p] = mul_rn(aux1, div_rn(1.0f, m.rho0[p]));
        m.cf[C_DRVX][p] = -div_rn(m.drho[p], m.rho0[p]);
    }
    if (ix < m.nx) {
        m.cf[C_RVZ][p] = div_rn(mul_rn(aux1, 1.0f), mul_rn(0.5f, add_rn(m.rho0[p + nz], m.rho0[p])));
        m.cf[C_DRVZ][p] = -add_rn(div_rn(m.drho[p + nz], m.rho0[p + nz]), div_rn(m.drho[p], m.rho0[p]));
    } else {
        m.cf[C_RVZ][p] = mul_rn(aux1, div_rn(1.0f, m.rho0[p]));
        m.cf[C_DRVZ][p] = -div_rn(m.drho[p], m.rho0[p]);
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
    m.cf[C_L][p] = l;
    m.cf[C_MI][p] = mi;
    m.cf[C_L2MI][p] = l2mi;
    m.cf[C_DL][p] = dl;
    m.cf[C_DMI][p] = dmi;
    m.cf[C_DL2MI][p] = dl2mi;
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
    int nz, nx, a, nseis, zrec, count;
    const float *w[2][NF];  // background, scattered new level
    float *seis[6];         // Vx, Vz, P, Vx_b, Vz_b, P_b: (nseis, nx - 2 abc)
};

__global__ void k_pml_record(const RecArgs r)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (ix > r.nx - 2 * r.a - 1) return;
    const long long nz = r.nz, c = ix + r.a;
    const long long q = (long long)(ix - 1) * r.nseis + r.count - 1;
    const long long pr = (c - 1) * nz + r.zrec - 1;  // (zrec, c)
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
    int nz, nx;
    long long off;
    const float *w[2][NF];
    float *snap[6];
};

__global__ void k_pml_snap(const SnapArgs s)
{
    const int iz = blockIdx.x * BZ + threadIdx.x + 1;
    const int ix = blockIdx.y * BX + threadIdx.y + 1;
    if (iz < 2 || iz > s.nz - 2 || ix < 2 || ix > s.nx - 2) return;
    const long long p = (long long)(ix - 1) * s.nz + iz - 1, o = s.off + p;
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

struct PmlState {
    DevBuf<float> buf;
    double last_ms = 0.0;
    long long launches = 0;
};
PmlState g_pml;

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
    const long long n = (long long)g.nz * g.nx;
    const long long ntab = 4LL * g.nz * g.abc + 4LL * g.abc * g.nx;
    TRY(g_pml.buf.alloc((size_t)(NC * n + 60 * n + ntab + 1)));
    float *cf = g_pml.buf.p, *fld = cf + NC * n, *tab = fld + 60 * n;
    RTM_CUDA(cudaMemsetAsync(fld, 0, sizeof(float) * 60 * n, st));
    for (int k = 0; k < 6; ++k) {
        RTM_CUDA(cudaMemsetAsync(seis[k], 0, sizeof(float) * g.seis_n(), st));
        RTM_CUDA(cudaMemsetAsync(snap[k], 0, sizeof(float) * g.snap_n(), st));
    }
    long long launches = 0;
    const dim3 blk(BZ, BX), grd(ceil_div(g.nz, BZ), ceil_div(g.nx, BX));
    {
        ModelArgs m;
        m.nz = g.nz;
        m.nx = g.nx;
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
    for (int k = 0; k < NC; ++k) a.cf[k] = cf + k * n;
    a.t = T;
    a.zs = g.zs;
    a.xs = g.xs;
    for (int it = 1; it <= g.nt; ++it) {
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
            if (w == 0) {
                a.src = pml_source(it, g.nsource, g.fp, g.dt, g.dx);
                k_pml_step<false><<<grd, blk, 0, st>>>(a);
            } else {
                a.src = 0.0f;
                k_pml_step<true><<<grd, blk, 0, st>>>(a);
            }
            RTM_CUDA(cudaGetLastError());
            ++launches;
        }
        if ((float)it > nsource2 && it % dseis == 0 && countseis <= g.nseis) {
            RecArgs r;
            r.nz = g.nz;
            r.nx = g.nx;
            r.a = g.abc == 0 ? 1 : g.abc;
            r.nseis = g.nseis;
            r.zrec = g.zrec;
            r.count = countseis;
            for (int w = 0; w < 2; ++w)
                for (int f = 0; f < NF; ++f) r.w[w][f] = lv[w][inew][f];
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
            SnapArgs s;
            s.nz = g.nz;
            s.nx = g.nx;
            s.off = (long long)(countsnap - 1) * n;
            for (int w = 0; w < 2; ++w)
                for (int f = 0; f < NF; ++f) s.w[w][f] = lv[w][inew][f];
            for (int k = 0; k < 6; ++k) s.snap[k] = snap[k];
            k_pml_snap<<<grd, blk, 0, st>>>(s);
            RTM_CUDA(cudaGetLastError());
            ++launches;
            countsnap++;
        }
        const int t = iold;
        iold = icur;
        icur = inew;
        inew = t;
    }
    g_pml.launches = launches;
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
    return pml_run(g, model, seis, snap, (cudaStream_t)stream);
}

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
    const long long n = (long long)nz * nx;
    static DevBuf<float> io;
    TRY(io.alloc((size_t)(6 * n + 6 * g.seis_n() + 6 * g.snap_n())));
    const float *host_in[6] = {vp0, vs0, rho0, dvp, dvs, drho};
    const float *dm[6];
    float *ds[6], *dc[6];
    for (int k = 0; k < 6; ++k) {
        float *p = io.p + k * n;
        RTM_CUDA(cudaMemcpyAsync(p, host_in[k], sizeof(float) * n, cudaMemcpyHostToDevice, 0));
        dm[k] = p;
        ds[k] = io.p + 6 * n + k * g.seis_n();
        dc[k] = io.p + 6 * n + 6 * g.seis_n() + k * g.snap_n();
    }
    TRY(pml_run(g, dm, ds, dc, 0));
    for (int k = 0; k < 6; ++k) {
        RTM_CUDA(cudaMemcpyAsync(seis[k], ds[k], sizeof(float) * g.seis_n(), cudaMemcpyDeviceToHost, 0));
        RTM_CUDA(cudaMemcpyAsync(snap[k], dc[k], sizeof(float) * g.snap_n(), cudaMemcpyDeviceToHost, 0));
    }
    RTM_CUDA(cudaStreamSynchronize(0));
    return RTM_OK;
}

extern "C" long long pml_born_launches(void) { return g_pml.launches; }
