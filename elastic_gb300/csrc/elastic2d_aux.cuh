// Setup and imaging kernels of the 2D elastic path (everything around the
// fused step kernel).  Planes use the column layout plane[ix*ld + iz].
#pragma once
#include "common.cuh"
#include "elastic2d.cuh"

namespace eg {

// model_op + rtmmod_init + aux_*_c (W/model-mod.f90:21-89,
// W/rtmlib-mod.f90:51-58, W/rtm-mod-adj.f90:111-113) for one cell.  The
// in-place Fortran sweeps are equivalent to: averaged lambda/mu at the
// clamped cell (min(max(i,1),n-2)); m1_x averages rho along z, m1_z along
// x, with 1/rho on the last row / column.  Outputs (unmasked):
// m1_x, m1_z (scaled by aux=dt/dx), lambda_avg, mu_avg, aux_m2, aux_m3,
// aux_m2m3.  Every operation is separately rounded in the reference order.
template <typename T>
__global__ void k_model_coef(int nz, int nx, const T *__restrict__ rho, const T *__restrict__ lam,
                             const T *__restrict__ mu, int ldin, T aux, T *m1x, T *m1z, T *m2o, T *m3o,
                             T *a2, T *a3, T *a23, int ldout)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iz >= nz || ix >= nx) return;
    auto R = [&](const T *p, int z, int x) { return p[(long long)x * ldin + z]; };
    const T one = T(1), half = T(0.5), four = T(4), two = T(2);
    T vx = (iz < nz - 1) ? div_rn(one, mul_rn(half, add_rn(R(rho, iz + 1, ix), R(rho, iz, ix)))) : div_rn(one, R(rho, iz, ix));
    T vz = (ix < nx - 1) ? div_rn(one, mul_rn(half, add_rn(R(rho, iz, ix + 1), R(rho, iz, ix)))) : div_rn(one, R(rho, iz, ix));
    const int cz = min(max(iz, 1), nz - 2), cx = min(max(ix, 1), nx - 2);
    const T l00 = R(lam, cz, cx), l10 = R(lam, cz + 1, cx), l01 = R(lam, cz, cx + 1), l11 = R(lam, cz + 1, cx + 1);
    const T m00 = R(mu, cz, cx), m10 = R(mu, cz + 1, cx), m01 = R(mu, cz, cx + 1), m11 = R(mu, cz + 1, cx + 1);
    T l = div_rn(four, add_rn(add_rn(add_rn(div_rn(one, l00), div_rn(one, l10)), div_rn(one, l01)), div_rn(one, l11)));
    T m;
    if (m00 == T(0) || m10 == T(0) || m01 == T(0) || m11 == T(0))
        m = T(0);
    else
        m = div_rn(four, add_rn(add_rn(add_rn(div_rn(one, m00), div_rn(one, m10)), div_rn(one, m01)), div_rn(one, m11)));
    const long long o = (long long)ix * ldout + iz;
    if (m1x) m1x[o] = mul_rn(aux, vx);
    if (m1z) m1z[o] = mul_rn(aux, vz);
    if (m2o) m2o[o] = l;
    if (m3o) m3o[o] = m;
    if (a2) a2[o] = mul_rn(aux, l);
    if (a3) a3[o] = mul_rn(aux, m);
    if (a23) a23[o] = mul_rn(aux, add_rn(l, mul_rn(two, m)));
}

// Masked coefficient planes: zero outside the loop ranges of the operator
// that uses each coefficient (W/rtmlib-modC.c:83-93, 0-based inclusive):
//   M1X  iz 4..nz-6, ix 5..nx-6      M1Z  iz 5..nz-6, ix 4..nx-6
//   A2, A23  iz 4..nz-6, ix 4..nx-6  A3   iz 5..nz-6, ix 5..nx-6
template <typename T>
__global__ void k_mask_coef(int nz, int nx, const T *m1x, const T *m1z, const T *a2, const T *a3, const T *a23,
                            int ldin, T *o_m1x, T *o_m1z, T *o_a2, T *o_a3, T *o_a23, int ldout)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iz >= nz || ix >= nx) return;
    const long long i = (long long)ix * ldin + iz, o = (long long)ix * ldout + iz;
    const bool z4 = iz >= 4 && iz <= nz - 6, z5 = iz >= 5 && iz <= nz - 6;
    const bool x4 = ix >= 4 && ix <= nx - 6, x5 = ix >= 5 && ix <= nx - 6;
    o_m1x[o] = (z4 && x5) ? m1x[i] : T(0);
    o_m1z[o] = (z5 && x4) ? m1z[i] : T(0);
    o_a2[o] = (z4 && x4) ? a2[i] : T(0);
    o_a3[o] = (z5 && x5) ? a3[i] : T(0);
    o_a23[o] = (z4 && x4) ? a23[i] : T(0);
}

// model_delta (W/model-mod.f90:91-171): thresholded harmonic averages of
// dlambda and dmu (dm1_x/dm1_z are unused by the reference and not formed).
template <typename T>
__global__ void k_model_delta(int nz, int nx, const T *__restrict__ dm2, const T *__restrict__ dm3, int ldin,
                              T *o2, T *o3, int ldout)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iz >= nz || ix >= nx) return;
    auto R = [&](const T *p, int z, int x) { return p[(long long)x * ldin + z]; };
    const int cz = min(max(iz, 1), nz - 2), cx = min(max(ix, 1), nx - 2);
    const T one = T(1), four = T(4), th = T(1e-2);
    auto avg = [&](const T *p) {
        const T v00 = R(p, cz, cx), v10 = R(p, cz + 1, cx), v01 = R(p, cz, cx + 1), v11 = R(p, cz + 1, cx + 1);
        if (v00 < th || v10 < th || v01 < th || v11 < th) return T(0);
        return div_rn(four, add_rn(add_rn(add_rn(div_rn(one, v00), div_rn(one, v10)), div_rn(one, v01)), div_rn(one, v11)));
    };
    const long long o = (long long)ix * ldout + iz;
    o2[o] = avg(dm2);
    o3[o] = avg(dm3);
}

// Source-wavefield partials of image_init (W/image-mod-rtm.f90:26-67) at
// one cell of one level, from the levels it and it+1 of Vx and Vz:
//   S1 = (1/dt)(Vx(it+1)-Vx(it))  (0 at the last level), S2 likewise for Vz
//   S4 = P-stencil_x(Vx)/dx  (ix,iz in 4..n-6 0-based), S5 = P-stencil_z(Vz)/dx
//   S3 = S4 + S5
//   S6 = M-stencil_z(Vx)/dx + M-stencil_x(Vz)/dx  (ix,iz in 5..n-6)
// `last` marks the last level.  Reads go through the read-only cache.
template <bool EXACT, typename T>
struct SrcPartials {
    T s1, s2, s3, s4, s5, s6;
};

template <bool EXACT, typename T>
__device__ __forceinline__ SrcPartials<EXACT, T> src_partials(const T *__restrict__ vx, const T *__restrict__ vz,
                                                               const T *__restrict__ vx1, const T *__restrict__ vz1,
                                                               bool last, long long o, int iz, int ix, int nz, int nx,
                                                               int ld, T inv_dt, T inv_dx)
{
    using A = Ar<EXACT>;
    SrcPartials<EXACT, T> p;
    if (!last) {
        p.s1 = A::mul(inv_dt, A::sub(__ldg(vx1 + o), __ldg(vx + o)));
        p.s2 = A::mul(inv_dt, A::sub(__ldg(vz1 + o), __ldg(vz + o)));
    } else {
        p.s1 = p.s2 = T(0);
    }
    p.s4 = p.s5 = p.s6 = T(0);
    if (iz >= 4 && iz <= nz - 6 && ix >= 4 && ix <= nx - 6) {
        T a = T(0), b = T(0);
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const T ta = A::mul(StagCoef<T>::c(k), A::sub(__ldg(vx + o + (long long)(5 - k) * ld), __ldg(vx + o + (long long)(-4 + k) * ld)));
            const T tb = A::mul(StagCoef<T>::c(k), A::sub(__ldg(vz + o + (5 - k)), __ldg(vz + o + (-4 + k))));
            a = k == 0 ? ta : A::add(a, ta);
            b = k == 0 ? tb : A::add(b, tb);
        }
        p.s4 = A::mul(a, inv_dx);
        p.s5 = A::mul(b, inv_dx);
    }
    p.s3 = A::add(p.s4, p.s5);
    if (iz >= 5 && iz <= nz - 6 && ix >= 5 && ix <= nx - 6) {
        T a = T(0), b = T(0);
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const T ta = A::mul(StagCoef<T>::c(k), A::sub(__ldg(vx + o + (4 - k)), __ldg(vx + o + (-5 + k))));
            const T tb = A::mul(StagCoef<T>::c(k), A::sub(__ldg(vz + o + (long long)(4 - k) * ld), __ldg(vz + o + (long long)(-5 + k) * ld)));
            a = k == 0 ? ta : A::add(a, ta);
            b = k == 0 ? tb : A::add(b, tb);
        }
        p.s6 = A::add(A::mul(a, inv_dx), A::mul(b, inv_dx));
    }
    return p;
}

// image_init as full histories S1..S6 (W/image-mod-rtm.f90:26-67).
template <typename T>
__global__ void k_image_init(int nz, int nx, int nt, const T *vx, const T *vz, T *S1, T *S2, T *S3, T *S4, T *S5,
                             T *S6, T inv_dt, T inv_dx)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y, it = blockIdx.z;
    if (iz >= nz) return;
    const long long plane = (long long)nz * nx;
    const long long o = (long long)ix * nz + iz, lv = (long long)it * plane;
    const bool last = it == nt - 1;
    auto p = src_partials<true, T>(vx + lv, vz + lv, last ? vx + lv : vx + lv + plane, last ? vz + lv : vz + lv + plane,
                                   last, o, iz, ix, nz, nx, nz, inv_dt, inv_dx);
    S1[lv + o] = p.s1; S2[lv + o] = p.s2; S3[lv + o] = p.s3;
    S4[lv + o] = p.s4; S5[lv + o] = p.s5; S6[lv + o] = p.s6;
}

// Imaging condition over full histories in forward time order, identical to
// image_op2(adj) (W/image-mod-rtm.f90:146-162): one thread per cell sums
// it = 1..nt with S computed on the fly from the source Vx, Vz history.
template <typename T>
__global__ void k_image_hist(int nz, int nx, int nt, const T *svx, const T *svz, const T *avx, const T *avz,
                             const T *axx, const T *azz, const T *axz, T *dm1, T *dm2, T *dm3, T inv_dt, T inv_dx)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iz >= nz) return;
    const long long plane = (long long)nz * nx;
    const long long o = (long long)ix * nz + iz;
    T r1 = T(0), r2 = T(0), r3 = T(0);
    const T two = T(2);
    for (int it = 0; it < nt; it++) {
        const long long lv = (long long)it * plane;
        const bool last = it == nt - 1;
        auto p = src_partials<true, T>(svx + lv, svz + lv, last ? svx + lv : svx + lv + plane,
                                       last ? svz + lv : svz + lv + plane, last, o, iz, ix, nz, nx, nz, inv_dt, inv_dx);
        const T vx = avx[lv + o], vz = avz[lv + o], xx = axx[lv + o], zz = azz[lv + o], xz = axz[lv + o];
        r1 = add_rn(add_rn(r1, mul_rn(vx, p.s1)), mul_rn(vz, p.s2));
        r2 = sub_rn(sub_rn(r2, mul_rn(xx, p.s3)), mul_rn(zz, p.s3));
        r3 = sub_rn(sub_rn(sub_rn(r3, mul_rn(mul_rn(xx, two), p.s4)), mul_rn(mul_rn(zz, two), p.s5)), mul_rn(xz, p.s6));
    }
    dm1[o] = r1;
    dm2[o] = r2;
    dm3[o] = r3;
}

// Born secondary sources of level it (image_op2 forward,
// W/image-mod-rtm.f90:164-179) added in place to the five planes `buf`
// (buf = s + buf, the reference's "Vx0(it) + Vx0(it-2)" order) or, with
// overwrite, written over them.  S comes from the source levels it, it+1.
template <bool EXACT, typename T>
__global__ void k_born_src(const ShotGeom *shots, int ld, const T *svx, const T *svz, const T *svx1, const T *svz1,
                           int last, const T *dm1, const T *dm2, const T *dm3, T *b0, T *b1, T *b2, T *b3, T *b4,
                           int overwrite, T inv_dt, T inv_dx)
{
    using A = Ar<EXACT>;
    const ShotGeom g = shots[blockIdx.z];
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iz >= g.nz || ix >= g.nx) return;
    const long long o = g.off + (long long)ix * ld + iz;
    auto p = src_partials<EXACT, T>(svx, svz, svx1, svz1, last != 0, o, iz, ix, g.nz, g.nx, ld, inv_dt, inv_dx);
    const T d1 = dm1[o], d2 = dm2[o], d3 = dm3[o], two = T(2);
    const T s0 = A::mul(d1, p.s1);
    const T s1 = A::mul(d1, p.s2);
    const T s2 = A::sub(-A::mul(d2, p.s3), A::mul(A::mul(d3, two), p.s4));
    const T s3 = A::sub(-A::mul(d2, p.s3), A::mul(A::mul(d3, two), p.s5));
    const T s4 = -A::mul(d3, p.s6);
    if (overwrite) {
        b0[o] = s0; b1[o] = s1; b2[o] = s2; b3[o] = s3; b4[o] = s4;
    } else {
        b0[o] = A::add(s0, b0[o]); b1[o] = A::add(s1, b1[o]); b2[o] = A::add(s2, b2[o]);
        b3[o] = A::add(s3, b3[o]); b4[o] = A::add(s4, b4[o]);
    }
}

// Imaging contribution of one adjoint level, accumulated into dm1..dm3 with
// Kahan compensation (c1..c3), S from the stored source levels it, it+1.
// Used by the streaming RTM, which visits levels in reverse time order.
template <typename T>
__device__ __forceinline__ void kahan_add(T &s, T &c, T v)
{
    const T y = v - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
}

template <bool EXACT, typename T>
__global__ void k_image_level(const ShotGeom *shots, int ld, const T *svx, const T *svz, const T *svx1, const T *svz1,
                              int last, const T *avx, const T *avz, const T *axx, const T *azz, const T *axz, T *dm1,
                              T *dm2, T *dm3, T *cm1, T *cm2, T *cm3, T inv_dt, T inv_dx)
{
    using A = Ar<EXACT>;
    const ShotGeom g = shots[blockIdx.z];
    const int iz = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y;
    if (iz >= g.nz || ix >= g.nx) return;
    const long long o = g.off + (long long)ix * ld + iz;
    auto p = src_partials<EXACT, T>(svx, svz, svx1, svz1, last != 0, o, iz, ix, g.nz, g.nx, ld, inv_dt, inv_dx);
    const T vx = avx[o], vz = avz[o], xx = axx[o], zz = azz[o], xz = axz[o], two = T(2);
    const T t1 = A::add(A::mul(vx, p.s1), A::mul(vz, p.s2));
    const T t2 = -A::add(A::mul(xx, p.s3), A::mul(zz, p.s3));
    const T t3 = -A::add(A::add(A::mul(A::mul(xx, two), p.s4), A::mul(A::mul(zz, two), p.s5)), A::mul(xz, p.s6));
    T s, c;
    s = dm1[o]; c = cm1[o]; kahan_add(s, c, t1); dm1[o] = s; cm1[o] = c;
    s = dm2[o]; c = cm2[o]; kahan_add(s, c, t2); dm2[o] = s; cm2[o] = c;
    s = dm3[o]; c = cm3[o]; kahan_add(s, c, t3); dm3[o] = s; cm3[o] = c;
}

// Receiver traces: Fortran (nt,nx) per component (column ix holds a trace)
// <-> device [it][slot][ix] of one shot.
template <typename T>
__global__ void k_traces_to_dev(int nt, int nx, int ncomp, const T *const *host_layout, T *dev)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int it = blockIdx.y, c = blockIdx.z;
    if (ix >= nx) return;
    dev[((long long)it * ncomp + c) * nx + ix] = host_layout[c][(long long)ix * nt + it];
}

template <typename T>
__global__ void k_traces_from_dev(int nt, int nx, int ncomp, const T *dev, T *const *host_layout)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    const int ix = blockIdx.y, c = blockIdx.z;
    if (it >= nt) return;
    host_layout[c][(long long)ix * nt + it] = dev[((long long)it * ncomp + c) * nx + ix];
}

}  // namespace eg
