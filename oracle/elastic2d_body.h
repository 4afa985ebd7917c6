/*
 * CPU restatement of the 2D elastic RTM/Born hot path of lgan/elastic.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests/, the smoke check
 * and bench.py's CPU-baseline leg call it as the checker.  The product
 * (elastic_gb300/csrc) never links or calls it.
 *
 * This body is included twice by elastic2d.c: once with R=float (the
 * reference's own precision, default REAL in the Fortran) and once with
 * R=double (the FP64 oracle for error statements and dot-product tests).
 *
 * Layout follows the Fortran exactly: column-major (nz,nx[,nt]), z fastest.
 * Indices in the loops below are 1-based, as in the Fortran, and mapped with
 * I2/I3.  Every loop keeps the reference's bounds and every expression keeps
 * its left-to-right evaluation order, so that the float build reproduces the
 * reference bit for bit when compiled with -ffp-contract=off.
 *
 * Reference files (paths inside the lgan/elastic project):
 *   W = 2d_rtm_restart/Src_working
 *   W/model-mod.f90, W/rtmlib-mod.f90, W/source-mod.f90, W/abc-mod.f90,
 *   W/rtm-mod-adj.f90, W/image-mod-rtm.f90, W/rtmlib-modC.c
 */

#define I2(iz, ix) ((size_t)((iz) - 1) + (size_t)nz * (size_t)((ix) - 1))
#define I3(iz, ix, it) (I2(iz, ix) + (size_t)nz * (size_t)nx * (size_t)((it) - 1))
#define PLANE ((size_t)nz * (size_t)nx)

/* 10th-order staggered coefficients, W/rtmlib-mod.f90:15 (single-precision
   division in Fortran; the float rounding of the double quotient is the same
   for all five, checked in tests/test_oracle.py,
   test_stagger_coefficients_single_precision). */
static const R FN(c1) = (R)(35.0 / 294912.0);
static const R FN(c2) = (R)(-405.0 / 229376.0);
static const R FN(c3) = (R)(567.0 / 40960.0);
static const R FN(c4) = (R)(-735.0 / 8192.0);
static const R FN(c5) = (R)(19845.0 / 16384.0);

/* ---------------------------------------------------------------- a1 ---- */
/* model_op: W/model-mod.f90:21-89.  m1 = rho, m2 = lambda, m3 = mu (m2, m3
   are replaced in place by their staggered harmonic averages). */
void FN(ora_model_op)(int nz, int nx, const R *m1, R *m2, R *m3, R *m1_x, R *m1_z)
{
    int iz, ix;
    for (ix = 1; ix <= nx; ix++)
        for (iz = 1; iz <= nz - 1; iz++)
            m1_x[I2(iz, ix)] = (R)1.0 / ((R)0.5 * (m1[I2(iz + 1, ix)] + m1[I2(iz, ix)]));
    for (ix = 1; ix <= nx - 1; ix++)
        for (iz = 1; iz <= nz; iz++)
            m1_z[I2(iz, ix)] = (R)1.0 / ((R)0.5 * (m1[I2(iz, ix + 1)] + m1[I2(iz, ix)]));
    for (iz = 1; iz <= nz; iz++) m1_z[I2(iz, nx)] = ((R)1.0 / m1[I2(iz, nx)]);
    for (ix = 1; ix <= nx; ix++) m1_x[I2(nz, ix)] = ((R)1.0 / m1[I2(nz, ix)]);
    for (ix = 2; ix <= nx - 1; ix++)
        for (iz = 2; iz <= nz - 1; iz++) {
            m2[I2(iz, ix)] = (R)4.0 / (((((R)1.0 / m2[I2(iz, ix)]) + ((R)1.0 / m2[I2(iz + 1, ix)])) +
                                       ((R)1.0 / m2[I2(iz, ix + 1)])) + ((R)1.0 / m2[I2(iz + 1, ix + 1)]));
            if (m3[I2(iz, ix)] == 0 || m3[I2(iz + 1, ix)] == 0 || m3[I2(iz, ix + 1)] == 0 ||
                m3[I2(iz + 1, ix + 1)] == 0)
                m3[I2(iz, ix)] = (R)0.0;
            else
                m3[I2(iz, ix)] = (R)4.0 / (((((R)1.0 / m3[I2(iz, ix)]) + ((R)1.0 / m3[I2(iz + 1, ix)])) +
                                           ((R)1.0 / m3[I2(iz, ix + 1)])) + ((R)1.0 / m3[I2(iz + 1, ix + 1)]));
        }
    for (ix = 1; ix <= nx; ix++) {
        m2[I2(1, ix)] = m2[I2(2, ix)];
        m2[I2(nz, ix)] = m2[I2(nz - 1, ix)];
        m3[I2(1, ix)] = m3[I2(2, ix)];
        m3[I2(nz, ix)] = m3[I2(nz - 1, ix)];
    }
    for (iz = 1; iz <= nz; iz++) {
        m2[I2(iz, 1)] = m2[I2(iz, 2)];
        m2[I2(iz, nx)] = m2[I2(iz, nx - 1)];
        m3[I2(iz, 1)] = m3[I2(iz, 2)];
        m3[I2(iz, nx)] = m3[I2(iz, nx - 1)];
    }
}

/* ---------------------------------------------------------------- a2 ---- */
/* rtmmod_init (W/rtmlib-mod.f90:51-58) plus the aux_*_c arrays of rtm_init
   (W/rtm-mod-adj.f90:111-113), which are the same products. */
void FN(ora_rtmmod_init)(int nz, int nx, R dx, R dt, R *m1_x, R *m1_z, const R *m2, const R *m3,
                         R *aux_m2, R *aux_m3, R *aux_m2m3)
{
    size_t i, n = PLANE;
    R aux = dt / dx;
    for (i = 0; i < n; i++) {
        m1_x[i] = aux * m1_x[i];
        m1_z[i] = aux * m1_z[i];
        aux_m2[i] = aux * m2[i];
        aux_m3[i] = aux * m3[i];
        aux_m2m3[i] = aux * (m2[i] + (R)2.0 * m3[i]);
    }
}

/* ---------------------------------------------------------------- a3 ---- */
/* source_op2: W/source-mod.f90:31-44 (Ricker, nsource samples of delay). */
void FN(ora_source_op2)(int nt, R dt, R fp, int nsource, R *source)
{
    int it, ft = nsource / 10;
    R pi = (R)3.14159265, aux, t;
    for (it = 0; it < nt; it++) source[it] = 0;
    for (it = ft; it <= nt; it++) {
        if (it < 1) continue; /* Fortran array is 1-based */
        t = ((R)it * dt) - (((R)nsource * dt) / (R)2.0);
        aux = ((((pi * pi) * fp) * fp) * t) * t;
#if R_IS_DOUBLE
        source[it - 1] = ((R)10.0e7 * ((R)1.0 - (R)2.0 * aux)) * exp(-aux);
#else
        source[it - 1] = ((R)10.0e7 * ((R)1.0 - (R)2.0 * aux)) * expf(-aux);
#endif
    }
}

/* ---------------------------------------------------------------- a4 ---- */
/* abc_init: W/abc-mod.f90:20-57.  filter has abc+5 entries (0-based here:
   filter[i-1] = Fortran filter(i)).  abc=0 reads filter(0) out of bounds in
   the reference; the oracle defines it as "no sponge" (all ones). */
void FN(ora_abc_init)(int abc, R *filter)
{
    int ix, abc2 = abc + 5;
    R alfa = (R)0.09, aux;
    if (abc <= 0) {
        for (ix = 0; ix < abc2; ix++) filter[ix] = (R)1.0;
        return;
    }
    for (ix = 1; ix <= abc; ix++) {
        aux = ((R)1.0 * (R)ix) / ((R)1.0 * (R)abc);
#if R_IS_DOUBLE
        filter[ix - 1] = exp((-alfa * aux) * aux);
#else
        filter[ix - 1] = expf((-alfa * aux) * aux);
#endif
    }
    for (ix = abc + 1; ix <= abc2; ix++) filter[ix - 1] = filter[abc - 1];
}

/* K: W/abc-mod.f90:59-78.  Top/bottom strips first, then left/right strips;
   corner cells are multiplied twice. */
void FN(ora_K)(int nz, int nx, int abc, const R *filter, R *data)
{
    int iz, ix, abc2 = abc + 5;
    for (ix = 1; ix <= nx; ix++)
        for (iz = 1; iz <= abc2; iz++) {
            data[I2(iz, ix)] = data[I2(iz, ix)] * filter[(abc2 - iz + 1) - 1];
            data[I2(nz - abc2 + iz, ix)] = data[I2(nz - abc2 + iz, ix)] * filter[iz - 1];
        }
    for (ix = 1; ix <= abc2; ix++)
        for (iz = 1; iz <= nz; iz++) {
            data[I2(iz, ix)] = data[I2(iz, ix)] * filter[(abc2 - ix + 1) - 1];
            data[I2(iz, nx - abc2 + ix)] = data[I2(iz, nx - abc2 + ix)] * filter[ix - 1];
        }
}

/* ---------------------------------------------------------------- a5 ---- */
/* Forward staggered operators Ax..J (adj=.false., add=.true.),
   W/rtmlib-mod.f90:200-633.  A "P" stencil pairs (i+5,i-4)...(i+1,i), an "M"
   stencil pairs (i+4,i-5)...(i,i-1).  dir 0 = along z, 1 = along x. */

static void FN(fwd_op)(int nz, int nx, const R *coef, const R *model, R *data, int dir, int st,
                       int izlo, int ixlo)
{
    int iz, ix, k;
    const R c[5] = {FN(c1), FN(c2), FN(c3), FN(c4), FN(c5)};
#pragma omp parallel for private(iz, k) schedule(static)
    for (ix = ixlo; ix <= nx - 5; ix++)
        for (iz = izlo; iz <= nz - 5; iz++) {
            R poly = 0;
            for (k = 0; k < 5; k++) {
                int hi = (st == ST_P) ? 5 - k : 4 - k;  /* offset of the + sample */
                int lo = (st == ST_P) ? -4 + k : -5 + k; /* offset of the - sample */
                R a, b, term;
                if (dir == 0) {
                    a = model[I2(iz + hi, ix)];
                    b = model[I2(iz + lo, ix)];
                } else {
                    a = model[I2(iz, ix + hi)];
                    b = model[I2(iz, ix + lo)];
                }
                term = c[k] * (a - b);
                poly = (k == 0) ? term : poly + term;
            }
            data[I2(iz, ix)] = data[I2(iz, ix)] + coef[I2(iz, ix)] * poly;
        }
}

/* Operator table: stencil direction, type and lower bounds (upper bound is
   always n-5). */
void FN(ora_Ax)(int nz, int nx, const R *m1_x, const R *model, R *data) { FN(fwd_op)(nz, nx, m1_x, model, data, 1, ST_M, 5, 6); }
void FN(ora_Bx)(int nz, int nx, const R *m1_x, const R *model, R *data) { FN(fwd_op)(nz, nx, m1_x, model, data, 0, ST_P, 5, 6); }
void FN(ora_Az)(int nz, int nx, const R *m1_z, const R *model, R *data) { FN(fwd_op)(nz, nx, m1_z, model, data, 1, ST_P, 6, 5); }
void FN(ora_Bz)(int nz, int nx, const R *m1_z, const R *model, R *data) { FN(fwd_op)(nz, nx, m1_z, model, data, 0, ST_M, 6, 5); }
void FN(ora_D)(int nz, int nx, const R *aux_m2m3, const R *model, R *data) { FN(fwd_op)(nz, nx, aux_m2m3, model, data, 1, ST_P, 5, 5); }
void FN(ora_E)(int nz, int nx, const R *aux_m2, const R *model, R *data) { FN(fwd_op)(nz, nx, aux_m2, model, data, 0, ST_P, 5, 5); }
void FN(ora_F)(int nz, int nx, const R *aux_m2, const R *model, R *data) { FN(fwd_op)(nz, nx, aux_m2, model, data, 1, ST_P, 5, 5); }
void FN(ora_G)(int nz, int nx, const R *aux_m2m3, const R *model, R *data) { FN(fwd_op)(nz, nx, aux_m2m3, model, data, 0, ST_P, 5, 5); }
void FN(ora_H)(int nz, int nx, const R *aux_m3, const R *model, R *data) { FN(fwd_op)(nz, nx, aux_m3, model, data, 0, ST_M, 6, 6); }
void FN(ora_J)(int nz, int nx, const R *aux_m3, const R *model, R *data) { FN(fwd_op)(nz, nx, aux_m3, model, data, 1, ST_M, 6, 6); }

/* Adjoint scatter operators Ax_c..J_c, W/rtmlib-mod.f90:635-998 (the
   transposes of the forward operators above, same loop bounds).  P-type
   transposes scatter to offsets +5..-4, M-type to +4..-5. */
static void FN(adj_op)(int nz, int nx, const R *coef, R *model, const R *data, int dir, int st,
                       int izlo, int ixlo)
{
    int iz, ix, k;
    const R c[5] = {FN(c1), FN(c2), FN(c3), FN(c4), FN(c5)};
    for (ix = ixlo; ix <= nx - 5; ix++)
        for (iz = izlo; iz <= nz - 5; iz++) {
            /* plus side: offsets hi(k) for k=0..4 receive +c[k]; then minus side
               offsets lo(k) for k=4..0 receive -c[k] (statement order of the
               Fortran: +c1 at the far end first, -c1 at the other end last). */
            for (k = 0; k < 5; k++) {
                int hi = (st == ST_P) ? 5 - k : 4 - k;
                size_t o = dir == 0 ? I2(iz + hi, ix) : I2(iz, ix + hi);
                model[o] = model[o] + (coef[I2(iz, ix)] * c[k]) * data[I2(iz, ix)];
            }
            for (k = 4; k >= 0; k--) {
                int lo = (st == ST_P) ? -4 + k : -5 + k;
                size_t o = dir == 0 ? I2(iz + lo, ix) : I2(iz, ix + lo);
                model[o] = model[o] - (coef[I2(iz, ix)] * c[k]) * data[I2(iz, ix)];
            }
        }
}

void FN(ora_Ax_c)(int nz, int nx, R *model, const R *data, const R *m1_x) { FN(adj_op)(nz, nx, m1_x, model, data, 1, ST_M, 5, 6); }
void FN(ora_Bx_c)(int nz, int nx, R *model, const R *data, const R *m1_x) { FN(adj_op)(nz, nx, m1_x, model, data, 0, ST_P, 5, 6); }
void FN(ora_Az_c)(int nz, int nx, R *model, const R *data, const R *m1_z) { FN(adj_op)(nz, nx, m1_z, model, data, 1, ST_P, 6, 5); }
void FN(ora_Bz_c)(int nz, int nx, R *model, const R *data, const R *m1_z) { FN(adj_op)(nz, nx, m1_z, model, data, 0, ST_M, 6, 5); }
void FN(ora_D_c)(int nz, int nx, R *model, const R *data, const R *a) { FN(adj_op)(nz, nx, a, model, data, 1, ST_P, 5, 5); }
void FN(ora_E_c)(int nz, int nx, R *model, const R *data, const R *a) { FN(adj_op)(nz, nx, a, model, data, 0, ST_P, 5, 5); }
void FN(ora_F_c)(int nz, int nx, R *model, const R *data, const R *a) { FN(adj_op)(nz, nx, a, model, data, 1, ST_P, 5, 5); }
void FN(ora_G_c)(int nz, int nx, R *model, const R *data, const R *a) { FN(adj_op)(nz, nx, a, model, data, 0, ST_P, 5, 5); }
void FN(ora_H_c)(int nz, int nx, R *model, const R *data, const R *a) { FN(adj_op)(nz, nx, a, model, data, 0, ST_M, 6, 6); }
void FN(ora_J_c)(int nz, int nx, R *model, const R *data, const R *a) { FN(adj_op)(nz, nx, a, model, data, 1, ST_M, 6, 6); }

/* ---------------------------------------------------------------- a6 ---- */
/* One forward update of level `it` from it-1 (neighbours) and it-2 (own),
   W/rtm-mod-adj.f90:225-252.  Used for the source wavefield (srcval added
   at (zsrc,xsrc) to both normal stresses) and, with born=1, for the
   scattered field whose secondary sources are already in level it
   (W/rtm-mod-adj.f90:323-348).  level it-2 may be absent (it2 < 1). */
static void FN(fwd_level)(int nz, int nx, int it, int born, R *Vx, R *Vz, R *sxx, R *szz, R *sxz,
                          const R *m1_x, const R *m1_z, const R *aux_m2, const R *aux_m3,
                          const R *aux_m2m3, int abc, const R *filter, int sponge, R srcval,
                          int zsrc, int xsrc)
{
    size_t n = PLANE, i;
    R *vx = Vx + (size_t)(it - 1) * n, *vz = Vz + (size_t)(it - 1) * n;
    R *xx = sxx + (size_t)(it - 1) * n, *zz = szz + (size_t)(it - 1) * n, *xz = sxz + (size_t)(it - 1) * n;
    const R *vx1 = Vx + (size_t)(it - 2) * n, *vz1 = Vz + (size_t)(it - 2) * n;
    const R *xx1 = sxx + (size_t)(it - 2) * n, *zz1 = szz + (size_t)(it - 2) * n, *xz1 = sxz + (size_t)(it - 2) * n;
    int have2 = it >= 3;
    const R *vx2 = Vx + (size_t)(it - 3) * n, *vz2 = Vz + (size_t)(it - 3) * n;
    const R *xx2 = sxx + (size_t)(it - 3) * n, *zz2 = szz + (size_t)(it - 3) * n, *xz2 = sxz + (size_t)(it - 3) * n;

    /* Vx */
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; i++) vx[i] = born ? (have2 ? vx[i] + vx2[i] : vx[i]) : (have2 ? vx2[i] : 0);
    FN(ora_Ax)(nz, nx, m1_x, xx1, vx);
    FN(ora_Bx)(nz, nx, m1_x, xz1, vx);
    if (sponge) FN(ora_K)(nz, nx, abc, filter, vx);
    /* Vz */
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; i++) vz[i] = born ? (have2 ? vz[i] + vz2[i] : vz[i]) : (have2 ? vz2[i] : 0);
    FN(ora_Az)(nz, nx, m1_z, xz1, vz);
    FN(ora_Bz)(nz, nx, m1_z, zz1, vz);
    if (sponge) FN(ora_K)(nz, nx, abc, filter, vz);
    /* sigmaxx */
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; i++) xx[i] = born ? (have2 ? xx[i] + xx2[i] : xx[i]) : (have2 ? xx2[i] : 0);
    if (!born) xx[I2(zsrc, xsrc)] = xx[I2(zsrc, xsrc)] + srcval;
    FN(ora_D)(nz, nx, aux_m2m3, vx1, xx);
    FN(ora_E)(nz, nx, aux_m2, vz1, xx);
    if (sponge) FN(ora_K)(nz, nx, abc, filter, xx);
    /* sigmazz */
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; i++) zz[i] = born ? (have2 ? zz[i] + zz2[i] : zz[i]) : (have2 ? zz2[i] : 0);
    if (!born) zz[I2(zsrc, xsrc)] = zz[I2(zsrc, xsrc)] + srcval;
    FN(ora_F)(nz, nx, aux_m2, vx1, zz);
    FN(ora_G)(nz, nx, aux_m2m3, vz1, zz);
    if (sponge) FN(ora_K)(nz, nx, abc, filter, zz);
    /* sigmaxz */
#pragma omp parallel for schedule(static)
    for (i = 0; i < n; i++) xz[i] = born ? (have2 ? xz[i] + xz2[i] : xz[i]) : (have2 ? xz2[i] : 0);
    FN(ora_H)(nz, nx, aux_m3, vx1, xz);
    FN(ora_J)(nz, nx, aux_m3, vz1, xz);
    if (sponge) FN(ora_K)(nz, nx, abc, filter, xz);
}

/* Source wavefield over the full history, W/rtm-mod-adj.f90:178-261.
   zsrc/xsrc are 1-based (Fortran).  Levels 1 and 2 follow :186-198 (level 2
   holds dt*source(1) at the source and is not sponged); level 3 (:200-222)
   equals the general update with a zero level 1. */
void FN(ora_forward)(int nz, int nx, int nt, R dt, int zsrc, int xsrc, const R *source, int abc,
                     const R *filter, const R *m1_x, const R *m1_z, const R *aux_m2, const R *aux_m3,
                     const R *aux_m2m3, R *Vx, R *Vz, R *sxx, R *szz, R *sxz)
{
    size_t n = PLANE, i;
    int it;
    for (i = 0; i < n * (size_t)nt; i++) Vx[i] = Vz[i] = sxx[i] = szz[i] = sxz[i] = 0;
    if (nt >= 2) {
        sxx[(size_t)n + I2(zsrc, xsrc)] = sxx[(size_t)n + I2(zsrc, xsrc)] + dt * source[0];
        szz[(size_t)n + I2(zsrc, xsrc)] = szz[(size_t)n + I2(zsrc, xsrc)] + dt * source[0];
    }
    for (it = 3; it <= nt; it++)
        FN(fwd_level)(nz, nx, it, 0, Vx, Vz, sxx, szz, sxz, m1_x, m1_z, aux_m2, aux_m3, aux_m2m3, abc,
                      filter, 1, dt * source[it - 2], zsrc, xsrc);
}

/* ---------------------------------------------------------------- a7 ---- */
/* image_init: W/image-mod-rtm.f90:26-67 with T (:268-299), vxdx (:301-344),
   vzdz (:346-390), vxdz (:392-435), vzdx (:437-480).  S arrays are
   (nz,nx,nt); S1(nt)=S2(nt)=0.  dz=dx is assumed by the reference (1/dx
   is used for z derivatives too). */
void FN(ora_image_init)(int nz, int nx, int nt, R dx, R dt, const R *Vx, const R *Vz, R *S1, R *S2,
                        R *S3, R *S4, R *S5, R *S6)
{
    size_t n = PLANE, tot = n * (size_t)nt, i;
    int it, iz, ix, k;
    const R c[5] = {FN(c1), FN(c2), FN(c3), FN(c4), FN(c5)};
    R at = (R)1.0 / dt, ax = (R)1.0 / dx;
    for (i = 0; i < tot; i++) S1[i] = S2[i] = S3[i] = S4[i] = S5[i] = S6[i] = 0;
    for (it = 1; it <= nt - 1; it++)
        for (i = 0; i < n; i++) {
            size_t a = (size_t)(it - 1) * n + i;
            S1[a] = S1[a] + at * (Vx[a + n] - Vx[a]);
            S2[a] = S2[a] + at * (Vz[a + n] - Vz[a]);
        }
    for (it = 1; it <= nt; it++) {
        /* vxdx: P stencil along x, ix 5..nx-5, iz 5..nz-5 */
        for (ix = 5; ix <= nx - 5; ix++)
            for (iz = 5; iz <= nz - 5; iz++) {
                R p = 0;
                for (k = 0; k < 5; k++) {
                    R t = c[k] * (Vx[I3(iz, ix + 5 - k, it)] - Vx[I3(iz, ix - 4 + k, it)]);
                    p = k == 0 ? t : p + t;
                }
                S4[I3(iz, ix, it)] = S4[I3(iz, ix, it)] + p * ax;
            }
        /* vzdz: P stencil along z */
        for (ix = 5; ix <= nx - 5; ix++)
            for (iz = 5; iz <= nz - 5; iz++) {
                R p = 0;
                for (k = 0; k < 5; k++) {
                    R t = c[k] * (Vz[I3(iz + 5 - k, ix, it)] - Vz[I3(iz - 4 + k, ix, it)]);
                    p = k == 0 ? t : p + t;
                }
                S5[I3(iz, ix, it)] = S5[I3(iz, ix, it)] + p * ax;
            }
    }
    for (i = 0; i < tot; i++) S3[i] = S4[i] + S5[i];
    for (it = 1; it <= nt; it++) {
        /* vxdz: M stencil along z, ix 6..nx-5, iz 6..nz-5 */
        for (ix = 6; ix <= nx - 5; ix++)
            for (iz = 6; iz <= nz - 5; iz++) {
                R p = 0;
                for (k = 0; k < 5; k++) {
                    R t = c[k] * (Vx[I3(iz + 4 - k, ix, it)] - Vx[I3(iz - 5 + k, ix, it)]);
                    p = k == 0 ? t : p + t;
                }
                S6[I3(iz, ix, it)] = S6[I3(iz, ix, it)] + p * ax;
            }
    }
    for (it = 1; it <= nt; it++) {
        /* vzdx: M stencil along x, added to S6 */
        for (ix = 6; ix <= nx - 5; ix++)
            for (iz = 6; iz <= nz - 5; iz++) {
                R p = 0;
                for (k = 0; k < 5; k++) {
                    R t = c[k] * (Vz[I3(iz, ix + 4 - k, it)] - Vz[I3(iz, ix - 5 + k, it)]);
                    p = k == 0 ? t : p + t;
                }
                S6[I3(iz, ix, it)] = S6[I3(iz, ix, it)] + p * ax;
            }
    }
}

/* ---------------------------------------------------------------- a8 ---- */
/* model_delta: W/model-mod.f90:91-171.  dm1_x/dm1_z are computed by the
   reference but never used afterwards; dm2/dm3 are replaced in place. */
void FN(ora_model_delta)(int nz, int nx, const R *dm1, R *dm1_x, R *dm1_z, R *dm2, R *dm3)
{
    int iz, ix;
    size_t i;
    for (i = 0; i < PLANE; i++) dm1_x[i] = dm1_z[i] = 0;
    for (ix = 1; ix <= nx; ix++)
        for (iz = 1; iz <= nz - 1; iz++)
            dm1_x[I2(iz, ix)] = (dm1[I2(iz + 1, ix)] <= (R)1.0e-1 || dm1[I2(iz, ix)] <= (R)1.0e-1)
                                    ? (R)0.0
                                    : (R)0.5 * (dm1[I2(iz + 1, ix)] + dm1[I2(iz, ix)]);
    for (ix = 1; ix <= nx - 1; ix++)
        for (iz = 1; iz <= nz; iz++)
            dm1_z[I2(iz, ix)] = (dm1[I2(iz, ix + 1)] <= (R)1.0e-1 || dm1[I2(iz, ix)] <= (R)1.0e-1)
                                    ? (R)0.0
                                    : (R)0.5 * (dm1[I2(iz, ix + 1)] + dm1[I2(iz, ix)]);
    for (iz = 1; iz <= nz; iz++) dm1_z[I2(iz, nx)] = dm1[I2(iz, nx)] <= (R)1.0e-1 ? (R)0.0 : dm1[I2(iz, nx)];
    for (ix = 1; ix <= nx; ix++) dm1_x[I2(nz, ix)] = dm1[I2(nz, ix)] <= (R)1.0e-1 ? (R)0.0 : dm1[I2(nz, ix)];
    for (ix = 2; ix <= nx - 1; ix++)
        for (iz = 2; iz <= nz - 1; iz++) {
            if (dm2[I2(iz, ix)] < (R)1e-2 || dm2[I2(iz + 1, ix)] < (R)1e-2 || dm2[I2(iz, ix + 1)] < (R)1e-2 ||
                dm2[I2(iz + 1, ix + 1)] < (R)1e-2)
                dm2[I2(iz, ix)] = (R)0.0;
            else
                dm2[I2(iz, ix)] = (R)4.0 / (((((R)1.0 / dm2[I2(iz, ix)]) + ((R)1.0 / dm2[I2(iz + 1, ix)])) +
                                            ((R)1.0 / dm2[I2(iz, ix + 1)])) + ((R)1.0 / dm2[I2(iz + 1, ix + 1)]));
            if (dm3[I2(iz, ix)] < (R)1e-2 || dm3[I2(iz + 1, ix)] < (R)1e-2 || dm3[I2(iz, ix + 1)] < (R)1e-2 ||
                dm3[I2(iz + 1, ix + 1)] < (R)1e-2)
                dm3[I2(iz, ix)] = (R)0.0;
            else
                dm3[I2(iz, ix)] = (R)4.0 / (((((R)1.0 / dm3[I2(iz, ix)]) + ((R)1.0 / dm3[I2(iz + 1, ix)])) +
                                            ((R)1.0 / dm3[I2(iz, ix + 1)])) + ((R)1.0 / dm3[I2(iz + 1, ix + 1)]));
        }
    for (ix = 1; ix <= nx; ix++) {
        dm2[I2(1, ix)] = dm2[I2(2, ix)];
        dm2[I2(nz, ix)] = dm2[I2(nz - 1, ix)];
        dm3[I2(1, ix)] = dm3[I2(2, ix)];
        dm3[I2(nz, ix)] = dm3[I2(nz - 1, ix)];
    }
    for (iz = 1; iz <= nz; iz++) {
        dm2[I2(iz, 1)] = dm2[I2(iz, 2)];
        dm2[I2(iz, nx)] = dm2[I2(iz, nx - 1)];
        dm3[I2(iz, 1)] = dm3[I2(iz, 2)];
        dm3[I2(iz, nx)] = dm3[I2(iz, nx - 1)];
    }
}

/* image_op2 for the Lame parameterisation, W/image-mod-rtm.f90:145-180.
   adj=1: dm1 (drho), dm2 (dlambda), dm3 (dmu) += imaging sums over it=1..nt
   (add=0 zeroes them first).  adj=0: the wavefield arrays receive the Born
   secondary sources (add=0 zeroes them first). */
void FN(ora_image_op2)(int nz, int nx, int nt, int adj, int add, R *dm1, R *dm2, R *dm3, R *Vx, R *Vz,
                       R *sxx, R *szz, R *sxz, const R *S1, const R *S2, const R *S3, const R *S4,
                       const R *S5, const R *S6)
{
    size_t n = PLANE, i;
    int it;
    if (adj) {
        if (!add)
            for (i = 0; i < n; i++) dm1[i] = dm2[i] = dm3[i] = 0;
        for (it = 1; it <= nt; it++)
            for (i = 0; i < n; i++) {
                size_t a = (size_t)(it - 1) * n + i;
                dm1[i] = (dm1[i] + (Vx[a] * S1[a])) + (Vz[a] * S2[a]);
                dm2[i] = (dm2[i] - (sxx[a] * S3[a])) - (szz[a] * S3[a]);
                dm3[i] = ((dm3[i] - ((sxx[a] * (R)2.0) * S4[a])) - ((szz[a] * (R)2.0) * S5[a])) - (sxz[a] * S6[a]);
            }
    } else {
        if (!add)
            for (i = 0; i < n * (size_t)nt; i++) Vx[i] = Vz[i] = sxx[i] = szz[i] = sxz[i] = 0;
        for (it = 1; it <= nt; it++)
            for (i = 0; i < n; i++) {
                size_t a = (size_t)(it - 1) * n + i;
                Vx[a] = Vx[a] + (dm1[i] * S1[a]);
                Vz[a] = Vz[a] + (dm1[i] * S2[a]);
                sxx[a] = (sxx[a] - (dm2[i] * S3[a])) - ((dm3[i] * (R)2.0) * S4[a]);
                szz[a] = (szz[a] - (dm2[i] * S3[a])) - ((dm3[i] * (R)2.0) * S5[a]);
                sxz[a] = sxz[a] - (dm3[i] * S6[a]);
            }
    }
}

/* ---------------------------------------------------------------- a9 ---- */
/* Born scattered propagation with secondary sources already stored in the
   five arrays (W/rtm-mod-adj.f90:291-357), then receiver sampling of all
   five components at row zrec (1-based) into (nt,nx) arrays (:361-375). */
void FN(ora_born_scatter)(int nz, int nx, int nt, int zrec, int abc, const R *filter, const R *m1_x,
                          const R *m1_z, const R *aux_m2, const R *aux_m3, const R *aux_m2m3, R *Vx,
                          R *Vz, R *sxx, R *szz, R *sxz, R *dVx, R *dVz, R *dsxx, R *dszz, R *dsxz)
{
    int it, ix;
    FN(ora_K)(nz, nx, abc, filter, Vx);
    FN(ora_K)(nz, nx, abc, filter, Vz);
    FN(ora_K)(nz, nx, abc, filter, sxx);
    FN(ora_K)(nz, nx, abc, filter, szz);
    FN(ora_K)(nz, nx, abc, filter, sxz);
    for (it = 2; it <= nt; it++)
        FN(fwd_level)(nz, nx, it, 1, Vx, Vz, sxx, szz, sxz, m1_x, m1_z, aux_m2, aux_m3, aux_m2m3, abc, filter,
                      1, 0, 1, 1);
    for (ix = 1; ix <= nx; ix++)
        for (it = 1; it <= nt; it++) {
            size_t d = (size_t)(it - 1) + (size_t)nt * (size_t)(ix - 1);
            dVx[d] = Vx[I3(zrec, ix, it)];
            dVz[d] = Vz[I3(zrec, ix, it)];
            dsxx[d] = sxx[I3(zrec, ix, it)];
            dszz[d] = szz[I3(zrec, ix, it)];
            dsxz[d] = sxz[I3(zrec, ix, it)];
        }
}

/* --------------------------------------------------------------- a11 ---- */
/* rtm_op3_c_: the C gather recursion, W/rtmlib-modC.c:29-313, restated on
   unpadded arrays.  Coefficients are masked to the forward operators' loop
   ranges as at :83-93 and neighbours outside the grid read as zero.  Levels
   are 0-based here as in the C: it = nt-3 .. 0. */
static R FN(mask_get)(int nz, int nx, const R *a, int iz, int ix, int lz, int hz, int lx, int hx)
{
    if (iz < lz || iz > hz || ix < lx || ix > hx) return 0;
    return a[(size_t)iz + (size_t)nz * (size_t)ix];
}

/* One cell of the recursion.  checked = 1: every neighbour and coefficient
   read goes through the reference's masks and the grid bounds (border
   cells); checked = 0: the cell lies at least 10 cells inside the grid,
   where every mask passes and every neighbour exists, so the reads are
   direct.  Both evaluate the same products in the same order. */
static inline __attribute__((always_inline)) void FN(gather_cell)(int nz, int nx, int iz, int ix, size_t n, int it,
                                                                   R *Vx0, R *Vz0, R *sxx0,
                                   R *szz0, R *sxz0, const R *m1_x, const R *m1_z, const R *aux_m2_c,
                                   const R *aux_m3_c, const R *aux_m2m3_c, const R *c, const int checked)
{
    int k;
    /* masks, 0-based inclusive ranges (W/rtmlib-modC.c:83-93) */
    const int zlo4 = 4, zhi = nz - 6, xlo4 = 4, xhi = nx - 6;
    size_t o = (size_t)iz + (size_t)nz * (size_t)ix + n * (size_t)it;
    size_t o2 = o + 2 * n;
    R v;
#define CF(a, z, x, lz, hz, lx, hx) (checked ? FN(mask_get)(nz, nx, a, z, x, lz, hz, lx, hx) : (a)[(size_t)(z) + (size_t)nz * (size_t)(x)])
#define AM2M3(z, x) CF(aux_m2m3_c, z, x, zlo4, zhi, xlo4, xhi)
#define AM2(z, x) CF(aux_m2_c, z, x, zlo4, zhi, xlo4, xhi)
#define AM3(z, x) CF(aux_m3_c, z, x, 5, zhi, 5, xhi)
#define M1X(z, x) CF(m1_x, z, x, zlo4, zhi, 5, xhi)
#define M1Z(z, x) CF(m1_z, z, x, 5, zhi, xlo4, xhi)
#define FLD(f, z, x, t) ((checked && ((z) < 0 || (z) >= nz || (x) < 0 || (x) >= nx)) ? (R)0 : (f)[(size_t)(z) + (size_t)nz * (size_t)(x) + n * (size_t)(t)])
    /* Vx: x-M5(aux_m2m3, sxx), x-M5(aux_m2, szz), z-P5(aux_m3, sxz) */
    v = Vx0[o] + Vx0[o2];
    for (k = 0; k < 5; k++) v = v + (AM2M3(iz, ix - 5 + k) * c[k]) * FLD(sxx0, iz, ix - 5 + k, it + 1);
    for (k = 4; k >= 0; k--) v = v - (AM2M3(iz, ix + 4 - k) * c[k]) * FLD(sxx0, iz, ix + 4 - k, it + 1);
    for (k = 0; k < 5; k++) v = v + (AM2(iz, ix - 5 + k) * c[k]) * FLD(szz0, iz, ix - 5 + k, it + 1);
    for (k = 4; k >= 0; k--) v = v - (AM2(iz, ix + 4 - k) * c[k]) * FLD(szz0, iz, ix + 4 - k, it + 1);
    for (k = 0; k < 5; k++) v = v + (AM3(iz - 4 + k, ix) * c[k]) * FLD(sxz0, iz - 4 + k, ix, it + 1);
    for (k = 4; k >= 0; k--) v = v - (AM3(iz + 5 - k, ix) * c[k]) * FLD(sxz0, iz + 5 - k, ix, it + 1);
    Vx0[o] = v;
    /* Vz: z-M5(aux_m2, sxx), z-M5(aux_m2m3, szz), x-P5(aux_m3, sxz) */
    v = Vz0[o] + Vz0[o2];
    for (k = 0; k < 5; k++) v = v + (AM2(iz - 5 + k, ix) * c[k]) * FLD(sxx0, iz - 5 + k, ix, it + 1);
    for (k = 4; k >= 0; k--) v = v - (AM2(iz + 4 - k, ix) * c[k]) * FLD(sxx0, iz + 4 - k, ix, it + 1);
    for (k = 0; k < 5; k++) v = v + (AM2M3(iz - 5 + k, ix) * c[k]) * FLD(szz0, iz - 5 + k, ix, it + 1);
    for (k = 4; k >= 0; k--) v = v - (AM2M3(iz + 4 - k, ix) * c[k]) * FLD(szz0, iz + 4 - k, ix, it + 1);
    for (k = 0; k < 5; k++) v = v + (AM3(iz, ix - 4 + k) * c[k]) * FLD(sxz0, iz, ix - 4 + k, it + 1);
    for (k = 4; k >= 0; k--) v = v - (AM3(iz, ix + 5 - k) * c[k]) * FLD(sxz0, iz, ix + 5 - k, it + 1);
    Vz0[o] = v;
    /* sxx: x-P5(m1_x, Vx) */
    v = sxx0[o] + sxx0[o2];
    for (k = 0; k < 5; k++) v = v + (M1X(iz, ix - 4 + k) * c[k]) * FLD(Vx0, iz, ix - 4 + k, it + 1);
    for (k = 4; k >= 0; k--) v = v - (M1X(iz, ix + 5 - k) * c[k]) * FLD(Vx0, iz, ix + 5 - k, it + 1);
    sxx0[o] = v;
    /* szz: z-P5(m1_z, Vz) */
    v = szz0[o] + szz0[o2];
    for (k = 0; k < 5; k++) v = v + (M1Z(iz - 4 + k, ix) * c[k]) * FLD(Vz0, iz - 4 + k, ix, it + 1);
    for (k = 4; k >= 0; k--) v = v - (M1Z(iz + 5 - k, ix) * c[k]) * FLD(Vz0, iz + 5 - k, ix, it + 1);
    szz0[o] = v;
    /* sxz: z-M5(m1_x, Vx), x-M5(m1_z, Vz) */
    v = sxz0[o] + sxz0[o2];
    for (k = 0; k < 5; k++) v = v + (M1X(iz - 5 + k, ix) * c[k]) * FLD(Vx0, iz - 5 + k, ix, it + 1);
    for (k = 4; k >= 0; k--) v = v - (M1X(iz + 4 - k, ix) * c[k]) * FLD(Vx0, iz + 4 - k, ix, it + 1);
    for (k = 0; k < 5; k++) v = v + (M1Z(iz, ix - 5 + k) * c[k]) * FLD(Vz0, iz, ix - 5 + k, it + 1);
    for (k = 4; k >= 0; k--) v = v - (M1Z(iz, ix + 4 - k) * c[k]) * FLD(Vz0, iz, ix + 4 - k, it + 1);
    sxz0[o] = v;
#undef CF
#undef AM2M3
#undef AM2
#undef AM3
#undef M1X
#undef M1Z
#undef FLD
}

void FN(ora_rtm_op3_c)(int nt, int nz, int nx, R *Vx0, R *Vz0, R *sxx0, R *szz0, R *sxz0, const R *m1_x,
                       const R *m1_z, const R *aux_m2_c, const R *aux_m3_c, const R *aux_m2m3_c)
{
    int it, iz, ix;
    size_t n = PLANE;
    const R c[5] = {FN(c1), FN(c2), FN(c3), FN(c4), FN(c5)};
    for (it = nt - 3; it >= 0; it--) {
#pragma omp parallel for private(iz) schedule(static)
        for (ix = 0; ix < nx; ix++)
            for (iz = 0; iz < nz; iz++) {
                if (iz >= 10 && iz <= nz - 11 && ix >= 10 && ix <= nx - 11)
                    FN(gather_cell)(nz, nx, iz, ix, n, it, Vx0, Vz0, sxx0, szz0, sxz0, m1_x, m1_z, aux_m2_c, aux_m3_c,
                                    aux_m2m3_c, c, 0);
                else
                    FN(gather_cell)(nz, nx, iz, ix, n, it, Vx0, Vz0, sxx0, szz0, sxz0, m1_x, m1_z, aux_m2_c, aux_m3_c,
                                    aux_m2m3_c, c, 1);
            }
    }
}

/* --------------------------------------------------------------- a10 ---- */
/* rtm_op3 (W/rtmlib-mod.f90:72-196): zero the five histories, write the
   receiver rows (row zrec, 1-based) for every level, compute level nt-1
   with the scatter operators, then run the C recursion for the rest.
   Receiver arrays are (nt,nx).  With exact=1 the sponge K is applied to
   every adjoint level (the true transpose of the sponged Born operator);
   exact=0 is the reference (no sponge in the adjoint). */
void FN(ora_rtm_op3)(int nt, int nz, int nx, int zrec, R *Vx0, R *Vz0, R *sxx0, R *szz0, R *sxz0,
                     const R *dVx, const R *dVz, const R *dsxx, const R *dszz, const R *dsxz, const R *m1_x,
                     const R *m1_z, const R *aux_m2_c, const R *aux_m3_c, const R *aux_m2m3_c, int exact,
                     int abc, const R *filter)
{
    size_t n = PLANE, i;
    int it, ix;
    for (i = 0; i < n * (size_t)nt; i++) Vx0[i] = Vz0[i] = sxx0[i] = szz0[i] = sxz0[i] = 0;
#define INJ(it_)                                                                         \
    for (ix = 1; ix <= nx; ix++) {                                                       \
        size_t d = (size_t)((it_) - 1) + (size_t)nt * (size_t)(ix - 1);                  \
        Vx0[I3(zrec, ix, it_)] = dVx[d];                                                 \
        Vz0[I3(zrec, ix, it_)] = dVz[d];                                                 \
        sxx0[I3(zrec, ix, it_)] = dsxx[d];                                               \
        szz0[I3(zrec, ix, it_)] = dszz[d];                                               \
        sxz0[I3(zrec, ix, it_)] = dsxz[d];                                               \
    }
#define KLEV(it_)                                                                        \
    if (exact) {                                                                         \
        FN(ora_K)(nz, nx, abc, filter, Vx0 + (size_t)((it_) - 1) * n);                   \
        FN(ora_K)(nz, nx, abc, filter, Vz0 + (size_t)((it_) - 1) * n);                   \
        FN(ora_K)(nz, nx, abc, filter, sxx0 + (size_t)((it_) - 1) * n);                  \
        FN(ora_K)(nz, nx, abc, filter, szz0 + (size_t)((it_) - 1) * n);                  \
        FN(ora_K)(nz, nx, abc, filter, sxz0 + (size_t)((it_) - 1) * n);                  \
    }
    INJ(nt);
    KLEV(nt);
    if (nt >= 2) {
        R *l = Vx0 + (size_t)(nt - 2) * n, *zl = Vz0 + (size_t)(nt - 2) * n;
        R *xxl = sxx0 + (size_t)(nt - 2) * n, *zzl = szz0 + (size_t)(nt - 2) * n, *xzl = sxz0 + (size_t)(nt - 2) * n;
        const R *xxn = sxx0 + (size_t)(nt - 1) * n, *zzn = szz0 + (size_t)(nt - 1) * n, *xzn = sxz0 + (size_t)(nt - 1) * n;
        const R *vxn = Vx0 + (size_t)(nt - 1) * n, *vzn = Vz0 + (size_t)(nt - 1) * n;
        INJ(nt - 1);
        FN(ora_D_c)(nz, nx, l, xxn, aux_m2m3_c);
        FN(ora_F_c)(nz, nx, l, zzn, aux_m2_c);
        FN(ora_H_c)(nz, nx, l, xzn, aux_m3_c);
        FN(ora_E_c)(nz, nx, zl, xxn, aux_m2_c);
        FN(ora_G_c)(nz, nx, zl, zzn, aux_m2m3_c);
        FN(ora_J_c)(nz, nx, zl, xzn, aux_m3_c);
        FN(ora_Ax_c)(nz, nx, xxl, vxn, m1_x);
        FN(ora_Bz_c)(nz, nx, zzl, vzn, m1_z);
        FN(ora_Bx_c)(nz, nx, xzl, vxn, m1_x);
        FN(ora_Az_c)(nz, nx, xzl, vzn, m1_z);
        KLEV(nt - 1);
    }
    for (it = nt - 2; it >= 1; it--) { INJ(it); }
    if (!exact) {
        FN(ora_rtm_op3_c)(nt, nz, nx, Vx0, Vz0, sxx0, szz0, sxz0, m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c);
    } else {
        /* same recursion one level at a time, each level sponged */
        for (it = nt - 2; it >= 1; it--) {
            /* run the gather for the single 0-based level it-1 by viewing the
               histories from level it-1 with a 3-level window */
            R *w[5] = {Vx0 + (size_t)(it - 1) * n, Vz0 + (size_t)(it - 1) * n, sxx0 + (size_t)(it - 1) * n,
                       szz0 + (size_t)(it - 1) * n, sxz0 + (size_t)(it - 1) * n};
            FN(ora_rtm_op3_c)(3, nz, nx, w[0], w[1], w[2], w[3], w[4], m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c);
            KLEV(it);
        }
    }
#undef INJ
#undef KLEV
}

/* --------------------------------------------------------------- a13 ---- */
/* rtm_op2 (W/rtm-mod-adj.f90:132-496) for lame=.true.: forward source
   wavefield, image_init, then Born (adj=0: model_delta, secondary sources,
   scattered loop, receivers) or RTM (adj=1: rtm_op3 and the imaging
   condition).  The model inputs follow rtm_init (:43-117): m1=rho, m2=lambda,
   m3=mu (raw, averaged here).  dm2/dm3 are modified in place by Born as in
   the reference.  Work arrays: 11 volumes of nz*nx*nt. */
void FN(ora_rtm_op2)(int adj, int nz, int nx, int nt, R dx, R dt, int zsrc, int xsrc, int zrec, R fp,
                     int nsource, int abc, const R *rho, const R *lambda, const R *mu, R *dm1, R *dm2,
                     R *dm3, R *dVx, R *dVz, R *dsxx, R *dszz, R *dsxz, int exact)
{
    size_t n = PLANE, tot = n * (size_t)nt;
    R *m2 = (R *)malloc(n * sizeof(R)), *m3 = (R *)malloc(n * sizeof(R));
    R *m1_x = (R *)calloc(n, sizeof(R)), *m1_z = (R *)calloc(n, sizeof(R));
    R *a2 = (R *)malloc(n * sizeof(R)), *a3 = (R *)malloc(n * sizeof(R)), *a23 = (R *)malloc(n * sizeof(R));
    R *src = (R *)malloc((size_t)nt * sizeof(R)), *filt = (R *)malloc((size_t)(abc + 5) * sizeof(R));
    R *W[11];
    int i;
    for (i = 0; i < 11; i++) W[i] = (R *)malloc(tot * sizeof(R));
    memcpy(m2, lambda, n * sizeof(R));
    memcpy(m3, mu, n * sizeof(R));
    FN(ora_model_op)(nz, nx, rho, m2, m3, m1_x, m1_z);
    FN(ora_source_op2)(nt, dt, fp, nsource, src);
    FN(ora_abc_init)(abc, filt);
    FN(ora_rtmmod_init)(nz, nx, dx, dt, m1_x, m1_z, m2, m3, a2, a3, a23);
    FN(ora_forward)(nz, nx, nt, dt, zsrc, xsrc, src, abc, filt, m1_x, m1_z, a2, a3, a23, W[0], W[1], W[2], W[3], W[4]);
    FN(ora_image_init)(nz, nx, nt, dx, dt, W[0], W[1], W[5], W[6], W[7], W[8], W[9], W[10]);
    if (!adj) {
        if (!exact) {
            R *t1 = (R *)malloc(n * sizeof(R)), *t2 = (R *)malloc(n * sizeof(R));
            FN(ora_model_delta)(nz, nx, dm1, t1, t2, dm2, dm3);
            free(t1);
            free(t2);
        }
        FN(ora_image_op2)(nz, nx, nt, 0, 0, dm1, dm2, dm3, W[0], W[1], W[2], W[3], W[4], W[5], W[6], W[7], W[8], W[9], W[10]);
        FN(ora_born_scatter)(nz, nx, nt, zrec, abc, filt, m1_x, m1_z, a2, a3, a23, W[0], W[1], W[2], W[3], W[4],
                             dVx, dVz, dsxx, dszz, dsxz);
    } else {
        FN(ora_rtm_op3)(nt, nz, nx, zrec, W[0], W[1], W[2], W[3], W[4], dVx, dVz, dsxx, dszz, dsxz, m1_x, m1_z, a2,
                        a3, a23, exact, abc, filt);
        FN(ora_image_op2)(nz, nx, nt, 1, 0, dm1, dm2, dm3, W[0], W[1], W[2], W[3], W[4], W[5], W[6], W[7], W[8], W[9], W[10]);
    }
    for (i = 0; i < 11; i++) free(W[i]);
    free(m2); free(m3); free(m1_x); free(m1_z); free(a2); free(a3); free(a23); free(src); free(filt);
}

/* ------------------------------------------------- a6..a13, low memory ---- */
/* The RTM of ora_rtm_op2 (adj=1) with the working set cut from 11 full
   histories to 2 (Vx and Vz of the source wavefield, which image_init
   differentiates in time): the forward stresses and the five adjoint fields
   live in 3-level windows and S1..S6 are formed one level at a time.  Every
   level is computed with the same operations in the same order as
   ora_rtm_op2; only the imaging sums run over it = nt..1 instead of 1..nt,
   so in double precision the images agree with ora_rtm_op2 to rounding
   (~1e-15).  Used as the float64 reference where full histories would not
   fit in host memory (the 2000 x 800 survey geometry). */
static void FN(s_level)(int nz, int nx, int nt, int it, R dx, R dt, const R *Vx, const R *Vz, R *S)
{
    /* S1..S6 of level it (1-based) into S[0..5]; W/image-mod-rtm.f90:26-67 */
    size_t n = PLANE, i;
    int iz, ix, k;
    const R c[5] = {FN(c1), FN(c2), FN(c3), FN(c4), FN(c5)};
    R at = (R)1.0 / dt, ax = (R)1.0 / dx;
    const R *vx = Vx + (size_t)(it - 1) * n, *vz = Vz + (size_t)(it - 1) * n;
    R *S1 = S, *S2 = S + n, *S3 = S + 2 * n, *S4 = S + 3 * n, *S5 = S + 4 * n, *S6 = S + 5 * n;
    for (i = 0; i < 6 * n; i++) S[i] = 0;
    if (it <= nt - 1)
        for (i = 0; i < n; i++) {
            S1[i] = S1[i] + at * (vx[i + n] - vx[i]);
            S2[i] = S2[i] + at * (vz[i + n] - vz[i]);
        }
#define P2(a, z, x) (a)[I2(z, x)]
#pragma omp parallel for private(iz, k) schedule(static)
    for (ix = 5; ix <= nx - 5; ix++)
        for (iz = 5; iz <= nz - 5; iz++) {
            R p = 0;
            for (k = 0; k < 5; k++) {
                R t = c[k] * (P2(vx, iz, ix + 5 - k) - P2(vx, iz, ix - 4 + k));
                p = k == 0 ? t : p + t;
            }
            S4[I2(iz, ix)] = S4[I2(iz, ix)] + p * ax;
        }
#pragma omp parallel for private(iz, k) schedule(static)
    for (ix = 5; ix <= nx - 5; ix++)
        for (iz = 5; iz <= nz - 5; iz++) {
            R p = 0;
            for (k = 0; k < 5; k++) {
                R t = c[k] * (P2(vz, iz + 5 - k, ix) - P2(vz, iz - 4 + k, ix));
                p = k == 0 ? t : p + t;
            }
            S5[I2(iz, ix)] = S5[I2(iz, ix)] + p * ax;
        }
    for (i = 0; i < n; i++) S3[i] = S4[i] + S5[i];
#pragma omp parallel for private(iz, k) schedule(static)
    for (ix = 6; ix <= nx - 5; ix++)
        for (iz = 6; iz <= nz - 5; iz++) {
            R p = 0;
            for (k = 0; k < 5; k++) {
                R t = c[k] * (P2(vx, iz + 4 - k, ix) - P2(vx, iz - 5 + k, ix));
                p = k == 0 ? t : p + t;
            }
            S6[I2(iz, ix)] = S6[I2(iz, ix)] + p * ax;
        }
#pragma omp parallel for private(iz, k) schedule(static)
    for (ix = 6; ix <= nx - 5; ix++)
        for (iz = 6; iz <= nz - 5; iz++) {
            R p = 0;
            for (k = 0; k < 5; k++) {
                R t = c[k] * (P2(vz, iz, ix + 4 - k) - P2(vz, iz, ix - 5 + k));
                p = k == 0 ? t : p + t;
            }
            S6[I2(iz, ix)] = S6[I2(iz, ix)] + p * ax;
        }
#undef P2
}

void FN(ora_rtm_lowmem)(int nz, int nx, int nt, R dx, R dt, int zsrc, int xsrc, int zrec, R fp, int nsource,
                        int abc, const R *rho, const R *lambda, const R *mu, R *dm1, R *dm2, R *dm3,
                        const R *dVx, const R *dVz, const R *dsxx, const R *dszz, const R *dsxz, int exact)
{
    size_t n = PLANE, i;
    int it, ix, f;
    R *m2 = (R *)malloc(n * sizeof(R)), *m3 = (R *)malloc(n * sizeof(R));
    R *m1_x = (R *)calloc(n, sizeof(R)), *m1_z = (R *)calloc(n, sizeof(R));
    R *a2 = (R *)malloc(n * sizeof(R)), *a3 = (R *)malloc(n * sizeof(R)), *a23 = (R *)malloc(n * sizeof(R));
    R *src = (R *)malloc((size_t)nt * sizeof(R)), *filt = (R *)malloc((size_t)(abc + 5) * sizeof(R));
    R *Vx = (R *)calloc(n * (size_t)nt, sizeof(R)), *Vz = (R *)calloc(n * (size_t)nt, sizeof(R));
    R *w = (R *)calloc(3 * 3 * n, sizeof(R));  /* forward stress windows: levels it-2, it-1, it */
    R *A[5], *S = (R *)malloc(6 * n * sizeof(R));
    const R *dd[5] = {dVx, dVz, dsxx, dszz, dsxz};
    for (f = 0; f < 5; f++) A[f] = (R *)calloc(3 * n, sizeof(R));  /* adjoint windows: levels it, it+1, it+2 */
    memcpy(m2, lambda, n * sizeof(R));
    memcpy(m3, mu, n * sizeof(R));
    FN(ora_model_op)(nz, nx, rho, m2, m3, m1_x, m1_z);
    FN(ora_source_op2)(nt, dt, fp, nsource, src);
    FN(ora_abc_init)(abc, filt);
    FN(ora_rtmmod_init)(nz, nx, dx, dt, m1_x, m1_z, m2, m3, a2, a3, a23);

    /* source wavefield (ora_forward): level 1 zero, level 2 the source */
    if (nt >= 2) {
        w[n + I2(zsrc, xsrc)] = w[n + I2(zsrc, xsrc)] + dt * src[0];
        w[3 * n + n + I2(zsrc, xsrc)] = w[3 * n + n + I2(zsrc, xsrc)] + dt * src[0];
    }
    for (it = 3; it <= nt; it++) {
        FN(fwd_level)(nz, nx, 3, 0, Vx + (size_t)(it - 3) * n, Vz + (size_t)(it - 3) * n, w, w + 3 * n,
                      w + 6 * n, m1_x, m1_z, a2, a3, a23, abc, filt, 1, dt * src[it - 2], zsrc, xsrc);
        for (f = 0; f < 3; f++) memmove(w + 3 * n * f, w + 3 * n * f + n, 2 * n * sizeof(R));
    }

    /* adjoint (ora_rtm_op3) with the imaging condition (ora_image_op2) level by level */
    for (i = 0; i < n; i++) dm1[i] = dm2[i] = dm3[i] = 0;
#define INJ1(plane, it_)                                                                     \
    for (ix = 1; ix <= nx; ix++)                                                             \
        for (f = 0; f < 5; f++)                                                              \
            A[f][(plane) * n + I2(zrec, ix)] = dd[f][(size_t)((it_) - 1) + (size_t)nt * (size_t)(ix - 1)];
#define KLEV1(plane)                                                                         \
    if (exact)                                                                               \
        for (f = 0; f < 5; f++) FN(ora_K)(nz, nx, abc, filt, A[f] + (plane) * n);
#define IMG1(plane, it_)                                                                     \
    FN(s_level)(nz, nx, nt, it_, dx, dt, Vx, Vz, S);                                         \
    _Pragma("omp parallel for schedule(static)")                                             \
    for (i = 0; i < n; i++) {                                                                \
        size_t a = (plane) * n + i;                                                          \
        dm1[i] = (dm1[i] + (A[0][a] * S[i])) + (A[1][a] * S[n + i]);                         \
        dm2[i] = (dm2[i] - (A[2][a] * S[2 * n + i])) - (A[3][a] * S[2 * n + i]);             \
        dm3[i] = ((dm3[i] - ((A[2][a] * (R)2.0) * S[3 * n + i])) - ((A[3][a] * (R)2.0) * S[4 * n + i])) \
                 - (A[4][a] * S[5 * n + i]);                                                 \
    }
    INJ1(1, nt);
    KLEV1(1);
    if (nt >= 2) {
        INJ1(0, nt - 1);
        FN(ora_D_c)(nz, nx, A[0], A[2] + n, a23);
        FN(ora_F_c)(nz, nx, A[0], A[3] + n, a2);
        FN(ora_H_c)(nz, nx, A[0], A[4] + n, a3);
        FN(ora_E_c)(nz, nx, A[1], A[2] + n, a2);
        FN(ora_G_c)(nz, nx, A[1], A[3] + n, a23);
        FN(ora_J_c)(nz, nx, A[1], A[4] + n, a3);
        FN(ora_Ax_c)(nz, nx, A[2], A[0] + n, m1_x);
        FN(ora_Bz_c)(nz, nx, A[3], A[1] + n, m1_z);
        FN(ora_Bx_c)(nz, nx, A[4], A[0] + n, m1_x);
        FN(ora_Az_c)(nz, nx, A[4], A[1] + n, m1_z);
        KLEV1(0);
    }
    IMG1(1, nt);
    if (nt >= 2) { IMG1(0, nt - 1); }
    for (it = nt - 2; it >= 1; it--) {
        for (f = 0; f < 5; f++) {
            memmove(A[f] + n, A[f], 2 * n * sizeof(R));
            memset(A[f], 0, n * sizeof(R));
        }
        INJ1(0, it);
        FN(ora_rtm_op3_c)(3, nz, nx, A[0], A[1], A[2], A[3], A[4], m1_x, m1_z, a2, a3, a23);
        KLEV1(0);
        IMG1(0, it);
    }
#undef INJ1
#undef KLEV1
#undef IMG1
    for (f = 0; f < 5; f++) free(A[f]);
    free(S); free(w); free(Vx); free(Vz);
    free(m2); free(m3); free(m1_x); free(m1_z); free(a2); free(a3); free(a23); free(src); free(filt);
}

#undef I2
#undef I3
#undef PLANE
