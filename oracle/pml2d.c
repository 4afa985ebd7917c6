/* Oracle (test infrastructure only): the reference's split-field PML Born
 * modelling program, restated cell by cell.
 *
 *   2d_rtm_restart/working_Src/born-mod.f90:80-776   elastic_op2: model
 *       set-up (:331-389), time loop (:425-745), pointer rotation
 *   working_Src/bornlib-mod.f90:45-617               operators Ax..J, S1..S8
 *   working_Src/pml-mod.f90:23-259                   pml_init and K..R
 *   working_Src/source-mod.f90:42-56                 Ricker source_op2
 *   working_Src/seis-mod-born.f90:36-98              receiver lines
 *   working_Src/snap-mod-born.f90:33-68              snapshots
 *
 * Every field is split into an x part and a z part (Vx = Vx_x + Vx_z, ...);
 * each part advances with three time levels:
 *     new = K1 * ( op(a_x) + op(a_z) + K0 * old [+ source] [+ Born terms] )
 * where op is one of four 10-tap stencils (below), K0 / K1 are the PML's
 * pml0 / pml1 factors on that part's axis (plain or averaged over two
 * neighbouring PML columns or rows), a_x, a_z are the two parts of the field
 * the operator differentiates at the current level.  Background and
 * scattered wavefields advance in the same loop; the scattered one adds the
 * Born terms S1..S8 built from the background's new and current levels.
 * Every product and sum is rounded separately in the reference's order
 * (compiled with -ffp-contract=off), so the result is bit-exact against the
 * reference's execution.  Arrays are Fortran-ordered (nz, nx), z fastest.
 *
 * Two details of the reference are kept as they are:
 *  - the model set-up leaves the outermost rows and columns of lambda, mu
 *    unaveraged (and, for lame = 1, lambda + 2 mu zero there);
 *  - the PML damping d0 of both sides is taken from the first abc columns
 *    (x) or rows (z) of vp (pml-mod.f90:63-89).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

enum { VXX, VXZ, VZX, VZZ, SXXX, SXXZ, SZZX, SZZZ, SXZX, SXZZ, NF };

/* stencil kinds: axis x or z; the five pairs are (p + (5-k+s)*st, p - (6-k-s)*st)
 * with coefficients c_k, k = 1..5.  Index ranges are 1-based, inclusive. */
enum { XA, XD, ZB, ZH };
static const struct {
    int axis, s, z0, zoff, x0, xoff;
} ST[4] = {
    {0, 0, 6, 0, 6, 4},  /* XA: Ax, J, S8          (bornlib-mod.f90:62-72, 386-396) */
    {0, 1, 6, 0, 5, 5},  /* XD: Az, D, F, S3, S5   (:143-153, 196-206, 270-280) */
    {1, 1, 6, 5, 1, 0},  /* ZB: Bx, E, G, S4, S6   (:96-106, 233-243, 307-317) */
    {1, 0, 6, 4, 1, 0},  /* ZH: Bz, H, S7          (:170-180, 344-354) */
};

/* per output part: stencil, coefficient (0 rho_Vx, 1 rho_Vz, 2 l, 3 mi,
 * 4 l2mi), its two inputs, PML axis (0 x, 1 z), averaged PML, source */
static const struct {
    int st, coef, a, b, axis, avg, src;
} PART[NF] = {
    {XA, 0, SXXX, SXXZ, 0, 0, 0}, /* Vx_x   born-mod.f90:431-438  Ax; L, K */
    {ZB, 0, SXZX, SXZZ, 1, 0, 0}, /* Vx_z   :440-447  Bx; N, M */
    {XD, 1, SXZX, SXZZ, 0, 1, 0}, /* Vz_x   :449-456  Az; P, O */
    {ZH, 1, SZZX, SZZZ, 1, 1, 0}, /* Vz_z   :458-465  Bz; R, Q */
    {XD, 4, VXX, VXZ, 0, 1, 1},   /* sxx_x  :467-472  D;  P, O, source */
    {ZB, 2, VZX, VZZ, 1, 1, 1},   /* sxx_z  :474-479  E;  R, Q, source */
    {XD, 2, VXX, VXZ, 0, 1, 1},   /* szz_x  :481-486  F;  P, O, source */
    {ZB, 4, VZX, VZZ, 1, 1, 1},   /* szz_z  :488-493  G;  R, Q, source */
    {ZH, 3, VXX, VXZ, 0, 0, 0},   /* sxz_x  :495-501  H;  L, K */
    {XA, 3, VZX, VZZ, 1, 0, 0},   /* sxz_z  :503-509  J;  N, M */
};

/* Born terms of the scattered parts (born-mod.f90:514-600): velocities add
 * (bg new - bg cur) * drho (S1, S2, pointwise on rows 6..nz-5); stresses add
 * a stencil of the background's new velocity parts (S3..S8) scaled by a
 * perturbation coefficient (5 dl, 6 dmi, 7 dl2mi). */
static const struct {
    int st, coef, a, b;
} BORN[NF] = {
    {-1, 0, VXX, -1}, {-1, 0, VXZ, -1}, {-1, 1, VZX, -1}, {-1, 1, VZZ, -1},
    {XD, 7, VXX, VXZ}, /* S3 */
    {ZB, 5, VZX, VZZ}, /* S4 */
    {XD, 5, VXX, VXZ}, /* S5 */
    {ZB, 7, VZX, VZZ}, /* S6 */
    {ZH, 6, VXX, VXZ}, /* S7 */
    {XA, 6, VZX, VZZ}, /* S8 */
};

static void coefs(float c[5])
{
    c[0] = 35.0f / 294912.0f;
    c[1] = -405.0f / 229376.0f;
    c[2] = 567.0f / 40960.0f;
    c[3] = -735.0f / 8192.0f;
    c[4] = 19845.0f / 16384.0f;
}

static int in_range(int k, int nz, int nx, int iz, int ix)
{
    return iz >= ST[k].z0 && iz <= nz - ST[k].zoff && ix >= ST[k].x0 && ix <= nx - ST[k].xoff;
}

/* c1*(m[hi1]-m[lo1]) + ... + c5*(m[hi5]-m[lo5]), left to right */
static float stencil(const float *m, int k, long p, long sx, const float c[5])
{
    const long st = ST[k].axis == 0 ? sx : 1;
    const int s = ST[k].s;
    float acc = 0.0f;
    for (int j = 1; j <= 5; ++j) {
        const float d = m[p + (5 - j + s) * st] - m[p - (6 - j - s) * st];
        const float t = c[j - 1] * d;
        acc = j == 1 ? t : acc + t;
    }
    return acc;
}

/* PML factor tables (pml-mod.f90:23-89): t[side][i][...] with side 0 left /
 * top, 1 right / bottom; pml0 and pml1 on x (nz x abc each side) and z
 * (abc x nx each side), Fortran order. */
typedef struct {
    float *x0[2], *x1[2], *z0[2], *z1[2];
} Pml;

static void pml_init(Pml *P, int nz, int nx, float dx, float dt, int abc, const float *vp, int free_surface)
{
    const float R = 0.001f;
    const float L = logf(1.0f / R);
    float *filter = (float *)calloc(abc + 1, sizeof(float));
    for (int i = 1; i <= abc; ++i)
        filter[i] = ((float)i / (1.0f * (float)abc)) * ((float)i / (1.0f * (float)abc));
    for (int s = 0; s < 2; ++s) {
        P->x0[s] = (float *)calloc((size_t)nz * abc + 1, sizeof(float));
        P->x1[s] = (float *)calloc((size_t)nz * abc + 1, sizeof(float));
        P->z0[s] = (float *)calloc((size_t)abc * nx + 1, sizeof(float));
        P->z1[s] = (float *)calloc((size_t)abc * nx + 1, sizeof(float));
    }
    const float den = (float)abc * dx;
#define D0(iz, ix) ((L * (1.5f * vp[((long)(ix)-1) * nz + (iz)-1])) / den)
    for (int ix = 1; ix <= abc; ++ix)
        for (int iz = 1; iz <= nz; ++iz) {
            const long q = (long)(ix - 1) * nz + iz - 1;
            const float dl = D0(iz, ix) * filter[abc - ix + 1], dr = D0(iz, ix) * filter[ix];
            P->x0[0][q] = 1.0f - ((dt * dl) / 2.0f);
            P->x0[1][q] = 1.0f - ((dt * dr) / 2.0f);
            P->x1[0][q] = 1.0f / (1.0f + ((dt * dl) / 2.0f));
            P->x1[1][q] = 1.0f / (1.0f + ((dt * dr) / 2.0f));
        }
    for (int ix = 1; ix <= nx; ++ix)
        for (int iz = 1; iz <= abc; ++iz) {
            const long q = (long)(ix - 1) * abc + iz - 1;
            const float dt_ = D0(iz, ix) * filter[abc - iz + 1], db = D0(iz, ix) * filter[iz];
            P->z0[0][q] = free_surface ? 1.0f : 1.0f - ((dt * dt_) / 2.0f);
            P->z0[1][q] = 1.0f - ((dt * db) / 2.0f);
            P->z1[0][q] = free_surface ? 1.0f : 1.0f / (1.0f + ((dt * dt_) / 2.0f));
            P->z1[1][q] = 1.0f / (1.0f + ((dt * db) / 2.0f));
        }
#undef D0
    free(filter);
}

/* v * (PML factor of one part at (iz, ix)): left / top side first, then
 * right / bottom (K..R apply their two loops in that order).  which: 0 the
 * pml0 table (L, N, P, R on the old level), 1 the pml1 table (K, M, O, Q). */
static float pml_apply(const Pml *P, int nz, int nx, int abc, int axis, int avg, int which, int iz, int ix,
                       float v)
{
    if (abc <= 0)
        return v;
    for (int side = 0; side < 2; ++side) {
        if (axis == 0) {
            const float *t = which ? P->x1[side] : P->x0[side];
            const int i = side == 0 ? ix - 5 : ix - (nx - abc - 5); /* PML column index, 1..abc */
            if (!avg && i >= 1 && i <= abc)
                v = t[(long)(i - 1) * nz + iz - 1] * v;
            if (avg && i >= 1 && i <= abc - 1)
                v = (0.5f * (t[(long)i * nz + iz - 1] + t[(long)(i - 1) * nz + iz - 1])) * v;
        } else {
            const float *t = which ? P->z1[side] : P->z0[side];
            const int i = side == 0 ? iz - 5 : iz - (nz - abc - 5);
            if (!avg && i >= 1 && i <= abc)
                v = t[(long)(ix - 1) * abc + i - 1] * v;
            if (avg && i >= 2 && i <= abc)
                v = (0.5f * (t[(long)(ix - 1) * abc + i - 1] + t[(long)(ix - 1) * abc + i - 2])) * v;
        }
    }
    return v;
}

/* Model set-up, born-mod.f90:331-389.  C[0..9] = rho_Vx, rho_Vz, l, mi,
 * l2mi, dl, dmi, dl2mi, drho_Vx, drho_Vz. */
static void model_setup(int nz, int nx, float dx, float dt, int lame, const float *vp0, const float *vs0,
                        const float *rho0, const float *dvp, const float *dvs, const float *drho, float **C)
{
    const long n = (long)nz * nx;
    float *l0 = C[2], *mi0 = C[3], *l2mi0 = C[4], *dl = C[5], *dmi = C[6], *dl2mi = C[7];
    for (long p = 0; p < n; ++p) {
        if (lame) {
            l0[p] = vp0[p];
            mi0[p] = vs0[p];
            dl[p] = dvp[p];
            dmi[p] = dvs[p];
            l2mi0[p] = 0.0f;
            dl2mi[p] = 0.0f;
        } else {
            mi0[p] = (vs0[p] * vs0[p]) * rho0[p];
            l0[p] = ((vp0[p] * vp0[p]) * rho0[p]) - (2.0f * mi0[p]);
            l2mi0[p] = l0[p] + (2.0f * mi0[p]);
            dmi[p] = (dvs[p] * dvs[p]) * drho[p];
            dl[p] = ((dvp[p] * dvp[p]) * drho[p]) - (2.0f * dmi[p]);
            dl2mi[p] = dl[p] + (2.0f * dmi[p]);
        }
    }
    const float aux1 = dt / dx;
    float *rvx = C[0], *rvz = C[1], *drvx = C[8], *drvz = C[9];
    memset(rvx, 0, sizeof(float) * n);
    memset(rvz, 0, sizeof(float) * n);
    memset(drvx, 0, sizeof(float) * n);
    memset(drvz, 0, sizeof(float) * n);
#define I(iz, ix) (((long)(ix)-1) * nz + (iz)-1)
    for (int ix = 1; ix <= nx; ++ix)
        for (int iz = 1; iz <= nz - 1; ++iz) {
            rvx[I(iz, ix)] = (aux1 * 1.0f) / (0.5f * (rho0[I(iz + 1, ix)] + rho0[I(iz, ix)]));
            drvx[I(iz, ix)] = -((drho[I(iz + 1, ix)] / rho0[I(iz + 1, ix)]) + (drho[I(iz, ix)] / rho0[I(iz, ix)]));
        }
    for (int ix = 1; ix <= nx - 1; ++ix)
        for (int iz = 1; iz <= nz; ++iz) {
            rvz[I(iz, ix)] = (aux1 * 1.0f) / (0.5f * (rho0[I(iz, ix + 1)] + rho0[I(iz, ix)]));
            drvz[I(iz, ix)] = -((drho[I(iz, ix + 1)] / rho0[I(iz, ix + 1)]) + (drho[I(iz, ix)] / rho0[I(iz, ix)]));
        }
    for (int iz = 1; iz <= nz; ++iz) {
        rvz[I(iz, nx)] = aux1 * (1.0f / rho0[I(iz, nx)]);
        drvz[I(iz, nx)] = -(drho[I(iz, nx)] / rho0[I(iz, nx)]);
    }
    for (int ix = 1; ix <= nx; ++ix) {
        rvx[I(nz, ix)] = aux1 * (1.0f / rho0[I(nz, ix)]);
        drvx[I(nz, ix)] = -(drho[I(nz, ix)] / rho0[I(nz, ix)]);
    }
    /* in place, column by column: every read of a neighbour (iz+1 or ix+1)
     * sees the value before averaging, so the originals are kept aside */
    float *o[4];
    float *src[4] = {l0, mi0, dl, dmi};
    for (int k = 0; k < 4; ++k) {
        o[k] = (float *)malloc(sizeof(float) * n);
        memcpy(o[k], src[k], sizeof(float) * n);
    }
    const float num = aux1 * 4.0f;
#define HARM(a, iz, ix) \
    (num / ((((1.0f / a[I(iz, ix)]) + (1.0f / a[I(iz + 1, ix)])) + (1.0f / a[I(iz, ix + 1)])) + (1.0f / a[I(iz + 1, ix + 1)])))
    for (int ix = 2; ix <= nx - 1; ++ix)
        for (int iz = 2; iz <= nz - 1; ++iz) {
            const float *L0 = o[0], *M0 = o[1], *DL = o[2], *DM = o[3];
            l0[I(iz, ix)] = HARM(L0, iz, ix);
            if (M0[I(iz, ix)] == 0 || M0[I(iz + 1, ix)] == 0 || M0[I(iz, ix + 1)] == 0 || M0[I(iz + 1, ix + 1)] == 0)
                mi0[I(iz, ix)] = 0.0f;
            else
                mi0[I(iz, ix)] = HARM(M0, iz, ix);
            if (DL[I(iz, ix)] < 1e-2f || DL[I(iz + 1, ix)] < 1e-2f || DL[I(iz, ix + 1)] < 1e-2f ||
                DL[I(iz + 1, ix + 1)] < 1e-2f)
                dl[I(iz, ix)] = 0.0f;
            else
                dl[I(iz, ix)] = HARM(DL, iz, ix);
            if (DM[I(iz, ix)] < 1e-2f || DM[I(iz + 1, ix)] < 1e-2f || DM[I(iz, ix + 1)] < 1e-2f ||
                DM[I(iz + 1, ix + 1)] < 1e-2f)
                dmi[I(iz, ix)] = 0.0f;
            else
                dmi[I(iz, ix)] = HARM(DM, iz, ix);
            l2mi0[I(iz, ix)] = l0[I(iz, ix)] + (2.0f * mi0[I(iz, ix)]);
            dl2mi[I(iz, ix)] = dl[I(iz, ix)] + (2.0f * dmi[I(iz, ix)]);
        }
#undef HARM
#undef I
    for (int k = 0; k < 4; ++k)
        free(o[k]);
}

/* Export of the model set-up (for the GPU tests' staging checks). */
void ora_pml_model(int nz, int nx, float dx, float dt, int lame, const float *vp0, const float *vs0,
                   const float *rho0, const float *dvp, const float *dvs, const float *drho, float *const *C)
{
    model_setup(nz, nx, dx, dt, lame, vp0, vs0, rho0, dvp, dvs, drho, (float **)C);
}

/* Ricker sample of level it, source-mod.f90:42-56, then the scaling of
 * born-mod.f90:424-428. */
static float source_at(int it, int nsource, float fp, float dt, float dx)
{
    float src = 0.0f;
    if (it < nsource) {
        const float pi = 3.14159265f;
        const float t = ((float)it * dt) - (((float)nsource * dt) / 2.0f);
        const float aux = ((((pi * pi) * fp) * fp) * t) * t;
        src = (1.0f - (2.0f * aux)) * expf(-aux);
        if (it <= nsource / 10)
            src = 0.0f;
        src = 10.0e7f * src;
    }
    return ((0.7e7f * src) * (dt / (dx * dx))) * 0.25f;
}

/* One level of one wavefield (background: born = 0; scattered: born = 1
 * with bgn / bgc the background's new and current parts). */
static void advance(int nz, int nx, int abc, const Pml *P, float *const *C, const float c[5], float *const *nw,
                    float *const *cur, float *const *old, int born, float *const *bgn, float *const *bgc, int zs,
                    int xs, float src)
{
    const long sx = nz;
#pragma omp parallel for schedule(static)
    for (int ix = 1; ix <= nx; ++ix)
        for (int iz = 1; iz <= nz; ++iz) {
            const long p = (long)(ix - 1) * nz + iz - 1;
            for (int f = 0; f < NF; ++f) {
                const int k = PART[f].st;
                float v = 0.0f;
                if (in_range(k, nz, nx, iz, ix)) {
                    const float cf = C[PART[f].coef][p];
                    v = v + cf * stencil(cur[PART[f].a], k, p, sx, c);
                    v = v + cf * stencil(cur[PART[f].b], k, p, sx, c);
                }
                v = v + pml_apply(P, nz, nx, abc, PART[f].axis, PART[f].avg, 0, iz, ix, old[f][p]);
                if (!born && PART[f].src && iz == zs && ix == xs)
                    v = v + src;
                if (born) {
                    const int kb = BORN[f].st;
                    if (kb < 0) {
                        if (iz >= 6 && iz <= nz - 5)
                            v = v + (bgn[BORN[f].a][p] - bgc[BORN[f].a][p]) * C[8 + BORN[f].coef][p];
                    } else if (in_range(kb, nz, nx, iz, ix)) {
                        const float cf = C[BORN[f].coef][p];
                        v = v + cf * stencil(bgn[BORN[f].a], kb, p, sx, c);
                        v = v + cf * stencil(bgn[BORN[f].b], kb, p, sx, c);
                    }
                }
                nw[f][p] = pml_apply(P, nz, nx, abc, PART[f].axis, PART[f].avg, 1, iz, ix, v);
            }
        }
}

/* Receiver lines, seis-mod-born.f90:36-98 (abc = 0 reads as 1 there). */
static void record(int nz, int nx, int abc, int nseis, int zrec, int count, float *const *f, float *svx, float *svz,
                   float *sp)
{
    (void)nz;
    const int a = abc == 0 ? 1 : abc;
#define F(k, iz, ix) f[k][((long)(ix)-1) * nz + (iz)-1]
    for (int ix = 1; ix <= nx - 2 * a - 1; ++ix) {
        const int c = ix + a;
        const long q = (long)(ix - 1) * nseis + count - 1;
        svx[q] = 0.5f * (((F(VXX, zrec, c) + F(VXZ, zrec, c)) + F(VXX, zrec - 1, c)) + F(VXZ, zrec - 1, c));
        svz[q] = 0.5f * (((F(VZX, zrec, c) + F(VZZ, zrec, c)) + F(VZX, zrec, c - 1)) + F(VZZ, zrec, c - 1));
        sp[q] = 0.5f * (((F(SXXX, zrec, c) + F(SXXZ, zrec, c)) + F(SZZX, zrec - 1, c)) + F(SZZZ, zrec - 1, c));
    }
#undef F
}

/* Snapshots, snap-mod-born.f90:33-68. */
static void snapshot(int nz, int nx, int count, float *const *f, float *vx, float *vz, float *pr)
{
    const long off = (long)(count - 1) * nz * nx;
    for (int ix = 2; ix <= nx - 2; ++ix)
        for (int iz = 2; iz <= nz - 2; ++iz) {
            const long p = (long)(ix - 1) * nz + iz - 1;
            vx[off + p] = f[VXX][p] + f[VXZ][p];
            vz[off + p] = f[VZX][p] + f[VZZ][p];
            pr[off + p] = 0.5f * (((f[SXXX][p] + f[SXXZ][p]) + f[SZZX][p]) + f[SZZZ][p]);
        }
}

/* The whole program after its parameter and file I/O (born.f90:270-296):
 * elastic_init + elastic_op.  Outputs are written where the reference
 * writes them; other cells keep the caller's values.  seis[0..5] = Vx, Vz,
 * P, Vx_b, Vz_b, P_b (nseis x (nx-2abc)); snap[0..5] likewise (nz x nx x
 * nsnap).  Requires nsnap <= nt (the reference divides by nt/nsnap) and
 * abc <= min(nz, nx). */
void ora_pml_born(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp,
                  int nsnap, int nseis, int abc, int zrec, int free_surface, int lame, const float *vp0,
                  const float *vs0, const float *rho0, const float *dvp, const float *dvs, const float *drho,
                  float *const *seis, float *const *snap)
{
    const long n = (long)nz * nx;
    float *C[10];
    for (int k = 0; k < 10; ++k)
        C[k] = (float *)calloc(n, sizeof(float));
    model_setup(nz, nx, dx, dt, lame, vp0, vs0, rho0, dvp, dvs, drho, C);
    Pml P;
    pml_init(&P, nz, nx, dx, dt, abc, vp0, free_surface);
    float c[5];
    coefs(c);
    float *buf = (float *)calloc((size_t)(6 * NF) * n, sizeof(float));
    float *lv[2][3][NF];
    for (int w = 0; w < 2; ++w)
        for (int l = 0; l < 3; ++l)
            for (int f = 0; f < NF; ++f)
                lv[w][l][f] = buf + ((long)(w * 3 + l) * NF + f) * n;
    int inew = 0, icur = 1, iold = 2;
    const int dseis = nt / nseis + 1, dsnap = nt / nsnap;
    const float nsource2 = (float)(2 * (int)lroundf(((sqrtf(6.0f) / 3.14159265f) / fp) / dt));
    int countseis = 1, countsnap = 1;
    /* ORA_PML_PLANT=1 (tests only): one ulp added to the largest scattered
     * sxx_x value half-way through, to show that the comparisons see it */
    const char *plant = getenv("ORA_PML_PLANT");
    for (int it = 1; it <= nt; ++it) {
        const float src = source_at(it, nsource, fp, dt, dx);
        if (plant && plant[0] == '1' && it == nt / 2) {
            float *f = lv[1][icur][SXXX];
            long qmax = 0;
            for (long q = 1; q < n; ++q)
                if (fabsf(f[q]) > fabsf(f[qmax]))
                    qmax = q;
            f[qmax] = nextafterf(f[qmax], INFINITY);
        }
        advance(nz, nx, abc, &P, C, c, lv[0][inew], lv[0][icur], lv[0][iold], 0, 0, 0, zsource, xsource, src);
        advance(nz, nx, abc, &P, C, c, lv[1][inew], lv[1][icur], lv[1][iold], 1, lv[0][inew], lv[0][icur], zsource,
                xsource, 0.0f);
        if ((float)it > nsource2 && it % dseis == 0) {
            record(nz, nx, abc, nseis, zrec, countseis, lv[0][inew], seis[0], seis[1], seis[2]);
            record(nz, nx, abc, nseis, zrec, countseis, lv[1][inew], seis[3], seis[4], seis[5]);
            countseis++;
        }
        if (it % dsnap == 0 && countsnap <= nsnap) {
            snapshot(nz, nx, countsnap, lv[0][inew], snap[0], snap[1], snap[2]);
            snapshot(nz, nx, countsnap, lv[1][inew], snap[3], snap[4], snap[5]);
            countsnap++;
        }
        const int t = iold;
        iold = icur;
        icur = inew;
        inew = t;
    }
    free(buf);
    for (int k = 0; k < 10; ++k)
        free(C[k]);
    for (int s = 0; s < 2; ++s) {
        free(P.x0[s]);
        free(P.x1[s]);
        free(P.z0[s]);
        free(P.z1[s]);
    }
}

/* Export of the PML tables (tests): x0l, x0r, x1l, x1r as (nz, abc) and
 * z0t, z0b, z1t, z1b as (abc, nx), pml-mod.f90's pml0_xl .. pml1_zb. */
void ora_pml_tables(int nz, int nx, float dx, float dt, int abc, const float *vp, int free_surface, float *const *out)
{
    Pml P;
    pml_init(&P, nz, nx, dx, dt, abc, vp, free_surface);
    const size_t nxz = (size_t)nz * abc, nzx = (size_t)abc * nx;
    memcpy(out[0], P.x0[0], sizeof(float) * nxz);
    memcpy(out[1], P.x0[1], sizeof(float) * nxz);
    memcpy(out[2], P.x1[0], sizeof(float) * nxz);
    memcpy(out[3], P.x1[1], sizeof(float) * nxz);
    memcpy(out[4], P.z0[0], sizeof(float) * nzx);
    memcpy(out[5], P.z0[1], sizeof(float) * nzx);
    memcpy(out[6], P.z1[0], sizeof(float) * nzx);
    memcpy(out[7], P.z1[1], sizeof(float) * nzx);
    for (int s = 0; s < 2; ++s) {
        free(P.x0[s]);
        free(P.x1[s]);
        free(P.z0[s]);
        free(P.z1[s]);
    }
}
