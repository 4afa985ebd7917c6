/*
 * CPU restatement of the single-domain 3D acoustic propagator of
 * lgan/elastic, raised from 8th to 10th order in space.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for tests/, the smoke check and
 * bench.py's CPU-baseline leg.  The product never links it.
 *
 * Reference (paths inside the lgan/elastic project, W = 2d_rtm_restart/Src_working):
 *   W/wave_fkernel.3d8o.cu:26-27   coefficient table (8th order there)
 *   W/wave_fkernel.3d8o.cu:31-106  p2 = vel*(stencil(p1)) + p1 + p1 - p0, vel = v^2 dt^2
 *   W/wave_fkernel.3d8o.cu:183-210 sponge: p0,p1 *= exp(-b(a-edge)) where the factor is < 1
 *   W/gpu_funcs_3d.cu:64-75        source injection after the update (sign dir)
 *   W/gpu_funcs_3d.cu:95-109       receiver extraction
 *   W/gpu_funcs_3d.cu:111-120      imaging img += 1e-6*rec*src
 *   W/gpu_funcs_3d.cu:133-315      source propagation, undamped, returns the last two slices
 *   W/gpu_funcs_3d.cu:509-712      adjoint: damped receiver field, source field propagated
 *                                  backwards from its last two slices (reverse-time restart)
 *
 * Differences from the reference, each deliberate: radius 5 and the
 * 10th-order Taylor coefficients (-5269/1800, 5/3, -5/21, 5/126, -5/1008,
 * 1/3150); injection and extraction on the grid at every step (the reference
 * interpolates subsampled traces with an 8-tap sinc table); the sponge edge
 * distance is symmetric (0 at the first and at the last interior cell).
 *
 * Layout: addr = iz + n1*(ix + n2*iy); interior cells are [5, n-5) on every
 * axis, the 5-cell rim stays zero.  Compile with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define RAD 5
#define A3(iz, ix, iy) ((size_t)(iz) + (size_t)n1 * ((size_t)(ix) + (size_t)n2 * (size_t)(iy)))

/* coef[0] = C0, coef[1+3(k-1)+{0,1,2}] = (z,x,y) coefficient of offset k. */
void ora3d_coeffs(double d1, double d2, double d3, float *coef)
{
    const double c[6] = {-5269.0 / 1800.0, 5.0 / 3.0, -5.0 / 21.0, 5.0 / 126.0, -5.0 / 1008.0, 1.0 / 3150.0};
    double i1 = 1.0 / (d1 * d1), i2 = 1.0 / (d2 * d2), i3 = 1.0 / (d3 * d3);
    int k;
    coef[0] = (float)(c[0] * (i1 + i2 + i3));
    for (k = 1; k <= 5; k++) {
        coef[1 + 3 * (k - 1) + 0] = (float)(c[k] * i1);
        coef[1 + 3 * (k - 1) + 1] = (float)(c[k] * i2);
        coef[1 + 3 * (k - 1) + 2] = (float)(c[k] * i3);
    }
}

/* table[e] = expf(-b*(a-e)) for e = 0..a-1 (W/wave_fkernel.3d8o.cu:201). */
void ora3d_damp_table(int a, float b, float *table)
{
    int e;
    for (e = 0; e < a; e++) table[e] = expf(-b * (float)(a - e));
}

static int edge_of(int i, int n) /* distance from the nearest interior face */
{
    int lo = i - RAD, hi = (n - 1 - RAD) - i;
    return lo < hi ? lo : hi;
}

/* Multiply p0 and p1 by the sponge factor where it is below one. */
void ora3d_damp(int n1, int n2, int n3, int a, const float *table, float *p0, float *p1)
{
    int iz, ix, iy;
    for (iy = RAD; iy < n3 - RAD; iy++)
        for (ix = RAD; ix < n2 - RAD; ix++)
            for (iz = RAD; iz < n1 - RAD; iz++) {
                int e = edge_of(iz, n1), t;
                t = edge_of(ix, n2);
                if (t < e) e = t;
                t = edge_of(iy, n3);
                if (t < e) e = t;
                if (e >= 0 && e < a && table[e] < 1.0f) {
                    size_t o = A3(iz, ix, iy);
                    p1[o] = p1[o] * table[e];
                    p0[o] = p0[o] * table[e];
                }
            }
}

/* p2 = vel*L(p1) + p1 + p1 - p0 on the interior; p2 may alias p0. */
void ora3d_step(int n1, int n2, int n3, const float *p0, const float *p1, float *p2, const float *vel,
                const float *coef)
{
    int iz, ix, iy, k;
    size_t s2 = (size_t)n1, s3 = (size_t)n1 * (size_t)n2;
    for (iy = RAD; iy < n3 - RAD; iy++)
        for (ix = RAD; ix < n2 - RAD; ix++)
            for (iz = RAD; iz < n1 - RAD; iz++) {
                size_t o = A3(iz, ix, iy);
                float acc = coef[0] * p1[o];
                for (k = 1; k <= 5; k++) {
                    acc = acc + coef[1 + 3 * (k - 1) + 0] * (p1[o + k] + p1[o - k]);
                    acc = acc + coef[1 + 3 * (k - 1) + 1] * (p1[o + k * s2] + p1[o - k * s2]);
                    acc = acc + coef[1 + 3 * (k - 1) + 2] * (p1[o + k * s3] + p1[o - k * s3]);
                }
                p2[o] = ((vel[o] * acc + p1[o]) + p1[o]) - p0[o];
            }
}

/* Forward modelling: nt steps from rest; source wavelet src[it] added at
   (zs,xs,ys) after each update with sign dir; receivers on the plane
   iz=zr recorded into d[it][iy][ix] when d is non-NULL; the sponge is
   applied before each update when damp_a > 0.  On return p0/p1 hold the
   last two slices (levels nt-2 and nt-1). */
void ora3d_forward(int n1, int n2, int n3, int nt, const float *vel, const float *coef, int damp_a,
                   const float *damp_table, int zs, int xs, int ys, const float *src, float dir, int zr,
                   float *d, float *p0, float *p1)
{
    size_t tot = (size_t)n1 * n2 * n3;
    int it, ix, iy;
    float *a = p0, *b = p1, *tmp;
    memset(a, 0, tot * sizeof(float));
    memset(b, 0, tot * sizeof(float));
    for (it = 0; it < nt; it++) {
        if (damp_a > 0) ora3d_damp(n1, n2, n3, damp_a, damp_table, a, b);
        ora3d_step(n1, n2, n3, a, b, a, vel, coef); /* level it written over it-2 */
        a[A3(zs, xs, ys)] = a[A3(zs, xs, ys)] + dir * src[it];
        if (d)
            for (iy = 0; iy < n3; iy++)
                for (ix = 0; ix < n2; ix++) d[(size_t)it * n2 * n3 + (size_t)iy * n2 + ix] = a[A3(zr, ix, iy)];
        tmp = a; a = b; b = tmp;
    }
    /* after the loop b holds level nt-1 and a level nt-2 */
    if (a != p0) {
        /* swap contents so that p0 = level nt-2, p1 = level nt-1 */
        float *t2 = (float *)malloc(tot * sizeof(float));
        memcpy(t2, p0, tot * sizeof(float));
        memcpy(p0, p1, tot * sizeof(float));
        memcpy(p1, t2, tot * sizeof(float));
        free(t2);
    }
}

/* 3D RTM with reverse-time restart of the source wavefield
   (W/gpu_funcs_3d.cu:509-712 restated on the grid):
   1. the source field S is propagated forward, undamped, for nt steps and
      only its last two slices S(nt-2), S(nt-1) are kept;
   2. for it = nt-1 .. 0 the receiver field R steps backwards (sponged) and
      receives d[it] on the plane zr after each update; the source field is
      rebuilt backwards: the forward recursion
         S(t) = vel*L S(t-1) + 2 S(t-1) - S(t-2) + w(t) delta_src
      solved for its oldest level gives
         S(t-2) = vel*L S(t-1) + 2 S(t-1) - (S(t) - w(t) delta_src),
      i.e. the same update with the newest slice, minus its wavelet, in the
      role of "p0" (the reference's dir=-1 injection);
   3. every jt-th level the image accumulates (1e-6*R)*S in float (the
      reference promotes this product to double through the literal). */
void ora3d_rtm(int n1, int n2, int n3, int nt, int jt, const float *vel, const float *coef, int damp_a,
               const float *damp_table, int zs, int xs, int ys, const float *src, int zr, const float *d,
               float *img)
{
    size_t tot = (size_t)n1 * n2 * n3, i;
    float *X = (float *)malloc(tot * sizeof(float)), *Y = (float *)malloc(tot * sizeof(float));
    float *r0 = (float *)calloc(tot, sizeof(float)), *r1 = (float *)calloc(tot, sizeof(float));
    float *tmp;
    const float *S;
    int it, ix, iy;
    ora3d_forward(n1, n2, n3, nt, vel, coef, 0, damp_table, zs, xs, ys, src, 1.0f, zr, NULL, X, Y);
    /* X = S(nt-2), Y = S(nt-1) */
    memset(img, 0, tot * sizeof(float));
    for (it = nt - 1; it >= 0; it--) {
        if (damp_a > 0) ora3d_damp(n1, n2, n3, damp_a, damp_table, r0, r1);
        ora3d_step(n1, n2, n3, r0, r1, r0, vel, coef);
        /* traces enter at interior receivers only (rim cells are never
           updated, so injecting there would accumulate) */
        for (iy = RAD; iy < n3 - RAD; iy++)
            for (ix = RAD; ix < n2 - RAD; ix++)
                r0[A3(zr, ix, iy)] = r0[A3(zr, ix, iy)] + d[(size_t)it * n2 * n3 + (size_t)iy * n2 + ix];
        tmp = r0; r0 = r1; r1 = tmp; /* r1 = R(it) */
        if (it == nt - 1)
            S = Y;
        else if (it == nt - 2)
            S = X;
        else {
            /* X = S(it+1), Y = S(it+2) */
            Y[A3(zs, xs, ys)] = Y[A3(zs, xs, ys)] - src[it + 2];
            ora3d_step(n1, n2, n3, Y, X, Y, vel, coef);
            tmp = X; X = Y; Y = tmp; /* X = S(it), Y = S(it+1) */
            S = X;
        }
        if (it % jt == 0)
            for (i = 0; i < tot; i++) img[i] = img[i] + (1e-6f * r1[i]) * S[i];
    }
    free(X); free(Y); free(r0); free(r1);
}

/* Forward modelling keeping every level: hist[it] = level it (as stored by
   ora3d_forward before the next damping).  Test helper for the reverse-time
   restart property. */
void ora3d_forward_history(int n1, int n2, int n3, int nt, const float *vel, const float *coef, const float *src,
                           int zs, int xs, int ys, float *hist)
{
    size_t tot = (size_t)n1 * n2 * n3;
    float *a = (float *)calloc(tot, sizeof(float)), *b = (float *)calloc(tot, sizeof(float)), *tmp;
    int it;
    for (it = 0; it < nt; it++) {
        ora3d_step(n1, n2, n3, a, b, a, vel, coef);
        a[A3(zs, xs, ys)] = a[A3(zs, xs, ys)] + src[it];
        memcpy(hist + (size_t)it * tot, a, tot * sizeof(float));
        tmp = a; a = b; b = tmp;
    }
    free(a); free(b);
}

/* 3D RTM imaging with the source field read from a stored history instead
   of the reverse-time restart (same receiver side as ora3d_rtm). */
void ora3d_rtm_stored(int n1, int n2, int n3, int nt, int jt, const float *vel, const float *coef, int damp_a,
                      const float *damp_table, const float *hist, int zr, const float *d, float *img)
{
    size_t tot = (size_t)n1 * n2 * n3, i;
    float *r0 = (float *)calloc(tot, sizeof(float)), *r1 = (float *)calloc(tot, sizeof(float)), *tmp;
    int it, ix, iy;
    memset(img, 0, tot * sizeof(float));
    for (it = nt - 1; it >= 0; it--) {
        if (damp_a > 0) ora3d_damp(n1, n2, n3, damp_a, damp_table, r0, r1);
        ora3d_step(n1, n2, n3, r0, r1, r0, vel, coef);
        for (iy = RAD; iy < n3 - RAD; iy++)
            for (ix = RAD; ix < n2 - RAD; ix++)
                r0[A3(zr, ix, iy)] = r0[A3(zr, ix, iy)] + d[(size_t)it * n2 * n3 + (size_t)iy * n2 + ix];
        tmp = r0; r0 = r1; r1 = tmp;
        if (it % jt == 0)
            for (i = 0; i < tot; i++) img[i] = img[i] + (1e-6f * r1[i]) * hist[(size_t)it * tot + i];
    }
    free(r0); free(r1);
}
