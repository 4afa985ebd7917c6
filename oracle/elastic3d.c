/* Oracle (test infrastructure only): one step of the reference's 3D elastic
 * kernel test, kernel_3d_test/rtmlib-modC.c:277-570 (the CPU step that
 * kernel_3d_test's main checks its GPU kernel against,
 * kernel_3d_test/rtmlib-modC.c:31-43 and :697-705).
 *
 * Nine fields (Vy, Vx, Vz, syy, sxx, szz, sxy, sxz, syz, the reference's
 * argument order, kernel_3d_test/gpu.h:71-79) and six coefficient planes
 * (m1_y, m1_x, m1_z, m2, m3, m2m3) on padded grids (ny+10)(nx+10)(nz+10),
 * z fastest, interior cells at padded index +5 on every axis.  Each output
 * field is updated in place:
 *     out = out + in1 + sum over its groups, in order, of the ten taps of
 *           the group in order: +/- (m[p'] * c_k) * f[p'],
 * where a group names a coefficient plane m, an input field f of the level
 * `in`, an axis and a stagger: taps at offsets -5..4 ("P") or -4..5 ("M")
 * along that axis, the first five added with c1..c5, the last five
 * subtracted with c5..c1.  Every product and sum is rounded separately in
 * the reference's left-to-right order (compiled with -ffp-contract=off).
 * The group table below is the reference's expressions written as data.
 */
#include <stddef.h>

enum { K3_VY, K3_VX, K3_VZ, K3_SYY, K3_SXX, K3_SZZ, K3_SXY, K3_SXZ, K3_SYZ };
enum { K3_M1Y, K3_M1X, K3_M1Z, K3_M2, K3_M3, K3_M2M3 };
enum { AX_Z = 0, AX_X = 1, AX_Y = 2 };
enum { ST_P = 0, ST_M = 1 };

typedef struct {
    int coef, field, axis, stag;
} K3Group;

/* groups of each output field, in the order the reference sums them;
 * n = number of groups */
static const struct {
    int n;
    K3Group g[5];
} K3_TABLE[9] = {
    /* Vy  (:350-413) */
    {5, {{K3_M2M3, K3_SYY, AX_Y, ST_P}, {K3_M2, K3_SZZ, AX_Y, ST_P}, {K3_M2, K3_SXX, AX_Y, ST_P},
         {K3_M3, K3_SYZ, AX_Z, ST_M}, {K3_M3, K3_SXY, AX_X, ST_M}}},
    /* Vx  (:288-349) */
    {5, {{K3_M2M3, K3_SXX, AX_X, ST_P}, {K3_M2, K3_SYY, AX_X, ST_P}, {K3_M2, K3_SZZ, AX_X, ST_P},
         {K3_M3, K3_SXY, AX_Y, ST_M}, {K3_M3, K3_SXZ, AX_Z, ST_M}}},
    /* Vz  (:414-472) */
    {5, {{K3_M2M3, K3_SZZ, AX_Z, ST_P}, {K3_M2, K3_SXX, AX_Z, ST_P}, {K3_M2, K3_SYY, AX_Z, ST_P},
         {K3_M3, K3_SYZ, AX_Y, ST_M}, {K3_M3, K3_SXZ, AX_X, ST_M}}},
    /* syy (:490-501) */
    {1, {{K3_M1Y, K3_VY, AX_Y, ST_M}}},
    /* sxx (:477-488) */
    {1, {{K3_M1X, K3_VX, AX_X, ST_M}}},
    /* szz (:503-514) */
    {1, {{K3_M1Z, K3_VZ, AX_Z, ST_M}}},
    /* sxy (:518-541) */
    {2, {{K3_M1Y, K3_VY, AX_X, ST_M}, {K3_M1X, K3_VX, AX_Y, ST_M}}},
    /* sxz (:543-564) */
    {2, {{K3_M1X, K3_VX, AX_Z, ST_M}, {K3_M1Z, K3_VZ, AX_X, ST_M}}},
    /* syz (:566-589) */
    {2, {{K3_M1Y, K3_VY, AX_Z, ST_M}, {K3_M1Z, K3_VZ, AX_Y, ST_M}}},
};

/* the reference's constants (kernel_3d_test/rtmlib-modC.c:60), computed in
 * double and stored as float */
static void k3_coefs(float c[5])
{
    c[0] = (float)(35.0 / 294912.0);
    c[1] = (float)(-405.0 / 229376.0);
    c[2] = (float)(567.0 / 40960.0);
    c[3] = (float)(-735.0 / 8192.0);
    c[4] = (float)(19845.0 / 16384.0);
}

/* Export of the group table for the GPU tests' documentation checks:
 * t[o*5*4 + g*4 + {0..3}] = coef, field, axis, stagger; n[o] groups. */
void ora_k3_table(int *n, int *t)
{
    for (int o = 0; o < 9; o++) {
        n[o] = K3_TABLE[o].n;
        for (int g = 0; g < 5; g++) {
            const K3Group *q = &K3_TABLE[o].g[g];
            t[(o * 5 + g) * 4 + 0] = g < K3_TABLE[o].n ? q->coef : -1;
            t[(o * 5 + g) * 4 + 1] = g < K3_TABLE[o].n ? q->field : -1;
            t[(o * 5 + g) * 4 + 2] = g < K3_TABLE[o].n ? q->axis : -1;
            t[(o * 5 + g) * 4 + 3] = g < K3_TABLE[o].n ? q->stag : -1;
        }
    }
}

/* One step: in[9] (level t+1 of the adjoint recursion), in1[9] (level t+2),
 * out[9] (level t, updated in place), m[6]; padded (ny+10)(nx+10)(nz+10). */
void ora_k3_step(int ny, int nz, int nx, const float *const *in, const float *const *in1, float *const *out,
                 const float *const *m)
{
    float c[5];
    k3_coefs(c);
    const ptrdiff_t sz = 1, sx = nz + 10, sy = (ptrdiff_t)(nz + 10) * (nx + 10);
    const ptrdiff_t stride[3] = {sz, sx, sy};
#pragma omp parallel for collapse(2) schedule(static)
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                const ptrdiff_t p = (iy + 5) * sy + (ix + 5) * sx + (iz + 5);
                for (int o = 0; o < 9; o++) {
                    float acc = out[o][p] + in1[o][p];
                    for (int g = 0; g < K3_TABLE[o].n; g++) {
                        const K3Group *q = &K3_TABLE[o].g[g];
                        const float *mm = m[q->coef], *ff = in[q->field];
                        const ptrdiff_t st = stride[q->axis];
                        const int first = q->stag == ST_P ? -5 : -4;
                        for (int t = 0; t < 10; t++) {
                            const ptrdiff_t pp = p + (first + t) * st;
                            const float term = (mm[pp] * c[t < 5 ? t : 9 - t]) * ff[pp];
                            acc = t < 5 ? acc + term : acc - term;
                        }
                    }
                    out[o][p] = acc;
                }
            }
}
