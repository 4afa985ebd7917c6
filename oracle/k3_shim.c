/* Test infrastructure: the GPU hand-off of the reference's 3D elastic kernel
 * test (kernel_3d_test/gpu.h:68-79, rtm_gpu_init/func/final) served by the
 * oracle's step, so that the reference's own main -- random fields, the
 * hand-off, its CPU step, func_check at 1e-13 (kernel_3d_test/rtmlib-modC.c:
 * 31-43, 48-705) -- checks the oracle against its CPU code.  The reference
 * source is compiled unchanged with its three entry points renamed on the
 * command line to the k3o_* functions below. */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

void ora_k3_step(int ny, int nz, int nx, const float *const *in, const float *const *in1, float *const *out,
                 const float *const *m);

void k3o_init(int ny, int nz, int nx) { (void)ny; (void)nz; (void)nx; }
void k3o_final(void) {}

void k3o_func(int ny, int nz, int nx, float *vy0, float *vx0, float *vz0, float *syy0, float *sxx0, float *szz0,
              float *sxy0, float *sxz0, float *syz0, float *vy1, float *vx1, float *vz1, float *syy1, float *sxx1,
              float *szz1, float *sxy1, float *sxz1, float *syz1, float *vyo, float *vxo, float *vzo, float *syyo,
              float *sxxo, float *szzo, float *sxyo, float *sxzo, float *syzo, float *m1y, float *m1x, float *m1z,
              float *m2, float *m3, float *m2m3, float *debug, float *t)
{
    const float *in[9] = {vy0, vx0, vz0, syy0, sxx0, szz0, sxy0, sxz0, syz0};
    const float *in1[9] = {vy1, vx1, vz1, syy1, sxx1, szz1, sxy1, sxz1, syz1};
    float *out[9] = {vyo, vxo, vzo, syyo, sxxo, szzo, sxyo, sxzo, syzo};
    const float *m[6] = {m1y, m1x, m1z, m2, m3, m2m3};
    (void)debug;
    ora_k3_step(ny, nz, nx, in, in1, out, m);
    /* K3_PLANT=1: a planted mistake (one cell of Vx moved by one unit in
     * the last place), which the reference's check must report */
    const char *e = getenv("K3_PLANT");
    if (e && atoi(e) == 1) {
        const size_t p = ((size_t)(ny / 2 + 5) * (nx + 10) + (nx / 2 + 5)) * (nz + 10) + nz / 2 + 5;
        vxo[p] = nextafterf(vxo[p], INFINITY);
    }
    if (t) t[0] = t[1] = t[2] = 1.0f;
}
