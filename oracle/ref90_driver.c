/* Driver for the reference's Fortran RTM modules translated by f90c.py
 * (test infrastructure only).
 *
 * It takes the place of the reference's main program (2d_rtm_restart/
 * Src_working/rtm.f90:30-170), whose only other work is SEPlib parameter and
 * file I/O: the model, the perturbation or the receiver gathers come in as
 * arrays, and the call sequence is the main program's:
 *   rtm_init(nz,dz,nx,dx,dt,xsource,zsource,zrec,fp,nt,abc,free_surface,
 *            rho,lambda,mu,lame)                      (rtm.f90:150)
 *   stat = rtm_op(adj,drho,dl,dmu,Vx_rec,...,sigmaxz_rec)   (rtm.f90:155)
 * Arrays are Fortran-ordered: a model plane is (nz,nx), a gather (nt,nx).
 * rtm_init averages lambda and mu in place (model_op), as in the reference.
 *
 * ref90_hook_forward runs just before rtm_op2 calls image_init, when the five
 * source-wavefield histories are complete; when the caller asked for them it
 * copies them out.  ref90_get copies any real module array out by name
 * ("module.variable") after a call. */
#include <stdlib.h>
#include <string.h>
#include "ref90.h"

int F_rtm_mod_adj_rtm_op(int *a_adj, rarr a_dm1_in, rarr a_dm2_in, rarr a_dm3_in, rarr a_vx_in, rarr a_vz_in,
                         rarr a_sigmaxx_in, rarr a_sigmazz_in, rarr a_sigmaxz_in);
void F_image_mod_rtm_image_init(int *a_nx_in, float *a_dx_in, int *a_nz_in, float *a_dz_in, int *a_nt_in,
                                float *a_dt_in, rarr a_vx0_in, rarr a_vz0_in, int *a_lame_in);
void F_image_mod_rtm_image_init2(rarr a_m1_in, rarr a_m2_in, rarr a_m3_in);
void F_image_mod_rtm_image_op2(int *a_adj, int *a_add, float *a_dm1_p, float *a_dm2_p, float *a_dm3_p, float *a_vx_p,
                               float *a_vz_p, float *a_sigmaxx_p, float *a_sigmazz_p, float *a_sigmaxz_p);

static float *hook_dst[5];

static const rarr *find(const char *name)
{
    for (const struct ref90_var *v = ref90_vars; v->name; ++v)
        if (strcmp(v->name, name) == 0)
            return v->arr;
    return 0;
}

void ref90_hook_forward(void)
{
    static const char *names[5] = {"rtm_mod_adj.vx0", "rtm_mod_adj.vz0", "rtm_mod_adj.sigmaxx0",
                                   "rtm_mod_adj.sigmazz0", "rtm_mod_adj.sigmaxz0"};
    for (int k = 0; k < 5; ++k) {
        if (!hook_dst[k])
            continue;
        const rarr *a = find(names[k]);
        memcpy(hook_dst[k], a->p, sizeof(float) * (size_t)(a->n[0] * a->n[1] * a->n[2]));
    }
}

/* One rtm_init + rtm_op.  fwd: five (nz,nx,nt) buffers for the source
 * wavefield, or NULL.  Returns rtm_op's status (0 ok). */
int ref90_rtm(int adj, int lame, int nz, int nx, int nt, float dz, float dx, float dt, int xsource, int zsource,
              int zrec, float fp, int abc, float *m1, float *m2, float *m3, float *dm1, float *dm2, float *dm3,
              float *d1, float *d2, float *d3, float *d4, float *d5, float **fwd)
{
    int free_surface = 0;
    rarr M1 = {m1, {nz, nx, 1}}, M2 = {m2, {nz, nx, 1}}, M3 = {m3, {nz, nx, 1}};
    rarr DM1 = {dm1, {nz, nx, 1}}, DM2 = {dm2, {nz, nx, 1}}, DM3 = {dm3, {nz, nx, 1}};
    rarr D1 = {d1, {nt, nx, 1}}, D2 = {d2, {nt, nx, 1}}, D3 = {d3, {nt, nx, 1}}, D4 = {d4, {nt, nx, 1}},
         D5 = {d5, {nt, nx, 1}};
    for (int k = 0; k < 5; ++k)
        hook_dst[k] = fwd ? fwd[k] : 0;
    F_rtm_mod_adj_rtm_init(&nz, &dz, &nx, &dx, &dt, &xsource, &zsource, &zrec, &fp, &nt, &abc, &free_surface,
                           M1, M2, M3, &lame);
    int st = F_rtm_mod_adj_rtm_op(&adj, DM1, DM2, DM3, D1, D2, D3, D4, D5);
    for (int k = 0; k < 5; ++k)
        hook_dst[k] = 0;
    return st;
}

/* Copies module array `name` into dst (up to n floats); returns its size,
 * or -1 when there is no such array. */
long ref90_get(const char *name, float *dst, long n)
{
    const rarr *a = find(name);
    if (!a)
        return -1;
    long size = a->p ? a->n[0] * a->n[1] * a->n[2] : 0;
    if (dst && size)
        memcpy(dst, a->p, sizeof(float) * (size_t)(size < n ? size : n));
    return size;
}

/* The reference's imaging operator alone (W/image-mod-rtm.f90): image_init on
 * the source histories Vx0, Vz0 (nz,nx,nt), image_init2 with (m1,m2,m3) when
 * lame = 0 (velocity parameterisation: rho, vp, vs), then image_op2(adj,
 * add=.false.): adj = 1 images the five histories h1..h5 into dm1..dm3,
 * adj = 0 writes the Born secondary sources of dm1..dm3 into h1..h5. */
int ref90_image(int adj, int lame, int nz, int nx, int nt, float dx, float dt, float *Vx0, float *Vz0, float *m1,
                float *m2, float *m3, float *dm1, float *dm2, float *dm3, float *h1, float *h2, float *h3, float *h4,
                float *h5)
{
    rarr VX = {Vx0, {nz, nx, nt}}, VZ = {Vz0, {nz, nx, nt}};
    rarr M1 = {m1, {nz, nx, 1}}, M2 = {m2, {nz, nx, 1}}, M3 = {m3, {nz, nx, 1}};
    int add = 0;
    F_image_mod_rtm_image_init(&nx, &dx, &nz, &dx, &nt, &dt, VX, VZ, &lame);
    if (!lame)
        F_image_mod_rtm_image_init2(M1, M2, M3);
    F_image_mod_rtm_image_op2(&adj, &add, dm1, dm2, dm3, h1, h2, h3, h4, h5);
    return 0;
}
