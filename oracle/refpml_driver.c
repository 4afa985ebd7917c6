/* Driver for the reference's PML Born modelling modules translated by
 * f90c.py --set pml (test infrastructure only).
 *
 * It takes the place of the reference's main program (2d_rtm_restart/
 * working_Src/born.f90:6-317), whose other work is SEPlib parameter and file
 * I/O: the models come in as arrays and the call sequence is the main
 * program's,
 *   elastic_init(nz,dz,nx,dx,nt,dt,xsource,zsource,nsource,fp,nsnap,nseis,
 *                abc,zrec,free_surface)                        (born.f90:282)
 *   stat = elastic_op(vp0,vs0,rho0,dvp,dvs,drho, seis x6, snap x6, lame)
 *                                                              (born.f90:285-293)
 * Arrays are Fortran-ordered: a model plane is (nz,nx), a receiver line
 * (nseis, nx-2*abc), a snapshot cube (nz,nx,nsnap).  The caller computes
 * nt, dt, nsource and nseis as the main program does. */
#include <string.h>

#include "refpml.h"

void F_born_mod_elastic_init(int *a_nz_in, float *a_dz_in, int *a_nx_in, float *a_dx_in, int *a_nt_in,
                             float *a_dt_in, int *a_xsource_in, int *a_zsource_in, int *a_nsource_in,
                             float *a_fp_in, int *a_nsnap_in, int *a_nseis_in, int *a_abc_in, int *a_zrec_in,
                             int *a_free_surface_in);
int F_born_mod_elastic_op(rarr a_vp0, rarr a_vs0, rarr a_rho0, rarr a_dvp, rarr a_dvs, rarr a_drho, rarr a_seis_vx,
                          rarr a_seis_vz, rarr a_seis_p, rarr a_seis_vx_b, rarr a_seis_vz_b, rarr a_seis_p_b,
                          rarr a_snap_vx, rarr a_snap_vz, rarr a_snap_p, rarr a_snap_vx_b, rarr a_snap_vz_b,
                          rarr a_snap_p_b, int *a_lame);

/* Returns elastic_op's status (0 ok). */
int refpml_born(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp,
                int nsnap, int nseis, int abc, int zrec, int free_surface, int lame, float *vp0, float *vs0,
                float *rho0, float *dvp, float *dvs, float *drho, float **seis, float **snap)
{
    float dz = dx;
    rarr m[6];
    float *mp[6] = {vp0, vs0, rho0, dvp, dvs, drho};
    for (int k = 0; k < 6; ++k) {
        m[k].p = mp[k];
        m[k].n[0] = nz;
        m[k].n[1] = nx;
        m[k].n[2] = 1;
    }
    rarr s[6], c[6];
    for (int k = 0; k < 6; ++k) {
        s[k].p = seis[k];
        s[k].n[0] = nseis;
        s[k].n[1] = nx - 2 * abc;
        s[k].n[2] = 1;
        c[k].p = snap[k];
        c[k].n[0] = nz;
        c[k].n[1] = nx;
        c[k].n[2] = nsnap;
    }
    F_born_mod_elastic_init(&nz, &dz, &nx, &dx, &nt, &dt, &xsource, &zsource, &nsource, &fp, &nsnap, &nseis, &abc,
                            &zrec, &free_surface);
    return F_born_mod_elastic_op(m[0], m[1], m[2], m[3], m[4], m[5], s[0], s[1], s[2], s[3], s[4], s[5], c[0], c[1],
                                 c[2], c[3], c[4], c[5], &lame);
}

/* Copies module array `name` ("module.variable", e.g. "pml_mod.pml0_xl")
 * into dst (up to n floats); returns its size, or -1 when there is none. */
long refpml_get(const char *name, float *dst, long n)
{
    for (const struct ref90_var *v = ref90_vars; v->name; ++v) {
        if (strcmp(v->name, name) != 0)
            continue;
        const rarr *a = v->arr;
        long size = a->p ? a->n[0] * a->n[1] * a->n[2] : 0;
        if (dst && size)
            memcpy(dst, a->p, sizeof(float) * (size_t)(size < n ? size : n));
        return size;
    }
    return -1;
}
