/*
 * elastic_rtm.h -- C-ABI of libelastic_rtm.so, the GB300 (sm_103a) engine for
 * the 2D elastic RTM / Born hot path of lgan/elastic and its single-domain 3D
 * acoustic propagator.
 *
 * Conventions (all entry points):
 *  - Arrays are plain pointers in the reference's Fortran layout:
 *    planes (nz,nx) column-major, z fastest; wavefield histories (nz,nx,nt);
 *    receiver gathers (nt,nx), one per component.
 *  - Grid positions (xsrc, zsrc, zrec) are 1-based, as in the Fortran.
 *  - Pointers are host memory unless the name ends in _dev.
 *  - int-returning functions return 0 on success or an RtmStatus code
 *    (1 bad argument, 2 out of memory, 3 CUDA error, 4 device wait timed
 *    out, 5 bad call order); rtm_last_error() gives the message.
 *  - The library uses CUDA device 0 unless ELASTIC_RTM_DEVICE names another.
 *    Every entry point is synchronous with respect to the host.
 *  - "exact" arithmetic reproduces the reference's CPU code bit for bit
 *    (every product and sum separately rounded, in the reference's order);
 *    "fast" arithmetic may fuse multiply-adds and reassociate the adjoint
 *    stencil (results agree to ~1e-6 relative L2).
 *
 * Reference paths below are inside the lgan/elastic project, with
 * W = 2d_rtm_restart/Src_working.
 */
#ifndef ELASTIC_RTM_H
#define ELASTIC_RTM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
const char *rtm_last_error(void);
/* Status of the last void drop-in call (rtm_op3_c_, rtm_gpu_*). */
int rtm_last_status(void);
/* Select exact (1, default) or fast (0) arithmetic for the drop-in calls. */
void rtm_set_exact(int exact);
/* Step-kernel generation: 0 automatic (default), 1 the shared-memory tile
 * kernel, 2 the cp.async-staged kernel (used only where planes are 16-byte
 * aligned with a pitch that is a multiple of 4 floats; otherwise 1). */
void rtm_set_kernel_version(int version);

/* ------------------------------------------------- drop-in replacements */
/* Adjoint recursion for levels nt-3 .. 0 (0-based) on full histories, in
 * place.  Replaces rtm_op3_c_ of W/rtmlib-modC.c:29-313 as bound by
 * W/rtmlib-modF.f90:27-52 (bind(c, name='rtm_op3_c_'), value scalars).
 * Coefficients are the unmasked (nz,nx) planes already scaled by dt/dx; the
 * reference's masks (W/rtmlib-modC.c:83-93) are applied on the device.
 * zrec is unused, as in the reference.  Errors: rtm_last_status(). */
void rtm_op3_c_(int nt, int nz, int nx, int zrec, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                float *sigmaxz0, float *m1_x, float *m1_z, float *aux_m2_c, float *aux_m3_c, float *aux_m2m3_c);

/* Allocation-free variant of rtm_op3_c_ (no counterpart in the reference):
 * the same adjoint recursion, exact arithmetic, on caller-owned DEVICE
 * buffers -- five (nz,nx,nt) histories updated in place and five unmasked
 * (nz,nx) coefficient planes -- for callers that cannot allocate device
 * memory at that point (their allocator owns the device heap, or an
 * allocation there would synchronise or fail).  It never calls cudaMalloc or
 * cudaFree: its scratch (masked coefficients, work-item table) is a fixed
 * 10 MiB device array of this library, so nz*nx must not exceed
 * RTM_NOALLOC_MAX_CELLS (larger grids are rejected with status 1).  The
 * first call on each device looks the scratch up (cudaGetSymbolAddress);
 * make it before any stream capture.  Calls whose GPU work overlaps race on
 * the shared scratch.  stream: a cudaStream_t, or NULL for the default
 * stream; returns after the work has finished. */
#define RTM_NOALLOC_MAX_CELLS 524288
int rtm_op3_dev_noalloc(int nt, int nz, int nx, float *Vx0_dev, float *Vz0_dev, float *sigmaxx0_dev,
                        float *sigmazz0_dev, float *sigmaxz0_dev, const float *m1_x_dev, const float *m1_z_dev,
                        const float *aux_m2_c_dev, const float *aux_m3_c_dev, const float *aux_m2m3_c_dev,
                        void *stream);

/* The reference's internal C<->CUDA layer (W/rtmlib-modC-gpu.cu:35,77,100,
 * 115,425), same arguments and padded layout: arrays (nz+10,nx+10[,nt+10])
 * with a 5-cell offset on every axis (W/gpu.h:9,13), masked coefficients.
 * rtm_gpu_func runs levels it_max .. 0, copying in and out itself, and
 * stores the device time per step (seconds) in gpu_kernel_time_ps[0];
 * `debug` is ignored. */
void rtm_gpu_init(int nt, int nz, int nx);
void rtm_gpu_copy_in(int nt, int nz, int nx, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                     float *sigmaxz0, float *ex_m1_x, float *ex_m1_z, float *ex_aux_m2_c, float *ex_aux_m3_c,
                     float *ex_aux_m2m3_c);
void rtm_gpu_copy_out(int nt, int nz, int nx, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                      float *sigmaxz0);
void rtm_gpu_func(int it_max, int nt, int nz, int nx, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                  float *sigmaxz0, float *ex_m1_x, float *ex_m1_z, float *ex_aux_m2_c, float *ex_aux_m3_c,
                  float *ex_aux_m2m3_c, float *debug, double *gpu_kernel_time_ps);
void rtm_gpu_final(void);

/* ------------------------------------------- siblings (one per reference
 * routine of the path; the Fortran calls them through bind(c) in the same
 * style as rtm_op3_c_) */

/* model_op + rtmmod_init + aux_*_c (W/model-mod.f90:21-89,
 * W/rtmlib-mod.f90:23-65, W/rtm-mod-adj.f90:99-113).  lambda and mu are
 * replaced in place by their staggered harmonic averages, as in the
 * reference.  Outputs m1_x, m1_z (scaled by dt/dx) and aux_m2_c, aux_m3_c,
 * aux_m2m3_c. */
int rtm_model_op_c_(int nz, int nx, float dx, float dt, const float *rho, float *lambda, float *mu, float *m1_x,
                    float *m1_z, float *aux_m2_c, float *aux_m3_c, float *aux_m2m3_c);

/* Ricker wavelet (W/source-mod.f90:31-44): source[nt]. */
int rtm_source_c_(int nt, float dt, float fp, int nsource, float *source);

/* Sponge filter table (W/abc-mod.f90:20-57): filter[abc+5].  abc=0 (which
 * reads out of bounds in the reference) gives an all-ones table. */
int rtm_abc_c_(int abc, float *filter);

/* Forward source wavefield history (W/rtm-mod-adj.f90:178-261): five
 * (nz,nx,nt) outputs.  Coefficients as returned by rtm_model_op_c_. */
int rtm_fwd_c_(int nt, int nz, int nx, float dt, int xsrc, int zsrc, int abc, const float *source,
               const float *m1_x, const float *m1_z, const float *aux_m2_c, const float *aux_m3_c,
               const float *aux_m2m3_c, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0, float *sigmaxz0);

/* image_init (W/image-mod-rtm.f90:26-67): S1..S6 histories from Vx0, Vz0. */
int rtm_image_init_c_(int nt, int nz, int nx, float dx, float dt, const float *Vx0, const float *Vz0, float *S1,
                      float *S2, float *S3, float *S4, float *S5, float *S6);

/* model_delta (W/model-mod.f90:91-171): dlambda, dmu averaged in place. */
int rtm_model_delta_c_(int nz, int nx, const float *drho, float *dlambda, float *dmu);

/* image_op2, Lame parameterisation (W/image-mod-rtm.f90:145-180).
 * adj=1: images (drho,dlambda,dmu) = imaging sums over the five histories;
 * adj=0: the five histories = Born secondary sources of the images. */
int rtm_image_op_c_(int adj, int nt, int nz, int nx, float *drho, float *dlambda, float *dmu, float *Vx0,
                    float *Vz0, float *sigmaxx0, float *sigmazz0, float *sigmaxz0, const float *S1, const float *S2,
                    const float *S3, const float *S4, const float *S5, const float *S6);

/* Born scattered propagation with the secondary sources already in the five
 * histories (W/rtm-mod-adj.f90:291-357), in place, then receiver sampling
 * of all five components at row zrec into (nt,nx) gathers (:361-375). */
int rtm_born_scatter_c_(int nt, int nz, int nx, int zrec, int abc, const float *m1_x, const float *m1_z,
                        const float *aux_m2_c, const float *aux_m3_c, const float *aux_m2m3_c, float *Vx0,
                        float *Vz0, float *sigmaxx0, float *sigmazz0, float *sigmaxz0, float *Vx, float *Vz,
                        float *sigmaxx, float *sigmazz, float *sigmaxz);

/* rtm_op3 (W/rtmlib-mod.f90:72-196): the five (nt,nx) receiver gathers are
 * written at row zrec and propagated backwards; outputs the five adjoint
 * histories.  exact_adjoint=1 applies the sponge to every adjoint level
 * (the transpose of the sponged Born operator); 0 is the reference. */
int rtm_op3_full_c_(int nt, int nz, int nx, int zrec, int abc, int exact_adjoint, const float *Vx,
                    const float *Vz, const float *sigmaxx, const float *sigmazz, const float *sigmaxz,
                    const float *m1_x, const float *m1_z, const float *aux_m2_c, const float *aux_m3_c,
                    const float *aux_m2m3_c, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                    float *sigmaxz0);

/* Whole rtm_op (W/rtm-mod-adj.f90:120-496, lame=.true.) for one shot, on
 * the raw model (rho, lambda, mu).  adj=1 (RTM): gathers in -> images
 * (drho, dlambda, dmu) out.  adj=0 (Born): images in -> gathers out; with
 * linear=0 dlambda and dmu are averaged in place by model_delta as in the
 * reference, linear=1 skips model_delta (the linear Born operator whose
 * transpose is adj=1 with exact_adjoint=1).  Full histories are kept on the
 * device (11 volumes of nz*nx*nt floats at most). */
int rtm_op_c_(int adj, int nz, int nx, int nt, float dx, float dt, int xsrc, int zsrc, int zrec, float fp,
              int nsource, int abc, const float *rho, const float *lambda, const float *mu, float *drho,
              float *dlambda, float *dmu, float *Vx, float *Vz, float *sigmaxx, float *sigmazz, float *sigmaxz,
              int linear, int exact_adjoint);
/* Least-squares RTM (no counterpart in the reference, which only intends an
 * iterative solver, W/rtm-mod-adj.f90:5-7): niter iterations of conjugate
 * gradients on the normal equations (CGLS) for the linear Born operator of
 * rtm_op_c_ (linear=1) over nshots shots on the full grid, with its exact
 * adjoint (exact_adjoint=1) as transpose, starting from a zero model.
 * xsrc/zsrc: 1-based source positions per shot; data: per shot the five
 * gathers of rtm_op_c_ (Vx, Vz, sigmaxx, sigmazz, sigmaxz, each (nt,nx)
 * Fortran order), shots consecutive.  dm: three (nz,nx) planes (drho,
 * dlambda, dmu) out.  resid (optional, niter+1 doubles): ||d - L m_k||.
 * comp_mask selects the recorded components as in rtm_born_migrate_c_
 * (the operator is mask * L).  Each shot's source history (5 nz*nx*nt
 * volumes) stays on the device. */
int rtm_lsrtm_c_(int nz, int nx, int nt, float dx, float dt, float fp, int nsource, int abc, int nshots,
                 const int *xsrc, const int *zsrc, int zrec, int comp_mask, const float *rho, const float *lambda,
                 const float *mu, const float *data, int niter, float *dm, double *resid);
int rtm_lsrtm_d_(int nz, int nx, int nt, double dx, double dt, double fp, int nsource, int abc, int nshots,
                 const int *xsrc, const int *zsrc, int zrec, int comp_mask, const double *rho, const double *lambda,
                 const double *mu, const double *data, int niter, double *dm, double *resid);

/* Velocity parameterisation (lame=.false., W/image-mod-rtm.f90:182-225; its
 * initialisation is commented out in W/rtmlib-mod.f90:59-63, so the
 * background Lame parameters are computed from the velocities here).
 * rtm_velocity_model_*: lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2.
 * rtm_velocity_jacobian_*: adj=1 maps the Lame images (drho, dlambda, dmu)
 * of rtm_op_c_ to the velocity images (drho, dvp, dvs) -- the reference's
 * velocity imaging condition, cell by cell the transpose of the Jacobian of
 * (rho, lambda, mu) with respect to (rho, vp, vs); adj=0 maps velocity
 * perturbations to the Lame perturbations whose Born sources the reference's
 * velocity branch injects.  All planes (nz,nx), host arrays. */
int rtm_velocity_model_c_(int nz, int nx, const float *rho, const float *vp, const float *vs, float *lambda, float *mu);
int rtm_velocity_model_d_(int nz, int nx, const double *rho, const double *vp, const double *vs, double *lambda,
                          double *mu);
int rtm_velocity_jacobian_c_(int adj, int nz, int nx, const float *rho, const float *vp, const float *vs,
                             const float *in1, const float *in2, const float *in3, float *out1, float *out2,
                             float *out3);
int rtm_velocity_jacobian_d_(int adj, int nz, int nx, const double *rho, const double *vp, const double *vs,
                             const double *in1, const double *in2, const double *in3, double *out1, double *out2,
                             double *out3);

/* Nonlinear elastic forward modelling of one shot (W/elastic-mod.f90:95-240,
 * the driver of elastic.x): the forward time loop of rtm_op on the raw
 * model (rho, lambda, mu), keeping two levels per field instead of the
 * reference's full histories, with the five receiver gathers at row zrec
 * (each (nt,nx) Fortran order, as W/elastic-mod.f90:226-234 samples them).
 * 1-based positions. */
int rtm_model_c_(int nz, int nx, int nt, float dx, float dt, int xsrc, int zsrc, int zrec, float fp, int nsource,
                 int abc, const float *rho, const float *lambda, const float *mu, float *Vx_rec, float *Vz_rec,
                 float *sigmaxx_rec, float *sigmazz_rec, float *sigmaxz_rec);

/* Born modelling and migration of a batch of npairs model perturbations
 * for one shot on the full grid, the source wavefield computed once (no
 * counterpart in the reference; builds the learned preconditioner's
 * training pairs).  With dm (npairs x 3 planes drho, dlambda, dmu): data_k =
 * L dm_k (linear Born, written to data when not null) and, when img is not
 * null, img_k = L^T data_k with the exact adjoint.  With data_in instead of
 * dm: img_k = L^T data_in_k.  Gathers as in rtm_op_c_ (5 x (nt,nx) per pair).
 * comp_mask (bit c for Vx, Vz, sigmaxx, sigmazz, sigmaxz; 31 = all) selects
 * the recorded components: the others are zero in data and ignored in
 * data_in (the operator is mask * L).  on_device=1: all arrays are device
 * pointers. */
int rtm_born_migrate_c_(int nz, int nx, int nt, float dx, float dt, int xsrc, int zsrc, int zrec, float fp,
                        int nsource, int abc, int comp_mask, const float *rho, const float *lambda, const float *mu,
                        int npairs, const float *dm, float *data, const float *data_in, float *img, int on_device);

/* Double-precision twin of rtm_op_c_ (used for the FP64 oracle comparison
 * and the adjoint dot-product test). */
int rtm_op_d_(int adj, int nz, int nx, int nt, double dx, double dt, int xsrc, int zsrc, int zrec, double fp,
              int nsource, int abc, const double *rho, const double *lambda, const double *mu, double *drho,
              double *dlambda, double *dmu, double *Vx, double *Vz, double *sigmaxx, double *sigmazz,
              double *sigmaxz, int linear, int exact_adjoint);

/* ------------------------------------------------- 3D acoustic (a14, a15)
 * Single-domain 3D acoustic propagator, 10th order in space (the
 * reference's W/wave_fkernel.3d8o.cu:31-106 is 8th order), sponge of
 * W/wave_fkernel.3d8o.cu:183-210 with factor expf(-damp_b*(damp_a-edge)) for
 * edge distances below damp_a, point source added after each update,
 * receivers on the plane iz=zr (1-based; 0 = none) recorded into
 * data[it][iy][ix].  Layout p[(iy*n2+ix)*n1+iz]; vel2 = v^2 dt^2.  Only the
 * interior [5, n-5) of every axis is updated.  on_device selects device
 * pointers; *ms receives the device time of the propagation.
 * acoustic3d_fwd_c_ returns the traces and the last two levels (the state
 * the reverse-time restart starts from); acoustic3d_rtm_c_ propagates the
 * source undamped, restarts it backwards from its last two levels
 * (W/gpu_funcs_3d.cu:509-712) and images every jt-th level. */
int acoustic3d_fwd_c_(int n1, int n2, int n3, int nt, float d1, float d2, float d3, const float *vel2, int damp_a,
                      float damp_b, int zs, int xs, int ys, const float *wavelet, int zr, float *data,
                      float *p_last0, float *p_last1, int on_device, double *ms);
int acoustic3d_rtm_c_(int n1, int n2, int n3, int nt, float d1, float d2, float d3, const float *vel2, int damp_a,
                      float damp_b, int zs, int xs, int ys, const float *wavelet, int zr, const float *data, int jt,
                      float *img, int on_device, double *ms);
/* Kernel shape of the 3D propagator: tile width 8 or 16 columns and the
 * number of chunks the y march is split into (0 = chosen from the SM count).
 * The tile width applies to the cp.async-pipelined kernel; the slice-ring
 * kernel uses 16 columns. */
int acoustic3d_set(int tile_x, int ychunks);
/* Step kernel where n1 % 4 == 0 (other n1 run a scalar kernel):
 *   0 (default) slab kernel: every operand arrives by bulk tensor copies
 *     issued slices ahead (p1 slabs with their x/z halo, p0 and v^2 dt^2
 *     boxes), the y taps from an unrolled register queue;
 *   1 slice-ring kernel: every tap from a 13-slice shared-memory ring filled
 *     by bulk tensor copies;
 *   2 cp.async-pipelined kernel with a shifted register queue;
 *   3 the slab kernel with paired FP32 instructions in fast arithmetic.
 * All are bit-identical in exact arithmetic.  A kernel whose copy does not
 * land within about a second stops; the entry point then returns
 * RTM_ERR_TIMEOUT (4). */
int acoustic3d_set_kernel(int kind);

/* ----------------------------------- 3D elastic kernel test (kernel_3d_test)
 * One step of the reference's 3D elastic kernel (kernel_3d_test/
 * rtmlib-modC.c:277-590): nine fields Vy, Vx, Vz, syy, sxx, szz, sxy, sxz,
 * syz and six coefficient planes m1_y, m1_x, m1_z, m2, m3, m2m3, each a
 * padded (ny+10)(nx+10)(nz+10) float plane, z fastest, interior at +5;
 * out = out + in1 + 10th-order staggered differences of coefficient x
 * field taps of `in` along z, x and y.
 * rtm3d_gpu_init / rtm3d_gpu_func / rtm3d_gpu_final have the signatures and
 * meaning of the reference's rtm_gpu_init / rtm_gpu_func / rtm_gpu_final
 * for this test (kernel_3d_test/gpu.h:68-79, rtmlib-modC-gpu.cu:65,218,698):
 * host planes in, one step, the nine outputs copied back, gpu_kernel_time
 * = {copy in, step, copy out} in seconds.  They carry an rtm3d_ prefix
 * because the 2D drop-in already exports the reference's rtm_gpu_* names;
 * the reference's test binds them by renaming on its compile line
 * (INTEGRATION.md).  Status in rtm_last_status().  Exact arithmetic (the
 * default, rtm3d_set_exact(1)) is bit-identical to the reference's CPU
 * step; rtm3d_set_exact(0) lets the compiler fuse multiply-adds.
 * rtm3d_step_dev: the same step on device planes (in[9], in1[9], out[9],
 * m[6] arrays of device pointers), on the default stream. */
void rtm3d_gpu_init(int ny, int nz, int nx);
void rtm3d_gpu_func(int ny, int nz, int nx, float *vy0, float *vx0, float *vz0, float *syy0, float *sxx0, float *szz0,
                    float *sxy0, float *sxz0, float *syz0, float *vy1, float *vx1, float *vz1, float *syy1, float *sxx1,
                    float *szz1, float *sxy1, float *sxz1, float *syz1, float *vyo, float *vxo, float *vzo, float *syyo,
                    float *sxxo, float *szzo, float *sxyo, float *sxzo, float *syzo, float *m1y, float *m1x, float *m1z,
                    float *m2, float *m3, float *m2m3, float *debug, float *gpu_kernel_time);
void rtm3d_gpu_final(void);
int rtm3d_set_exact(int exact);
/* Step kernel form, every form bit-identical: 0 one cell a thread; 1 two z
 * cells a thread with 8-byte taps (where nz is even and the planes 8-byte
 * aligned, else the one-cell form); + 2 requests the own cells' lines into
 * L2 first; + 4 bounds registers to 4 blocks of 256 threads an SM
 * (default 5). */
int rtm3d_set_kernel(int kind);
int rtm3d_step_dev(int ny, int nz, int nx, const float *const *in, const float *const *in1, float *const *out,
                   const float *const *m, int exact);

/* -------------------------------------------- split-field PML Born modelling
 * The reference's PML Born modelling program (2d_rtm_restart/working_Src/
 * born.f90 -> born_mod's elastic_init + elastic_op, born-mod.f90:32-78):
 * background and scattered wavefields with split-field PML (pml-mod.f90),
 * Ricker source at (zsource, xsource), receiver lines at row zrec, nsnap
 * snapshots.  Arguments are elastic_init's and elastic_op's (dz is unused
 * by the reference and omitted); grid indices are 1-based; planes are
 * Fortran-ordered (nz, nx).  nt, dt, nsource and nseis are derived by the
 * caller as the reference's main program does (born.f90:67-73, 251, 255).
 * lame = 0: vp0, vs0, rho0 / dvp, dvs, drho are velocities and densities;
 * lame = 1: vp0, vs0 hold lambda, mu (and dvp, dvs their perturbations).
 * seis[6] = Vx, Vz, P, Vx_b, Vz_b, P_b receiver lines (nseis, nx - 2 abc);
 * snap[6] the same six as (nz, nx, nsnap) cubes.  Every output is fully
 * written; cells the reference never sets are zero.  Requires nz, nx >= 11,
 * 1 <= nsnap <= nt, 0 <= abc <= min(nz, nx), 2 <= zrec <= nz.  Bit-identical
 * to the reference's CPU execution.
 * pml_born_c_: host arrays.  pml_born_dev: model[6] = vp0, vs0, rho0, dvp,
 * dvs, drho and the outputs are device pointers, work on `stream` (a
 * cudaStream_t, NULL for the default stream) and returns when it is done.
 * Calls of a process are serialized (one set of working planes).
 * pml_born_launches: kernels launched by the last call.
 * pml_set_kernel: step kernel form, kind & 15: 0 four rows per thread, 1 one
 * cell per thread, 4 tiles staged by bulk tensor copies, 8 one launch a
 * level for both wavefields (scattered one level behind); + 2 to request
 * each thread's first-touch lines into L2 first; kind >> 4 (one-cell form):
 * 0, or a register bound of 5, 6 or 8 blocks of 256 threads an SM.  Default
 * 3 + 6 * 16.  Every form gives the same bits.  A staged tile whose copies do not arrive within about a
 * second makes the call return status 4. */
int pml_born_c_(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp, int nsnap,
                int nseis, int abc, int zrec, int free_surface, int lame, const float *vp0, const float *vs0,
                const float *rho0, const float *dvp, const float *dvs, const float *drho, float *const *seis,
                float *const *snap);
int pml_born_dev(int nz, int nx, int nt, float dx, float dt, int xsource, int zsource, int nsource, float fp, int nsnap,
                 int nseis, int abc, int zrec, int free_surface, int lame, const float *const *model,
                 float *const *seis, float *const *snap, void *stream);
long long pml_born_launches(void);
int pml_set_kernel(int kind);
/* Test hook of the failure path: with on = 1, the staged-tile form's first
 * launch of every later call waits on a flag that nothing sets instead of
 * its copies, gives up after about a second, and the call returns status 4
 * (no copy is in flight when a CTA gives up).  0 restores normal runs. */
int pml_set_test_stall(int on);

/* -------------------------------------------- batched multi-shot RTM
 * No counterpart in the reference (one shot per run, W/rtm.f90:46-47): the
 * shots of a survey, each on its own subgrid [x0, x0+nxs) of the full model
 * (uneven widths), are migrated in groups of up to group_max shots.  Each
 * time level of a group is one launch over all its shots; the nt-level
 * loops of both passes are captured as one CUDA graph per group.  The
 * source side keeps per-level FP16 snapshots of Vx, Vz (per-snapshot
 * scaled); propagation and image accumulation (Kahan) are FP32; fast
 * arithmetic.  Positions are 1-based in the full grid.  comp_mask selects
 * the recorded components (bit 0 Vx, 1 Vz, 2 sigma_xx, 3 sigma_zz,
 * 4 sigma_xz).  exact_adjoint=1 applies the sponge in the adjoint. */
typedef struct rtm_batch rtm_batch;
rtm_batch *rtm_batch_create(int nz, int nx, int nt, float dx, float dt, float fp, int nsource, int abc,
                            const float *rho, const float *lambda, const float *mu, int nshots, const int *x0,
                            const int *nxs, const int *xsrc, const int *zsrc, const int *zrec, int comp_mask,
                            int group_max, int exact_adjoint);
/* Migrate shots [shot0, shot0+nshot) (nshot <= group_max).  traces: for
 * each shot in order, for each selected component, an (nt, nxs) gather in
 * the reference layout.  image: three (nz,nx) planes (drho, dlambda, dmu)
 * to which the group's images are added.  *_on_device selects device or
 * host pointers. */
int rtm_batch_migrate(rtm_batch *b, int shot0, int nshot, const float *traces, int traces_on_device, float *image,
                      int image_on_device);
/* out[0..43] (pass an array of at least 44 doubles): forward ms, adjoint
 * ms, cells of the last group, kernels launched, total ms of the last call,
 * forward tile width, forward work items, adjoint tile width; [8..13] the
 * autotuner's best ms per step for tile widths 8, 16, 32 (forward, then
 * adjoint); [14..15] staging buffers per CTA (1 or 2) of the forward and
 * adjoint pass; [16..39] the autotuner's ms per step for every tile width
 * (8, 16, 32) and launch shape (1 stage, 2 stages, each with 256 then 512
 * threads), forward then adjoint, -1 where a shape does not fit in a block;
 * [40..41] threads per CTA of the forward and adjoint pass; [42] checkpoint
 * interval (0 = every level's snapshots kept); [43] 1 with TMA staging. */
int rtm_batch_stats(const rtm_batch *b, double *out);
/* Autotuner: times `steps` launches of each pass for every tile width and
 * staging depth on the geometry of shots [shot0, shot0+nshot) and keeps the
 * fastest per pass for the following rtm_batch_migrate calls. */
int rtm_batch_autotune(rtm_batch *b, int shot0, int nshot, int steps);
/* use_graph=0 launches the time loop kernel by kernel; tile_x selects the
 * tile width of the step kernel (8, 16 or 32; 0 = automatic). */
int rtm_batch_set(rtm_batch *b, int use_graph, int tile_x);
/* Launch shape of the forward and adjoint step kernels: staging buffers per
 * CTA (1, or 2 to stage the next tile while computing the current one) and
 * threads per CTA (256, or 512 at tile widths >= 16).  A shape that does not
 * fit in a block with the tile width in use falls back to 1 stage and 256
 * threads. */
int rtm_batch_set_stages(rtm_batch *b, int fwd, int adj, int threads_fwd, int threads_adj);
/* Checkpoint-restart of the source wavefield.  interval = 0 keeps the FP16
 * snapshots of every level (4 bytes per cell and level); interval = k keeps
 * the full forward state every k levels (40 bytes per cell each) and a ring
 * of k + 1 snapshot levels, and the adjoint pass recomputes each k-level
 * segment from its checkpoint before migrating through it (one more forward
 * propagation; images bit-identical to interval 0).  rtm_batch_create picks
 * k ~ sqrt(10 nt) by itself when every level's snapshots would not fit in 80 %
 * of the free device memory.  out[42] of rtm_batch_stats reports k. */
int rtm_batch_set_checkpoint(rtm_batch *b, int interval);
/* on=1 (the default): the step kernels stage their tiles with
 * tensor-memory-access bulk loads (one thread per tile, completion on a
 * shared-memory barrier with a time limit; a load that does not complete
 * fails the call with status 4); on=0: per-thread asynchronous copies.
 * Results are bit-identical.  out[43] of rtm_batch_stats reports the
 * setting. */
int rtm_batch_set_tma(rtm_batch *b, int on);
/* Forward and adjoint passes by the marching kernels (one CTA per SM walks
 * 128-row strips column chunk by column chunk, operands loaded by tensor-map
 * copies ahead of the compute; needs tensor-map staging): mode -1 = the
 * autotuner's choice per pass (on until rtm_batch_autotune has run), else a
 * bit mask: 1 forward, 2 adjoint (0 = tile kernels for both).  The marching
 * forward is bit-identical to the tile kernel; the marching adjoint sums the
 * two pairs of coefficient x field products that share a stencil before
 * differencing them, which agrees with the tile kernel to rounding (fast
 * arithmetic).  rtm_batch_stats: out[44] / out[46] whether the forward /
 * adjoint marching kernel runs, out[45] / out[47] their autotuner times (ms
 * per launch, -1 when not timed). */
int rtm_batch_set_march(rtm_batch *b, int mode);
/* Test hook for the timeout path (no counterpart in the reference): with
 * on != 0 the forward pass's first marching launch of every following
 * migration waits on a device flag that nothing sets.  The wait gives up
 * after about a second, before the kernel has issued any copy, and
 * rtm_batch_migrate returns RTM_ERR_TIMEOUT (4) for that group; with on = 0
 * the engine migrates normally again.  Needs the marching forward kernel
 * (rtm_batch_set_march with bit 1). */
int rtm_batch_set_test_stall(rtm_batch *b, int on);
void rtm_batch_destroy(rtm_batch *b);
/* Page-locked host memory for fast host<->device traces and images. */
void *rtm_host_alloc(size_t bytes);
void rtm_host_free(void *p);

/* Checks of the tensor-core building blocks (no counterpart in the
 * reference).  rtm_debug_umma_desc: out[0] = the tcgen05 instruction
 * descriptor (.kind::f16, M x N, BF16 or F16 operands, F32 or F16
 * accumulator), out[1] = the shared-memory matrix descriptor of a matrix at
 * shared address addr with byte offsets lbo (along K) and sbo (along M/N)
 * and the given swizzle mode.  rtm_debug_umma_probe: one 128 x N x 16 BF16
 * MMA (A 128x16 and B Nx16 row-major BF16 on the host, K contiguous) with the
 * operands stored K-major without swizzle (core matrices 128 bytes apart
 * along K, 256 along M/N) and the descriptors built with lbo/sbo; D (128 x N,
 * FP32) comes back from tensor memory. */
int rtm_debug_umma_desc(int M, int N, int bf16, int f32, unsigned addr, unsigned lbo, unsigned sbo, unsigned swizzle,
                        unsigned long long *out);
int rtm_debug_umma_probe(int N, unsigned lbo, unsigned sbo, const unsigned short *A, const unsigned short *B,
                         float *D);
/* rtm_debug_umma_probe_sw: A (128 x K) and B (N x K), K = 64 or 32, placed
 * in shared memory in the 128-byte (K = 64) or 64-byte (K = 32) swizzled
 * K-major layout that bulk tensor copies produce, multiplied by K/16 MMAs
 * whose descriptors advance 32 bytes along K: D = A B^T (128 x N, FP32). */
int rtm_debug_umma_probe_sw(int N, int K, const unsigned short *A, const unsigned short *B, float *D);
/* rtm_debug_umma_probe2: layout variants.  mode 0: A ((128+shift) x K,
 * K = 32 or 64) in the swizzled K-major layout, the descriptor starting
 * `shift` rows in (base-offset field (start >> 7) & 7 when boff), D = A[shift
 * .. shift+127] B^T.  mode 1: A (128 x 32) and B (N x 32, N = 64 or 128)
 * MN-major with the 128-byte swizzle, atoms of 8 K-rows x 64 MN elements
 * placed lbo apart along MN and sbo apart along K ((4096, 1024) or
 * (1024, 2048)), D = A B^T.  mode 2: the same with the 64-byte swizzle (atoms
 * of 8 K-rows x 32 MN elements, N = 32 .. 128, (lbo, sbo) = (2048, 512) or
 * (512, 2048)). */
int rtm_debug_umma_probe2(int N, int K, int mode, int shift, int boff, unsigned lbo, unsigned sbo,
                          const unsigned short *A, const unsigned short *B, float *D);

/* ------------------------------------------ learned image preconditioner
 * (no counterpart in the reference).  A 4-level 3->3 channel U-Net
 * (channels 32/64/96/128, 3x3 convolutions with leaky ReLU (slope 0.1), 2x2 average pooling,
 * nearest upsampling with skip concatenation, 1x1 output convolution;
 * ~0.9M parameters) with BF16 weights and activations and FP32 accumulation
 * on the tensor cores, trained with Adam on the mean squared error.  Images
 * are FP32 NHWC (n, H, W, 3); H and W multiples of 8.  Parameters are one
 * flat FP32 vector: per layer (15 convolutions in the order e1a e1b e2a e2b
 * e3a e3b ba bb d3a d3b d2a d2b d1a d1b out) the weights [coutp][kp] with
 * k = (ky*3+kx)*cin + ci (zero-padded to kp), then the bias [coutp]. */
typedef struct unet unet;
unet *unet_create(int H, int W, int max_batch, unsigned seed);
void unet_destroy(unet *u);
long long unet_num_params(const unet *u);
/* info[0..8]: ks, cin, cout, coutp, kp, weight offset, bias offset, H, W */
int unet_layer_info(const unet *u, int layer, long long *info);
int unet_get_params(const unet *u, float *w);
/* also resets the Adam moments and step count */
int unet_set_params(unet *u, const float *w);
/* y (n, H, W, 3) = net(x); *_on_device selects device or host pointers */
int unet_forward(unet *u, const float *x, int n, float *y, int on_device);
/* loss = mean((net(x) - t)^2) and its gradient (flat, like the parameters;
 * grad may be null) without updating the weights */
int unet_loss_grad(unet *u, const float *x, const float *t, int n, int on_device, double *loss, float *grad);
/* one Adam step (bias-corrected) on the batch; loss before the update */
int unet_train_step(unet *u, const float *x, const float *t, int n, int on_device, float lr, float beta1, float beta2,
                    float eps, double *loss);
/* GEMM path of the forward and backward-data passes: 2 (default) tcgen05
 * MMAs with tensor-memory accumulators, the 3x3 convolutions fed by bulk
 * tensor copies of shifted activation boxes (zero padding from the copies'
 * out-of-range fill), other GEMMs by the thread-gathered kernel of 1; 1 the
 * thread-gathered tcgen05 kernel for every such GEMM; 0 the mma.sync
 * kernel.  The backward-weights pass always runs mma.sync.  A tensor-core
 * GEMM whose bounded wait runs out makes the call return RTM_ERR_TIMEOUT (4). */
int unet_set_gemm(int tensor_core);

#ifdef __cplusplus
}
#endif
#endif /* ELASTIC_RTM_H */
