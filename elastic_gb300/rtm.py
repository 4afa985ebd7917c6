"""Python mirror of the reference's operator interface for the elastic RTM path.

The names, argument meanings and error behaviour follow the Fortran modules
of lgan/elastic (W = 2d_rtm_restart/Src_working):

* ``rtm_init`` / ``RtmOperator.rtm_op`` -- W/rtm-mod-adj.f90:43-129
  (``rtm_op`` returns stat 0 on success; failures raise ``RtmError``).
* ``rtm_op3`` -- the Fortran->C call of W/rtmlib-mod.f90:158 into
  ``rtm_op3_c_`` (W/rtmlib-modC.c:29), in place on full histories.
* ``model_op``, ``source_op2``, ``abc_init``, ``image_init``, ``image_op2``,
  ``model_delta``, ``born_scatter``, ``rtm_op3_full`` -- one per reference
  routine of the path.

Arrays are numpy, C-ordered views of the Fortran layout: a plane (nz,nx) is
``a[ix, iz]``, a history (nz,nx,nt) is ``h[it, ix, iz]``, a gather (nt,nx) is
``d[ix, it]``.  Grid positions are 1-based.  Every computation runs in
libelastic_rtm.so on the GPU.
"""
import numpy as np

from ._lib import check, check_void, load, ptr

F32 = np.float32


def _f32(a):
    return np.ascontiguousarray(a, dtype=F32)


def set_exact(exact=True):
    """Exact (reference bit-identical) or fast arithmetic for the drop-in calls."""
    load().rtm_set_exact(1 if exact else 0)


def set_kernel_version(version=0):
    """0 automatic, 1 shared-memory tile kernel, 2 cp.async-staged kernel."""
    load().rtm_set_kernel_version(int(version))


# ----------------------------------------------------------------- a1..a4
def model_op(rho, lam, mu, dx, dt):
    """model_op + rtmmod_init + aux_*_c.  Returns (m1_x, m1_z, aux_m2_c,
    aux_m3_c, aux_m2m3_c, lambda_avg, mu_avg)."""
    rho, lam, mu = _f32(rho), _f32(lam).copy(), _f32(mu).copy()
    nx, nz = rho.shape
    out = [np.zeros_like(rho) for _ in range(5)]
    check(load().rtm_model_op_c_(nz, nx, dx, dt, ptr(rho), ptr(lam), ptr(mu), *[ptr(o) for o in out]))
    return (*out, lam, mu)


def source_op2(nt, dt, fp, nsource=250):
    s = np.zeros(nt, F32)
    check(load().rtm_source_c_(nt, dt, fp, nsource, ptr(s)))
    return s


def abc_init(abc):
    f = np.zeros(abc + 5, F32)
    check(load().rtm_abc_c_(abc, ptr(f)))
    return f


# ----------------------------------------------------------------- a6..a13
def forward(coefs, nt, dt, xsrc, zsrc, abc, source):
    """Source wavefield histories (Vx0, Vz0, sxx0, szz0, sxz0)."""
    coefs = [_f32(c) for c in coefs]
    nx, nz = coefs[0].shape
    H = [np.zeros((nt, nx, nz), F32) for _ in range(5)]
    check(load().rtm_fwd_c_(nt, nz, nx, dt, xsrc, zsrc, abc, ptr(_f32(source)), *[ptr(c) for c in coefs],
                            *[ptr(h) for h in H]))
    return H


def image_init(Vx0, Vz0, dx, dt):
    Vx0, Vz0 = _f32(Vx0), _f32(Vz0)
    nt, nx, nz = Vx0.shape
    S = [np.zeros_like(Vx0) for _ in range(6)]
    check(load().rtm_image_init_c_(nt, nz, nx, dx, dt, ptr(Vx0), ptr(Vz0), *[ptr(s) for s in S]))
    return S


def model_delta(drho, dlambda, dmu):
    dl, dm = _f32(dlambda).copy(), _f32(dmu).copy()
    nx, nz = dl.shape
    check(load().rtm_model_delta_c_(nz, nx, ptr(_f32(drho)), ptr(dl), ptr(dm)))
    return dl, dm


def image_op2(adj, S, images=None, H=None):
    """adj=True: histories H -> images (drho, dlambda, dmu);
    adj=False: images -> five secondary-source histories."""
    S = [_f32(s) for s in S]
    nt, nx, nz = S[0].shape
    if adj:
        H = [_f32(h) for h in H]
        img = [np.zeros((nx, nz), F32) for _ in range(3)]
    else:
        img = [_f32(i).copy() for i in images]
        H = [np.zeros((nt, nx, nz), F32) for _ in range(5)]
    check(load().rtm_image_op_c_(1 if adj else 0, nt, nz, nx, *[ptr(i) for i in img], *[ptr(h) for h in H],
                                 *[ptr(s) for s in S]))
    return img if adj else H


def born_scatter(H, coefs, zrec, abc):
    """Scattered propagation in place on H; returns five gathers [nx, nt]."""
    H = [np.ascontiguousarray(h, F32) for h in H]
    nt, nx, nz = H[0].shape
    D = [np.zeros((nx, nt), F32) for _ in range(5)]
    check(load().rtm_born_scatter_c_(nt, nz, nx, zrec, abc, *[ptr(_f32(c)) for c in coefs], *[ptr(h) for h in H],
                                     *[ptr(d) for d in D]))
    return H, D


def rtm_op3_full(D, coefs, nz, zrec, abc=0, exact_adjoint=False):
    """rtm_op3: five gathers [nx, nt] -> five adjoint histories."""
    D = [_f32(d) for d in D]
    nx, nt = D[0].shape
    H = [np.zeros((nt, nx, nz), F32) for _ in range(5)]
    check(load().rtm_op3_full_c_(nt, nz, nx, zrec, abc, 1 if exact_adjoint else 0, *[ptr(d) for d in D],
                                 *[ptr(_f32(c)) for c in coefs], *[ptr(h) for h in H]))
    return H


def rtm_op3(nt, nz, nx, zrec, Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0, m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c):
    """Drop-in rtm_op3_c_: adjoint recursion in place on the five histories."""
    arrs = [Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0, m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c]
    for a in arrs:
        if a.dtype != F32 or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("rtm_op3 works in place on C-contiguous float32 arrays")
    load().rtm_op3_c_(nt, nz, nx, zrec, *[ptr(a) for a in arrs])
    check_void()


# ----------------------------------------------------------------- rtm_op
class RtmOperator:
    """rtm_init + rtm_op of W/rtm-mod-adj.f90 for the Lame parameterisation.

    ``rtm_op(adj, drho, dlambda, dmu, Vx, Vz, sigmaxx, sigmazz, sigmaxz)``
    follows the reference: adj=True migrates the five gathers into the three
    images (overwritten in place); adj=False Born-models the images into the
    gathers (dlambda/dmu are averaged in place by model_delta unless
    linear=True).  Returns stat 0.
    """

    def __init__(self, nz, dz, nx, dx, dt, xsource, zsource, zrec, fp, nt, abc, rho, lam, mu, nsource=250,
                 dtype=F32, linear=False, exact_adjoint=False, lame=True):
        """With lame=False the model is (rho, vp, vs) in place of (rho,
        lambda, mu) and the images / perturbations are (drho, dvp, dvs)
        (W/image-mod-rtm.f90:182-225); lambda and mu are derived from the
        velocities."""
        self.nz, self.nx, self.nt = nz, nx, nt
        self.dz, self.dx, self.dt = dz, dx, dt
        self.xsource, self.zsource, self.zrec = xsource, zsource, zrec
        self.fp, self.abc, self.nsource = fp, abc, nsource
        self.dtype = np.dtype(dtype)
        self.lame = lame
        self.rho = np.ascontiguousarray(rho, self.dtype)
        if lame:
            self.lam = np.ascontiguousarray(lam, self.dtype)
            self.mu = np.ascontiguousarray(mu, self.dtype)
        else:
            self.vp = np.ascontiguousarray(lam, self.dtype)
            self.vs = np.ascontiguousarray(mu, self.dtype)
            self.lam, self.mu = velocity_model(self.rho, self.vp, self.vs)
        self.linear, self.exact_adjoint = linear, exact_adjoint

    def rtm_op(self, adj, drho, dlambda, dmu, Vx, Vz, sigmaxx, sigmazz, sigmaxz):
        if not self.lame:
            return self._rtm_op_velocity(adj, drho, dlambda, dmu, Vx, Vz, sigmaxx, sigmazz, sigmaxz)
        return self._rtm_op_lame(adj, drho, dlambda, dmu, Vx, Vz, sigmaxx, sigmazz, sigmaxz)

    def _rtm_op_velocity(self, adj, drho, dvp, dvs, *gathers):
        if adj:
            im = [np.zeros_like(drho) for _ in range(3)]
            self._rtm_op_lame(True, *im, *gathers)
            out = velocity_jacobian(True, self.rho, self.vp, self.vs, *im)
        else:
            dl = velocity_jacobian(False, self.rho, self.vp, self.vs, drho, dvp, dvs)
            self._rtm_op_lame(False, *dl, *gathers)
            return 0
        for dst, src in zip((drho, dvp, dvs), out):
            dst[...] = src
        return 0

    def _rtm_op_lame(self, adj, drho, dlambda, dmu, Vx, Vz, sigmaxx, sigmazz, sigmaxz):
        arrs = [drho, dlambda, dmu, Vx, Vz, sigmaxx, sigmazz, sigmaxz]
        for a in arrs:
            if a.dtype != self.dtype or not a.flags["C_CONTIGUOUS"]:
                raise TypeError(f"rtm_op works in place on C-contiguous {self.dtype} arrays")
        fn = load().rtm_op_d_ if self.dtype == np.float64 else load().rtm_op_c_
        check(fn(1 if adj else 0, self.nz, self.nx, self.nt, self.dx, self.dt, self.xsource, self.zsource,
                 self.zrec, self.fp, self.nsource, self.abc, ptr(self.rho), ptr(self.lam), ptr(self.mu),
                 *[ptr(a) for a in arrs], 1 if self.linear else 0, 1 if self.exact_adjoint else 0))
        return 0


def lsrtm(rho, lam, mu, data, xsrc, zsrc, zrec, dx, dt, nt, fp, abc, niter=10, nsource=250, dtype=F32, comp_mask=31):
    """Least-squares RTM by CGLS on the linear Born operator of ``rtm_op``
    (linear=True) with its exact adjoint, over all shots stacked.

    rho, lam, mu: (nx, nz) models.  data: (nshots, 5, nx, nt) gathers in the
    order Vx, Vz, sigmaxx, sigmazz, sigmaxz.  xsrc, zsrc: 1-based source
    positions per shot.  Returns (dm, resid): dm (3, nx, nz) = (drho,
    dlambda, dmu) after niter iterations from zero, resid (niter+1,) the
    data residual norms ||d - L m_k||.  comp_mask selects the recorded
    components (bit c: Vx, Vz, sigmaxx, sigmazz, sigmaxz); the others are
    ignored.
    """
    dtype = np.dtype(dtype)
    rho, lam, mu = (np.ascontiguousarray(a, dtype) for a in (rho, lam, mu))
    nx, nz = rho.shape
    data = np.ascontiguousarray(data, dtype)
    nshots = data.shape[0]
    if data.shape != (nshots, 5, nx, nt):
        raise ValueError(f"data must be (nshots, 5, {nx}, {nt}), got {data.shape}")
    xs = np.ascontiguousarray(xsrc, np.int32)
    zs = np.ascontiguousarray(zsrc, np.int32)
    if xs.shape != (nshots,) or zs.shape != (nshots,):
        raise ValueError("one source position per shot")
    dm = np.zeros((3, nx, nz), dtype)
    resid = np.zeros(niter + 1, np.float64)
    fn = load().rtm_lsrtm_d_ if dtype == np.float64 else load().rtm_lsrtm_c_
    check(fn(nz, nx, nt, dx, dt, fp, nsource, abc, nshots, ptr(xs), ptr(zs), zrec, comp_mask, ptr(rho), ptr(lam),
             ptr(mu), ptr(data), niter, ptr(dm), ptr(resid)))
    return dm, resid


def model(rho, lam, mu, dx, dt, nt, xsrc, zsrc, zrec, fp, abc, nsource=250):
    """Nonlinear elastic modelling of one shot (elastic.x of the reference):
    returns the five receiver gathers (Vx, Vz, sigmaxx, sigmazz, sigmaxz),
    each (nx, nt) -- the C view of Fortran (nt, nx).  1-based positions;
    rho, lam, mu are (nx, nz) float32."""
    rho, lam, mu = (np.ascontiguousarray(a, F32) for a in (rho, lam, mu))
    nx, nz = rho.shape
    D = [np.zeros((nx, nt), F32) for _ in range(5)]
    check(load().rtm_model_c_(nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, ptr(rho), ptr(lam), ptr(mu),
                              *[ptr(d) for d in D]))
    return D


def velocity_model(rho, vp, vs):
    """lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2 on the GPU; (nx, nz)
    planes, float32 or float64."""
    d = np.asarray(rho).dtype if np.asarray(rho).dtype == np.float64 else F32
    rho, vp, vs = (np.ascontiguousarray(a, d) for a in (rho, vp, vs))
    nx, nz = rho.shape
    lam, mu = np.zeros_like(rho), np.zeros_like(rho)
    fn = load().rtm_velocity_model_d_ if d == np.float64 else load().rtm_velocity_model_c_
    check(fn(nz, nx, ptr(rho), ptr(vp), ptr(vs), ptr(lam), ptr(mu)))
    return lam, mu


def velocity_jacobian(adj, rho, vp, vs, a, b, c):
    """adj=True: Lame images (drho, dlambda, dmu) -> velocity images (drho,
    dvp, dvs); adj=False: velocity perturbations -> Lame perturbations."""
    d = np.asarray(rho).dtype if np.asarray(rho).dtype == np.float64 else F32
    ins = [np.ascontiguousarray(x, d) for x in (rho, vp, vs, a, b, c)]
    nx, nz = ins[0].shape
    out = [np.zeros_like(ins[0]) for _ in range(3)]
    fn = load().rtm_velocity_jacobian_d_ if d == np.float64 else load().rtm_velocity_jacobian_c_
    check(fn(1 if adj else 0, nz, nx, *[ptr(x) for x in ins], *[ptr(o) for o in out]))
    return out
