"""ctypes front end for the C oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker.  The product never imports it.

Array conventions mirror the Fortran memory layout with C-ordered numpy
arrays: a wavefield history (nz,nx,nt) column-major is ``H[it, ix, iz]``; a
model plane (nz,nx) is ``M[ix, iz]``; receiver data (nt,nx) is ``D[ix, it]``.
Grid indices passed to the C functions (zsrc, xsrc, zrec) are 1-based as in
the Fortran.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "librefc.so")
REF90_PATH = os.path.join(HERE, "_ref", "libref90.so")
REF_ROOT = os.environ.get("REFERENCE_ROOT", "/root/reference")
# unmodified copy of the reference's source files of this path (make stage)
STAGED_ROOT = os.path.join(os.path.dirname(HERE), "baseline", "_ref")

_lib = None
_ref = None
_ref90 = None


def ref_root():
    """The reference tree, else its staged copy in baseline/_ref, else None."""
    for r in (REF_ROOT, STAGED_ROOT):
        if os.path.isdir(os.path.join(r, "2d_rtm_restart", "Src_working")):
            return r
    return None


def build(ref=False):
    """Compile liboracle.so (and, when the reference's sources exist, _ref).
    Where the reference tree exists its sources are also staged into
    baseline/_ref for machines that lack it."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref and os.path.isdir(REF_ROOT):
        subprocess.run(["make", "-s", "-C", HERE, "stage", "REFROOT=" + REF_ROOT], check=True)
    root = ref_root() if ref else None
    if root:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REFROOT=" + os.path.abspath(root)], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def ref_available():
    return os.path.exists(REF_PATH) or ref_root() is not None


def ref90_available():
    return os.path.exists(REF90_PATH) or ref_root() is not None


def ref():
    """The reference's own rtmlib-modC.c compiled CPU-only (see Makefile)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            build(ref=True)
        _ref = ctypes.CDLL(REF_PATH)
    return _ref


def _p(a):
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)


def _sfx(dtype):
    return "_d" if np.dtype(dtype) == np.float64 else "_f"


def _R(dtype):
    return ctypes.c_double if np.dtype(dtype) == np.float64 else ctypes.c_float


# ------------------------------------------------------------------ a1..a4
def model_op(rho, lam, mu):
    """model_op: returns (m1_x, m1_z, lambda_avg, mu_avg)."""
    dt = rho.dtype
    nx, nz = rho.shape
    m2, m3 = lam.copy(), mu.copy()
    m1x, m1z = np.zeros_like(rho), np.zeros_like(rho)
    getattr(lib(), "ora_model_op" + _sfx(dt))(nz, nx, _p(rho), _p(m2), _p(m3), _p(m1x), _p(m1z))
    return m1x, m1z, m2, m3


def rtmmod_init(m1x, m1z, m2, m3, dx, dt):
    """Scale m1_x, m1_z by dt/dx; return (m1_x, m1_z, aux_m2, aux_m3, aux_m2m3)."""
    d = m1x.dtype
    nx, nz = m1x.shape
    m1x, m1z = m1x.copy(), m1z.copy()
    a2, a3, a23 = (np.zeros_like(m1x) for _ in range(3))
    R = _R(d)
    getattr(lib(), "ora_rtmmod_init" + _sfx(d))(nz, nx, R(dx), R(dt), _p(m1x), _p(m1z), _p(m2), _p(m3),
                                                _p(a2), _p(a3), _p(a23))
    return m1x, m1z, a2, a3, a23


def coefficients(rho, lam, mu, dx, dt):
    """model_op + rtmmod_init: the five scaled coefficient planes."""
    m1x, m1z, m2, m3 = model_op(rho, lam, mu)
    return rtmmod_init(m1x, m1z, m2, m3, dx, dt)


def source_op2(nt, dt, fp, nsource=250, dtype=np.float32):
    s = np.zeros(nt, dtype)
    R = _R(dtype)
    getattr(lib(), "ora_source_op2" + _sfx(dtype))(nt, R(dt), R(fp), nsource, _p(s))
    return s


def abc_init(abc, dtype=np.float32):
    f = np.zeros(abc + 5, dtype)
    getattr(lib(), "ora_abc_init" + _sfx(dtype))(abc, _p(f))
    return f


def K(data, abc, filt):
    d = data.copy()
    nx, nz = d.shape
    getattr(lib(), "ora_K" + _sfx(d.dtype))(nz, nx, abc, _p(filt), _p(d))
    return d


# ------------------------------------------------------------------ a6..a13
def forward(coefs, nt, dt, zsrc, xsrc, source, abc, filt):
    """Source wavefield history: returns (Vx, Vz, sxx, szz, sxz), each [nt,nx,nz]."""
    m1x = coefs[0]
    d = m1x.dtype
    nx, nz = m1x.shape
    H = [np.zeros((nt, nx, nz), d) for _ in range(5)]
    getattr(lib(), "ora_forward" + _sfx(d))(nz, nx, nt, _R(d)(dt), zsrc, xsrc, _p(source), abc, _p(filt),
                                            *[_p(c) for c in coefs], *[_p(h) for h in H])
    return H


def image_init(Vx, Vz, dx, dt):
    d = Vx.dtype
    nt, nx, nz = Vx.shape
    S = [np.zeros_like(Vx) for _ in range(6)]
    R = _R(d)
    getattr(lib(), "ora_image_init" + _sfx(d))(nz, nx, nt, R(dx), R(dt), _p(Vx), _p(Vz), *[_p(s) for s in S])
    return S


def model_delta(dm1, dm2, dm3):
    d = dm1.dtype
    nx, nz = dm1.shape
    dm2, dm3 = dm2.copy(), dm3.copy()
    t1, t2 = np.zeros_like(dm1), np.zeros_like(dm1)
    getattr(lib(), "ora_model_delta" + _sfx(d))(nz, nx, _p(dm1), _p(t1), _p(t2), _p(dm2), _p(dm3))
    return dm2, dm3


def image_adj(H, S):
    """Imaging condition: returns (dm1, dm2, dm3) from adjoint history H and S1..S6."""
    d = H[0].dtype
    nt, nx, nz = H[0].shape
    dm = [np.zeros((nx, nz), d) for _ in range(3)]
    H = [h.copy() for h in H]
    getattr(lib(), "ora_image_op2" + _sfx(d))(nz, nx, nt, 1, 0, *[_p(x) for x in dm], *[_p(h) for h in H],
                                              *[_p(s) for s in S])
    return dm


def image_fwd(dm1, dm2, dm3, S):
    """Born secondary sources: returns 5 histories."""
    d = dm1.dtype
    nt, nx, nz = S[0].shape
    H = [np.zeros((nt, nx, nz), d) for _ in range(5)]
    getattr(lib(), "ora_image_op2" + _sfx(d))(nz, nx, nt, 0, 0, _p(dm1), _p(dm2), _p(dm3), *[_p(h) for h in H],
                                              *[_p(s) for s in S])
    return H


def born_scatter(H, coefs, zrec, abc, filt):
    """Scattered propagation in place on H (5 histories); returns 5 gathers [nx,nt]."""
    d = H[0].dtype
    nt, nx, nz = H[0].shape
    D = [np.zeros((nx, nt), d) for _ in range(5)]
    getattr(lib(), "ora_born_scatter" + _sfx(d))(nz, nx, nt, zrec, abc, _p(filt), *[_p(c) for c in coefs],
                                                 *[_p(h) for h in H], *[_p(x) for x in D])
    return D


def rtm_op3_c(H, coefs):
    """The C gather recursion (restated) in place on 5 histories."""
    d = H[0].dtype
    nt, nx, nz = H[0].shape
    getattr(lib(), "ora_rtm_op3_c" + _sfx(d))(nt, nz, nx, *[_p(h) for h in H], *[_p(c) for c in coefs])
    return H


def rtm_op3(D, coefs, nz, zrec, exact=False, abc=0, filt=None):
    """rtm_op3: receivers D (5 gathers [nx,nt]) -> 5 adjoint histories."""
    d = D[0].dtype
    nx, nt = D[0].shape
    H = [np.zeros((nt, nx, nz), d) for _ in range(5)]
    if filt is None:
        filt = abc_init(abc, d)
    getattr(lib(), "ora_rtm_op3" + _sfx(d))(nt, nz, nx, zrec, *[_p(h) for h in H], *[_p(x) for x in D],
                                            *[_p(c) for c in coefs], int(exact), abc, _p(filt))
    return H


def rtm_op2(adj, rho, lam, mu, dm, D, dx, dt, nt, zsrc, xsrc, zrec, fp, abc, nsource=250, exact=False):
    """Whole rtm_op2.  adj=True: D (5 gathers [nx,nt]) -> image (dm1,dm2,dm3).
    adj=False: dm (3 planes) -> 5 gathers.  Returns (dm, D) after the call."""
    d = rho.dtype
    nx, nz = rho.shape
    R = _R(d)
    dm = [x.copy() for x in dm]
    D = [x.copy() for x in D]
    getattr(lib(), "ora_rtm_op2" + _sfx(d))(int(adj), nz, nx, nt, R(dx), R(dt), zsrc, xsrc, zrec, R(fp), nsource,
                                            abc, _p(rho), _p(lam), _p(mu), *[_p(x) for x in dm],
                                            *[_p(x) for x in D], int(exact))
    return dm, D


def rtm_lowmem(rho, lam, mu, D, dx, dt, nt, zsrc, xsrc, zrec, fp, abc, nsource=250, exact=False):
    """The RTM of rtm_op2(adj=True) holding 2 histories instead of 11 (see
    ora_rtm_lowmem): images (drho, dlambda, dmu) of the 5 gathers D [nx,nt].
    Same arithmetic per level; the imaging sums run backwards in time."""
    d = rho.dtype
    nx, nz = rho.shape
    R = _R(d)
    dm = [np.zeros((nx, nz), d) for _ in range(3)]
    D = [np.ascontiguousarray(x, d) for x in D]
    getattr(lib(), "ora_rtm_lowmem" + _sfx(d))(nz, nx, nt, R(dx), R(dt), zsrc, xsrc, zrec, R(fp), nsource, abc,
                                               _p(rho), _p(np.ascontiguousarray(lam, d)),
                                               _p(np.ascontiguousarray(mu, d)), *[_p(x) for x in dm],
                                               *[_p(x) for x in D], int(exact))
    return dm


# ------------------------------------------------------------------ reference C
def ref_rtm_op3_c(H, coefs, zrec=1):
    """Run the reference's own rtm_op3_c_ (CPU-only build) in place on float32 histories."""
    r = ref()
    nt, nx, nz = H[0].shape
    f = r.rtm_op3_c_
    f.restype = None
    f(ctypes.c_int(nt), ctypes.c_int(nz), ctypes.c_int(nx), ctypes.c_int(zrec), *[_p(h) for h in H],
      *[_p(c) for c in coefs])
    return H


# ------------------------------------------------------------------ reference Fortran (translated)
def ref90():
    """The reference's Fortran RTM modules translated to C (f90c.py), linked
    with its rtmlib-modC.c and driven like its main program (ref90_driver.c)."""
    global _ref90
    if _ref90 is None:
        if not os.path.exists(REF90_PATH):
            build(ref=True)
        _ref90 = ctypes.CDLL(REF90_PATH)
        _ref90.ref90_get.restype = ctypes.c_long
    return _ref90


REF90_STATE = ("rtm_mod_adj.m1_x", "rtm_mod_adj.m1_z", "rtm_mod_adj.aux_m2_c", "rtm_mod_adj.aux_m3_c",
               "rtm_mod_adj.aux_m2m3_c", "rtm_mod_adj.source", "abc_mod.filter", "image_mod_rtm.s1",
               "image_mod_rtm.s2", "image_mod_rtm.s3", "image_mod_rtm.s4", "image_mod_rtm.s5", "image_mod_rtm.s6")


def ref90_get(name, shape):
    r = ref90()
    out = np.zeros(shape, np.float32)
    n = r.ref90_get(name.encode(), _p(out), ctypes.c_long(out.size))
    if n != out.size:
        raise ValueError("%s holds %d values, %d expected" % (name, n, out.size))
    return out


def ref90_rtm(adj, rho, lam, mu, dm, D, dx, dt, nt, zsrc, xsrc, zrec, fp, abc, forward=False, state=()):
    """One rtm_init + rtm_op of the reference's own Fortran, as its main
    program calls them (rtm.f90:150-156), lame=.true., float32.

    adj=True: D (5 gathers [nx,nt]) -> images (drho, dlambda, dmu);
    adj=False: dm (3 planes [nx,nz]) -> 5 Born gathers.  Returns a dict with
    "dm", "D", the source-wavefield histories "fwd" ([nt,nx,nz] x5) when
    forward=True, and the module arrays named in `state` after the call."""
    r = ref90()
    nx, nz = rho.shape
    m = [np.array(x, np.float32, order="C") for x in (rho, lam, mu)]
    dm = [np.array(x, np.float32, order="C") for x in dm]
    D = [np.array(x, np.float32, order="C") for x in D]
    fwd = [np.zeros((nt, nx, nz), np.float32) for _ in range(5)] if forward else None
    arr = (ctypes.c_void_p * 5)(*[_p(f).value for f in fwd]) if forward else None
    F = ctypes.c_float
    st = r.ref90_rtm(int(adj), 1, nz, nx, nt, F(dx), F(dx), F(dt), xsrc, zsrc, zrec, F(fp), abc,
                     *[_p(x) for x in m], *[_p(x) for x in dm], *[_p(x) for x in D], arr)
    if st != 0:
        raise RuntimeError("reference rtm_op returned %d" % st)
    out = {"dm": dm, "D": D, "fwd": fwd}
    for name in state:
        if name.startswith("image_mod_rtm.s"):
            shape = (nt, nx, nz)
        elif name == "rtm_mod_adj.source":
            shape = (nt,)
        elif name == "abc_mod.filter":
            shape = (abc + 5,)
        else:
            shape = (nx, nz)
        out[name] = ref90_get(name, shape)
    return out


def ref90_image(adj, lame, m, Vx0, Vz0, dx, dt, dm=None, H=None):
    """The reference's image_init (+ image_init2 for lame=False) and
    image_op2 (W/image-mod-rtm.f90:26-225), float32.  m = (m1, m2, m3)
    planes [nx,nz] (rho, lambda, mu or rho, vp, vs); Vx0, Vz0 source
    histories [nt,nx,nz].  adj=True: H (5 histories) -> images (dm1, dm2,
    dm3); adj=False: dm -> 5 histories of Born secondary sources."""
    r = ref90()
    nt, nx, nz = Vx0.shape
    m = [np.array(x, np.float32, order="C") for x in m]
    V = [np.array(x, np.float32, order="C") for x in (Vx0, Vz0)]
    dm = [np.zeros((nx, nz), np.float32) for _ in range(3)] if dm is None else [np.array(x, np.float32) for x in dm]
    H = [np.zeros((nt, nx, nz), np.float32) for _ in range(5)] if H is None else [np.array(x, np.float32) for x in H]
    F = ctypes.c_float
    r.ref90_image(int(adj), int(lame), nz, nx, nt, F(dx), F(dt), _p(V[0]), _p(V[1]), *[_p(x) for x in m],
                  *[_p(x) for x in dm], *[_p(x) for x in H])
    return dm if adj else H


# ------------------------------------------------------------------ 3D acoustic
def acoustic_coeffs(d1, d2, d3):
    c = np.zeros(16, np.float32)
    lib().ora3d_coeffs(ctypes.c_double(d1), ctypes.c_double(d2), ctypes.c_double(d3), _p(c))
    return c


def acoustic_damp_table(a, b):
    t = np.zeros(max(a, 1), np.float32)
    if a > 0:
        lib().ora3d_damp_table(a, ctypes.c_float(b), _p(t))
    return t


def acoustic_forward(vel2, coef, damp_a, table, src_pos, wavelet, zr, record=True):
    """vel2 [n3,n2,n1] (v^2 dt^2).  Returns (d [nt,n3,n2] or None, p0, p1)."""
    n3, n2, n1 = vel2.shape
    nt = wavelet.shape[0]
    p0 = np.zeros_like(vel2)
    p1 = np.zeros_like(vel2)
    d = np.zeros((nt, n3, n2), np.float32) if record else None
    zs, xs, ys = src_pos
    lib().ora3d_forward(n1, n2, n3, nt, _p(vel2), _p(coef), damp_a, _p(table), zs, xs, ys, _p(wavelet),
                        ctypes.c_float(1.0), zr, _p(d) if record else None, _p(p0), _p(p1))
    return d, p0, p1


def acoustic_rtm(vel2, coef, damp_a, table, src_pos, wavelet, zr, d, jt):
    n3, n2, n1 = vel2.shape
    nt = wavelet.shape[0]
    img = np.zeros_like(vel2)
    zs, xs, ys = src_pos
    lib().ora3d_rtm(n1, n2, n3, nt, jt, _p(vel2), _p(coef), damp_a, _p(table), zs, xs, ys, _p(wavelet), zr,
                    _p(np.ascontiguousarray(d)), _p(img))
    return img


def acoustic_forward_history(vel2, coef, src_pos, wavelet):
    n3, n2, n1 = vel2.shape
    nt = wavelet.shape[0]
    h = np.zeros((nt, n3, n2, n1), np.float32)
    zs, xs, ys = src_pos
    lib().ora3d_forward_history(n1, n2, n3, nt, _p(vel2), _p(coef), _p(wavelet), zs, xs, ys, _p(h))
    return h


def acoustic_rtm_stored(vel2, coef, damp_a, table, hist, zr, d, jt):
    n3, n2, n1 = vel2.shape
    nt = hist.shape[0]
    img = np.zeros_like(vel2)
    lib().ora3d_rtm_stored(n1, n2, n3, nt, jt, _p(vel2), _p(coef), damp_a, _p(table), _p(np.ascontiguousarray(hist)),
                           zr, _p(np.ascontiguousarray(d)), _p(img))
    return img


# ------------------------------------------------ 3D elastic kernel test (K3)
K3_FIELDS = ("vy", "vx", "vz", "syy", "sxx", "szz", "sxy", "sxz", "syz")
K3_COEFS = ("m1y", "m1x", "m1z", "m2", "m3", "m2m3")


def _pp(arrs):
    P = ctypes.c_void_p * len(arrs)
    return P(*[a.ctypes.data_as(ctypes.c_void_p) for a in arrs])


def k3_step(inp, in1, out, m):
    """One step of the reference's 3D elastic kernel test
    (kernel_3d_test/rtmlib-modC.c:277-590) in float32: inp, in1, out lists
    of nine padded (ny+10, nx+10, nz+10) arrays (Vy, Vx, Vz, syy, sxx, szz,
    sxy, sxz, syz), m six (m1y, m1x, m1z, m2, m3, m2m3).  out is updated in
    place and returned."""
    L = lib()
    ny, nx, nz = (d - 10 for d in out[0].shape)
    for a in list(inp) + list(in1) + list(out) + list(m):
        assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and a.shape == out[0].shape
    L.ora_k3_step(ctypes.c_int(ny), ctypes.c_int(nz), ctypes.c_int(nx), _pp(inp), _pp(in1), _pp(out), _pp(m))
    return out


def k3_table():
    n = np.zeros(9, np.int32)
    t = np.zeros(9 * 5 * 4, np.int32)
    lib().ora_k3_table(_p(n), _p(t))
    return n, t.reshape(9, 5, 4)


K3_CHECK = os.path.join(HERE, "_ref", "k3_check_oracle")


def k3_reference_check(binary=K3_CHECK, plant=False, timeout=600):
    """Run the reference's own 3D elastic kernel test main (random 200^3
    fields, the hand-off, its CPU step, func_check at 1e-13) with the
    hand-off served by `binary`'s implementation; returns its stderr."""
    env = dict(os.environ)
    if plant:
        env["K3_PLANT"] = "1"
    r = subprocess.run([binary], capture_output=True, text=True, env=env, timeout=timeout)
    return r.stderr


# ------------------------------------------------------------------ PML Born modelling (working_Src)
REFPML_PATH = os.path.join(HERE, "_ref", "librefpml.so")
_refpml = None
PML_SEIS = ("Vx", "Vz", "P", "Vx_b", "Vz_b", "P_b")


def pml_params(nz, nx, dx, Tt, fp=25.0, dtseis=0.002):
    """nt, dt, nsource and nseis as the reference's main program derives them
    (working_Src/born.f90:67-73, 251, 255): dt = 0.2 dx / (sqrt(2) 2000)."""
    F = np.float32
    dt = F(F(F(0.2) * F(dx)) / F(F(np.sqrt(F(2.0))) * F(2000.0)))
    nseis = int(F(F(Tt) / F(dtseis)) + F(1))
    nt = int(F(F(Tt) / dt))
    x = F(F(F(F(np.sqrt(F(6.0))) / F(3.14159265)) / F(fp)) / dt)
    nsource = 4 * int(np.floor(x + 0.5))  # NINT: halves away from zero
    return {"nt": nt, "dt": float(dt), "nsource": nsource, "nseis": nseis}


def refpml_available():
    return os.path.exists(REFPML_PATH) or ref_root() is not None


def refpml():
    """The reference's PML Born modules translated to C (f90c.py --set pml),
    driven like its main program (refpml_driver.c)."""
    global _refpml
    if _refpml is None:
        if not os.path.exists(REFPML_PATH):
            build(ref=True)
        _refpml = ctypes.CDLL(REFPML_PATH)
    return _refpml


def _pml_call(fn, vp0, vs0, rho0, dvp, dvs, drho, dx, dt, nt, xsource, zsource, nsource, fp, nsnap, nseis, abc,
              zrec, free_surface, lame):
    nx, nz = vp0.shape
    m = [np.array(x, np.float32, order="C") for x in (vp0, vs0, rho0, dvp, dvs, drho)]
    seis = [np.zeros((nx - 2 * abc, nseis), np.float32) for _ in range(6)]
    snap = [np.zeros((nsnap, nx, nz), np.float32) for _ in range(6)]
    S = (ctypes.c_void_p * 6)(*[_p(a).value for a in seis])
    C = (ctypes.c_void_p * 6)(*[_p(a).value for a in snap])
    F = ctypes.c_float
    st = fn(nz, nx, nt, F(dx), F(dt), xsource, zsource, nsource, F(fp), nsnap, nseis, abc, zrec, int(free_surface),
            int(lame), *[_p(x) for x in m], S, C)
    return st, seis, snap


def refpml_born(vp0, vs0, rho0, dvp, dvs, drho, dx, dt, nt, xsource, zsource, nsource, fp, nsnap, nseis, abc, zrec,
                free_surface=False, lame=False):
    """elastic_init + elastic_op of the reference's PML Born modelling
    program (working_Src/born.f90:282-293), float32.  Model planes [nx, nz];
    grid indices 1-based.  Returns (seis, snap): six receiver lines
    [nx-2abc, nseis] (Vx, Vz, P, then the scattered Vx_b, Vz_b, P_b) and six
    snapshot cubes [nsnap, nx, nz]."""
    st, seis, snap = _pml_call(refpml().refpml_born, vp0, vs0, rho0, dvp, dvs, drho, dx, dt, nt, xsource, zsource,
                               nsource, fp, nsnap, nseis, abc, zrec, free_surface, lame)
    if st != 0:
        raise RuntimeError("reference elastic_op returned %d" % st)
    return seis, snap


def pml_born(vp0, vs0, rho0, dvp, dvs, drho, dx, dt, nt, xsource, zsource, nsource, fp, nsnap, nseis, abc, zrec,
             free_surface=False, lame=False):
    """The oracle's restatement of the same program (pml2d.c); same
    arguments and results as refpml_born."""
    L = lib()
    L.ora_pml_born.restype = None
    _, seis, snap = _pml_call(L.ora_pml_born, vp0, vs0, rho0, dvp, dvs, drho, dx, dt, nt, xsource, zsource, nsource,
                              fp, nsnap, nseis, abc, zrec, free_surface, lame)
    return seis, snap


def pml_model(vp0, vs0, rho0, dvp, dvs, drho, dx, dt, lame=False):
    """The program's model set-up (born-mod.f90:331-389): rho_Vx, rho_Vz, l,
    mi, l2mi, dl, dmi, dl2mi, drho_Vx, drho_Vz as [nx, nz] planes."""
    nx, nz = vp0.shape
    m = [np.array(x, np.float32, order="C") for x in (vp0, vs0, rho0, dvp, dvs, drho)]
    C = [np.zeros((nx, nz), np.float32) for _ in range(10)]
    Cp = (ctypes.c_void_p * 10)(*[_p(a).value for a in C])
    lib().ora_pml_model(nz, nx, ctypes.c_float(dx), ctypes.c_float(dt), int(lame), *[_p(x) for x in m], Cp)
    return C


PML_TABLES = ("pml0_xl", "pml0_xr", "pml1_xl", "pml1_xr", "pml0_zt", "pml0_zb", "pml1_zt", "pml1_zb")


def pml_tables(vp0, dx, dt, abc, free_surface=False):
    """The oracle's PML factor tables (pml-mod.f90:23-89) in PML_TABLES
    order: x tables [abc, nz], z tables [nx, abc] (Fortran (nz, abc) and
    (abc, nx))."""
    nx, nz = vp0.shape
    vp = np.ascontiguousarray(vp0, np.float32)
    out = [np.zeros((abc, nz), np.float32) for _ in range(4)] + [np.zeros((nx, abc), np.float32) for _ in range(4)]
    P = (ctypes.c_void_p * 8)(*[_p(a).value for a in out])
    lib().ora_pml_tables(nz, nx, ctypes.c_float(dx), ctypes.c_float(dt), abc, _p(vp), int(free_surface), P)
    return out


def refpml_get(name, shape):
    """A module array of the translated reference after a refpml_born call."""
    r = refpml()
    r.refpml_get.restype = ctypes.c_long
    out = np.zeros(shape, np.float32)
    n = r.refpml_get(name.encode(), _p(out), ctypes.c_long(out.size))
    if n != out.size:
        raise ValueError("%s holds %d values, %d expected" % (name, n, out.size))
    return out
