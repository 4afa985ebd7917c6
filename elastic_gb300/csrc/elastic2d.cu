// Host orchestration and C-ABI of the 2D elastic path (see
// include/elastic_rtm.h for the contract of every entry point).
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <type_traits>
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "../../include/elastic_rtm.h"
#include "elastic2d.cuh"
#include "elastic2d_aux.cuh"
#include "elastic2d_v2.cuh"
#include "engine.h"

using namespace eg;

// ------------------------------------------------------------------ errors
static thread_local char g_err[1024] = "";
static thread_local int g_last_status = 0;
static int g_exact = 1;

void rtm_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}
extern "C" const char *rtm_last_error(void) { return g_err; }
extern "C" int rtm_last_status(void) { return g_last_status; }
// status of a void drop-in entry point (read back by rtm_last_status); a
// failure is also reported on stderr, the void entry points' only channel
void rtm_set_status(int s, const char *where)
{
    g_last_status = s;
    if (s) fprintf(stderr, "%s: %s\n", where, g_err);
}
extern "C" void rtm_set_exact(int exact) { g_exact = exact ? 1 : 0; }
static int g_kernel_version = 0;
extern "C" void rtm_set_kernel_version(int v) { g_kernel_version = (v == 1 || v == 2) ? v : 0; }
int eg::kernel_version() { return g_kernel_version; }

namespace eg {

int ensure_device()
{
    static int dev = -1;
    if (dev < 0) {
        const char *s = getenv("ELASTIC_RTM_DEVICE");
        dev = s ? atoi(s) : 0;
    }
    RTM_CUDA(cudaSetDevice(dev));
    return RTM_OK;
}

int device_sm_count()
{
    static int nsm[RTM_MAX_DEVICES] = {};
    const int dev = rtm_current_device();
    std::lock_guard<std::mutex> lk(rtm_device_state_lock());
    if (!nsm[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        nsm[dev] = v > 0 ? v : 1;
    }
    return nsm[dev];
}

// ------------------------------------------------------------ step launch
template <typename T, bool EXACT, bool ADJ, int TX>
static int launch_step_tx(const Step2DArgs<T> &a, int grid_cap, cudaStream_t st)
{
    auto kern = k_step2d<T, EXACT, ADJ, TZ_TILE, TX>;
    const bool img = ADJ && a.img[0] != nullptr;
    const size_t smem = step2d_smem<T, EXACT, ADJ, TZ_TILE, TX>(img);
    static int grid_max[RTM_MAX_DEVICES][2] = {};
    const int dev = rtm_current_device();
    const int nsm = device_sm_count();
    int gm;
    {
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!grid_max[dev][img]) {
            const size_t smax = step2d_smem<T, EXACT, ADJ, TZ_TILE, TX>(true);
            RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax));
            int nb = 0;
            RTM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 256, smem));
            grid_max[dev][img] = (nb > 0 ? nb : 1) * nsm;
        }
        gm = grid_max[dev][img];
    }
    int grid = a.ntiles < gm ? a.ntiles : gm;
    if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
    if (grid <= 0) return RTM_OK;
    kern<<<grid, 256, smem, st>>>(a);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

template <typename T, bool EXACT, bool ADJ>
static int launch_step_e(const Step2DArgs<T> &a, int tx, int grid_cap, cudaStream_t st)
{
    switch (tx) {
    case 8: return launch_step_tx<T, EXACT, ADJ, 8>(a, grid_cap, st);
    case 16: return launch_step_tx<T, EXACT, ADJ, 16>(a, grid_cap, st);
    case 32: return launch_step_tx<T, EXACT, ADJ, 32>(a, grid_cap, st);
    default: rtm_set_error("unsupported tile width %d", tx); return RTM_ERR_ARG;
    }
}

int max_smem_optin()
{
    static int optin[RTM_MAX_DEVICES] = {};
    const int dev = rtm_current_device();
    std::lock_guard<std::mutex> lk(rtm_device_state_lock());
    if (!optin[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        optin[dev] = v > 0 ? v : 48 * 1024;
    }
    return optin[dev];
}

template <int TX>
static size_t v2_bytes_tx(bool adj, bool exact)
{
    if (adj) return exact ? v2_smem<true, true, TX>(true) : v2_smem<true, false, TX>(true);
    return exact ? v2_smem<false, true, TX>(false) : v2_smem<false, false, TX>(false);
}

size_t v2_stage_bytes(bool adj, bool exact, int tx)
{
    switch (tx) {
    case 8: return v2_bytes_tx<8>(adj, exact);
    case 16: return v2_bytes_tx<16>(adj, exact);
    case 32: return v2_bytes_tx<32>(adj, exact);
    default: return 0;
    }
}

bool v2_fits(bool adj, bool exact, int tx) { return v2_fits(adj, exact, tx, 1); }

bool v2_threads_ok(bool exact, int tx, int threads)
{
    return threads == 256 || (threads == 512 && !exact && tx >= 16);
}

bool v2_fits(bool adj, bool exact, int tx, int stages, int threads)
{
    if (stages < 1 || stages > 2 || !v2_threads_ok(exact, tx, threads)) return false;
    const size_t b = v2_stage_bytes(adj, exact, tx);
    return b > 0 && (size_t)stages * b + V2_SMEM_EXTRA <= (size_t)max_smem_optin();
}

template <bool EXACT, bool ADJ, int TX>
static int launch_v2_tx(const Step2DArgs<float> &a, int grid_cap, cudaStream_t st, int stages, int threads)
{
    auto kern = k_step2d_v2<EXACT, ADJ, TX>;
    const bool img = ADJ && a.img[0] != nullptr;
    RTM_CHECK_ARG(v2_fits(ADJ, EXACT, TX, stages, threads),
                  "tile width %d with %d stages and %d threads does not fit in a block", TX, stages, threads);
    const size_t smem = (size_t)stages * v2_smem<ADJ, EXACT, TX>(img) + V2_SMEM_EXTRA;
    static bool attr_set[RTM_MAX_DEVICES] = {};
    static int grid_max[RTM_MAX_DEVICES][2][2][2] = {};
    const int dev = rtm_current_device();
    const int optin = max_smem_optin();
    const int nsm = device_sm_count();
    int gm;
    {
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!attr_set[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
            attr_set[dev] = true;
        }
        int &g = grid_max[dev][img][stages - 1][threads == 512];
        if (!g) {
            int nb = 0;
            RTM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem));
            g = (nb > 0 ? nb : 1) * nsm;
        }
        gm = g;
    }
    int grid = a.ntiles < gm ? a.ntiles : gm;
    if (grid_cap > 0 && grid > grid_cap) grid = grid_cap;
    if (grid <= 0) return RTM_OK;
    kern<<<grid, threads, smem, st>>>(a);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

template <bool EXACT, bool ADJ>
static int launch_v2(const Step2DArgs<float> &a, int tx, int grid_cap, cudaStream_t st, int stages, int threads)
{
    switch (tx) {
    case 8: return launch_v2_tx<EXACT, ADJ, 8>(a, grid_cap, st, stages, threads);
    case 16: return launch_v2_tx<EXACT, ADJ, 16>(a, grid_cap, st, stages, threads);
    case 32: return launch_v2_tx<EXACT, ADJ, 32>(a, grid_cap, st, stages, threads);
    default: rtm_set_error("unsupported tile width %d", tx); return RTM_ERR_ARG;
    }
}

// v2 needs float planes whose columns start on 16-byte boundaries.
static bool v2_layout_ok(const Step2DArgs<float> &a)
{
    if (a.ldz % 4) return false;
    auto al = [](const void *p) { return ((uintptr_t)p & 15u) == 0; };
    for (int f = 0; f < 5; f++) {
        if (!al(a.out[f]) || !al(a.own2[f]) || !al(a.nb[f]) || !al(a.coef[f])) return false;
        if (a.inplane[f] && !al(a.inplane[f])) return false;
    }
    return true;
}

bool v2_usable(bool is_float, int ldz, const void *const *ptrs, int n)
{
    if (!is_float || kernel_version() == 1 || ldz % 4) return false;
    for (int i = 0; i < n; i++)
        if (ptrs[i] && ((uintptr_t)ptrs[i] & 15u)) return false;
    return true;
}

template <typename T>
int launch_step(const Step2DArgs<T> &a, bool adj, bool exact, int tx, int grid_cap, cudaStream_t st, int tz, int stages,
                int threads)
{
    if constexpr (std::is_same<T, float>::value) {
        if (tz == TZ_TILE2) {
            if (!v2_layout_ok(a)) {
                rtm_set_error("v2 step launched on an unaligned layout");
                return RTM_ERR_ARG;
            }
            if (adj)
                return exact ? launch_v2<true, true>(a, tx, grid_cap, st, stages, threads)
                             : launch_v2<false, true>(a, tx, grid_cap, st, stages, threads);
            return exact ? launch_v2<true, false>(a, tx, grid_cap, st, stages, threads)
                         : launch_v2<false, false>(a, tx, grid_cap, st, stages, threads);
        }
    }
    if (adj) return exact ? launch_step_e<T, true, true>(a, tx, grid_cap, st) : launch_step_e<T, false, true>(a, tx, grid_cap, st);
    return exact ? launch_step_e<T, true, false>(a, tx, grid_cap, st) : launch_step_e<T, false, false>(a, tx, grid_cap, st);
}
template int launch_step<float>(const Step2DArgs<float> &, bool, bool, int, int, cudaStream_t, int, int, int);
template int launch_step<double>(const Step2DArgs<double> &, bool, bool, int, int, cudaStream_t, int, int, int);

// ------------------------------------------------------------- batch table
int ShotTable::build(int tx_, int tz_)
{
    tx = tx_;
    tz = tz_;
    std::vector<ShotGeom> g(shots.size());
    int t = 0;
    for (size_t s = 0; s < shots.size(); s++) {
        const HostShot &h = shots[s];
        g[s].off = h.off;
        g[s].doff = h.doff;
        g[s].nz = h.nz;
        g[s].nx = h.nx;
        g[s].src_iz = h.src_iz;
        g[s].src_ix = h.src_ix;
        g[s].rec_iz = h.rec_iz;
        g[s].tile0 = t;
        g[s].ntz = ceil_div(h.nz, tz);
        g[s].pad = 0;
        t += g[s].ntz * ceil_div(h.nx, tx);
    }
    ntiles = t;
    if (d_geom) cudaFree(d_geom);
    d_geom = nullptr;
    RTM_CUDA(cudaMalloc(&d_geom, g.size() * sizeof(ShotGeom)));
    RTM_CUDA(cudaMemcpy(d_geom, g.data(), g.size() * sizeof(ShotGeom), cudaMemcpyHostToDevice));
    return RTM_OK;
}

ShotTable::~ShotTable()
{
    if (d_geom) cudaFree(d_geom);
}

// ---------------------------------------------------------- model set-up
template <typename T>
int model_coefs(int nz, int nx, T dx, T dt, const T *d_rho, const T *d_lam, const T *d_mu, int ldin, T *m1x, T *m1z,
                T *m2o, T *m3o, T *a2, T *a3, T *a23, int ldout, cudaStream_t st)
{
    const T aux = dt / dx;
    RTM_CHECK_ARG(nz > 0 && nx > 0 && nx <= 65535, "model_coefs: bad grid %d x %d", nz, nx);
    dim3 b(128), g(ceil_div(nz, 128), nx);
    k_model_coef<T><<<g, b, 0, st>>>(nz, nx, d_rho, d_lam, d_mu, ldin, aux, m1x, m1z, m2o, m3o, a2, a3, a23, ldout);
    {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            rtm_set_error("k_model_coef launch (grid %u x %u, stream %p): %s", g.x, g.y, (void *)st,
                          cudaGetErrorString(e));
            return RTM_ERR_CUDA;
        }
    }
    return RTM_OK;
}
template int model_coefs<float>(int, int, float, float, const float *, const float *, const float *, int, float *,
                                float *, float *, float *, float *, float *, float *, int, cudaStream_t);
template int model_coefs<double>(int, int, double, double, const double *, const double *, const double *, int,
                                 double *, double *, double *, double *, double *, double *, double *, int,
                                 cudaStream_t);

template <typename T>
int mask_coefs(int nz, int nx, const T *const in[5], int ldin, T *const out[5], int ldout, cudaStream_t st)
{
    dim3 b(128), g(ceil_div(nz, 128), nx);
    k_mask_coef<T><<<g, b, 0, st>>>(nz, nx, in[0], in[1], in[2], in[3], in[4], ldin, out[0], out[1], out[2], out[3],
                                    out[4], ldout);
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}
template int mask_coefs<float>(int, int, const float *const[5], int, float *const[5], int, cudaStream_t);
template int mask_coefs<double>(int, int, const double *const[5], int, double *const[5], int, cudaStream_t);

// Host tables shared with the reference semantics (computed with the host
// libm, as the reference's Fortran does on the host).
template <typename T>
void host_abc_filter(int abc, T *filter)
{
    const int abc2 = abc + 5;
    if (abc <= 0) {
        for (int i = 0; i < abc2; i++) filter[i] = T(1);
        return;
    }
    const T alfa = T(0.09);
    for (int ix = 1; ix <= abc; ix++) {
        const T aux = (T(1) * T(ix)) / (T(1) * T(abc));
        const T arg = (-alfa * aux) * aux;
        filter[ix - 1] = sizeof(T) == 4 ? (T)expf((float)arg) : (T)exp((double)arg);
    }
    for (int ix = abc + 1; ix <= abc2; ix++) filter[ix - 1] = filter[abc - 1];
}
template void host_abc_filter<float>(int, float *);
template void host_abc_filter<double>(int, double *);

template <typename T>
void host_ricker(int nt, T dt, T fp, int nsource, T *source)
{
    for (int it = 0; it < nt; it++) source[it] = T(0);
    const T pi = T(3.14159265);
    for (int it = nsource / 10; it <= nt; it++) {
        if (it < 1) continue;
        const T t = (T(it) * dt) - ((T(nsource) * dt) / T(2));
        const T aux = ((((pi * pi) * fp) * fp) * t) * t;
        const T e = sizeof(T) == 4 ? (T)expf((float)-aux) : (T)exp((double)-aux);
        source[it - 1] = (T(10.0e7) * (T(1) - T(2) * aux)) * e;
    }
}
template void host_ricker<float>(int, float, float, int, float *);
template void host_ricker<double>(int, double, double, int, double *);

}  // namespace eg

// =====================================================================
// Single-shot full-history pipeline (the reference's own decomposition).
// Every history is (nz,nx,nt) in the reference layout on the device.
// =====================================================================
namespace {

template <typename T>
struct Hist {
    int nz = 0, nx = 0, nt = 0;
    size_t plane = 0;
    cudaStream_t st = 0;
    bool exact = true;
    ShotTable tab;
    DevBuf<T> zero, cm, filt, coefraw;
    T *cmp[5] = {};  // masked coefficient planes (ld = nz)
    int abc2 = 5;

    int init(int nz_, int nx_, int nt_, bool exact_)
    {
        nz = nz_; nx = nx_; nt = nt_; exact = exact_;
        plane = (size_t)nz * nx;
        TRY(ensure_device());
        TRY(zero.alloc(plane));
        RTM_CUDA(cudaMemset(zero.p, 0, plane * sizeof(T)));
        tab.shots.assign(1, HostShot{0, 0, nz, nx, -1, -1, -1});
        tab.ldz = nz;
        // v2 when every level of every history starts on a 16-byte boundary
        // (cudaMalloc bases, plane = nz*nx floats)
        const bool v2 = kernel_version() != 1 && std::is_same<T, float>::value && nz % 4 == 0 && (plane % 4) == 0;
        const int tz = v2 ? TZ_TILE2 : TZ_TILE;
        int tx = pick_tile_width(nz, nx, tz);
        while (v2 && tx > 8 && !v2_fits(true, exact, tx)) tx /= 2;
        TRY(tab.build(tx, tz));
        return RTM_OK;
    }
    // coefficient planes (unmasked, device) -> masked planes
    int set_coefs_dev(T *const raw[5])
    {
        TRY(cm.alloc(5 * plane));
        for (int i = 0; i < 5; i++) cmp[i] = cm.p + i * plane;
        const T *in[5] = {raw[0], raw[1], raw[2], raw[3], raw[4]};
        return mask_coefs<T>(nz, nx, in, nz, cmp, nz, st);
    }
    int set_coefs_host(const T *const raw[5])
    {
        TRY(coefraw.alloc(5 * plane));
        T *r[5];
        for (int i = 0; i < 5; i++) {
            r[i] = coefraw.p + i * plane;
            RTM_CUDA(cudaMemcpy(r[i], raw[i], plane * sizeof(T), cudaMemcpyHostToDevice));
        }
        return set_coefs_dev(r);
    }
    int set_abc(int abc)
    {
        abc2 = abc + 5;
        RTM_CHECK_ARG(nz >= abc2 && nx >= abc2, "grid %dx%d smaller than the sponge strip abc+5=%d", nz, nx, abc2);
        std::vector<T> f(abc2);
        host_abc_filter<T>(abc, f.data());
        TRY(filt.alloc(abc2));
        RTM_CUDA(cudaMemcpy(filt.p, f.data(), abc2 * sizeof(T), cudaMemcpyHostToDevice));
        return RTM_OK;
    }
    Step2DArgs<T> args() const
    {
        Step2DArgs<T> a;
        memset(&a, 0, sizeof a);
        for (int i = 0; i < 5; i++) a.coef[i] = cmp[i];
        a.shots = tab.d_geom;
        a.nshots = 1;
        a.ntiles = tab.ntiles;
        a.ldz = nz;
        a.filt = filt.p;
        a.abc2 = abc2;
        return a;
    }
    T *lev(T *h, int L) const { return h + (size_t)(L - 1) * plane; }  // 1-based level
    int step(const Step2DArgs<T> &a, bool adj) { return launch_step<T>(a, adj, exact, tab.tx, 0, st, tab.tz); }

    // Source wavefield, W/rtm-mod-adj.f90:178-261.  src[] = dt*source(it).
    int forward(T *const H[5], const std::vector<T> &dtsrc, int zsrc0, int xsrc0)
    {
        for (int f = 0; f < 5; f++) RTM_CUDA(cudaMemsetAsync(H[f], 0, plane * nt * sizeof(T), st));
        ShotTable &tb = tab;
        tb.shots[0].src_iz = zsrc0;
        tb.shots[0].src_ix = xsrc0;
        TRY(tb.build(tb.tx, tb.tz));
        for (int L = 2; L <= nt; L++) {
            Step2DArgs<T> a = args();
            for (int f = 0; f < 5; f++) {
                a.out[f] = lev(H[f], L);
                a.own2[f] = L >= 3 ? lev(H[f], L - 2) : zero.p;
                a.nb[f] = lev(H[f], L - 1);
            }
            a.sponge = L >= 3;
            a.has_src = 1;
            a.srcval = dtsrc[L - 2];
            TRY(step(a, false));
        }
        tb.shots[0].src_iz = tb.shots[0].src_ix = -1;
        return tb.build(tb.tx, tb.tz);
    }

    // Nonlinear forward modelling (W/elastic-mod.f90:95-240, the same time
    // loop as the source wavefield): two rolling levels per field in B[f]
    // (2 planes each; level L in plane L & 1, written over level L-2 in
    // place) and the five components of row zrec0 of every level recorded
    // into rec ([it][5][nx], level 1 zero).
    int model(T *const B[5], const std::vector<T> &dtsrc, int zsrc0, int xsrc0, int zrec0, T *rec)
    {
        for (int f = 0; f < 5; f++) RTM_CUDA(cudaMemsetAsync(B[f], 0, 2 * plane * sizeof(T), st));
        RTM_CUDA(cudaMemsetAsync(rec, 0, (size_t)nt * 5 * nx * sizeof(T), st));
        tab.shots[0].src_iz = zsrc0;
        tab.shots[0].src_ix = xsrc0;
        tab.shots[0].rec_iz = zrec0;
        tab.shots[0].doff = 0;
        TRY(tab.build(tab.tx, tab.tz));
        for (int L = 2; L <= nt; L++) {
            Step2DArgs<T> a = args();
            for (int f = 0; f < 5; f++) {
                a.out[f] = B[f] + (L & 1) * plane;
                a.own2[f] = L >= 3 ? a.out[f] : zero.p;
                a.nb[f] = B[f] + ((L - 1) & 1) * plane;
            }
            a.sponge = L >= 3;
            a.has_src = 1;
            a.srcval = dtsrc[L - 2];
            a.rec = rec;
            a.comp_mask = 31;
            a.ncomp = 5;
            a.it = L - 1;
            TRY(step(a, false));
        }
        tab.shots[0].src_iz = tab.shots[0].src_ix = tab.shots[0].rec_iz = -1;
        return tab.build(tab.tx, tab.tz);
    }

    // Born scattered loop (W/rtm-mod-adj.f90:291-357) on histories already
    // holding the secondary sources; records five gathers at zrec0 into
    // rec ([it][5][nx] device) when rec != null.
    int born_scatter(T *const H[5], int zrec0, T *rec)
    {
        tab.shots[0].rec_iz = zrec0;
        tab.shots[0].doff = 0;
        TRY(tab.build(tab.tx, tab.tz));
        for (int L = 1; L <= nt; L++) {
            Step2DArgs<T> a = args();
            for (int f = 0; f < 5; f++) {
                a.out[f] = lev(H[f], L);
                a.inplane[f] = lev(H[f], L);
                a.own2[f] = L >= 3 ? lev(H[f], L - 2) : zero.p;
                a.nb[f] = L >= 2 ? lev(H[f], L - 1) : zero.p;
            }
            a.sponge = 1;
            a.rec = rec;
            a.comp_mask = 31;
            a.ncomp = 5;
            a.it = L - 1;
            TRY(step(a, false));
        }
        tab.shots[0].rec_iz = -1;
        return tab.build(tab.tx, tab.tz);
    }

    // rtm_op3 (W/rtmlib-mod.f90:72-196) + the C recursion: H holds the
    // receiver rows (all levels, zero elsewhere) on entry.
    int adjoint(T *const H[5], bool exact_adj)
    {
        if (exact_adj) TRY(sponge_level(H, nt));
        for (int L = nt - 1; L >= 1; L--) {
            Step2DArgs<T> a = args();
            for (int f = 0; f < 5; f++) {
                a.out[f] = lev(H[f], L);
                a.inplane[f] = lev(H[f], L);
                a.own2[f] = L + 2 <= nt ? lev(H[f], L + 2) : zero.p;
                a.nb[f] = lev(H[f], L + 1);
            }
            a.sponge = exact_adj;
            TRY(step(a, true));
        }
        return RTM_OK;
    }
    // K applied alone to one level (a zero stencil step with sponge).
    int sponge_level(T *const H[5], int L)
    {
        Step2DArgs<T> a = args();
        for (int f = 0; f < 5; f++) {
            a.out[f] = lev(H[f], L);
            a.own2[f] = lev(H[f], L);
            a.nb[f] = zero.p;
        }
        a.sponge = 1;
        return step(a, false);
    }
};

template <typename T>
__global__ void k_put_rows(int nt, int nx, int nz, int zrec0, const T *d0, const T *d1, const T *d2, const T *d3,
                           const T *d4, T *h0, T *h1, T *h2, T *h3, T *h4)
{
    // gathers (nt,nx) Fortran -> row zrec0 of every level
    const int it = blockIdx.x * blockDim.x + threadIdx.x, ix = blockIdx.y;
    if (it >= nt) return;
    const size_t d = (size_t)ix * nt + it, o = (size_t)it * nz * nx + (size_t)ix * nz + zrec0;
    h0[o] = d0[d]; h1[o] = d1[d]; h2[o] = d2[d]; h3[o] = d3[d]; h4[o] = d4[d];
}

template <typename T>
__global__ void k_gather_from_rec(int nt, int nx, const T *rec, T *g0, T *g1, T *g2, T *g3, T *g4)
{
    // device traces [it][5][nx] -> five (nt,nx) Fortran gathers
    const int it = blockIdx.x * blockDim.x + threadIdx.x, ix = blockIdx.y;
    if (it >= nt) return;
    const size_t d = (size_t)ix * nt + it, r = ((size_t)it * 5) * nx + ix;
    g0[d] = rec[r]; g1[d] = rec[r + nx]; g2[d] = rec[r + 2 * nx]; g3[d] = rec[r + 3 * nx]; g4[d] = rec[r + 4 * nx];
}

template <typename T>
int copy_h2d(T *d, const T *h, size_t n, cudaStream_t st) {
    RTM_CUDA(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return RTM_OK;
}
template <typename T>
int copy_d2h(T *h, const T *d, size_t n, cudaStream_t st) {
    RTM_CUDA(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, st));
    return RTM_OK;
}

// One shot of rtm_op2 (W/rtm-mod-adj.f90:132-496, lame=.true.) on the full
// grid, with the shot's source wavefield history resident on the device:
// born() is the Born operator (image_op2 forward, W/image-mod-rtm.f90:164-179,
// then the scattered loop and receiver sampling, :291-375) and adjoint() the
// RTM (rtm_op3 then image_op2 adjoint, W/image-mod-rtm.f90:146-162).  With
// exact_adj the adjoint is the exact transpose of born() (sponge applied in
// transposed order), which LSRTM needs.
template <typename T>
struct BornShot {
    Hist<T> h;
    DevBuf<T> S;  // source wavefield, 5 histories of nt levels
    int nz = 0, nx = 0, nt = 0, zrec0 = 0;
    int comp_mask = 31;  // recorded components (bit c: Vx, Vz, sxx, szz, sxz)
    size_t plane = 0, vol = 0;
    T inv_dt = 0, inv_dx = 0;

    // model: device planes rho, lambda, mu (raw, averaged here as model_op)
    int init(int nz_, int nx_, int nt_, T dx, T dt, int xsrc, int zsrc, int zrec, T fp, int nsource, int abc,
             const T *model, bool exact)
    {
        RTM_CHECK_ARG(nz_ >= 11 && nx_ >= 11 && nt_ >= 3, "grid too small (nz=%d nx=%d nt=%d)", nz_, nx_, nt_);
        RTM_CHECK_ARG(zsrc >= 1 && zsrc <= nz_ && xsrc >= 1 && xsrc <= nx_ && zrec >= 1 && zrec <= nz_,
                      "source/receiver position outside the grid");
        nz = nz_; nx = nx_; nt = nt_; zrec0 = zrec - 1;
        TRY(h.init(nz, nx, nt, exact));
        TRY(h.set_abc(abc));
        plane = h.plane;
        vol = plane * nt;
        DevBuf<T> raw;
        TRY(raw.alloc(5 * plane));
        T *r[5];
        for (int i = 0; i < 5; i++) r[i] = raw.p + i * plane;
        TRY(model_coefs<T>(nz, nx, dx, dt, model, model + plane, model + 2 * plane, nz, r[M1X], r[M1Z], nullptr,
                           nullptr, r[A2], r[A3], r[A23], nz, h.st));
        TRY(h.set_coefs_dev(r));
        // source wavelet scaled by dt (host, as the reference)
        std::vector<T> src(nt), dtsrc(nt);
        host_ricker<T>(nt, dt, fp, nsource, src.data());
        for (int i = 0; i < nt; i++) dtsrc[i] = dt * src[i];
        TRY(S.alloc(5 * vol));
        T *Sp[5];
        for (int f = 0; f < 5; f++) Sp[f] = S.p + f * vol;
        TRY(h.forward(Sp, dtsrc, zsrc - 1, xsrc - 1));
        inv_dt = T(1) / dt;
        inv_dx = T(1) / dx;
        return RTM_OK;
    }
    T *sv(int f) const { return S.p + f * vol; }
    size_t gather_size() const { return (size_t)nt * nx; }

    // data (5 gathers of (nt,nx) in Fortran order, device) = Born(dm1..dm3).
    // A: 5 work histories, rec: nt*5*nx work.
    int born(const T *dm1, const T *dm2, const T *dm3, T *const A[5], T *rec, T *data)
    {
        for (int L = 1; L <= nt; L++) {
            const size_t lv = (size_t)(L - 1) * plane, lv1 = L < nt ? lv + plane : lv;
            dim3 b(128), g(ceil_div(nz, 128), nx, 1);
            if (h.exact)
                k_born_src<true, T><<<g, b, 0, h.st>>>(h.tab.d_geom, nz, sv(VX) + lv, sv(VZ) + lv, sv(VX) + lv1,
                                                       sv(VZ) + lv1, L == nt, dm1, dm2, dm3, A[0] + lv, A[1] + lv,
                                                       A[2] + lv, A[3] + lv, A[4] + lv, 1, inv_dt, inv_dx);
            else
                k_born_src<false, T><<<g, b, 0, h.st>>>(h.tab.d_geom, nz, sv(VX) + lv, sv(VZ) + lv, sv(VX) + lv1,
                                                        sv(VZ) + lv1, L == nt, dm1, dm2, dm3, A[0] + lv, A[1] + lv,
                                                        A[2] + lv, A[3] + lv, A[4] + lv, 1, inv_dt, inv_dx);
            RTM_CUDA(cudaGetLastError());
        }
        TRY(h.born_scatter(A, zrec0, rec));
        dim3 b(128), gr(ceil_div(nt, 128), nx);
        const size_t gs = gather_size();
        k_gather_from_rec<T><<<gr, b, 0, h.st>>>(nt, nx, rec, data, data + gs, data + 2 * gs, data + 3 * gs,
                                                 data + 4 * gs);
        RTM_CUDA(cudaGetLastError());
        // components that are not recorded are zero (L := mask * L)
        return mask_data(data);
    }
    // zero the unrecorded components of device gathers in place
    int mask_data(T *data)
    {
        const size_t gs = gather_size();
        for (int c = 0; c < 5; c++)
            if (!(comp_mask & (1 << c))) RTM_CUDA(cudaMemsetAsync(data + c * gs, 0, gs * sizeof(T), h.st));
        return RTM_OK;
    }

    // img (3 planes, overwritten) = RTM(data); A: 5 work histories.
    int adjoint(const T *data, T *const A[5], T *img, bool exact_adj)
    {
        for (int f = 0; f < 5; f++) RTM_CUDA(cudaMemsetAsync(A[f], 0, vol * sizeof(T), h.st));
        const size_t gs = gather_size();
        dim3 b(128), gr(ceil_div(nt, 128), nx);
        k_put_rows<T><<<gr, b, 0, h.st>>>(nt, nx, nz, zrec0, data, data + gs, data + 2 * gs, data + 3 * gs,
                                          data + 4 * gs, A[0], A[1], A[2], A[3], A[4]);
        RTM_CUDA(cudaGetLastError());
        TRY(h.adjoint(A, exact_adj));
        dim3 gi(ceil_div(nz, 128), nx);
        k_image_hist<T><<<gi, b, 0, h.st>>>(nz, nx, nt, sv(VX), sv(VZ), A[0], A[1], A[2], A[3], A[4], img,
                                            img + plane, img + 2 * plane, inv_dt, inv_dx);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    }
};

// Whole rtm_op2 for one shot (W/rtm-mod-adj.f90:132-496), host arrays in
// and out.
template <typename T>
int rtm_op_impl(int adj, int nz, int nx, int nt, T dx, T dt, int xsrc, int zsrc, int zrec, T fp, int nsource,
                int abc, const T *rho, const T *lam, const T *mu, T *dm1, T *dm2, T *dm3, T *const D[5], int linear,
                int exact_adj, bool exact)
{
    RTM_CHECK_ARG(nz >= 11 && nx >= 11 && nt >= 3, "grid too small (nz=%d nx=%d nt=%d)", nz, nx, nt);
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx;
    DevBuf<T> model;
    TRY(model.alloc(3 * plane));
    RTM_CUDA(cudaMemcpy(model.p, rho, plane * sizeof(T), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(model.p + plane, lam, plane * sizeof(T), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(model.p + 2 * plane, mu, plane * sizeof(T), cudaMemcpyHostToDevice));
    BornShot<T> sh;
    TRY(sh.init(nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, model.p, exact));
    const size_t vol = sh.vol, gs = sh.gather_size();
    cudaStream_t st = sh.h.st;
    DevBuf<T> W, img, g;
    TRY(W.alloc(5 * vol));
    T *A[5];
    for (int f = 0; f < 5; f++) A[f] = W.p + f * vol;
    TRY(img.alloc(3 * plane));
    TRY(g.alloc(5 * gs));
    if (!adj) {
        // images in; Born
        TRY(copy_h2d(img.p, dm1, plane, st));
        TRY(copy_h2d(img.p + plane, dm2, plane, st));
        TRY(copy_h2d(img.p + 2 * plane, dm3, plane, st));
        T *i2 = img.p + plane, *i3 = img.p + 2 * plane;
        DevBuf<T> avg;
        if (!linear) {
            TRY(avg.alloc(2 * plane));
            dim3 b(128), gm(ceil_div(nz, 128), nx);
            k_model_delta<T><<<gm, b, 0, st>>>(nz, nx, i2, i3, nz, avg.p, avg.p + plane, nz);
            RTM_CUDA(cudaGetLastError());
            i2 = avg.p;
            i3 = avg.p + plane;
            // the reference averages dlambda/dmu in place
            TRY(copy_d2h(dm2, i2, plane, st));
            TRY(copy_d2h(dm3, i3, plane, st));
        }
        DevBuf<T> rec;
        TRY(rec.alloc((size_t)nt * 5 * nx));
        TRY(sh.born(img.p, i2, i3, A, rec.p, g.p));
        for (int c = 0; c < 5; c++) TRY(copy_d2h(D[c], g.p + c * gs, gs, st));
    } else {
        // gathers in; RTM
        for (int c = 0; c < 5; c++) TRY(copy_h2d(g.p + c * gs, D[c], gs, st));
        TRY(sh.adjoint(g.p, A, img.p, exact_adj != 0));
        TRY(copy_d2h(dm1, img.p, plane, st));
        TRY(copy_d2h(dm2, img.p + plane, plane, st));
        TRY(copy_d2h(dm3, img.p + 2 * plane, plane, st));
    }
    RTM_CUDA(cudaStreamSynchronize(st));
    return RTM_OK;
}

// ------------------------------------------------------------------ LSRTM
// Deterministic dot product in double: per-block partial sums, then one
// block adds the partials in order.
template <typename T>
__global__ void k_dot_partial(size_t n, const T *x, const T *y, double *part)
{
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        acc += (double)x[i] * (double)y[i];
    __shared__ double red[32];
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
        if (threadIdx.x == 0) part[blockIdx.x] = v;
    }
}
__global__ void k_sum_partials(int n, const double *part, double *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < n; i++) s += part[i];
        *out = s;
    }
}
// y += a * x
template <typename T>
__global__ void k_axpy(size_t n, T a, const T *x, T *y)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] += a * x[i];
}
// p = s + b * p
template <typename T>
__global__ void k_xpby(size_t n, const T *s, T b, T *p)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = s[i] + b * p[i];
}

constexpr int DOT_BLOCKS = 1024;

template <typename T>
struct Vec {
    cudaStream_t st = 0;
    DevBuf<double> part;
    int init(cudaStream_t s)
    {
        st = s;
        return part.alloc(DOT_BLOCKS + 1);
    }
    int grid(size_t n) const { return (int)std::min<size_t>(DOT_BLOCKS, std::max<size_t>(1, (n + 255) / 256)); }
    int dot(size_t n, const T *x, const T *y, double *out)
    {
        const int g = grid(n);
        k_dot_partial<T><<<g, 256, 0, st>>>(n, x, y, part.p);
        RTM_CUDA(cudaGetLastError());
        k_sum_partials<<<1, 32, 0, st>>>(g, part.p, part.p + DOT_BLOCKS);
        RTM_CUDA(cudaGetLastError());
        RTM_CUDA(cudaMemcpyAsync(out, part.p + DOT_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, st));
        RTM_CUDA(cudaStreamSynchronize(st));
        return RTM_OK;
    }
    int axpy(size_t n, double a, const T *x, T *y)
    {
        k_axpy<T><<<grid(n), 256, 0, st>>>(n, (T)a, x, y);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    }
    int xpby(size_t n, const T *s, double b, T *p)
    {
        k_xpby<T><<<grid(n), 256, 0, st>>>(n, s, (T)b, p);
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    }
};

// Least-squares RTM: niter iterations of conjugate gradients on the normal
// equations (CGLS) for the linear Born operator L of all shots stacked,
// min || L m - d ||^2 with m = (drho, dlambda, dmu), starting from m = 0.
// L^T is the exact adjoint.  resid[k] = ||d - L m_k|| (k = 0..niter).
template <typename T>
int lsrtm_impl(int nz, int nx, int nt, T dx, T dt, T fp, int nsource, int abc, int nshots, const int *xsrc,
               const int *zsrc, int zrec, int comp_mask, const T *rho, const T *lam, const T *mu, const T *data,
               int niter, T *dm, double *resid, bool exact)
{
    RTM_CHECK_ARG(nshots >= 1 && niter >= 0 && xsrc && zsrc && data && dm, "bad LSRTM arguments");
    RTM_CHECK_ARG(comp_mask >= 1 && comp_mask <= 31, "comp_mask must select 1 to 5 components");
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx, nm = 3 * plane, gs = (size_t)nt * nx, nd1 = 5 * gs,
                 nd = nd1 * (size_t)nshots;
    DevBuf<T> model;
    TRY(model.alloc(3 * plane));
    RTM_CUDA(cudaMemcpy(model.p, rho, plane * sizeof(T), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(model.p + plane, lam, plane * sizeof(T), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(model.p + 2 * plane, mu, plane * sizeof(T), cudaMemcpyHostToDevice));
    std::vector<std::unique_ptr<BornShot<T>>> shots;
    for (int s = 0; s < nshots; s++) {
        shots.emplace_back(new BornShot<T>());
        TRY(shots.back()->init(nz, nx, nt, dx, dt, xsrc[s], zsrc[s], zrec, fp, nsource, abc, model.p, exact));
        shots.back()->comp_mask = comp_mask;
    }
    cudaStream_t st = shots[0]->h.st;
    const size_t vol = shots[0]->vol;
    DevBuf<T> W, rec, x, r, sv, p, q, tmp;
    TRY(W.alloc(5 * vol));
    T *A[5];
    for (int f = 0; f < 5; f++) A[f] = W.p + f * vol;
    TRY(rec.alloc((size_t)nt * 5 * nx));
    TRY(x.alloc(nm)); TRY(sv.alloc(nm)); TRY(p.alloc(nm)); TRY(tmp.alloc(nm));
    TRY(r.alloc(nd)); TRY(q.alloc(nd));
    RTM_CUDA(cudaMemsetAsync(x.p, 0, nm * sizeof(T), st));
    RTM_CUDA(cudaMemcpyAsync(r.p, data, nd * sizeof(T), cudaMemcpyHostToDevice, st));
    for (int s = 0; s < nshots; s++) TRY(shots[s]->mask_data(r.p + (size_t)s * nd1));
    Vec<T> v;
    TRY(v.init(st));
    // L m for all shots (data of shot s at offset s*nd1)
    auto apply = [&](const T *m, T *out) -> int {
        for (int s = 0; s < nshots; s++)
            TRY(shots[s]->born(m, m + plane, m + 2 * plane, A, rec.p, out + (size_t)s * nd1));
        return RTM_OK;
    };
    // L^T d summed over shots
    auto apply_t = [&](const T *d, T *out) -> int {
        for (int s = 0; s < nshots; s++) {
            TRY(shots[s]->adjoint(d + (size_t)s * nd1, A, s ? tmp.p : out, true));
            if (s) TRY(v.axpy(nm, 1.0, tmp.p, out));
        }
        return RTM_OK;
    };
    double rr = 0, gamma = 0, qq = 0;
    TRY(v.dot(nd, r.p, r.p, &rr));
    if (resid) resid[0] = std::sqrt(rr);
    TRY(apply_t(r.p, sv.p));
    TRY(v.dot(nm, sv.p, sv.p, &gamma));
    RTM_CUDA(cudaMemcpyAsync(p.p, sv.p, nm * sizeof(T), cudaMemcpyDeviceToDevice, st));
    for (int k = 1; k <= niter; k++) {
        if (gamma <= 0) {  // exact solution reached
            if (resid) for (int j = k; j <= niter; j++) resid[j] = std::sqrt(rr);
            break;
        }
        TRY(apply(p.p, q.p));
        TRY(v.dot(nd, q.p, q.p, &qq));
        if (qq <= 0) {
            if (resid) for (int j = k; j <= niter; j++) resid[j] = std::sqrt(rr);
            break;
        }
        const double alpha = gamma / qq;
        TRY(v.axpy(nm, alpha, p.p, x.p));
        TRY(v.axpy(nd, -alpha, q.p, r.p));
        TRY(v.dot(nd, r.p, r.p, &rr));
        if (resid) resid[k] = std::sqrt(rr);
        TRY(apply_t(r.p, sv.p));
        double gnew = 0;
        TRY(v.dot(nm, sv.p, sv.p, &gnew));
        const double beta = gnew / gamma;
        gamma = gnew;
        TRY(v.xpby(nm, sv.p, beta, p.p));
    }
    RTM_CUDA(cudaMemcpyAsync(dm, x.p, nm * sizeof(T), cudaMemcpyDeviceToHost, st));
    RTM_CUDA(cudaStreamSynchronize(st));
    return RTM_OK;
}

// Born modelling and migration of a batch of model perturbations for one
// shot with the source wavefield computed once: data_k = L dm_k and
// img_k = L^T data_k (exact adjoint), or img_k = L^T data_in_k.  Every
// array may be on the device (on_device=1) or the host.
template <typename T>
int born_migrate_impl(int nz, int nx, int nt, T dx, T dt, int xsrc, int zsrc, int zrec, T fp, int nsource, int abc,
                      int comp_mask, const T *rho, const T *lam, const T *mu, int npairs, const T *dm, T *data,
                      const T *data_in, T *img, int on_device, bool exact)
{
    RTM_CHECK_ARG(npairs >= 1, "npairs must be >= 1");
    RTM_CHECK_ARG(comp_mask >= 1 && comp_mask <= 31, "comp_mask must select 1 to 5 components");
    RTM_CHECK_ARG(dm || data_in, "need model perturbations or data");
    RTM_CHECK_ARG(!dm || !data_in, "give model perturbations or data, not both");
    RTM_CHECK_ARG(data || img, "nothing to compute");
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx;
    const cudaMemcpyKind h2d = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind d2h = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    DevBuf<T> model;
    TRY(model.alloc(3 * plane));
    RTM_CUDA(cudaMemcpy(model.p, rho, plane * sizeof(T), h2d));
    RTM_CUDA(cudaMemcpy(model.p + plane, lam, plane * sizeof(T), h2d));
    RTM_CUDA(cudaMemcpy(model.p + 2 * plane, mu, plane * sizeof(T), h2d));
    BornShot<T> sh;
    TRY(sh.init(nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, model.p, exact));
    sh.comp_mask = comp_mask;
    const size_t vol = sh.vol, nd = 5 * sh.gather_size();
    cudaStream_t st = sh.h.st;
    DevBuf<T> W, rec, m, d, im;
    TRY(W.alloc(5 * vol));
    T *A[5];
    for (int f = 0; f < 5; f++) A[f] = W.p + f * vol;
    TRY(rec.alloc((size_t)nt * 5 * nx));
    TRY(m.alloc(3 * plane));
    TRY(d.alloc(nd));
    TRY(im.alloc(3 * plane));
    for (int k = 0; k < npairs; k++) {
        if (dm) {
            RTM_CUDA(cudaMemcpyAsync(m.p, dm + k * 3 * plane, 3 * plane * sizeof(T), h2d, st));
            TRY(sh.born(m.p, m.p + plane, m.p + 2 * plane, A, rec.p, d.p));
            if (data) RTM_CUDA(cudaMemcpyAsync(data + k * nd, d.p, nd * sizeof(T), d2h, st));
        } else {
            RTM_CUDA(cudaMemcpyAsync(d.p, data_in + k * nd, nd * sizeof(T), h2d, st));
            TRY(sh.mask_data(d.p));
        }
        if (img) {
            TRY(sh.adjoint(d.p, A, im.p, true));
            RTM_CUDA(cudaMemcpyAsync(img + k * 3 * plane, im.p, 3 * plane * sizeof(T), d2h, st));
        }
    }
    RTM_CUDA(cudaStreamSynchronize(st));
    return RTM_OK;
}

// Nonlinear elastic modelling of one shot (W/elastic-mod.f90:95-240):
// gathers of the five components at row zrec (Fortran (nt,nx) each).
template <typename T>
int model_impl(int nz, int nx, int nt, T dx, T dt, int xsrc, int zsrc, int zrec, T fp, int nsource, int abc,
               const T *rho, const T *lam, const T *mu, T *const D[5], bool exact)
{
    RTM_CHECK_ARG(nz >= 11 && nx >= 11 && nt >= 3, "grid too small (nz=%d nx=%d nt=%d)", nz, nx, nt);
    RTM_CHECK_ARG(zsrc >= 1 && zsrc <= nz && xsrc >= 1 && xsrc <= nx && zrec >= 1 && zrec <= nz,
                  "source/receiver position outside the grid");
    for (int c = 0; c < 5; c++) RTM_CHECK_ARG(D[c], "null gather pointer");
    TRY(ensure_device());
    Hist<T> h;
    TRY(h.init(nz, nx, nt, exact));
    TRY(h.set_abc(abc));
    const size_t plane = h.plane, gs = (size_t)nt * nx;
    DevBuf<T> model, raw, B, rec, g;
    TRY(model.alloc(3 * plane));
    RTM_CUDA(cudaMemcpy(model.p, rho, plane * sizeof(T), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(model.p + plane, lam, plane * sizeof(T), cudaMemcpyHostToDevice));
    RTM_CUDA(cudaMemcpy(model.p + 2 * plane, mu, plane * sizeof(T), cudaMemcpyHostToDevice));
    TRY(raw.alloc(5 * plane));
    T *r[5];
    for (int i = 0; i < 5; i++) r[i] = raw.p + i * plane;
    TRY(model_coefs<T>(nz, nx, dx, dt, model.p, model.p + plane, model.p + 2 * plane, nz, r[M1X], r[M1Z], nullptr,
                       nullptr, r[A2], r[A3], r[A23], nz, h.st));
    TRY(h.set_coefs_dev(r));
    std::vector<T> src(nt), dtsrc(nt);
    host_ricker<T>(nt, dt, fp, nsource, src.data());
    for (int i = 0; i < nt; i++) dtsrc[i] = dt * src[i];
    TRY(B.alloc(10 * plane));
    T *Bp[5];
    for (int f = 0; f < 5; f++) Bp[f] = B.p + 2 * f * plane;
    TRY(rec.alloc((size_t)nt * 5 * nx));
    TRY(h.model(Bp, dtsrc, zsrc - 1, xsrc - 1, zrec - 1, rec.p));
    TRY(g.alloc(5 * gs));
    dim3 b(128), gr(ceil_div(nt, 128), nx);
    k_gather_from_rec<T><<<gr, b, 0, h.st>>>(nt, nx, rec.p, g.p, g.p + gs, g.p + 2 * gs, g.p + 3 * gs, g.p + 4 * gs);
    RTM_CUDA(cudaGetLastError());
    for (int c = 0; c < 5; c++) RTM_CUDA(cudaMemcpyAsync(D[c], g.p + c * gs, gs * sizeof(T), cudaMemcpyDeviceToHost, h.st));
    RTM_CUDA(cudaStreamSynchronize(h.st));
    return RTM_OK;
}

// Velocity parameterisation (lame=.false., W/image-mod-rtm.f90:182-225).
// With lambda = rho (vp^2 - 2 vs^2) and mu = rho vs^2, the reference's
// velocity imaging condition is, cell by cell, the transpose J^T of the
// Jacobian d(rho, lambda, mu)/d(rho, vp, vs) applied to the Lame images, and
// its Born sources are those of the Lame perturbation J (drho, dvp, dvs).
// adj=1: (drho, dlambda, dmu) images -> (drho, dvp, dvs) images;
// adj=0: (drho, dvp, dvs) -> (drho, dlambda, dmu) perturbations.
template <typename T>
__global__ void k_vel_jacobian(long long n, int adj, const T *rho, const T *vp, const T *vs, const T *a, const T *b,
                               const T *c, T *o1, T *o2, T *o3)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T r = rho[i], p = vp[i], q = vs[i];
        const T p2 = p * p, q2 = q * q, l2 = p2 - T(2) * q2;
        const T x = a[i], y = b[i], z = c[i];
        if (adj) {
            o1[i] = x + l2 * y + q2 * z;
            o2[i] = T(2) * r * p * y;
            o3[i] = T(2) * r * q * z - T(4) * r * q * y;
        } else {
            o1[i] = x;
            o2[i] = l2 * x + T(2) * r * p * y - T(4) * r * q * z;
            o3[i] = q2 * x + T(2) * r * q * z;
        }
    }
}
// lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2
template <typename T>
__global__ void k_vel_model(long long n, const T *rho, const T *vp, const T *vs, T *lam, T *mu)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const T r = rho[i], p = vp[i], q = vs[i];
        lam[i] = r * (p * p - T(2) * q * q);
        mu[i] = r * q * q;
    }
}

template <typename T>
int velocity_impl(int mode, int nz, int nx, const T *rho, const T *vp, const T *vs, const T *i1, const T *i2,
                  const T *i3, T *o1, T *o2, T *o3)
{
    RTM_CHECK_ARG(nz >= 1 && nx >= 1 && rho && vp && vs && o1 && o2, "bad velocity-parameterisation arguments");
    TRY(ensure_device());
    const long long n = (long long)nz * nx;
    DevBuf<T> buf;
    TRY(buf.alloc(9 * (size_t)n));
    T *d[9];
    for (int k = 0; k < 9; k++) d[k] = buf.p + k * n;
    const T *src[6] = {rho, vp, vs, i1, i2, i3};
    const int nin = mode == 2 ? 3 : 6;
    for (int k = 0; k < nin; k++) {
        RTM_CHECK_ARG(src[k], "null input");
        RTM_CUDA(cudaMemcpy(d[k], src[k], n * sizeof(T), cudaMemcpyHostToDevice));
    }
    const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
    if (mode == 2) {
        k_vel_model<T><<<grid, 256>>>(n, d[0], d[1], d[2], d[6], d[7]);
    } else {
        RTM_CHECK_ARG(o3, "null output");
        k_vel_jacobian<T><<<grid, 256>>>(n, mode, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]);
    }
    RTM_CUDA(cudaGetLastError());
    T *outs[3] = {o1, o2, o3};
    for (int k = 0; k < (mode == 2 ? 2 : 3); k++)
        RTM_CUDA(cudaMemcpy(outs[k], d[6 + k], n * sizeof(T), cudaMemcpyDeviceToHost));
    return RTM_OK;
}

}  // namespace

// ===================================================================== C-ABI
extern "C" int rtm_op_c_(int adj, int nz, int nx, int nt, float dx, float dt, int xsrc, int zsrc, int zrec, float fp,
                         int nsource, int abc, const float *rho, const float *lambda, const float *mu, float *drho,
                         float *dlambda, float *dmu, float *Vx, float *Vz, float *sigmaxx, float *sigmazz,
                         float *sigmaxz, int linear, int exact_adjoint)
{
    float *D[5] = {Vx, Vz, sigmaxx, sigmazz, sigmaxz};
    return rtm_op_impl<float>(adj, nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, rho, lambda, mu, drho,
                              dlambda, dmu, D, linear, exact_adjoint, g_exact != 0);
}

extern "C" int rtm_velocity_jacobian_c_(int adj, int nz, int nx, const float *rho, const float *vp, const float *vs,
                                        const float *in1, const float *in2, const float *in3, float *out1, float *out2,
                                        float *out3)
{
    RTM_CHECK_ARG(adj == 0 || adj == 1, "adj must be 0 or 1");
    return velocity_impl<float>(adj, nz, nx, rho, vp, vs, in1, in2, in3, out1, out2, out3);
}

extern "C" int rtm_velocity_jacobian_d_(int adj, int nz, int nx, const double *rho, const double *vp,
                                        const double *vs, const double *in1, const double *in2, const double *in3,
                                        double *out1, double *out2, double *out3)
{
    RTM_CHECK_ARG(adj == 0 || adj == 1, "adj must be 0 or 1");
    return velocity_impl<double>(adj, nz, nx, rho, vp, vs, in1, in2, in3, out1, out2, out3);
}

extern "C" int rtm_velocity_model_c_(int nz, int nx, const float *rho, const float *vp, const float *vs,
                                     float *lambda, float *mu)
{
    return velocity_impl<float>(2, nz, nx, rho, vp, vs, nullptr, nullptr, nullptr, lambda, mu, nullptr);
}

extern "C" int rtm_velocity_model_d_(int nz, int nx, const double *rho, const double *vp, const double *vs,
                                     double *lambda, double *mu)
{
    return velocity_impl<double>(2, nz, nx, rho, vp, vs, nullptr, nullptr, nullptr, lambda, mu, nullptr);
}

extern "C" int rtm_model_c_(int nz, int nx, int nt, float dx, float dt, int xsrc, int zsrc, int zrec, float fp,
                            int nsource, int abc, const float *rho, const float *lambda, const float *mu, float *Vx_rec,
                            float *Vz_rec, float *sigmaxx_rec, float *sigmazz_rec, float *sigmaxz_rec)
{
    float *D[5] = {Vx_rec, Vz_rec, sigmaxx_rec, sigmazz_rec, sigmaxz_rec};
    return model_impl<float>(nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, rho, lambda, mu, D, g_exact != 0);
}

extern "C" int rtm_born_migrate_c_(int nz, int nx, int nt, float dx, float dt, int xsrc, int zsrc, int zrec, float fp,
                                   int nsource, int abc, int comp_mask, const float *rho, const float *lambda,
                                   const float *mu, int npairs, const float *dm, float *data, const float *data_in,
                                   float *img, int on_device)
{
    return born_migrate_impl<float>(nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, comp_mask, rho, lambda, mu,
                                    npairs, dm, data, data_in, img, on_device, g_exact != 0);
}

extern "C" int rtm_lsrtm_c_(int nz, int nx, int nt, float dx, float dt, float fp, int nsource, int abc, int nshots,
                            const int *xsrc, const int *zsrc, int zrec, int comp_mask, const float *rho,
                            const float *lambda, const float *mu, const float *data, int niter, float *dm,
                            double *resid)
{
    return lsrtm_impl<float>(nz, nx, nt, dx, dt, fp, nsource, abc, nshots, xsrc, zsrc, zrec, comp_mask, rho, lambda,
                             mu, data, niter, dm, resid, g_exact != 0);
}

extern "C" int rtm_lsrtm_d_(int nz, int nx, int nt, double dx, double dt, double fp, int nsource, int abc,
                            int nshots, const int *xsrc, const int *zsrc, int zrec, int comp_mask, const double *rho,
                            const double *lambda, const double *mu, const double *data, int niter, double *dm,
                            double *resid)
{
    return lsrtm_impl<double>(nz, nx, nt, dx, dt, fp, nsource, abc, nshots, xsrc, zsrc, zrec, comp_mask, rho, lambda,
                              mu, data, niter, dm, resid, true);
}

extern "C" int rtm_op_d_(int adj, int nz, int nx, int nt, double dx, double dt, int xsrc, int zsrc, int zrec,
                         double fp, int nsource, int abc, const double *rho, const double *lambda, const double *mu,
                         double *drho, double *dlambda, double *dmu, double *Vx, double *Vz, double *sigmaxx,
                         double *sigmazz, double *sigmaxz, int linear, int exact_adjoint)
{
    double *D[5] = {Vx, Vz, sigmaxx, sigmazz, sigmaxz};
    return rtm_op_impl<double>(adj, nz, nx, nt, dx, dt, xsrc, zsrc, zrec, fp, nsource, abc, rho, lambda, mu, drho,
                               dlambda, dmu, D, linear, exact_adjoint, true);
}

extern "C" int rtm_model_op_c_(int nz, int nx, float dx, float dt, const float *rho, float *lambda, float *mu,
                               float *m1_x, float *m1_z, float *aux_m2_c, float *aux_m3_c, float *aux_m2m3_c)
{
    RTM_CHECK_ARG(nz >= 3 && nx >= 3, "grid too small");
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx;
    DevBuf<float> b;
    TRY(b.alloc(10 * plane));
    float *p[10];
    for (int i = 0; i < 10; i++) p[i] = b.p + i * plane;
    TRY(copy_h2d(p[0], rho, plane, 0));
    TRY(copy_h2d(p[1], lambda, plane, 0));
    TRY(copy_h2d(p[2], mu, plane, 0));
    TRY(model_coefs<float>(nz, nx, dx, dt, p[0], p[1], p[2], nz, p[3], p[4], p[5], p[6], p[7], p[8], p[9], nz, 0));
    float *outs[7] = {m1_x, m1_z, lambda, mu, aux_m2_c, aux_m3_c, aux_m2m3_c};
    for (int i = 0; i < 7; i++) TRY(copy_d2h(outs[i], p[3 + i], plane, 0));
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

extern "C" int rtm_source_c_(int nt, float dt, float fp, int nsource, float *source)
{
    RTM_CHECK_ARG(nt >= 1 && source, "bad arguments");
    host_ricker<float>(nt, dt, fp, nsource, source);
    return RTM_OK;
}

extern "C" int rtm_abc_c_(int abc, float *filter)
{
    RTM_CHECK_ARG(abc >= 0 && filter, "bad arguments");
    host_abc_filter<float>(abc, filter);
    return RTM_OK;
}

extern "C" int rtm_fwd_c_(int nt, int nz, int nx, float dt, int xsrc, int zsrc, int abc, const float *source,
                          const float *m1_x, const float *m1_z, const float *aux_m2_c, const float *aux_m3_c,
                          const float *aux_m2m3_c, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                          float *sigmaxz0)
{
    RTM_CHECK_ARG(nz >= 11 && nx >= 11 && nt >= 2, "grid too small");
    RTM_CHECK_ARG(zsrc >= 1 && zsrc <= nz && xsrc >= 1 && xsrc <= nx, "source outside the grid");
    Hist<float> h;
    TRY(h.init(nz, nx, nt, g_exact != 0));
    TRY(h.set_abc(abc));
    const float *raw[5] = {m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c};
    TRY(h.set_coefs_host(raw));
    std::vector<float> dtsrc(nt);
    for (int i = 0; i < nt; i++) dtsrc[i] = dt * source[i];
    const size_t vol = h.plane * nt;
    DevBuf<float> W;
    TRY(W.alloc(5 * vol));
    float *H[5];
    for (int f = 0; f < 5; f++) H[f] = W.p + f * vol;
    TRY(h.forward(H, dtsrc, zsrc - 1, xsrc - 1));
    float *outs[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    for (int f = 0; f < 5; f++) TRY(copy_d2h(outs[f], H[f], vol, 0));
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

extern "C" int rtm_image_init_c_(int nt, int nz, int nx, float dx, float dt, const float *Vx0, const float *Vz0,
                                 float *S1, float *S2, float *S3, float *S4, float *S5, float *S6)
{
    RTM_CHECK_ARG(nz >= 11 && nx >= 11 && nt >= 1, "grid too small");
    TRY(ensure_device());
    const size_t vol = (size_t)nz * nx * nt;
    DevBuf<float> W;
    TRY(W.alloc(8 * vol));
    TRY(copy_h2d(W.p, Vx0, vol, 0));
    TRY(copy_h2d(W.p + vol, Vz0, vol, 0));
    float *S[6];
    for (int i = 0; i < 6; i++) S[i] = W.p + (2 + i) * vol;
    dim3 b(128), g(ceil_div(nz, 128), nx, nt);
    k_image_init<float><<<g, b>>>(nz, nx, nt, W.p, W.p + vol, S[0], S[1], S[2], S[3], S[4], S[5], 1.0f / dt, 1.0f / dx);
    RTM_CUDA(cudaGetLastError());
    float *outs[6] = {S1, S2, S3, S4, S5, S6};
    for (int i = 0; i < 6; i++) TRY(copy_d2h(outs[i], S[i], vol, 0));
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

extern "C" int rtm_model_delta_c_(int nz, int nx, const float *drho, float *dlambda, float *dmu)
{
    (void)drho;  // dm1_x/dm1_z are formed by the reference but never used
    RTM_CHECK_ARG(nz >= 3 && nx >= 3, "grid too small");
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx;
    DevBuf<float> b;
    TRY(b.alloc(4 * plane));
    TRY(copy_h2d(b.p, dlambda, plane, 0));
    TRY(copy_h2d(b.p + plane, dmu, plane, 0));
    dim3 bl(128), g(ceil_div(nz, 128), nx);
    k_model_delta<float><<<g, bl>>>(nz, nx, b.p, b.p + plane, nz, b.p + 2 * plane, b.p + 3 * plane, nz);
    RTM_CUDA(cudaGetLastError());
    TRY(copy_d2h(dlambda, b.p + 2 * plane, plane, 0));
    TRY(copy_d2h(dmu, b.p + 3 * plane, plane, 0));
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

namespace {
template <typename T>
__global__ void k_image_fwd_hist(int nz, int nx, int nt, const T *dm1, const T *dm2, const T *dm3, const T *S1,
                                 const T *S2, const T *S3, const T *S4, const T *S5, const T *S6, T *h0, T *h1, T *h2,
                                 T *h3, T *h4)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x, ix = blockIdx.y, it = blockIdx.z;
    if (iz >= nz) return;
    const size_t o = (size_t)ix * nz + iz, a = (size_t)it * nz * nx + o;
    const T two = T(2);
    h0[a] = mul_rn(dm1[o], S1[a]);
    h1[a] = mul_rn(dm1[o], S2[a]);
    h2[a] = sub_rn(-mul_rn(dm2[o], S3[a]), mul_rn(mul_rn(dm3[o], two), S4[a]));
    h3[a] = sub_rn(-mul_rn(dm2[o], S3[a]), mul_rn(mul_rn(dm3[o], two), S5[a]));
    h4[a] = -mul_rn(dm3[o], S6[a]);
}
template <typename T>
__global__ void k_image_adj_hist(int nz, int nx, int nt, const T *h0, const T *h1, const T *h2, const T *h3,
                                 const T *h4, const T *S1, const T *S2, const T *S3, const T *S4, const T *S5,
                                 const T *S6, T *dm1, T *dm2, T *dm3)
{
    const int iz = blockIdx.x * blockDim.x + threadIdx.x, ix = blockIdx.y;
    if (iz >= nz) return;
    const size_t o = (size_t)ix * nz + iz, plane = (size_t)nz * nx;
    T r1 = 0, r2 = 0, r3 = 0;
    const T two = T(2);
    for (int it = 0; it < nt; it++) {
        const size_t a = (size_t)it * plane + o;
        r1 = add_rn(add_rn(r1, mul_rn(h0[a], S1[a])), mul_rn(h1[a], S2[a]));
        r2 = sub_rn(sub_rn(r2, mul_rn(h2[a], S3[a])), mul_rn(h3[a], S3[a]));
        r3 = sub_rn(sub_rn(sub_rn(r3, mul_rn(mul_rn(h2[a], two), S4[a])), mul_rn(mul_rn(h3[a], two), S5[a])),
                    mul_rn(h4[a], S6[a]));
    }
    dm1[o] = r1; dm2[o] = r2; dm3[o] = r3;
}
}  // namespace

extern "C" int rtm_image_op_c_(int adj, int nt, int nz, int nx, float *drho, float *dlambda, float *dmu, float *Vx0,
                               float *Vz0, float *sigmaxx0, float *sigmazz0, float *sigmaxz0, const float *S1,
                               const float *S2, const float *S3, const float *S4, const float *S5, const float *S6)
{
    RTM_CHECK_ARG(nz >= 1 && nx >= 1 && nt >= 1, "bad sizes");
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx, vol = plane * nt;
    DevBuf<float> W;
    TRY(W.alloc(11 * vol + 3 * plane));
    const float *Sh[6] = {S1, S2, S3, S4, S5, S6};
    float *S[6], *H[5], *dm = W.p + 11 * vol;
    for (int i = 0; i < 6; i++) { S[i] = W.p + i * vol; TRY(copy_h2d(S[i], Sh[i], vol, 0)); }
    for (int f = 0; f < 5; f++) H[f] = W.p + (6 + f) * vol;
    float *hh[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    float *dh[3] = {drho, dlambda, dmu};
    dim3 b(128);
    if (adj) {
        for (int f = 0; f < 5; f++) TRY(copy_h2d(H[f], hh[f], vol, 0));
        k_image_adj_hist<float><<<dim3(ceil_div(nz, 128), nx), b>>>(nz, nx, nt, H[0], H[1], H[2], H[3], H[4], S[0], S[1],
                                                                   S[2], S[3], S[4], S[5], dm, dm + plane, dm + 2 * plane);
        RTM_CUDA(cudaGetLastError());
        for (int i = 0; i < 3; i++) TRY(copy_d2h(dh[i], dm + i * plane, plane, 0));
    } else {
        for (int i = 0; i < 3; i++) TRY(copy_h2d(dm + i * plane, dh[i], plane, 0));
        k_image_fwd_hist<float><<<dim3(ceil_div(nz, 128), nx, nt), b>>>(nz, nx, nt, dm, dm + plane, dm + 2 * plane, S[0],
                                                                       S[1], S[2], S[3], S[4], S[5], H[0], H[1], H[2],
                                                                       H[3], H[4]);
        RTM_CUDA(cudaGetLastError());
        for (int f = 0; f < 5; f++) TRY(copy_d2h(hh[f], H[f], vol, 0));
    }
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

extern "C" int rtm_born_scatter_c_(int nt, int nz, int nx, int zrec, int abc, const float *m1_x, const float *m1_z,
                                   const float *aux_m2_c, const float *aux_m3_c, const float *aux_m2m3_c, float *Vx0,
                                   float *Vz0, float *sigmaxx0, float *sigmazz0, float *sigmaxz0, float *Vx,
                                   float *Vz, float *sigmaxx, float *sigmazz, float *sigmaxz)
{
    RTM_CHECK_ARG(nz >= 11 && nx >= 11 && nt >= 1 && zrec >= 1 && zrec <= nz, "bad sizes");
    Hist<float> h;
    TRY(h.init(nz, nx, nt, g_exact != 0));
    TRY(h.set_abc(abc));
    const float *raw[5] = {m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c};
    TRY(h.set_coefs_host(raw));
    const size_t vol = h.plane * nt, gs = (size_t)nt * nx;
    DevBuf<float> W, rec, g;
    TRY(W.alloc(5 * vol));
    TRY(rec.alloc(5 * gs));
    TRY(g.alloc(5 * gs));
    float *hh[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    float *H[5];
    for (int f = 0; f < 5; f++) { H[f] = W.p + f * vol; TRY(copy_h2d(H[f], hh[f], vol, 0)); }
    TRY(h.born_scatter(H, zrec - 1, rec.p));
    dim3 b(128), gr(ceil_div(nt, 128), nx);
    k_gather_from_rec<float><<<gr, b>>>(nt, nx, rec.p, g.p, g.p + gs, g.p + 2 * gs, g.p + 3 * gs, g.p + 4 * gs);
    RTM_CUDA(cudaGetLastError());
    float *gh[5] = {Vx, Vz, sigmaxx, sigmazz, sigmaxz};
    for (int f = 0; f < 5; f++) {
        TRY(copy_d2h(hh[f], H[f], vol, 0));
        TRY(copy_d2h(gh[f], g.p + f * gs, gs, 0));
    }
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

extern "C" int rtm_op3_full_c_(int nt, int nz, int nx, int zrec, int abc, int exact_adjoint, const float *Vx,
                               const float *Vz, const float *sigmaxx, const float *sigmazz, const float *sigmaxz,
                               const float *m1_x, const float *m1_z, const float *aux_m2_c, const float *aux_m3_c,
                               const float *aux_m2m3_c, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                               float *sigmaxz0)
{
    RTM_CHECK_ARG(nz >= 11 && nx >= 11 && nt >= 2 && zrec >= 1 && zrec <= nz, "bad sizes");
    Hist<float> h;
    TRY(h.init(nz, nx, nt, g_exact != 0));
    TRY(h.set_abc(abc));
    const float *raw[5] = {m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c};
    TRY(h.set_coefs_host(raw));
    const size_t vol = h.plane * nt, gs = (size_t)nt * nx;
    DevBuf<float> W, g;
    TRY(W.alloc(5 * vol));
    TRY(g.alloc(5 * gs));
    float *H[5];
    const float *gh[5] = {Vx, Vz, sigmaxx, sigmazz, sigmaxz};
    for (int f = 0; f < 5; f++) {
        H[f] = W.p + f * vol;
        RTM_CUDA(cudaMemset(H[f], 0, vol * sizeof(float)));
        TRY(copy_h2d(g.p + f * gs, gh[f], gs, 0));
    }
    dim3 b(128), gr(ceil_div(nt, 128), nx);
    k_put_rows<float><<<gr, b>>>(nt, nx, nz, zrec - 1, g.p, g.p + gs, g.p + 2 * gs, g.p + 3 * gs, g.p + 4 * gs, H[0], H[1],
                                 H[2], H[3], H[4]);
    RTM_CUDA(cudaGetLastError());
    TRY(h.adjoint(H, exact_adjoint != 0));
    float *hh[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    for (int f = 0; f < 5; f++) TRY(copy_d2h(hh[f], H[f], vol, 0));
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}

// ===================================================== drop-in rtm_op3_c_
namespace {
// Device state shared by rtm_op3_c_ and the rtm_gpu_* layer; buffers grow on
// demand and are kept between calls.
struct DropIn {
    DevBuf<float> hist, coef, raw;
    int nt = 0, nz = 0, nx = 0;
    bool inited = false;
    double last_ms_per_step = 0;
} g_drop;

// Adjoint levels it_max..0 (0-based) on full histories with pitch ldz and
// plane stride pstride; `base[f]` points at level 0, cell (0,0).
int dropin_run(int it_max, int nt, int nz, int nx, int ldz, size_t pstride, float *const base[5],
               float *const cm[5], double *ms_per_step)
{
    Hist<float> h;  // only for the shot table and launch helpers
    h.nz = nz; h.nx = nx; h.nt = nt; h.plane = pstride; h.exact = g_exact != 0;
    TRY(ensure_device());
    h.tab.shots.assign(1, HostShot{0, 0, nz, nx, -1, -1, -1});
    h.tab.ldz = ldz;
    const void *ptrs[10];
    for (int f = 0; f < 5; f++) { ptrs[f] = base[f]; ptrs[5 + f] = cm[f]; }
    const bool v2 = v2_usable(true, ldz, ptrs, 10) && (pstride % 4) == 0;
    const int tz = v2 ? TZ_TILE2 : TZ_TILE;
    int tx = pick_tile_width(nz, nx, tz);
    while (v2 && tx > 8 && !v2_fits(true, h.exact, tx)) tx /= 2;
    TRY(h.tab.build(tx, tz));
    for (int i = 0; i < 5; i++) h.cmp[i] = cm[i];
    cudaEvent_t e0, e1;
    RTM_CUDA(cudaEventCreate(&e0));
    RTM_CUDA(cudaEventCreate(&e1));
    RTM_CUDA(cudaEventRecord(e0, h.st));
    for (int it = it_max; it >= 0; it--) {
        Step2DArgs<float> a = h.args();
        a.ldz = ldz;
        for (int f = 0; f < 5; f++) {
            a.out[f] = base[f] + (size_t)it * pstride;
            a.inplane[f] = a.out[f];
            a.own2[f] = base[f] + (size_t)(it + 2) * pstride;
            a.nb[f] = base[f] + (size_t)(it + 1) * pstride;
        }
        a.sponge = 0;
        TRY(h.step(a, true));
    }
    RTM_CUDA(cudaEventRecord(e1, h.st));
    RTM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    RTM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_per_step) *ms_per_step = it_max >= 0 ? ms / (it_max + 1) : 0;
    return RTM_OK;
}

int rtm_op3_impl(int nt, int nz, int nx, float *const H[5], const float *const coef[5])
{
    RTM_CHECK_ARG(nt >= 3 && nz >= 11 && nx >= 11, "rtm_op3_c_: grid too small (nt=%d nz=%d nx=%d)", nt, nz, nx);
    for (int f = 0; f < 5; f++) RTM_CHECK_ARG(H[f] && coef[f], "rtm_op3_c_: null array");
    TRY(ensure_device());
    const size_t plane = (size_t)nz * nx, vol = plane * nt;
    TRY(g_drop.hist.alloc(5 * vol));
    TRY(g_drop.raw.alloc(5 * plane));
    TRY(g_drop.coef.alloc(5 * plane));
    float *d[5], *r[5], *c[5];
    for (int f = 0; f < 5; f++) {
        d[f] = g_drop.hist.p + f * vol;
        r[f] = g_drop.raw.p + f * plane;
        c[f] = g_drop.coef.p + f * plane;
        TRY(copy_h2d(d[f], H[f], vol, 0));
        TRY(copy_h2d(r[f], coef[f], plane, 0));
    }
    const float *rc[5] = {r[0], r[1], r[2], r[3], r[4]};
    TRY(mask_coefs<float>(nz, nx, rc, nz, c, nz, 0));
    TRY(dropin_run(nt - 3, nt, nz, nx, nz, plane, d, c, &g_drop.last_ms_per_step));
    for (int f = 0; f < 5; f++) TRY(copy_d2h(H[f], d[f], vol, 0));
    RTM_CUDA(cudaDeviceSynchronize());
    return RTM_OK;
}
}  // namespace

extern "C" void rtm_op3_c_(int nt, int nz, int nx, int zrec, float *Vx0, float *Vz0, float *sigmaxx0,
                           float *sigmazz0, float *sigmaxz0, float *m1_x, float *m1_z, float *aux_m2_c,
                           float *aux_m3_c, float *aux_m2m3_c)
{
    (void)zrec;
    float *H[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    const float *C[5] = {m1_x, m1_z, aux_m2_c, aux_m3_c, aux_m2m3_c};
    g_last_status = rtm_op3_impl(nt, nz, nx, H, C);
    if (g_last_status) fprintf(stderr, "rtm_op3_c_: %s\n", g_err);
}

// ------------------------------------------------ rtm_gpu_* internal layer
extern "C" void rtm_gpu_init(int nt, int nz, int nx)
{
    g_last_status = RTM_OK;
    const size_t pe = (size_t)(nz + 10) * (nx + 10);
    int s = ensure_device();
    if (!s) s = g_drop.hist.alloc(5 * pe * (nt + 10));
    if (!s) s = g_drop.coef.alloc(5 * pe);
    if (!s) {
        g_drop.nt = nt; g_drop.nz = nz; g_drop.nx = nx; g_drop.inited = true;
        cudaMemset(g_drop.hist.p, 0, 5 * pe * (nt + 10) * sizeof(float));
        cudaMemset(g_drop.coef.p, 0, 5 * pe * sizeof(float));
    }
    g_last_status = s;
}

extern "C" void rtm_gpu_copy_in(int nt, int nz, int nx, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                                float *sigmaxz0, float *ex_m1_x, float *ex_m1_z, float *ex_aux_m2_c,
                                float *ex_aux_m3_c, float *ex_aux_m2m3_c)
{
    if (!g_drop.inited || g_drop.nt != nt || g_drop.nz != nz || g_drop.nx != nx) {
        rtm_set_error("rtm_gpu_copy_in: rtm_gpu_init(%d,%d,%d) not called", nt, nz, nx);
        g_last_status = RTM_ERR_STATE;
        return;
    }
    const size_t pe = (size_t)(nz + 10) * (nx + 10), ve = pe * (nt + 10);
    float *h[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    float *c[5] = {ex_m1_x, ex_m1_z, ex_aux_m2_c, ex_aux_m3_c, ex_aux_m2m3_c};
    int s = RTM_OK;
    for (int f = 0; f < 5 && !s; f++) s = copy_h2d(g_drop.hist.p + f * ve, h[f], ve, 0);
    for (int f = 0; f < 5 && !s; f++) s = copy_h2d(g_drop.coef.p + f * pe, c[f], pe, 0);
    if (!s && cudaDeviceSynchronize() != cudaSuccess) { rtm_set_error("copy_in failed"); s = RTM_ERR_CUDA; }
    g_last_status = s;
}

extern "C" void rtm_gpu_copy_out(int nt, int nz, int nx, float *Vx0, float *Vz0, float *sigmaxx0, float *sigmazz0,
                                 float *sigmaxz0)
{
    if (!g_drop.inited || g_drop.nt != nt || g_drop.nz != nz || g_drop.nx != nx) {
        rtm_set_error("rtm_gpu_copy_out: rtm_gpu_init(%d,%d,%d) not called", nt, nz, nx);
        g_last_status = RTM_ERR_STATE;
        return;
    }
    const size_t pe = (size_t)(nz + 10) * (nx + 10), ve = pe * (nt + 10);
    float *h[5] = {Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0};
    int s = RTM_OK;
    for (int f = 0; f < 5 && !s; f++) s = copy_d2h(h[f], g_drop.hist.p + f * ve, ve, 0);
    if (!s && cudaDeviceSynchronize() != cudaSuccess) { rtm_set_error("copy_out failed"); s = RTM_ERR_CUDA; }
    g_last_status = s;
}

extern "C" void rtm_gpu_func(int it_max, int nt, int nz, int nx, float *Vx0, float *Vz0, float *sigmaxx0,
                             float *sigmazz0, float *sigmaxz0, float *ex_m1_x, float *ex_m1_z, float *ex_aux_m2_c,
                             float *ex_aux_m3_c, float *ex_aux_m2m3_c, float *debug, double *gpu_kernel_time_ps)
{
    (void)debug;
    if (it_max < 0 || it_max > nt - 3) {
        rtm_set_error("rtm_gpu_func: it_max %d outside 0..nt-3", it_max);
        g_last_status = RTM_ERR_ARG;
        return;
    }
    rtm_gpu_copy_in(nt, nz, nx, Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0, ex_m1_x, ex_m1_z, ex_aux_m2_c, ex_aux_m3_c,
                    ex_aux_m2m3_c);
    if (g_last_status) return;
    const size_t pe = (size_t)(nz + 10) * (nx + 10), ve = pe * (nt + 10);
    const int ld = nz + 10;
    float *base[5], *cm[5];
    for (int f = 0; f < 5; f++) {
        base[f] = g_drop.hist.p + f * ve + 5 * pe + 5 * (size_t)ld + 5;  // level 0, cell (0,0)
        cm[f] = g_drop.coef.p + f * pe + 5 * (size_t)ld + 5;
    }
    double ms = 0;
    int s = dropin_run(it_max, nt, nz, nx, ld, pe, base, cm, &ms);
    if (s) { g_last_status = s; return; }
    if (gpu_kernel_time_ps) gpu_kernel_time_ps[0] = ms / 1000.0;
    rtm_gpu_copy_out(nt, nz, nx, Vx0, Vz0, sigmaxx0, sigmazz0, sigmaxz0);
}

extern "C" void rtm_gpu_final(void)
{
    g_drop.hist.release();
    g_drop.coef.release();
    g_drop.raw.release();
    g_drop.inited = false;
    g_last_status = RTM_OK;
}
