// Batched multi-shot 2D elastic RTM on one GPU.
//
// Shots live on their own subgrids (uneven widths) of a full model.  A batch
// ("group") of shots is propagated together: every time level is ONE launch
// of the fused step kernel over the work items of all shots of the group
// (a persistent grid of CTAs walking the (shot, tile) list), and the whole
// nt-level loop of both passes is captured once per group as a CUDA graph.
//
// Source side: the forward pass stores per-level FP16 snapshots of Vx, Vz
// (each plane scaled by 2^14/max|.|, the max being reduced by the kernel
// that wrote the level) -- the only part of the source wavefield the imaging
// condition needs (W/image-mod-rtm.f90:57-65 uses Vx0, Vz0 only).
// Receiver side: the adjoint pass injects the traces at the receiver row
// and applies the imaging condition of W/image-mod-rtm.f90:146-162 in the
// same kernel, accumulating the three images in FP32 with Kahan
// compensation.  Propagation stays FP32 throughout.
//
// Each shot is an independent problem on its subgrid (model_op, masks and
// sponge are those of the subgrid), so a shot migrated in a batch gives the
// same image as the single-shot pipeline on its subgrid (up to the FP16
// snapshot rounding and the summation order of the imaging condition).
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/elastic_rtm.h"
#include "elastic2d.cuh"
#include "elastic2d_aux.cuh"
#include "elastic2d_v2.cuh"
#include "engine.h"
#include "march2d.cuh"

using namespace eg;

namespace eg {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
typedef CUresult (*EncodeTiledFn_)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn_ encode_fn_impl()
{
    static EncodeTiledFn_ fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn_>(p);
        else
            cudaGetLastError();
    }
    return fn;
}


bool tensor_maps_available() { return encode_fn_impl() != nullptr; }

// 3D tensor map (ldz rows x cols columns x planes, plane stride plane_elems)
// with a box of box_rows rows x box_cols columns x 1 plane
int make_map(CUtensorMap *m, const void *base, bool half, int ldz, long long cols, long long planes,
             long long plane_elems, int box_rows, int box_cols)
{
    EncodeTiledFn_ fn = encode_fn_impl();
    RTM_CHECK_ARG(fn, "cuTensorMapEncodeTiled is not available from the driver");
    const cuuint64_t es = half ? 2 : 4;
    const cuuint64_t dims[3] = {(cuuint64_t)ldz, (cuuint64_t)cols, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)ldz * es, (cuuint64_t)plane_elems * es};
    const cuuint32_t box[3] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols, 1};
    const cuuint32_t el[3] = {1, 1, 1};
    const CUresult r = fn(m, half ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                          const_cast<void *>(base), dims, strides, box, el, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        rtm_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return RTM_ERR_CUDA;
    }
    return RTM_OK;
}

int make_map_nd(CUtensorMap *m, const void *base, bool bf16, int rank, const long long *dims, const long long *strides_b,
                const int *box, int swizzle)
{
    EncodeTiledFn_ fn = encode_fn_impl();
    RTM_CHECK_ARG(fn, "cuTensorMapEncodeTiled is not available from the driver");
    RTM_CHECK_ARG(rank >= 1 && rank <= 5, "tensor map rank %d", rank);
    cuuint64_t d[5], st[4];
    cuuint32_t bx[5], el[5];
    for (int i = 0; i < rank; i++) {
        d[i] = (cuuint64_t)dims[i];
        bx[i] = (cuuint32_t)box[i];
        el[i] = 1;
        if (i + 1 < rank) st[i] = (cuuint64_t)strides_b[i];
    }
    const CUtensorMapSwizzle sw = swizzle == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                  : swizzle == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                  : swizzle == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                                                  : CU_TENSOR_MAP_SWIZZLE_NONE;
    const CUresult r = fn(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank,
                          const_cast<void *>(base), d, st, bx, el, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        rtm_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return RTM_ERR_CUDA;
    }
    return RTM_OK;
}

}  // namespace eg

static char g_pending_at[128] = "";
static void note_pending(const char *where)
{
    if (!g_pending_at[0] && cudaPeekAtLastError() != cudaSuccess) snprintf(g_pending_at, sizeof g_pending_at, "%s", where);
}

namespace {

__global__ void k_snap_plane(const ShotGeom *shots, int ld, const float *vx, const float *vz, const float *maxes,
                             __half *s0, __half *s1)
{
    const ShotGeom g = shots[blockIdx.z];
    const int iz = blockIdx.x * blockDim.x + threadIdx.x, ix = blockIdx.y;
    if (iz >= g.nz || ix >= g.nx) return;
    const long long o = g.off + (long long)ix * ld + iz;
    const float m0 = maxes[2 * blockIdx.z], m1 = maxes[2 * blockIdx.z + 1];
    s0[o] = __float2half_rn(vx[o] * (m0 > 0.f ? SNAP_Q / m0 : 0.f));
    s1[o] = __float2half_rn(vz[o] * (m1 > 0.f ? SNAP_Q / m1 : 0.f));
}

// traces of one shot: reference layout comp-major (nt,nx) gathers -> [it][slot][ix]
__global__ void k_traces_in(int nt, int nx, int ncomp, const float *src, float *dst)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, it = blockIdx.y, c = blockIdx.z;
    if (ix >= nx) return;
    dst[((long long)it * ncomp + c) * nx + ix] = src[((long long)c * nx + ix) * nt + it];
}

// full image (3 planes, ld nz) += shot images (sum minus Kahan residual)
// One launch per shot: overlapping subgrids are summed in shot order.
__global__ void k_stack(const ShotGeom *shots, int shot, int ld, int nz, long long plane_full, const int *x0,
                        const float *img, const float *cmp, long long gplane, float *full)
{
    const ShotGeom g = shots[shot];
    const int iz = blockIdx.x * blockDim.x + threadIdx.x, ix = blockIdx.y;
    if (iz >= g.nz || ix >= g.nx) return;
    const long long o = g.off + (long long)ix * ld + iz;
    const long long f = (long long)(x0[shot] + ix) * nz + iz;
#pragma unroll
    for (int i = 0; i < 3; i++) full[i * plane_full + f] += img[i * gplane + o] - cmp[i * gplane + o];
}

// Blocked compensated imaging: totals (sum, compensation) += partial planes
// with Kahan's update, then the partials restart from zero.  The three image
// planes of a group are contiguous, so one launch covers n4 float4 words.
__global__ void k_fold(long long n4, float4 *sum, float4 *cmp, float4 *part)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = part[i];
        float4 sv = sum[i], cv = cmp[i];
        float *sa = &sv.x, *ca = &cv.x;
        const float pa[4] = {p.x, p.y, p.z, p.w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float y = pa[j] - ca[j];
            const float t = sa[j] + y;
            ca[j] = (t - sa[j]) - y;
            sa[j] = t;
        }
        sum[i] = sv;
        cmp[i] = cv;
        part[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// levels accumulated in FP32 partial planes between two folds
constexpr int IMG_FOLD = 32;
// zero guard columns after every shot of a group: a halo read across a shot's
// edge (5 columns) lands on zeros, so tile staging needs no per-shot masking
constexpr int GUARD = 5;

// Work of the marching kernels for `ctas` CTAs.  The units (shot, strip,
// 8-column chunk) are ordered by shot, column block (the shot's chunks in
// equal blocks of about one CTA's share), strip, chunk, and cut into `ctas` contiguous pieces of equal
// length; a piece's units form runs of consecutive chunks of one strip.  So
// the CTAs of vertically adjacent strips march over the same columns at the
// same time, and the 8-row halo that one strip's tiles share with the next is
// still in L2 when the second reads it.  Units weigh the same whatever their
// strip's depth: a partial last strip moves fewer bytes but keeps every warp
// issuing the full chunk's instructions.
void march_plan(const std::vector<HostShot> &shots, int ctas, std::vector<int4> &runs, std::vector<int> &lo)
{
    long long total = 0;
    for (const HostShot &h : shots) total += (long long)ceil_div(h.nx, MC) * ceil_div(h.nz, V2_TZ);
    const double share = (double)total / ctas;  // chunks per CTA
    runs.clear();
    lo.assign(ctas + 1, 0);
    long long before = 0;
    int cur = -1;
    for (size_t s = 0; s < shots.size(); s++) {
        const HostShot &h = shots[s];
        const int nch = ceil_div(h.nx, MC);
        // the shot's columns in nb blocks of equal length
        const int nb = std::max(1, (int)std::lround(nch / share));
        for (int q = 0; q < nb; q++)
            for (int t = 0; t * V2_TZ < h.nz; t++)
                for (int k = (int)((long long)q * nch / nb); k < (int)((long long)(q + 1) * nch / nb); k++, before++) {
                    const int cta = (int)(before * ctas / total);
                    if (cta != cur || runs.back().x != (int)s || runs.back().y != t * V2_TZ || runs.back().w != k) {
                        runs.push_back(make_int4((int)s, t * V2_TZ, k, k + 1));
                        for (int c = cur + 1; c <= cta; c++) lo[c] = (int)runs.size() - 1;
                        cur = cta;
                    } else {
                        runs.back().w = k + 1;
                    }
                }
    }
    for (int c = cur + 1; c <= ctas; c++) lo[c] = (int)runs.size();
}

// Launch with programmatic stream serialisation: the kernel may start
// before the previous kernel in the stream has finished (the marching
// kernels wait for it in their prologue, griddepcontrol.wait).
template <typename Args>
cudaError_t launch_pdl(void (*kernel)(Step2DArgs<float>, Args), int ctas, int threads, size_t smem, cudaStream_t st,
                       const Step2DArgs<float> &a, const Args &m)
{
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a, m);
}

int launch_march(const Step2DArgs<float> &a, const MarchArgs &m, int ctas, cudaStream_t st)
{
    static bool init[RTM_MAX_DEVICES] = {};
    {
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!init[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(k_fwd_march, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)M_SMEM));
            init[dev] = true;
        }
    }
    RTM_CHECK_ARG(!a.inplane[0] && a.tma && a.ldz % 4 == 0, "marching forward step: unsupported arguments");
    RTM_CUDA(launch_pdl(k_fwd_march, ctas, M_FWD_THREADS, M_SMEM, st, a, m));
    return RTM_OK;
}

int launch_march_adj(const Step2DArgs<float> &a, const MarchAdjArgs &m, int ctas, cudaStream_t st)
{
    static bool init[RTM_MAX_DEVICES] = {};
    {
        const int dev = rtm_current_device();
        std::lock_guard<std::mutex> lk(rtm_device_state_lock());
        if (!init[dev]) {
            RTM_CUDA(cudaFuncSetAttribute(k_adj_march, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MA_SMEM));
            init[dev] = true;
        }
    }
    RTM_CHECK_ARG(!a.inplane[0] && a.tma && a.ldz % 4 == 0 && a.img[0] && !a.imgc[0],
                  "marching adjoint step: unsupported arguments");
    RTM_CUDA(launch_pdl(k_adj_march, ctas, M_THREADS, MA_SMEM, st, a, m));
    return RTM_OK;
}

}  // namespace

struct rtm_batch {
    int nz = 0, nx = 0, nt = 0;
    float dx = 0, dt = 0, fp = 0;
    int nsource = 250, abc = 0, comp_mask = 3, ncomp = 2, group_max = 1, exact_adj = 0;
    std::vector<int> x0, nxs, xsrc, zsrc, zrec;  // 0-based
    int ldz = 0;
    long long cap_cols = 0, gplane = 0;
    DevBuf<float> model, coefraw, coef, F, A, zero, img, filt, maxes, traces, tstage, full;
    DevBuf<__half> snaps;
    // Checkpoint-restart: ckpt = 0 keeps the FP16 snapshots of every level;
    // ckpt = k keeps the full forward state (two levels of the five fields)
    // at the start of every k-level segment in `ck`, and a ring of k + 1
    // snapshot levels that the adjoint pass refills by recomputing each
    // segment from its checkpoint before migrating through it.
    int ckpt = 0;
    DevBuf<float> ck;
    bool use_tma = true;   // stage step tiles with tensor-memory-access loads
    // passes by the marching kernels: -1 automatic (the autotuner's choice
    // per pass, on until it has run), else bit 0 forward, bit 1 adjoint;
    // needs tensor-map staging
    int march = -1;
    bool march_tuned = true, march_tuned_a = true;  // per pass
    double tune_march_ms = -1, tune_march_ms_a = -1;
    DevBuf<int4> mruns;
    DevBuf<int> mlo;
    DevBuf<int> err;       // set by a step kernel whose tile load never completed
    // test hook: the forward pass's first marching launch waits on `stall`,
    // a zeroed device flag that nothing sets (rtm_batch_set_test_stall)
    bool test_stall = false;
    DevBuf<int> stall;
    DevBuf<int> dx0;
    ShotTable tab;    // forward pass work items (also used by the per-shot kernels)
    ShotTable tab_a;  // adjoint pass work items
    int tx_f = 0, tx_a = 0;          // tile widths chosen by the autotuner (0 = heuristic)
    int st_f = 1, st_a = 1;          // staging buffers per CTA chosen by the autotuner
    int th_f = 256, th_a = 256;      // threads per CTA chosen by the autotuner
    // measured ms per step, [pass][tx 8,16,32][variant: stages 1/2 x threads 256/512]
    double tune_ms[2][3][4] = {};
    std::vector<float> dtsrc;
    cudaStream_t st = nullptr;
    double last_fwd_ms = 0, last_adj_ms = 0, last_total_ms = 0;
    long long last_cells = 0;
    int kernels_last = 0;
    bool use_graph = true;
    int tile_x = 0;  // 0 = automatic

    ~rtm_batch()
    {
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

// A step kernel that gave up waiting for its staged tile sets b->err.
int check_tile_loads(rtm_batch *b)
{
    int e = 0;
    RTM_CUDA(cudaMemcpy(&e, b->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        RTM_CUDA(cudaMemset(b->err.p, 0, sizeof(int)));
        rtm_set_error("a step kernel's tile load did not complete within its time limit");
        return RTM_ERR_TIMEOUT;
    }
    return RTM_OK;
}

int batch_group(rtm_batch *b, int s0, int ns, const float *traces, int traces_dev, float *image, int image_dev,
                int tune_steps = 0)
{
    RTM_CHECK_ARG(s0 >= 0 && ns >= 1 && s0 + ns <= (int)b->x0.size() && ns <= b->group_max, "bad shot range");
    {
        const cudaError_t pend = cudaGetLastError();
        if (pend != cudaSuccess) {
            rtm_set_error("rtm_batch_migrate: CUDA error pending on entry: %s (first seen at %s)",
                          cudaGetErrorString(pend), g_pending_at[0] ? g_pending_at : "?");
            return RTM_ERR_CUDA;
        }
    }
    const int nz = b->nz, nt = b->nt, ld = b->ldz;
    cudaStream_t st = b->st;
    // ---- group geometry
    long long col = 0, doff = 0, tin = 0;
    b->tab.shots.clear();
    std::vector<int> x0g(ns);
    std::vector<long long> tin_off(ns);
    for (int i = 0; i < ns; i++) {
        const int s = s0 + i;
        HostShot h;
        h.off = col * ld;
        h.doff = doff;
        h.nz = nz;
        h.nx = b->nxs[s];
        h.src_iz = b->zsrc[s];
        h.src_ix = b->xsrc[s] - b->x0[s];
        h.rec_iz = b->zrec[s];
        b->tab.shots.push_back(h);
        x0g[i] = b->x0[s];
        tin_off[i] = tin;
        col += b->nxs[s] + GUARD;
        doff += (long long)nt * b->ncomp * b->nxs[s];
        tin += (long long)b->ncomp * b->nxs[s] * nt;
    }
    RTM_CHECK_ARG(col <= b->cap_cols, "group wider than the batch capacity");
    b->tab.ldz = ld;
    const int tz = kernel_version() == 1 ? TZ_TILE : TZ_TILE2;  // batch planes are always v2-aligned
    int stf = 1, sta = 1;      // staging buffers per CTA of the two passes
    int thf = 256, tha = 256;  // threads per CTA of the two passes
    {
        const int heur = pick_tile_width((long long)nz, col, tz);
        int heur_a = heur;
        while (tz == TZ_TILE2 && heur_a > 8 && !v2_fits(true, false, heur_a)) heur_a /= 2;
        const int txf = b->tile_x > 0 ? b->tile_x : (b->tx_f > 0 ? b->tx_f : heur);
        int txa = b->tile_x > 0 ? b->tile_x : (b->tx_a > 0 ? b->tx_a : heur_a);
        while (tz == TZ_TILE2 && txa > 8 && !v2_fits(true, false, txa)) txa /= 2;
        TRY(b->tab.build(txf, tz));
        b->tab_a.shots = b->tab.shots;
        b->tab_a.ldz = ld;
        TRY(b->tab_a.build(txa, tz));
        if (tz == TZ_TILE2 && v2_fits(false, false, txf, b->st_f, b->th_f)) { stf = b->st_f; thf = b->th_f; }
        if (tz == TZ_TILE2 && v2_fits(true, false, txa, b->st_a, b->th_a)) { sta = b->st_a; tha = b->th_a; }
    }
    RTM_CUDA(cudaMemcpyAsync(b->dx0.p, x0g.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st));
    const long long gp = b->gplane;
    // tensor maps of the staged planes (tile box of the pass's width)
    const bool tma_on = b->use_tma && tz == TZ_TILE2;
    CUtensorMap mF, mA, mC, mS;
    memset(&mF, 0, sizeof mF); memset(&mA, 0, sizeof mA); memset(&mC, 0, sizeof mC); memset(&mS, 0, sizeof mS);
    auto build_maps = [&](int txf, int txa) -> int {
        if (!tma_on) return RTM_OK;
        const long long cols = b->cap_cols;
        const long long nlev = b->ckpt ? b->ckpt + 1 : nt;
        TRY(make_map(&mF, b->F.p, false, ld, cols, 10, gp, V2_LZ, txf + 2 * HALO));
        TRY(make_map(&mA, b->A.p, false, ld, cols, 10, gp, V2_LZ, txa + 2 * HALO));
        TRY(make_map(&mC, b->coef.p, false, ld, cols, 5, gp, V2_LZ, txa + 2 * HALO));
        TRY(make_map(&mS, b->snaps.p, true, ld, cols, 2 * nlev, gp, V2_LZ, txa + 2 * HALO));
        return RTM_OK;
    };
    TRY(build_maps(b->tab.tx, b->tab_a.tx));
    // marching forward kernel: its run table and tensor maps
    const int mctas = device_sm_count();
    MarchArgs marg;
    memset(&marg, 0, sizeof marg);
    if (tma_on) {
        std::vector<int4> runs;
        std::vector<int> lo;
        march_plan(b->tab.shots, mctas, runs, lo);
        TRY(b->mruns.alloc(runs.size()));
        TRY(b->mlo.alloc(lo.size()));
        RTM_CUDA(cudaMemcpy(b->mruns.p, runs.data(), runs.size() * sizeof(int4), cudaMemcpyHostToDevice));
        RTM_CUDA(cudaMemcpy(b->mlo.p, lo.data(), lo.size() * sizeof(int), cudaMemcpyHostToDevice));
        marg.runs = b->mruns.p;
        marg.run_lo = b->mlo.p;
        TRY(make_map(&marg.tm_nb, b->F.p, false, ld, b->cap_cols, 10, gp, V2_LZ, MC));
        TRY(make_map(&marg.tm_own, b->F.p, false, ld, b->cap_cols, 10, gp, V2_TZ, MC));
        TRY(make_map(&marg.tm_coef, b->coef.p, false, ld, b->cap_cols, 5, gp, V2_TZ, MC));
    }
    MarchAdjArgs madj;
    memset(&madj, 0, sizeof madj);
    if (tma_on) {
        madj.runs = marg.runs;
        madj.run_lo = marg.run_lo;
        const long long nlev = b->ckpt ? b->ckpt + 1 : nt;
        TRY(make_map(&madj.tm_nb, b->A.p, false, ld, b->cap_cols, 10, gp, V2_LZ, MC));
        TRY(make_map(&madj.tm_coef, b->coef.p, false, ld, b->cap_cols, 5, gp, V2_LZ, MC));
        TRY(make_map(&madj.tm_snap, b->snaps.p, true, ld, b->cap_cols, 2 * nlev, gp, V2_LZ, MC));
    }
    const bool use_march = tma_on && (b->march < 0 ? b->march_tuned : (b->march & 1) != 0);
    const bool use_march_a = tma_on && (b->march < 0 ? b->march_tuned_a : (b->march & 2) != 0);
    // ---- coefficients of every shot's subgrid (guard columns and columns of
    // the previous group's shots are zero)
    RTM_CUDA(cudaMemsetAsync(b->coef.p, 0, 5 * gp * sizeof(float), st));
    for (int i = 0; i < ns; i++) {
        const HostShot &h = b->tab.shots[i];
        const long long mo = (long long)x0g[i] * nz;
        float *r[5], *c[5];
        for (int k = 0; k < 5; k++) {
            r[k] = b->coefraw.p + k * gp + h.off;
            c[k] = b->coef.p + k * gp + h.off;
        }
        const long long pf = (long long)nz * b->nx;
        TRY(model_coefs<float>(nz, h.nx, b->dx, b->dt, b->model.p + mo, b->model.p + pf + mo, b->model.p + 2 * pf + mo,
                               nz, r[M1X], r[M1Z], nullptr, nullptr, r[A2], r[A3], r[A23], ld, st));
        const float *rc[5] = {r[0], r[1], r[2], r[3], r[4]};
        TRY(mask_coefs<float>(nz, h.nx, rc, ld, c, ld, st));
    }
    // ---- traces -> device internal layout
    const float *tsrc = traces;
    if (!traces_dev) {
        RTM_CUDA(cudaMemcpyAsync(b->tstage.p, traces, tin * sizeof(float), cudaMemcpyHostToDevice, st));
        tsrc = b->tstage.p;
    }
    for (int i = 0; i < ns; i++) {
        const HostShot &h = b->tab.shots[i];
        dim3 blk(128), grd(ceil_div(h.nx, 128), nt, b->ncomp);
        k_traces_in<<<grd, blk, 0, st>>>(nt, h.nx, b->ncomp, tsrc + tin_off[i], b->traces.p + h.doff);
        RTM_CUDA(cudaGetLastError());
    }
    // ---- state
    RTM_CUDA(cudaMemsetAsync(b->F.p, 0, 10 * gp * sizeof(float), st));
    RTM_CUDA(cudaMemsetAsync(b->A.p, 0, 10 * gp * sizeof(float), st));
    RTM_CUDA(cudaMemsetAsync(b->img.p, 0, 9 * gp * sizeof(float), st));
    RTM_CUDA(cudaMemsetAsync(b->maxes.p, 0, (size_t)(nt + 2) * b->group_max * 2 * sizeof(float), st));

    auto fb = [&](int par, int f) { return b->F.p + (par * 5 + f) * gp; };
    auto ab = [&](int par, int f) { return b->A.p + (par * 5 + f) * gp; };
    // v2 images: FP32 partial planes folded every IMG_FOLD levels; the v1
    // kernel keeps per-level Kahan updates of the totals
    const bool blocked = tz == TZ_TILE2;
    auto set_img = [&](Step2DArgs<float> &a) {
        for (int i = 0; i < 3; i++) {
            a.img[i] = b->img.p + (blocked ? 6 + i : i) * gp;
            a.imgc[i] = blocked ? nullptr : b->img.p + (3 + i) * gp;
        }
    };
    auto fold = [&]() -> int {
        const long long n4 = 3 * gp / 4;
        const int grid = (int)std::min<long long>(ceil_div((int)std::min<long long>(n4, 1LL << 30), 256), 8LL * device_sm_count());
        k_fold<<<grid, 256, 0, st>>>(n4, reinterpret_cast<float4 *>(b->img.p), reinterpret_cast<float4 *>(b->img.p + 3 * gp),
                                    reinterpret_cast<float4 *>(b->img.p + 6 * gp));
        RTM_CUDA(cudaGetLastError());
        return RTM_OK;
    };
    // snapshot slot of level L (1-based): its own level, or a ring slot
    auto snap = [&](int L, int f) {
        const size_t slot = b->ckpt ? (size_t)(L % (b->ckpt + 1)) : (size_t)(L - 1);
        return b->snaps.p + (slot * 2 + f) * gp;
    };
    auto mx = [&](int L) { return b->maxes.p + (size_t)L * b->group_max * 2; };
    const float inv_dt = 1.0f / b->dt, inv_dx = 1.0f / b->dx;

    auto base_args = [&](bool adj) {
        const ShotTable &tb = adj ? b->tab_a : b->tab;
        Step2DArgs<float> a;
        memset(&a, 0, sizeof a);
        for (int k = 0; k < 5; k++) a.coef[k] = b->coef.p + k * gp;
        a.shots = tb.d_geom;
        a.nshots = ns;
        a.ntiles = tb.ntiles;
        a.ldz = ld;
        a.filt = b->filt.p;
        a.abc2 = b->abc + 5;
        a.inv_dt = inv_dt;
        a.inv_dx = inv_dx;
        if (tma_on) {
            a.tma = 1;
            a.err = b->err.p;
            a.tm[0] = adj ? mA : mF;
            a.tm[1] = mC;
            a.tm[2] = mS;
        }
        return a;
    };
    auto slot = [&](int L) { return b->ckpt ? L % (b->ckpt + 1) : L - 1; };
    // initialise launch configuration outside any capture
    {
        Step2DArgs<float> a = base_args(false);
        a.ntiles = 0;
        TRY(launch_step<float>(a, false, false, b->tab.tx, 0, st, b->tab.tz, stf, thf));
        a.img[0] = b->img.p;
        TRY(launch_step<float>(a, true, false, b->tab_a.tx, 0, st, b->tab_a.tz, sta, tha));
    }

    if (tune_steps > 0) {
        // Autotuner: time `tune_steps` launches of each pass for every tile
        // width on this group's geometry and keep the fastest per pass.
        cudaEvent_t t0, t1;
        RTM_CUDA(cudaEventCreate(&t0));
        RTM_CUDA(cudaEventCreate(&t1));
        const int cand[3] = {8, 16, 32};
        for (int pass = 0; pass < 2; pass++) {
            double best = 1e30;
            int bx = cand[0], bs = 1, bt = 256;
            for (int ci = 0; ci < 3; ci++)
                for (int var = 0; var < 4; var++) {
                    const int ns_ = 1 + (var & 1), nth = var >= 2 ? 512 : 256;
                    if (tz != TZ_TILE2 ? var > 0 : !v2_fits(pass == 1, false, cand[ci], ns_, nth)) {
                        b->tune_ms[pass][ci][var] = -1;  // not available or does not fit in a block
                        continue;
                    }
                    ShotTable &tb = pass ? b->tab_a : b->tab;
                    TRY(tb.build(cand[ci], tz));
                    TRY(build_maps(b->tab.tx, b->tab_a.tx));
                    for (int rep = 0; rep < 2; rep++) {  // the first repetition warms up
                        RTM_CUDA(cudaEventRecord(t0, st));
                        for (int k = 0; k < tune_steps; k++) {
                            const int L = 3 + (k & 1);
                            Step2DArgs<float> a = base_args(pass == 1);
                            for (int f = 0; f < 5; f++) {
                                a.out[f] = pass ? ab(L & 1, f) : fb(L & 1, f);
                                a.own2[f] = a.out[f];
                                a.nb[f] = pass ? ab((L + 1) & 1, f) : fb((L + 1) & 1, f);
                                a.nb_plane[f] = ((L + 1) & 1) * 5 + f;
                            }
                            a.snap_plane[0] = 2 * slot(1);
                            a.snap_plane[1] = 2 * slot(1) + 1;
                            if (!pass) {
                                a.sponge = 1;
                                a.snap_out[0] = snap(1, 0);
                                a.snap_out[1] = snap(1, 1);
                                a.snap_max_in = mx(1);
                                a.snap_max_out = mx(2);
                            } else {
                                a.rec = b->traces.p; a.comp_mask = b->comp_mask; a.ncomp = b->ncomp; a.it = 0;
                                a.isnap0[0] = snap(1, 0); a.isnap0[1] = snap(1, 1); a.imax0 = mx(1);
                                a.isnap1[0] = snap(2, 0); a.isnap1[1] = snap(2, 1); a.imax1 = mx(2);
                                set_img(a);
                            }
                            TRY(launch_step<float>(a, pass == 1, false, tb.tx, 0, st, tb.tz, ns_, nth));
                        }
                        RTM_CUDA(cudaEventRecord(t1, st));
                        RTM_CUDA(cudaEventSynchronize(t1));
                    }
                    float ms = 0;
                    RTM_CUDA(cudaEventElapsedTime(&ms, t0, t1));
                    b->tune_ms[pass][ci][var] = ms / tune_steps;
                    if (ms < best) { best = ms; bx = cand[ci]; bs = ns_; bt = nth; }
                }
            if (pass == 0 && tma_on) {
                // the marching forward kernel on the same levels
                for (int rep = 0; rep < 2; rep++) {
                    RTM_CUDA(cudaEventRecord(t0, st));
                    for (int k = 0; k < tune_steps; k++) {
                        const int L = 3 + (k & 1);
                        Step2DArgs<float> a = base_args(false);
                        MarchArgs m = marg;
                        for (int f = 0; f < 5; f++) {
                            a.out[f] = fb(L & 1, f);
                            a.own2[f] = a.out[f];
                            a.nb[f] = fb((L + 1) & 1, f);
                            a.nb_plane[f] = ((L + 1) & 1) * 5 + f;
                            m.own_plane[f] = (L & 1) * 5 + f;
                        }
                        a.sponge = 1;
                        a.snap_out[0] = snap(1, 0);
                        a.snap_out[1] = snap(1, 1);
                        a.snap_max_in = mx(1);
                        a.snap_max_out = mx(2);
                        TRY(launch_march(a, m, mctas, st));
                    }
                    RTM_CUDA(cudaEventRecord(t1, st));
                    RTM_CUDA(cudaEventSynchronize(t1));
                }
                float ms = 0;
                RTM_CUDA(cudaEventElapsedTime(&ms, t0, t1));
                b->tune_march_ms = ms / tune_steps;
                b->march_tuned = ms < best;
            }
            if (pass == 1 && tma_on) {
                // the marching adjoint kernel on the same levels
                for (int rep = 0; rep < 2; rep++) {
                    RTM_CUDA(cudaEventRecord(t0, st));
                    for (int k = 0; k < tune_steps; k++) {
                        const int L = 3 + (k & 1);
                        Step2DArgs<float> a = base_args(true);
                        for (int f = 0; f < 5; f++) {
                            a.out[f] = ab(L & 1, f);
                            a.own2[f] = a.out[f];
                            a.nb[f] = ab((L + 1) & 1, f);
                            a.nb_plane[f] = ((L + 1) & 1) * 5 + f;
                        }
                        a.snap_plane[0] = 2 * slot(1);
                        a.snap_plane[1] = 2 * slot(1) + 1;
                        a.rec = b->traces.p; a.comp_mask = b->comp_mask; a.ncomp = b->ncomp; a.it = 0;
                        a.isnap0[0] = snap(1, 0); a.isnap0[1] = snap(1, 1); a.imax0 = mx(1);
                        a.isnap1[0] = snap(2, 0); a.isnap1[1] = snap(2, 1); a.imax1 = mx(2);
                        set_img(a);
                        TRY(launch_march_adj(a, madj, mctas, st));
                    }
                    RTM_CUDA(cudaEventRecord(t1, st));
                    RTM_CUDA(cudaEventSynchronize(t1));
                }
                float ms = 0;
                RTM_CUDA(cudaEventElapsedTime(&ms, t0, t1));
                b->tune_march_ms_a = ms / tune_steps;
                b->march_tuned_a = ms < best;
            }
            if (pass) { b->st_a = bs; b->th_a = bt; } else { b->st_f = bs; b->th_f = bt; }
            if (pass) b->tx_a = bx; else b->tx_f = bx;
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        return check_tile_loads(b);
    }

    cudaEvent_t e0, e1, e2;
    RTM_CUDA(cudaEventCreate(&e0));
    RTM_CUDA(cudaEventCreate(&e1));
    RTM_CUDA(cudaEventCreate(&e2));
    int nkern = 0;
    // ---- forward pass: levels 2..nt (level 1 is zero), then the snapshot
    // of the last level.  One step of the forward recursion:
    auto fwd_step = [&](int L) -> int {
        Step2DArgs<float> a = base_args(false);
        for (int f = 0; f < 5; f++) {
            a.out[f] = fb(L & 1, f);
            a.own2[f] = fb(L & 1, f);
            a.nb[f] = fb((L - 1) & 1, f);
            a.nb_plane[f] = ((L - 1) & 1) * 5 + f;
        }
        a.sponge = L >= 3;
        a.has_src = 1;
        a.srcval = b->dtsrc[L - 2];
        a.snap_out[0] = snap(L - 1, 0);
        a.snap_out[1] = snap(L - 1, 1);
        a.snap_max_in = mx(L - 1);
        a.snap_max_out = mx(L);
        if (use_march) {
            MarchArgs m = marg;
            for (int f = 0; f < 5; f++) m.own_plane[f] = (L & 1) * 5 + f;
            if (b->test_stall && L == 2) m.stall = b->stall.p;
            TRY(launch_march(a, m, mctas, st));
        } else {
            TRY(launch_step<float>(a, false, false, b->tab.tx, 0, st, b->tab.tz, stf, thf));
        }
        nkern++;
        return RTM_OK;
    };
    auto snap_last = [&]() -> int {
        dim3 blk(128), grd(ceil_div(nz, 128), (unsigned)*std::max_element(b->nxs.begin() + s0, b->nxs.begin() + s0 + ns), ns);
        k_snap_plane<<<grd, blk, 0, st>>>(b->tab.d_geom, ld, fb(nt & 1, VX), fb(nt & 1, VZ), mx(nt), snap(nt, 0), snap(nt, 1));
        RTM_CUDA(cudaGetLastError());
        nkern++;
        return RTM_OK;
    };
    const int ck = b->ckpt;
    const int nseg = ck ? (nt + ck - 1) / ck : 1;
    // checkpoint of segment s >= 1: levels a-1, a (a = s*ck + 1) of F
    auto ck_state = [&](int sgm) { return b->ck.p + (size_t)(sgm - 1) * 10 * gp; };
    auto record_fwd_ckpt = [&]() -> int {
        for (int L = 2; L <= nt; L++) {
            TRY(fwd_step(L));
            if ((L - 1) % ck == 0)
                RTM_CUDA(cudaMemcpyAsync(ck_state((L - 1) / ck), b->F.p, 10 * gp * sizeof(float),
                                         cudaMemcpyDeviceToDevice, st));
        }
        return RTM_OK;
    };
    auto record_fwd = [&]() -> int {
        if (ck) return record_fwd_ckpt();
        for (int L = 2; L <= nt; L++) TRY(fwd_step(L));
        return snap_last();
    };
    // ---- adjoint pass with the imaging condition: levels nt..1
    auto adj_level = [&](int L) -> int {
        Step2DArgs<float> a = base_args(true);
        for (int f = 0; f < 5; f++) {
            a.out[f] = ab(L & 1, f);
            a.own2[f] = L + 2 <= nt ? ab(L & 1, f) : b->zero.p;
            a.nb[f] = L + 1 <= nt ? ab((L + 1) & 1, f) : b->zero.p;
            a.nb_plane[f] = L + 1 <= nt ? ((L + 1) & 1) * 5 + f : 10;  // past the last plane: zeros
        }
        a.snap_plane[0] = 2 * slot(L);
        a.snap_plane[1] = 2 * slot(L) + 1;
        a.sponge = b->exact_adj;
        a.rec = b->traces.p;
        a.comp_mask = b->comp_mask;
        a.ncomp = b->ncomp;
        a.it = L - 1;
        a.isnap0[0] = snap(L, 0);
        a.isnap0[1] = snap(L, 1);
        a.imax0 = mx(L);
        a.ilast = L == nt;
        a.isnap1[0] = L < nt ? snap(L + 1, 0) : snap(L, 0);
        a.isnap1[1] = L < nt ? snap(L + 1, 1) : snap(L, 1);
        a.imax1 = L < nt ? mx(L + 1) : mx(L);
        set_img(a);
        if (use_march_a) {
            TRY(launch_march_adj(a, madj, mctas, st));
        } else {
            TRY(launch_step<float>(a, true, false, b->tab_a.tx, 0, st, b->tab_a.tz, sta, tha));
        }
        nkern++;
        if (blocked && ((nt - L + 1) % IMG_FOLD == 0 || L == 1)) {
            TRY(fold());
            nkern++;
        }
        return RTM_OK;
    };
    // checkpoint-restart: per segment (last first) restore its forward state,
    // recompute its snapshots (and the next segment's first), migrate through it
    auto record_adj_ckpt = [&]() -> int {
        for (int sgm = nseg - 1; sgm >= 0; sgm--) {
            const int a0 = sgm * ck + 1, b0 = std::min((sgm + 1) * ck, nt);
            if (sgm == 0) {
                RTM_CUDA(cudaMemsetAsync(b->F.p, 0, 10 * gp * sizeof(float), st));
            } else {
                RTM_CUDA(cudaMemcpyAsync(b->F.p, ck_state(sgm), 10 * gp * sizeof(float), cudaMemcpyDeviceToDevice, st));
            }
            const int last = std::min(b0 + 2, nt);
            for (int L = a0 + 1; L <= last; L++) TRY(fwd_step(L));
            if (b0 + 2 > nt) TRY(snap_last());
            for (int L = b0; L >= a0; L--) TRY(adj_level(L));
        }
        return RTM_OK;
    };
    auto record_adj = [&]() -> int {
        if (ck) return record_adj_ckpt();
        for (int L = nt; L >= 1; L--) TRY(adj_level(L));
        return RTM_OK;
    };
    // capture one graph per pass; timing events stay outside the graphs
    cudaGraphExec_t gx[2] = {nullptr, nullptr};
    auto capture = [&](int which, cudaGraphExec_t *out) -> int {
        cudaGraph_t g = nullptr;
        RTM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int s = which == 0 ? record_fwd() : record_adj();
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (s) {
            if (g) cudaGraphDestroy(g);
            return s;
        }
        if (ce != cudaSuccess) {
            rtm_set_error("graph capture failed: %s", cudaGetErrorString(ce));
            return RTM_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            rtm_set_error("graph instantiation failed: %s", cudaGetErrorString(ie));
            return RTM_ERR_CUDA;
        }
        return RTM_OK;
    };
    int rc = RTM_OK;
    if (b->use_graph) {
        rc = capture(0, &gx[0]);
        if (!rc) rc = capture(1, &gx[1]);
        if (!rc) {
            RTM_CUDA(cudaEventRecord(e0, st));
            RTM_CUDA(cudaGraphLaunch(gx[0], st));
            RTM_CUDA(cudaEventRecord(e1, st));
            RTM_CUDA(cudaGraphLaunch(gx[1], st));
            RTM_CUDA(cudaEventRecord(e2, st));
        }
    } else {
        RTM_CUDA(cudaEventRecord(e0, st));
        rc = record_fwd();
        if (!rc) RTM_CUDA(cudaEventRecord(e1, st));
        if (!rc) rc = record_adj();
        if (!rc) RTM_CUDA(cudaEventRecord(e2, st));
    }
    if (rc) {
        for (auto &x : gx) if (x) cudaGraphExecDestroy(x);
        cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
        return rc;
    }
    // ---- stack into the full image
    {
        for (int i = 0; i < ns; i++) {
            dim3 blk(128), grd(ceil_div(nz, 128), b->nxs[s0 + i], 1);
            k_stack<<<grd, blk, 0, st>>>(b->tab.d_geom, i, ld, nz, (long long)nz * b->nx, b->dx0.p, b->img.p,
                                         b->img.p + 3 * gp, gp, b->full.p);
            RTM_CUDA(cudaGetLastError());
        }
    }
    const size_t pf = (size_t)nz * b->nx;
    if (image_dev) {
        RTM_CUDA(cudaMemcpyAsync(image, b->full.p, 3 * pf * sizeof(float), cudaMemcpyDeviceToDevice, st));
    } else {
        RTM_CUDA(cudaMemcpyAsync(image, b->full.p, 3 * pf * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    RTM_CUDA(cudaStreamSynchronize(st));
    TRY(check_tile_loads(b));
    float f_ms = 0, a_ms = 0;
    RTM_CUDA(cudaEventElapsedTime(&f_ms, e0, e1));
    RTM_CUDA(cudaEventElapsedTime(&a_ms, e1, e2));
    b->last_fwd_ms = f_ms;
    b->last_adj_ms = a_ms;
    b->kernels_last = nkern;
    long long cells = 0;
    for (int i = 0; i < ns; i++) cells += (long long)nz * b->nxs[s0 + i];
    b->last_cells = cells;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    for (auto &x : gx) if (x) cudaGraphExecDestroy(x);
    return RTM_OK;
}

}  // namespace

extern "C" rtm_batch *rtm_batch_create(int nz, int nx, int nt, float dx, float dt, float fp, int nsource, int abc,
                                       const float *rho, const float *lambda, const float *mu, int nshots,
                                       const int *x0, const int *nxs, const int *xsrc, const int *zsrc,
                                       const int *zrec, int comp_mask, int group_max, int exact_adjoint)
{
    auto fail = [](int code, const char *msg) -> rtm_batch * {
        if (msg) rtm_set_error("%s", msg);
        (void)code;
        return nullptr;
    };
    if (nz < 11 || nx < 11 || nt < 3 || nshots < 1 || group_max < 1 || !(comp_mask & 31))
        return fail(RTM_ERR_ARG, "rtm_batch_create: bad sizes");
    note_pending("create entry");
    if (ensure_device()) return nullptr;
    note_pending("after ensure_device");
    rtm_batch *b = new rtm_batch();
    b->nz = nz; b->nx = nx; b->nt = nt; b->dx = dx; b->dt = dt; b->fp = fp;
    b->nsource = nsource; b->abc = abc; b->comp_mask = comp_mask & 31; b->exact_adj = exact_adjoint ? 1 : 0;
    b->ncomp = __builtin_popcount(b->comp_mask);
    b->group_max = std::min(group_max, nshots);
    for (int s = 0; s < nshots; s++) {
        const int a0 = x0[s] - 1, w = nxs[s], xs = xsrc[s] - 1, zs = zsrc[s] - 1, zr = zrec[s] - 1;
        if (a0 < 0 || w < abc + 5 || w < 11 || a0 + w > nx || xs < a0 || xs >= a0 + w || zs < 0 || zs >= nz || zr < 0 ||
            zr >= nz || nz < abc + 5) {
            delete b;
            rtm_set_error("rtm_batch_create: shot %d geometry outside the grid or narrower than the sponge", s);
            return nullptr;
        }
        b->x0.push_back(a0); b->nxs.push_back(w); b->xsrc.push_back(xs); b->zsrc.push_back(zs); b->zrec.push_back(zr);
    }
    b->ldz = (nz + 31) / 32 * 32;
    // capacity: the group_max widest shots
    std::vector<int> w(b->nxs);
    std::sort(w.begin(), w.end(), std::greater<int>());
    long long cap = 0;
    for (int i = 0; i < b->group_max; i++) cap += w[i] + GUARD;
    b->cap_cols = cap;
    b->gplane = cap * b->ldz;
    long long tcap = 0;
    for (int i = 0; i < b->group_max; i++) tcap += (long long)w[i] * nt * b->ncomp;
    const size_t gp = (size_t)b->gplane, pf = (size_t)nz * nx;
    int s = 0;
    if (!s) s = b->model.alloc(3 * pf);
    if (!s) s = b->coefraw.alloc(5 * gp);
    if (!s) s = b->coef.alloc(5 * gp);
    if (!s) s = b->F.alloc(10 * gp);
    if (!s) s = b->A.alloc(10 * gp);
    if (!s) s = b->zero.alloc(gp);
    if (!s) s = b->img.alloc(9 * gp);  // sums, compensations, partials
    if (!s) s = b->filt.alloc(abc + 5);
    if (!s) s = b->maxes.alloc((size_t)(nt + 2) * b->group_max * 2);
    if (!s) s = b->traces.alloc((size_t)tcap);
    if (!s) s = b->tstage.alloc((size_t)tcap);
    if (!s) s = b->full.alloc(3 * pf);
    if (!s) {
        // keep every level's snapshots when they fit in 80 % of the free
        // device memory, otherwise checkpoint every ck levels (ck ~ sqrt(10 nt)
        // minimises ring + checkpoint storage)
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        const double full = (double)nt * 2 * gp * sizeof(__half);
        if (full > 0.8 * (double)free_b) {
            int k = (int)std::ceil(std::sqrt(10.0 * nt));
            b->ckpt = std::max(1, std::min(k, nt));
        }
        const int nlev = b->ckpt ? b->ckpt + 1 : nt;
        s = b->snaps.alloc((size_t)nlev * 2 * gp);
        if (!s && b->ckpt) {
            const int nseg = (nt + b->ckpt - 1) / b->ckpt;
            if (nseg > 1) s = b->ck.alloc((size_t)(nseg - 1) * 10 * gp);
        }
    }
    if (!s) s = b->dx0.alloc(b->group_max);
    if (!s) s = b->err.alloc(1);
    note_pending("after allocations");
    if (s) { delete b; return nullptr; }
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        rtm_set_error("stream creation failed");
        return nullptr;
    }
    note_pending("after stream");
    std::vector<float> f(abc + 5), src(nt);
    host_abc_filter<float>(abc, f.data());
    host_ricker<float>(nt, dt, fp, nsource, src.data());
    b->dtsrc.resize(nt);
    for (int i = 0; i < nt; i++) b->dtsrc[i] = dt * src[i];
    const struct { cudaError_t e; const char *what; } ops[] = {
        {cudaMemcpy(b->model.p, rho, pf * sizeof(float), cudaMemcpyHostToDevice), "rho upload"},
        {cudaMemcpy(b->model.p + pf, lambda, pf * sizeof(float), cudaMemcpyHostToDevice), "lambda upload"},
        {cudaMemcpy(b->model.p + 2 * pf, mu, pf * sizeof(float), cudaMemcpyHostToDevice), "mu upload"},
        {cudaMemset(b->zero.p, 0, gp * sizeof(float)), "zero plane"},
        {cudaMemset(b->err.p, 0, sizeof(int)), "error flag"},
        {cudaMemset(b->snaps.p, 0, b->snaps.n * sizeof(__half)), "snapshot store"},
        {cudaMemset(b->coefraw.p, 0, 5 * gp * sizeof(float)), "coefficient planes"},
        {cudaMemset(b->coef.p, 0, 5 * gp * sizeof(float)), "masked coefficient planes"},
        {cudaMemcpy(b->filt.p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice), "filter upload"},
        {cudaDeviceSynchronize(), "synchronize"},
    };
    for (const auto &op : ops)
        if (op.e != cudaSuccess) {
            rtm_set_error("rtm_batch_create: %s failed: %s", op.what, cudaGetErrorString(op.e));
            cudaGetLastError();
            delete b;
            return nullptr;
        }
    note_pending("end of create");
    return b;
}

extern "C" int rtm_batch_migrate(rtm_batch *b, int shot0, int nshot, const float *traces, int traces_on_device,
                                 float *image, int image_on_device)
{
    RTM_CHECK_ARG(b && traces && image, "rtm_batch_migrate: null argument");
    note_pending("migrate entry");
    TRY(ensure_device());
    note_pending("migrate after ensure_device");
    cudaEvent_t t0, t1;
    RTM_CUDA(cudaEventCreate(&t0));
    RTM_CUDA(cudaEventCreate(&t1));
    // the full image accumulates across calls: load the caller's image first
    const size_t pf = (size_t)b->nz * b->nx;
    RTM_CUDA(cudaEventRecord(t0, b->st));
    note_pending("migrate before image load");
    RTM_CUDA(cudaMemcpyAsync(b->full.p, image, 3 * pf * sizeof(float),
                             image_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->st));
    note_pending("migrate after image load");
    int s = batch_group(b, shot0, nshot, traces, traces_on_device, image, image_on_device);
    RTM_CUDA(cudaEventRecord(t1, b->st));
    RTM_CUDA(cudaEventSynchronize(t1));
    float ms = 0;
    if (!s) RTM_CUDA(cudaEventElapsedTime(&ms, t0, t1));
    b->last_total_ms = ms;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return s;
}

extern "C" int rtm_batch_stats(const rtm_batch *b, double *out)
{
    RTM_CHECK_ARG(b && out, "null argument");
    out[0] = b->last_fwd_ms;
    out[1] = b->last_adj_ms;
    out[2] = (double)b->last_cells;
    out[3] = (double)b->kernels_last;
    out[4] = b->last_total_ms;
    out[5] = (double)(b->tx_f > 0 ? b->tx_f : b->tab.tx);
    out[6] = (double)b->tab.ntiles;
    out[7] = (double)(b->tx_a > 0 ? b->tx_a : b->tab_a.tx);
    for (int p = 0; p < 2; p++)
        for (int i = 0; i < 3; i++) {
            double best = -1;
            for (int v = 0; v < 4; v++) {
                const double m = b->tune_ms[p][i][v];
                out[16 + 12 * p + 4 * i + v] = m;
                if (m >= 0 && (best < 0 || m < best)) best = m;
            }
            out[8 + 3 * p + i] = best;
        }
    out[14] = b->st_f;
    out[15] = b->st_a;
    out[40] = b->th_f;
    out[41] = b->th_a;
    out[42] = b->ckpt;
    out[43] = b->use_tma ? 1 : 0;
    out[44] = b->use_tma && (b->march < 0 ? b->march_tuned : (b->march & 1) != 0) ? 1 : 0;
    out[45] = b->tune_march_ms;
    out[46] = b->use_tma && (b->march < 0 ? b->march_tuned_a : (b->march & 2) != 0) ? 1 : 0;
    out[47] = b->tune_march_ms_a;
    return RTM_OK;
}

extern "C" int rtm_batch_set(rtm_batch *b, int use_graph, int tile_x)
{
    RTM_CHECK_ARG(b, "null argument");
    RTM_CHECK_ARG(tile_x == 0 || tile_x == 8 || tile_x == 16 || tile_x == 32, "tile_x must be 0, 8, 16 or 32");
    b->use_graph = use_graph != 0;
    b->tile_x = tile_x;
    return RTM_OK;
}

extern "C" int rtm_batch_set_tma(rtm_batch *b, int on)
{
    RTM_CHECK_ARG(b, "null argument");
    if (on) RTM_CHECK_ARG(tensor_maps_available(), "tensor maps are not available from the driver");
    b->use_tma = on != 0;
    return RTM_OK;
}

extern "C" int rtm_batch_set_march(rtm_batch *b, int mode)
{
    RTM_CHECK_ARG(b && mode >= -1 && mode <= 3, "mode must be -1 .. 3");
    b->march = mode;
    return RTM_OK;
}

extern "C" int rtm_batch_set_test_stall(rtm_batch *b, int on)
{
    RTM_CHECK_ARG(b, "null argument");
    if (on) {
        TRY(ensure_device());
        if (!b->stall.p) {
            TRY(b->stall.alloc(1));
            RTM_CUDA(cudaMemset(b->stall.p, 0, sizeof(int)));
        }
    }
    b->test_stall = on != 0;
    return RTM_OK;
}

extern "C" int rtm_batch_set_checkpoint(rtm_batch *b, int interval)
{
    RTM_CHECK_ARG(b && interval >= 0, "bad arguments");
    TRY(ensure_device());
    const int k = std::min(interval, b->nt);
    const size_t gp = (size_t)b->gplane;
    b->snaps.release();
    b->ck.release();
    b->ckpt = k;
    const int nlev = k ? k + 1 : b->nt;
    TRY(b->snaps.alloc((size_t)nlev * 2 * gp));
    RTM_CUDA(cudaMemset(b->snaps.p, 0, b->snaps.n * sizeof(__half)));
    if (k) {
        const int nseg = (b->nt + k - 1) / k;
        if (nseg > 1) TRY(b->ck.alloc((size_t)(nseg - 1) * 10 * gp));
    }
    return RTM_OK;
}

extern "C" int rtm_batch_set_stages(rtm_batch *b, int fwd, int adj, int threads_fwd, int threads_adj)
{
    RTM_CHECK_ARG(b, "null argument");
    RTM_CHECK_ARG(fwd >= 1 && fwd <= 2 && adj >= 1 && adj <= 2, "stages must be 1 or 2");
    RTM_CHECK_ARG((threads_fwd == 256 || threads_fwd == 512) && (threads_adj == 256 || threads_adj == 512),
                  "threads must be 256 or 512");
    b->st_f = fwd;
    b->st_a = adj;
    b->th_f = threads_fwd;
    b->th_a = threads_adj;
    return RTM_OK;
}

extern "C" int rtm_batch_autotune(rtm_batch *b, int shot0, int nshot, int steps)
{
    RTM_CHECK_ARG(b && steps > 0, "bad arguments");
    TRY(ensure_device());
    b->tx_f = b->tx_a = 0;
    b->st_f = b->st_a = 1;
    b->th_f = b->th_a = 256;
    b->march_tuned = b->march_tuned_a = true;
    b->tune_march_ms = b->tune_march_ms_a = -1;
    // traces are not read during tuning beyond the receiver row; use the
    // staging buffer content as is
    TRY(batch_group(b, shot0, nshot, b->tstage.p, 1, b->full.p, 1, steps));
    RTM_CUDA(cudaStreamSynchronize(b->st));
    return RTM_OK;
}

extern "C" void rtm_batch_destroy(rtm_batch *b) { delete b; }

// Diagnostic: the marching kernels' work plan for shots of widths nxs[] and
// depth nz over `ctas` CTAs (not part of the public header; no device use).
// runs[4 * i ..] = (shot, first row, first chunk, end chunk) of run i, lo[b]
// = first run of CTA b (ctas + 1 entries).  Returns the number of runs, or -1
// when max_runs is too small.
extern "C" int rtm_debug_march_plan(int nshots, const int *nxs, int nz, int ctas, int *runs, int max_runs, int *lo)
{
    if (nshots < 1 || nz < 1 || ctas < 1 || !nxs || !runs || !lo) return -1;
    std::vector<HostShot> shots(nshots);
    for (int i = 0; i < nshots; i++) {
        shots[i] = HostShot{};
        shots[i].nz = nz;
        shots[i].nx = nxs[i];
    }
    std::vector<int4> r;
    std::vector<int> l;
    march_plan(shots, ctas, r, l);
    if ((int)r.size() > max_runs) return -1;
    for (size_t i = 0; i < r.size(); i++) {
        runs[4 * i] = r[i].x;
        runs[4 * i + 1] = r[i].y;
        runs[4 * i + 2] = r[i].z;
        runs[4 * i + 3] = r[i].w;
    }
    for (int b = 0; b <= ctas; b++) lo[b] = l[b];
    return (int)r.size();
}

// Diagnostic: the pending CUDA error of this library's runtime and where it
// was first seen (not part of the public header).
extern "C" int rtm_debug_peek(char *where, int n)
{
    if (where && n > 0) snprintf(where, n, "%s", g_pending_at);
    return (int)cudaPeekAtLastError();
}

extern "C" void *rtm_host_alloc(size_t bytes)
{
    void *p = nullptr;
    note_pending("host_alloc entry");
    if (ensure_device()) return nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        rtm_set_error("cudaMallocHost of %zu bytes failed", bytes);
        return nullptr;
    }
    return p;
}

extern "C" void rtm_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}
