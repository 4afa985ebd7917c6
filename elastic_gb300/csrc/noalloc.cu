// rtm_op3_dev_noalloc: the adjoint recursion of rtm_op3_c_ on caller-owned
// device buffers, without allocating any memory.
//
// Who needs it: code that may not call cudaMalloc/cudaFree at the point where
// it migrates -- a host that has handed all device memory to its own pool
// allocator (a framework's caching allocator, an MPI/NCCL runtime that
// registered its buffers), a callback running where an allocation would
// implicitly synchronise the device or fail under memory pressure, or a
// long-running service that must not fragment the device heap.  Such a
// caller owns the five wavefield histories and the five coefficient planes
// on the device and passes them in; everything else this computation needs
// lives in the fixed scratch array below.
//
// Scratch: `g_noalloc_scratch`, a file-scope __device__ array holding the five
// masked coefficient planes (at most RTM_NOALLOC_MAX_CELLS cells each) and the
// one-shot work-item table.  It occupies 10 MiB (+256 B) on every GPU on which
// this library's kernels run, for the life of the process.  All calls share
// it and it keeps the previous call's contents: every call rewrites the
// planes it reads (masking zeroes everything outside the operator ranges)
// before the recursion uses them, and rewrites the table.  Two calls whose
// GPU work overlaps (different host threads, or different streams without
// ordering) race on the scratch and give wrong results.
//
// Set-up: the first call on a device looks up the device address of the
// array with cudaGetSymbolAddress (with that device current) and keeps it;
// make that first call before any stream capture is started on the device.
#include <mutex>

#include "../../include/elastic_rtm.h"
#include "elastic2d.cuh"
#include "engine.h"

using namespace eg;

namespace {

constexpr size_t kPlane = RTM_NOALLOC_MAX_CELLS;
constexpr size_t kGeomFloats = 64;  // >= sizeof(ShotGeom) / 4, rounded for alignment

static __device__ __align__(256) float g_noalloc_scratch[5 * kPlane + kGeomFloats];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
float *g_scratch_addr[kMaxDevices] = {};

int scratch_address(float **out)
{
    int dev = 0;
    RTM_CUDA(cudaGetDevice(&dev));
    RTM_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        RTM_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = static_cast<float *>(p);
    }
    *out = g_scratch_addr[dev];
    return RTM_OK;
}

}  // namespace

extern "C" int rtm_op3_dev_noalloc(int nt, int nz, int nx, float *Vx0_dev, float *Vz0_dev, float *sigmaxx0_dev,
                                   float *sigmazz0_dev, float *sigmaxz0_dev, const float *m1_x_dev,
                                   const float *m1_z_dev, const float *aux_m2_c_dev, const float *aux_m3_c_dev,
                                   const float *aux_m2m3_c_dev, void *stream)
{
    RTM_CHECK_ARG(nt >= 3 && nz >= 11 && nx >= 11, "rtm_op3_dev_noalloc: grid too small (nt=%d nz=%d nx=%d)", nt, nz,
                  nx);
    RTM_CHECK_ARG((size_t)nz * (size_t)nx <= kPlane,
                  "rtm_op3_dev_noalloc: nz*nx = %zu cells exceeds the fixed scratch of %zu cells per plane",
                  (size_t)nz * (size_t)nx, kPlane);
    float *H[5] = {Vx0_dev, Vz0_dev, sigmaxx0_dev, sigmazz0_dev, sigmaxz0_dev};
    const float *C[5] = {m1_x_dev, m1_z_dev, aux_m2_c_dev, aux_m3_c_dev, aux_m2m3_c_dev};
    for (int f = 0; f < 5; f++) RTM_CHECK_ARG(H[f] && C[f], "rtm_op3_dev_noalloc: null pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *scratch = nullptr;
    TRY(scratch_address(&scratch));
    const size_t plane = (size_t)nz * nx;
    float *cm[5];
    for (int f = 0; f < 5; f++) cm[f] = scratch + f * kPlane;
    ShotGeom *geom = reinterpret_cast<ShotGeom *>(scratch + 5 * kPlane);

    // masked coefficient planes (every cell rewritten)
    TRY(mask_coefs<float>(nz, nx, C, nz, cm, nz, st));

    // one-shot work-item table
    const void *ptrs[10];
    for (int f = 0; f < 5; f++) { ptrs[f] = H[f]; ptrs[5 + f] = cm[f]; }
    const bool v2 = v2_usable(true, nz, ptrs, 10) && (plane % 4) == 0;
    const int tz = v2 ? TZ_TILE2 : TZ_TILE;
    int tx = pick_tile_width(nz, nx, tz);
    while (v2 && tx > 8 && !v2_fits(true, true, tx)) tx /= 2;
    ShotGeom g;
    memset(&g, 0, sizeof g);
    g.nz = nz;
    g.nx = nx;
    g.src_iz = g.src_ix = g.rec_iz = -1;
    g.ntz = ceil_div(nz, tz);
    const int ntiles = g.ntz * ceil_div(nx, tx);
    RTM_CUDA(cudaMemcpyAsync(geom, &g, sizeof g, cudaMemcpyHostToDevice, st));

    // levels nt-3 .. 0, exact arithmetic (same kernels as rtm_op3_c_)
    for (int it = nt - 3; it >= 0; it--) {
        Step2DArgs<float> a;
        memset(&a, 0, sizeof a);
        for (int f = 0; f < 5; f++) {
            a.coef[f] = cm[f];
            a.out[f] = H[f] + (size_t)it * plane;
            a.inplane[f] = a.out[f];
            a.own2[f] = H[f] + (size_t)(it + 2) * plane;
            a.nb[f] = H[f] + (size_t)(it + 1) * plane;
        }
        a.shots = geom;
        a.nshots = 1;
        a.ntiles = ntiles;
        a.ldz = nz;
        TRY(launch_step<float>(a, true, true, tx, 0, st, tz));
    }
    RTM_CUDA(cudaStreamSynchronize(st));
    return RTM_OK;
}
