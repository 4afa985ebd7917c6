// Host-side building blocks shared by the 2D elastic entry points.
#pragma once
#include <cuda.h>

#include <vector>

#include "common.cuh"
#include "elastic2d.cuh"

#define TRY(x)                   \
    do {                         \
        int s_ = (x);            \
        if (s_) return s_;       \
    } while (0)

namespace eg {

constexpr int TZ_TILE = 32;   // v1 tile height (one warp along z)
constexpr int TZ_TILE2 = 128; // v2 tile height (32 lanes x 4 cells)

// Kernel version: 0 = automatic (v2 where the layout allows), 1 or 2 forced
// (a forced v2 on an unaligned layout runs v1).
int kernel_version();

int ensure_device();
int device_sm_count();

// Tensor maps for bulk tensor copies, encoded through the runtime's driver
// entry point (no link against the driver library).  make_map: a 3D map of
// ldz rows x cols columns x planes (plane stride plane_elems elements), FP32
// or FP16, box of box_rows x box_cols x 1, zero fill outside the tensor.
bool tensor_maps_available();
int make_map(CUtensorMap *m, const void *base, bool half, int ldz, long long cols, long long planes,
             long long plane_elems, int box_rows, int box_cols);
// Tensor map of rank 1..5 over BF16 (bf16) or FP32 elements: dims[i]
// elements along dimension i (0 innermost, unit stride), strides_b[i] bytes
// between elements of dimension i + 1, a box of box[i] elements, swizzle of
// 0, 32, 64 or 128 bytes, zero fill outside the tensor.
int make_map_nd(CUtensorMap *m, const void *base, bool bf16, int rank, const long long *dims, const long long *strides_b,
                const int *box, int swizzle);

// Owning device allocation that grows on demand.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count)
    {
        if (count <= n && p) return RTM_OK;
        release();
        if (count == 0) return RTM_OK;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            rtm_set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
            return RTM_ERR_NOMEM;
        }
        n = count;
        return RTM_OK;
    }
};

// One shot of a batch as the host sees it (0-based cells; -1 = none).
struct HostShot {
    long long off;   // element offset of the shot's planes
    long long doff;  // element offset of the shot's traces
    int nz, nx;
    int src_iz, src_ix;
    int rec_iz;
};

// Work-item table of a batch for a given tile width (device copy in d_geom).
struct ShotTable {
    std::vector<HostShot> shots;
    int ldz = 0;
    int tx = 16;
    int tz = TZ_TILE;
    int ntiles = 0;
    ShotGeom *d_geom = nullptr;
    ShotTable() = default;
    ShotTable(const ShotTable &) = delete;
    ShotTable &operator=(const ShotTable &) = delete;
    ~ShotTable();
    int build(int tx, int tz = TZ_TILE);
};

// Tile width giving at least two work items per SM when the grid allows.
inline int pick_tile_width(long long cells_z, long long cells_x, int tz = TZ_TILE)
{
    const long long ntz = (cells_z + tz - 1) / tz;
    const long long want = 2LL * device_sm_count();
    for (int tx : {32, 16}) if (ntz * ((cells_x + tx - 1) / tx) >= want) return tx;
    return 8;
}

template <typename T>
int launch_step(const Step2DArgs<T> &a, bool adj, bool exact, int tx, int grid_cap, cudaStream_t st, int tz = TZ_TILE,
                int stages = 1, int threads = 256);

// True when a float step on planes with pitch ldz starting at `ptrs` can use v2.
bool v2_usable(bool is_float, int ldz, const void *const *ptrs, int n);
// True when the v2 kernel of this flavour and tile width fits in shared memory.
bool v2_fits(bool adj, bool exact, int tx);
// v2 tile of width tx with `stages` staging buffers (1 or 2) and `threads`
// threads (256, or 512 for the fast kernels with tx >= 16) fits in a block
bool v2_fits(bool adj, bool exact, int tx, int stages, int threads = 256);
size_t v2_stage_bytes(bool adj, bool exact, int tx);
int max_smem_optin();

template <typename T>
int model_coefs(int nz, int nx, T dx, T dt, const T *d_rho, const T *d_lam, const T *d_mu, int ldin, T *m1x, T *m1z,
                T *m2o, T *m3o, T *a2, T *a3, T *a23, int ldout, cudaStream_t st);

template <typename T>
int mask_coefs(int nz, int nx, const T *const in[5], int ldin, T *const out[5], int ldout, cudaStream_t st);

template <typename T>
void host_abc_filter(int abc, T *filter);

template <typename T>
void host_ricker(int nt, T dt, T fp, int nsource, T *source);

}  // namespace eg
