// Single-domain 3D acoustic propagator, 10th order in space, 2nd in time,
// and 3D RTM with reverse-time restart of the source wavefield (sm_103a).
//
// Reference (lgan/elastic, W = 2d_rtm_restart/Src_working), raised from its
// 8th-order stencil to 10th order:
//   W/wave_fkernel.3d8o.cu:31-106   p2 = vel*L(p1) + p1 + p1 - p0, vel = v^2 dt^2
//   W/wave_fkernel.3d8o.cu:183-210  sponge p0, p1 *= exp(-b(a-edge)) before each step
//   W/gpu_funcs_3d.cu:64-131        source injection, receiver extraction, imaging
//   W/gpu_funcs_3d.cu:509-712       adjoint with the source wavefield restarted
//                                   backwards from its last two slices
//
// Layout: p[(iy*n2 + ix)*n1 + iz], iz fastest; interior cells [5, n-5) on
// every axis are updated, the 5-cell rim stays zero.
//
// Kernel (2.5-D): a CTA covers 128 z-rows x TX columns and marches along y.
// Each thread owns 4 consecutive z cells of one column: an 11-slice register
// queue of float4 gives the y taps; the current slice with its x and z halo
// sits in shared memory for the x and z taps.  DRAM traffic per cell-update
// is p1 + p0 + vel read, p2 written (16 B).
//
// Sponge, fused: planes are stored pre-damped.  The reference damps p1 and
// p0 in place before each step, so every stored level is multiplied by the
// factor once as "p1" and once more as "p0".  Writing f*p2 and reading
// f*p0 reproduces that exactly (same products, same rounding).  Receivers see
// the undamped level, as in the reference (they record before the next
// step's damping).
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/elastic_rtm.h"
#include "common.cuh"
#include "elastic2d_v2.cuh"
#include "engine.h"

using namespace eg;

namespace {

constexpr int AR = 5;            // stencil radius
constexpr int A_TZ = 128;        // tile rows (32 lanes x 4)
constexpr int A_ZH = 8;          // aligned z halo
constexpr int A_LZ = A_TZ + 2 * A_ZH;

struct Ac3DArgs {
    const float *p0;   // level t-1 (stored, pre-damped)
    const float *p1;   // level t   (stored, pre-damped)
    float *p2;         // level t+1 output (may alias p0)
    const float *vel;  // v^2 dt^2
    int n1, n2, n3;
    float coef[16];    // C0, then (z, x, y) per offset 1..5
    const float *damp; // factor per edge distance, damp_a entries (nullable)
    int damp_a;
    long long src_o;   // linear offset of the source cell, -1 none
    float src_val;     // added to the raw p2 at the source cell
    int zr;            // receiver plane (0-based), -1 none
    float *rec_out;    // record raw p2 at iz=zr into rec_out[iy*n2+ix]
    const float *rec_in;  // add rec_in[iy*n2+ix] to p2 at iz=zr
    float *img;        // img += (1e-6*p2_raw)*simg  (nullable)
    const float *simg;
    int y0, y1;        // y range of the march handled by a CTA chunk: [y0, y1)
    int ychunks;       // number of y chunks
    int *err;          // set by a kernel whose bounded wait ran out (ring kernel)
    int raw_out;       // store p2 undamped: the last level of a run, which the
                       // reference leaves raw (no later step damps it)
};

__device__ __forceinline__ int edge_dist(int i, int n)
{
    const int lo = i - AR, hi = (n - 1 - AR) - i;
    return lo < hi ? lo : hi;
}

template <bool EXACT>
__device__ __forceinline__ float damp_of(const Ac3DArgs &a, int iz, int ix, int iy)
{
    if (!a.damp) return 1.f;
    int e = edge_dist(iz, a.n1);
    e = min(e, edge_dist(ix, a.n2));
    e = min(e, edge_dist(iy, a.n3));
    if (e >= 0 && e < a.damp_a) {
        const float t = __ldg(a.damp + e);
        return t < 1.f ? t : 1.f;
    }
    return 1.f;
}

template <bool EXACT>
__device__ __forceinline__ float fm(float x, float y) { return EXACT ? __fmul_rn(x, y) : x * y; }
template <bool EXACT>
__device__ __forceinline__ float fa(float x, float y) { return EXACT ? __fadd_rn(x, y) : x + y; }
template <bool EXACT>
__device__ __forceinline__ float fs(float x, float y) { return EXACT ? __fsub_rn(x, y) : x - y; }

__device__ __forceinline__ float e4(const float4 &v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

// The complete update of a thread's 4 cells (rows z..z+3 of column x at
// slice y, offset o of row z): the sponge factor, the source, the receiver
// row, the imaging condition and the rim (rows outside the interior stay
// zero).  acc: the Laplacian sums, p: p1 at the cells.  Threads whose cells
// touch none of these take the straight-line update in the kernels instead
// (same arithmetic with a factor of one); this branch is rarely taken.
template <bool EXACT>
__device__ __forceinline__ float4 cells_full(const Ac3DArgs &a, int z, int x, int y, long long o, float4 acc4,
                                          float4 p4, float4 p0c, float4 velc)
{
    const float acc[4] = {acc4.x, acc4.y, acc4.z, acc4.w}, p[4] = {p4.x, p4.y, p4.z, p4.w};
    float out[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int zz = z + j;
        const bool inside = zz >= AR && zz < a.n1 - AR;
        const float f = damp_of<EXACT>(a, zz, x, y);
        const float p0v = e4(p0c, j);
        const float p0d = f == 1.f ? p0v : fm<EXACT>(f, p0v);
        float v = fs<EXACT>(fa<EXACT>(fa<EXACT>(fm<EXACT>(e4(velc, j), acc[j]), p[j]), p[j]), p0d);
        const long long oj = o + j;
        if (oj == a.src_o) v = fa<EXACT>(v, a.src_val);
        if (inside && zz == a.zr) {
            const long long ri = (long long)y * a.n2 + x;
            if (a.rec_in) v = fa<EXACT>(v, a.rec_in[ri]);
            if (a.rec_out) a.rec_out[ri] = v;
        }
        if (inside && a.img) a.img[oj] = fa<EXACT>(a.img[oj], fm<EXACT>(fm<EXACT>(1e-6f, v), a.simg[oj]));
        out[j] = inside ? ((f == 1.f || a.raw_out) ? v : fm<EXACT>(f, v)) : 0.f;
    }
    return make_float4(out[0], out[1], out[2], out[3]);
}

// True when none of a thread's 4 cells (rows z..z+3, column x) is on the
// rim, the source or the receiver row, and no image is formed: then, on a
// slice outside the sponge, the plain update applies.
__device__ __forceinline__ bool cells_plain(const Ac3DArgs &a, int z, int x)
{
    if (a.img || z < AR || z + 3 >= a.n1 - AR) return false;
    if ((a.rec_in || a.rec_out) && a.zr >= z && a.zr < z + 4) return false;
    if (a.src_o >= 0) {
        const long long s3 = (long long)a.n1 * a.n2;
        const long long r = a.src_o % s3;
        if (r / a.n1 == x && r % a.n1 >= z && r % a.n1 < z + 4) return false;
    }
    return true;
}

// Sponge distance of the thread's 4 rows and column (the slice's own
// distance is added per slice).
__device__ __forceinline__ int cells_edge(int z, int x, int n1, int n2)
{
    int e = edge_dist(x, n2);
#pragma unroll
    for (int j = 0; j < 4; j++) e = min(e, edge_dist(z + j, n1));
    return e;
}

template <bool EXACT, int TX>
__global__ void __launch_bounds__(TX * 32) k_acoustic3d(const __grid_constant__ Ac3DArgs a)
{
    __shared__ __align__(16) float sl[(TX + 2 * AR) * A_LZ];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;  // warp = column in tile
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3;
    const int ntz = (n1 - 2 * AR + A_TZ - 1) / A_TZ;
    const int ntx = (n2 - 2 * AR + TX - 1) / TX;
    int b = blockIdx.x;
    const int yc = b % a.ychunks;
    b /= a.ychunks;
    const int tzi = b % ntz, txi = b / ntz;
    const int z0 = AR + tzi * A_TZ, x0 = AR + txi * TX;
    const int ylen = (n3 - 2 * AR + a.ychunks - 1) / a.ychunks;
    const int ya = AR + yc * ylen, yb = min(n3 - AR, ya + ylen);
    if (ya >= yb) return;
    const int z = z0 + 4 * lane, x = x0 + warp;  // this thread's cells z..z+3 at column x
    const bool colok = x < n2 - AR;
    const long long s2 = n1, s3 = (long long)n1 * n2;
    // Interior rows start at 5, so the 4 cells of a thread are not 16-byte
    // aligned: the queue and the own-cell loads are scalar.
    // Queue q[k] = p1 at (z..z+3, x, y-5+k).
    float q[11][4];
#pragma unroll
    for (int k = 0; k < 11; k++)
#pragma unroll
        for (int j = 0; j < 4; j++) q[k][j] = 0.f;  // columns beyond the interior stay zero
    auto ld4 = [&](const float *p, long long o, float out[4]) {
#pragma unroll
        for (int j = 0; j < 4; j++) out[j] = (z + j < n1 - AR) ? __ldg(p + o + j) : 0.f;
    };
    const long long ocol = (long long)x * s2 + z;
    if (colok)
#pragma unroll
        for (int k = 0; k < 10; k++) ld4(a.p1, ocol + (long long)(ya - 5 + k) * s3, q[k + 1]);
    const float *coef = a.coef;
    for (int y = ya; y < yb; y++) {
        // advance the queue: q[0..9] <- q[1..10], q[10] <- p1(y+5)
#pragma unroll
        for (int k = 0; k < 10; k++)
#pragma unroll
            for (int j = 0; j < 4; j++) q[k][j] = q[k + 1][j];
        if (colok) ld4(a.p1, ocol + (long long)(y + 5) * s3, q[10]);
        __syncthreads();  // previous slice consumed
        // centre of the slice from the queue
        {
            float *d = sl + (warp + AR) * A_LZ + (4 * lane + A_ZH);
#pragma unroll
            for (int j = 0; j < 4; j++) d[j] = q[5][j];
        }
        // z halo (rows z0-8..z0-1 and z0+128..z0+135) and x halo (5 columns each side)
        {
            const long long sy = (long long)y * s3;
            for (int e = threadIdx.x; e < TX * 2 * A_ZH; e += blockDim.x) {
                const int c = e / (2 * A_ZH), r = e % (2 * A_ZH);
                const int zz = r < A_ZH ? z0 - A_ZH + r : z0 + A_TZ + (r - A_ZH);
                const int xx = x0 + c;
                const float v = (zz >= 0 && zz < n1 && xx < n2) ? __ldg(a.p1 + sy + (long long)xx * s2 + zz) : 0.f;
                sl[(c + AR) * A_LZ + (zz - z0 + A_ZH)] = v;
            }
            for (int e = threadIdx.x; e < 2 * AR * A_LZ; e += blockDim.x) {
                const int c = e / A_LZ, r = e % A_LZ;
                const int xx = c < AR ? x0 - AR + c : x0 + TX + (c - AR);
                const int zz = z0 - A_ZH + r;
                const float v = (zz >= 0 && zz < n1 && xx >= 0 && xx < n2) ? __ldg(a.p1 + sy + (long long)xx * s2 + zz) : 0.f;
                sl[(c < AR ? c : TX + c) * A_LZ + r] = v;
            }
        }
        __syncthreads();
        if (!colok) continue;
        const long long o = ocol + (long long)y * s3;
        float vel4[4], p04[4];
        ld4(a.vel, o, vel4);
        ld4(a.p0, o, p04);
        float w[20];  // z window rows z-8..z+11 at column x
        {
            const float *c = sl + (warp + AR) * A_LZ + (4 * lane + A_ZH) - 8;
#pragma unroll
            for (int i = 0; i < 20; i++) w[i] = c[i];
        }
        float outv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float p = q[5][j];
            float acc = fm<EXACT>(coef[0], p);
#pragma unroll
            for (int k = 1; k <= 5; k++) {
                const float zp = fa<EXACT>(w[8 + j + k], w[8 + j - k]);
                const float xp = fa<EXACT>(sl[(warp + AR + k) * A_LZ + (4 * lane + A_ZH + j)],
                                           sl[(warp + AR - k) * A_LZ + (4 * lane + A_ZH + j)]);
                const float yp = fa<EXACT>(q[5 + k][j], q[5 - k][j]);
                acc = fa<EXACT>(acc, fm<EXACT>(coef[1 + 3 * (k - 1)], zp));
                acc = fa<EXACT>(acc, fm<EXACT>(coef[2 + 3 * (k - 1)], xp));
                acc = fa<EXACT>(acc, fm<EXACT>(coef[3 + 3 * (k - 1)], yp));
            }
            const int zz = z + j;
            const float f = damp_of<EXACT>(a, zz, x, y);
            const float p0d = f == 1.f ? p04[j] : fm<EXACT>(f, p04[j]);
            float v = fs<EXACT>(fa<EXACT>(fa<EXACT>(fm<EXACT>(vel4[j], acc), p), p), p0d);
            const long long oj = o + j;
            if (oj == a.src_o) v = fa<EXACT>(v, a.src_val);
            if (zz == a.zr) {
                const long long ri = (long long)y * n2 + x;
                if (a.rec_in) v = fa<EXACT>(v, a.rec_in[ri]);
                if (a.rec_out) a.rec_out[ri] = v;
            }
            if (a.img && zz < n1 - AR) a.img[oj] = fa<EXACT>(a.img[oj], fm<EXACT>(fm<EXACT>(1e-6f, v), a.simg[oj]));
            outv[j] = (f == 1.f || a.raw_out) ? v : fm<EXACT>(f, v);
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (z + j < n1 - AR) a.p2[o + j] = outv[j];
    }
}

// Pipelined 2.5-D kernel for n1 % 4 == 0 (16-byte aligned columns).  Tiles
// start at row 4 + 128k so that every thread's 4 cells form one aligned
// float4; rows outside the interior are computed as zero and stay zero.
// Per y slice: the x/z halo of the NEXT slice is staged by cp.async into the
// other half of a double buffer and the next queue / p0 / vel values are
// loaded into registers while the current slice is computed; one barrier
// per slice.
__device__ __forceinline__ void acp16(float *smem, const float *gmem, bool ok)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(ok ? 16 : 0));
}

template <bool EXACT, int TX>
__global__ void __launch_bounds__(TX * 32, TX == 8 ? 2 : 1) k_acoustic3d_p(const __grid_constant__ Ac3DArgs a)
{
    __shared__ __align__(16) float buf[2][(TX + 2 * AR) * A_LZ];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3;
    const int ntz = (n1 - 9 + A_TZ - 1) / A_TZ;  // rows 4 .. n1-6 (interior plus row 4)
    const int ntx = (n2 - 2 * AR + TX - 1) / TX;
    int b = blockIdx.x;
    const int yc = b % a.ychunks;
    b /= a.ychunks;
    const int tzi = b % ntz, txi = b / ntz;
    const int z0 = 4 + tzi * A_TZ, x0 = AR + txi * TX;
    const int ylen = (n3 - 2 * AR + a.ychunks - 1) / a.ychunks;
    const int ya = AR + yc * ylen, yb = min(n3 - AR, ya + ylen);
    if (ya >= yb) return;
    const int z = z0 + 4 * lane, x = x0 + warp;
    const bool colok = x < n2 - AR;
    const bool grp = colok && z < n1;  // this thread's float4 exists
    const long long s2 = n1, s3 = (long long)n1 * n2;
    const long long ocol = (long long)x * s2 + z;
    const bool plain = cells_plain(a, z, x);
    const int ezx = cells_edge(z, x, n1, n2);
    auto L4 = [&](const float *p, long long o) -> float4 {
        return grp ? __ldg(reinterpret_cast<const float4 *>(p + o)) : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    // halo staging of slice y into buffer h (z halo rows of the tile columns,
    // x halo columns over all 144 rows), 16-byte chunks
    auto stage = [&](int y, float *h) {
        const long long sy = (long long)y * s3;
        constexpr int ZCH = 4 * TX, XCH = 2 * AR * (A_LZ / 4);
        for (int e = threadIdx.x; e < ZCH + XCH; e += blockDim.x) {
            int col, r4;
            if (e < ZCH) {
                col = AR + e / 4;
                const int q = e % 4;
                r4 = q < 2 ? 4 * q : A_ZH + A_TZ + 4 * (q - 2);
            } else {
                const int f = e - ZCH;
                const int c = f / (A_LZ / 4);
                col = c < AR ? c : TX + c;
                r4 = 4 * (f % (A_LZ / 4));
            }
            const int xx = x0 - AR + col, zz = z0 - A_ZH + r4;
            const bool ok = xx >= 0 && xx < n2 && zz >= 0 && zz < n1;
            acp16(h + col * A_LZ + r4, a.p1 + (ok ? sy + (long long)xx * s2 + zz : 0), ok);
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };
    float4 q[11];
#pragma unroll
    for (int k = 0; k < 11; k++) q[k] = L4(a.p1, ocol + (long long)(ya - 5 + k) * s3);
    stage(ya, buf[ya & 1]);
    // every column writes its centre (zero outside the interior): the
    // x taps of edge cells read these slots
    *reinterpret_cast<float4 *>(buf[ya & 1] + (warp + AR) * A_LZ + (4 * lane + A_ZH)) = q[5];
    float4 p0c = L4(a.p0, ocol + (long long)ya * s3), velc = L4(a.vel, ocol + (long long)ya * s3);
    asm volatile("cp.async.wait_group 0;\n" ::);
    __syncthreads();
    const float *coef = a.coef;
    for (int y = ya; y < yb; y++) {
        const bool more = y + 1 < yb;
        float4 qn = make_float4(0.f, 0.f, 0.f, 0.f), p0n = qn, veln = qn;
        if (more) {
            stage(y + 1, buf[(y + 1) & 1]);
            qn = L4(a.p1, ocol + (long long)(y + 6) * s3);
            p0n = L4(a.p0, ocol + (long long)(y + 1) * s3);
            veln = L4(a.vel, ocol + (long long)(y + 1) * s3);
        }
        if (grp) {
            const float *sl = buf[y & 1];
            const float *cz = sl + (warp + AR) * A_LZ + (4 * lane + A_ZH);
            float w[20];
#pragma unroll
            for (int i = 0; i < 20; i += 4) {
                const float4 t = *reinterpret_cast<const float4 *>(cz - 8 + i);
                w[i] = t.x; w[i + 1] = t.y; w[i + 2] = t.z; w[i + 3] = t.w;
            }
            const long long o = ocol + (long long)y * s3;
            // offset-outer, cell-inner: each cell's sum keeps the order
            // C0, then (z, x, y) for offsets 1..5
            float accv[4];
#pragma unroll
            for (int j = 0; j < 4; j++) accv[j] = fm<EXACT>(coef[0], e4(q[5], j));
#pragma unroll
            for (int k = 1; k <= 5; k++) {
                const float4 xm = *reinterpret_cast<const float4 *>(cz - k * A_LZ);
                const float4 xp = *reinterpret_cast<const float4 *>(cz + k * A_LZ);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float zp = fa<EXACT>(w[8 + j + k], w[8 + j - k]);
                    const float xq = fa<EXACT>(e4(xp, j), e4(xm, j));
                    const float yp = fa<EXACT>(e4(q[5 + k], j), e4(q[5 - k], j));
                    accv[j] = fa<EXACT>(accv[j], fm<EXACT>(coef[1 + 3 * (k - 1)], zp));
                    accv[j] = fa<EXACT>(accv[j], fm<EXACT>(coef[2 + 3 * (k - 1)], xq));
                    accv[j] = fa<EXACT>(accv[j], fm<EXACT>(coef[3 + 3 * (k - 1)], yp));
                }
            }
            float out[4], pv[4];
#pragma unroll
            for (int j = 0; j < 4; j++) pv[j] = e4(q[5], j);
            if (__builtin_expect(plain && (!a.damp || min(ezx, edge_dist(y, n3)) >= a.damp_a), 1)) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    out[j] = fs<EXACT>(fa<EXACT>(fa<EXACT>(fm<EXACT>(e4(velc, j), accv[j]), pv[j]), pv[j]), e4(p0c, j));
            } else {
                const float4 r = cells_full<EXACT>(a, z, x, y, o, make_float4(accv[0], accv[1], accv[2], accv[3]),
                                                   q[5], p0c, velc);
                out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
            }
            *reinterpret_cast<float4 *>(a.p2 + o) = make_float4(out[0], out[1], out[2], out[3]);
        }
        if (more) *reinterpret_cast<float4 *>(buf[(y + 1) & 1] + (warp + AR) * A_LZ + (4 * lane + A_ZH)) = q[6];
        asm volatile("cp.async.wait_group 0;\n" ::);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 10; k++) q[k] = q[k + 1];
        q[10] = qn;
        p0c = p0n;
        velc = veln;
    }
}

// wavelet injection on a stored plane (used for the reverse restart:
// S(t) - w(t) delta before the backward step)
__global__ void k_inject(float *p, long long o, float v)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) p[o] = p[o] + v;
}

// Ring kernel (default for n1 % 4 == 0): the same tiles, per-cell arithmetic
// and march as k_acoustic3d_p, with every tap read from shared memory.  A
// ring of T3_NR slices of p1 -- each the tile's 144 rows (8-row z halo) by
// T3_LX columns (5-column x halo) -- is filled by one tensor-memory-access
// box load per slice, issued by one thread seven slices ahead of the
// compute; slice y's x and z taps come from its ring slot, its y taps from
// the slots of slices y-5 .. y+5 (no register queue to shift).  The sponge
// factor, the source and the receiver row are resolved per thread before the
// march (a thread whose 4 cells and column lie outside the sponge needs no
// factor on interior slices).  One CTA-wide barrier per slice, which also
// carries the bounded waits' outcome: a CTA whose slice load did not land
// within about a second records it in the error flag and stops.
constexpr int T3_TX = 16;
constexpr int T3_LX = T3_TX + 2 * AR;   // staged columns (26)
constexpr int T3_NR = 13;               // slices y-5 .. y+5 in use, y+6 and y+7 loading
constexpr int T3_SLICE = A_LZ * T3_LX;  // floats per staged slice
constexpr size_t T3_SMEM = (size_t)T3_NR * T3_SLICE * sizeof(float) + 128 + T3_NR * 8;

struct Ac3DTArgs {
    Ac3DArgs a;
    CUtensorMap tm;           // p1: n1 x n2 x n3, box {A_LZ, T3_LX, 1}
};

template <bool EXACT, bool IMG>
__global__ void __launch_bounds__(T3_TX * 32, 1) k_acoustic3d_t(const __grid_constant__ Ac3DTArgs A)
{
    const Ac3DArgs &a = A.a;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *ring = reinterpret_cast<float *>(smem_raw + ((128u - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127u)) & 127u));
    unsigned long long *full = reinterpret_cast<unsigned long long *>(ring + T3_NR * T3_SLICE);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3;
    const int ntz = (n1 - 9 + A_TZ - 1) / A_TZ;  // rows 4 .. n1-6 (interior plus row 4)
    int b = blockIdx.x;
    const int yc = b % a.ychunks;
    b /= a.ychunks;
    const int tzi = b % ntz, txi = b / ntz;
    const int z0 = 4 + tzi * A_TZ, x0 = AR + txi * T3_TX;
    const int ylen = (n3 - 2 * AR + a.ychunks - 1) / a.ychunks;
    const int ya = AR + yc * ylen, yb = min(n3 - AR, ya + ylen);
    if (ya >= yb) return;
    const int z = z0 + 4 * lane, x = x0 + warp;
    const bool grp = x < n2 - AR && z < n1;  // this thread's float4 exists
    const long long s3 = (long long)n1 * n2;
    const long long ocol = (long long)x * n1 + z;
    // per-thread constants: the plain update applies (no rim, source or
    // receiver cell), sponge distance of the 4 rows and the column
    const bool plain = cells_plain(a, z, x);
    const int ezx = cells_edge(z, x, n1, n2);
    auto slot = [&](int s) { return (s - (ya - AR)) % T3_NR; };
    auto wrap = [](int t) { return t >= T3_NR ? t - T3_NR : t; };  // t in [0, 2 T3_NR)
    auto issue = [&](int s) {
        const int k = slot(s);
        mbar_expect_tx(&full[k], (unsigned)(T3_SLICE * sizeof(float)));
        tma_load_3d(ring + k * T3_SLICE, &A.tm, z0 - A_ZH, x0 - AR, s, &full[k]);
    };
    if (threadIdx.x == 0) {
        for (int k = 0; k < T3_NR; k++) mbar_init(&full[k]);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const int last = yb - 1 + AR;  // last slice the march reads
    if (threadIdx.x == 0)
        for (int s = ya - AR; s <= min(ya + 6, last); s++) issue(s);
    auto L4 = [&](const float *p, long long o) -> float4 {
        return grp ? __ldg(reinterpret_cast<const float4 *>(p + o)) : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    float4 p0c = L4(a.p0, ocol + (long long)ya * s3), velc = L4(a.vel, ocol + (long long)ya * s3);
    const float *coef = a.coef;
    const int cofs = (warp + AR) * A_LZ + (4 * lane + A_ZH);  // this thread's float4 within a slice
    int sy = AR;  // ring slot of slice y
    for (int y = ya; y < yb; y++, sy = wrap(sy + 1)) {
        // slices y-5 .. y+5 resident: wait for y+5 (and, first, for y-5 .. y+4)
        bool ok = true;
        for (int s = (y == ya ? ya - AR : y + AR); s <= y + AR; s++) {
            const int u = s - (ya - AR);
            ok = ok && mbar_wait(&full[u % T3_NR], (unsigned)((u / T3_NR) & 1));
        }
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0 && a.err) atomicExch(a.err, 1);
            return;
        }
        // every thread is past slice y-1, so the slot of slice y-6 (first
        // iteration: a slot not used yet) takes slice y+7
        if (threadIdx.x == 0 && y + 7 <= last) issue(y + 7);
        float4 p0n = make_float4(0.f, 0.f, 0.f, 0.f), veln = p0n;
        if (y + 1 < yb) {
            p0n = L4(a.p0, ocol + (long long)(y + 1) * s3);
            veln = L4(a.vel, ocol + (long long)(y + 1) * s3);
        }
        if (grp) {
            const float *cz = ring + sy * T3_SLICE + cofs;
            float w[20];
#pragma unroll
            for (int i = 0; i < 20; i += 4) {
                const float4 t = *reinterpret_cast<const float4 *>(cz - 8 + i);
                w[i] = t.x; w[i + 1] = t.y; w[i + 2] = t.z; w[i + 3] = t.w;
            }
            float accv[4];
#pragma unroll
            for (int j = 0; j < 4; j++) accv[j] = fm<EXACT>(coef[0], w[8 + j]);
#pragma unroll
            for (int k = 1; k <= AR; k++) {
                const float4 xm = *reinterpret_cast<const float4 *>(cz - k * A_LZ);
                const float4 xp = *reinterpret_cast<const float4 *>(cz + k * A_LZ);
                const float4 ym = *reinterpret_cast<const float4 *>(ring + wrap(sy + T3_NR - k) * T3_SLICE + cofs);
                const float4 yq = *reinterpret_cast<const float4 *>(ring + wrap(sy + k) * T3_SLICE + cofs);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float zp = fa<EXACT>(w[8 + j + k], w[8 + j - k]);
                    const float xq = fa<EXACT>(e4(xp, j), e4(xm, j));
                    const float yp = fa<EXACT>(e4(yq, j), e4(ym, j));
                    accv[j] = fa<EXACT>(accv[j], fm<EXACT>(coef[1 + 3 * (k - 1)], zp));
                    accv[j] = fa<EXACT>(accv[j], fm<EXACT>(coef[2 + 3 * (k - 1)], xq));
                    accv[j] = fa<EXACT>(accv[j], fm<EXACT>(coef[3 + 3 * (k - 1)], yp));
                }
            }
            const long long o = ocol + (long long)y * s3;
            float out[4];
            if (__builtin_expect(plain && (!a.damp || min(ezx, edge_dist(y, n3)) >= a.damp_a), 1)) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    out[j] = fs<EXACT>(fa<EXACT>(fa<EXACT>(fm<EXACT>(e4(velc, j), accv[j]), w[8 + j]), w[8 + j]),
                                       e4(p0c, j));
            } else {
                const float4 r = cells_full<EXACT>(a, z, x, y, o, make_float4(accv[0], accv[1], accv[2], accv[3]),
                                                   make_float4(w[8], w[9], w[10], w[11]), p0c, velc);
                out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
            }
            *reinterpret_cast<float4 *>(a.p2 + o) = make_float4(out[0], out[1], out[2], out[3]);
        }
        p0c = p0n;
        velc = veln;
    }
}

// Slab kernel (kinds 0 and 3).  The same tiles and march as k_acoustic3d_p,
// arranged so that every operand arrives by a bulk tensor copy issued
// slices ahead of its use and every thread runs the same straight-line code
// on every slice:
// - slab ring: slice s of p1 over the tile's 144 rows by 26 columns (x and z
//   halo) lands in slot s % S3_NS, issued when the march reaches slice
//   s - 7; slice y's x and z taps come from its slab;
// - the y taps come from a register queue of S3_Q float4 (slices y-5 .. y+5)
//   refilled from the centre of slab y+5 (landed two slices after its
//   issue); the march is unrolled by S3_Q so that each queue slot is a
//   fixed register and nothing is shifted;
// - p0 and v^2 dt^2 of the tile's cells (128 rows x 16 columns) land in a
//   ring of S3_NP slots, issued three slices ahead;
// - the sponge factor is a per-slice branch that is uniform across the CTA
//   (the tile's least edge distance against the slice's): inside the sponge
//   every cell looks its factor up, a factor of one leaving a value
//   unchanged; rim rows are zeroed by a select in the CTAs that hold any;
//   only the threads holding the source or the receiver row branch off;
// - with PK (kind 3, fast arithmetic only) the cells are updated in pairs
//   (cells 0-1 and 2-3 of a thread) by the paired single-precision
//   instructions, in the scalar form's order and roundings.  Measured: the
//   paired instructions round some subnormal results differently from the
//   scalar ones, which the wavefield's leading edge reaches, so exact
//   arithmetic runs the scalar form; and the paired form is no faster (the
//   kernel is bound by shared-memory latency, not by issue), so the
//   default is the scalar form.
// One CTA-wide barrier per slice; it also carries the bounded waits'
// outcome: a CTA whose copy does not land within about a second records it
// in the error flag, lets its copies in flight land and stops.
constexpr int S3_NS = 8;                 // slab slots (power of two)
constexpr int S3_LEAD = 7;               // slab s is issued at slice s - S3_LEAD
constexpr int S3_NP = 4;                 // p0 / vel slots (power of two), issued S3_NP - 1 slices ahead
constexpr int S3_Q = 11;                 // register queue depth = unroll of the march
constexpr int S3_BOX = A_TZ * T3_TX;     // floats of a p0 or vel box
constexpr size_t S3_SMEM = ((size_t)S3_NS * T3_SLICE + 2 * S3_NP * S3_BOX) * sizeof(float) + 128 + (S3_NS + S3_NP) * 8;

struct Ac3DSArgs {
    Ac3DArgs a;
    CUtensorMap tm;   // p1: box {A_LZ, T3_LX, 1}
    CUtensorMap tm0;  // p0: box {A_TZ, T3_TX, 1}
    CUtensorMap tmv;  // vel: box {A_TZ, T3_TX, 1}
};

template <bool PK>
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    if (PK) return __fadd2_rn(a, b);
    return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
template <bool PK>
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    if (PK) return __fmul2_rn(a, b);
    return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
template <bool PK>
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    if (PK) return __ffma2_rn(a, b, c);
    return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
}
// acc + c x: two roundings in exact mode, one (fused) in fast mode
template <bool EXACT, bool PK>
__device__ __forceinline__ float2 mac2(float2 acc, float2 c, float2 x)
{
    return EXACT ? add2<PK>(acc, mul2<PK>(c, x)) : fma2<PK>(c, x, acc);
}
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 bc2(float c) { return make_float2(c, c); }

template <bool EXACT, bool IMG, bool PK>
__global__ void __launch_bounds__(T3_TX * 32, 1) k_acoustic3d_s(const __grid_constant__ Ac3DSArgs A)
{
    const Ac3DArgs &a = A.a;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *slab = reinterpret_cast<float *>(smem_raw + ((128u - ((unsigned)__cvta_generic_to_shared(smem_raw) & 127u)) & 127u));
    float *p0b = slab + S3_NS * T3_SLICE, *velb = p0b + S3_NP * S3_BOX;
    unsigned long long *fulls = reinterpret_cast<unsigned long long *>(velb + S3_NP * S3_BOX);
    unsigned long long *fullp = fulls + S3_NS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n1 = a.n1, n2 = a.n2, n3 = a.n3;
    const int ntz = (n1 - 9 + A_TZ - 1) / A_TZ;  // rows 4 .. n1-6 (interior plus row 4)
    int b = blockIdx.x;
    const int yc = b % a.ychunks;
    b /= a.ychunks;
    const int tzi = b % ntz, txi = b / ntz;
    const int z0 = 4 + tzi * A_TZ, x0 = AR + txi * T3_TX;
    const int ylen = (n3 - 2 * AR + a.ychunks - 1) / a.ychunks;
    const int ya = AR + yc * ylen, yb = min(n3 - AR, ya + ylen);
    if (ya >= yb) return;
    const int z = z0 + 4 * lane, x = x0 + warp;
    const bool grp = x < n2 - AR && z < n1;  // this thread's float4 exists
    const long long s3 = (long long)n1 * n2;
    // tile constants (uniform): least sponge distance over the tile's
    // interior cells (edge_dist is smallest at a range's ends), rim rows
    const int zlo = max(z0, AR), zhi = min(z0 + A_TZ - 1, n1 - AR - 1), xhi = min(x0 + T3_TX - 1, n2 - AR - 1);
    const int tile_e = min(min(edge_dist(zlo, n1), edge_dist(zhi, n1)), min(edge_dist(x0, n2), edge_dist(xhi, n2)));
    const bool tile_rim = z0 < AR || z0 + A_TZ > n1 - AR;
    const bool damped = a.damp != nullptr;
    // per-thread special cells: the receiver row's component rj and the
    // source's component sj (at slice ys), -1 where none
    int rj = -1, sj = -1, ys = -1;
    if (grp && (a.rec_in || a.rec_out) && a.zr >= z && a.zr < z + 4 && a.zr >= AR && a.zr < n1 - AR) rj = a.zr - z;
    if (grp && a.src_o >= 0) {
        const long long r = a.src_o % s3;
        const int sx = (int)(r / n1), sz = (int)(r % n1);
        if (sx == x && sz >= z && sz < z + 4) {
            sj = sz - z;
            ys = (int)(a.src_o / s3);
        }
    }
    const int slab_last = yb - 1 + AR;  // the queue reads slabs up to here
    auto issue_slab = [&](int s) {
        const int k = (s - ya) & (S3_NS - 1);
        mbar_expect_tx(&fulls[k], (unsigned)(T3_SLICE * sizeof(float)));
        tma_load_3d(slab + k * T3_SLICE, &A.tm, z0 - A_ZH, x0 - AR, s, &fulls[k]);
    };
    auto issue_box = [&](int s) {
        const int k = (s - ya) & (S3_NP - 1);
        mbar_expect_tx(&fullp[k], (unsigned)(2 * S3_BOX * sizeof(float)));
        tma_load_3d(p0b + k * S3_BOX, &A.tm0, z0, x0, s, &fullp[k]);
        tma_load_3d(velb + k * S3_BOX, &A.tmv, z0, x0, s, &fullp[k]);
    };
    auto slab_ok = [&](int s) { return mbar_wait(&fulls[(s - ya) & (S3_NS - 1)], (unsigned)(((s - ya) / S3_NS) & 1)); };
    auto box_ok = [&](int s) { return mbar_wait(&fullp[(s - ya) & (S3_NP - 1)], (unsigned)(((s - ya) / S3_NP) & 1)); };
    if (threadIdx.x == 0) {
        for (int k = 0; k < S3_NS; k++) mbar_init(&fulls[k]);
        for (int k = 0; k < S3_NP; k++) mbar_init(&fullp[k]);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int s = ya; s <= min(ya + S3_LEAD - 1, slab_last); s++) issue_slab(s);
        for (int s = ya; s <= min(ya + S3_NP - 2, yb - 1); s++) issue_box(s);
    }
    float *pp2 = a.p2 + (long long)x * n1 + z;
    // queue slot of slice s: (s - ya + 5) % S3_Q; slices ya-5 .. ya+4 from
    // global memory, later ones from the slabs
    float4 q[S3_Q];
    {
        const float *pp1 = a.p1 + (long long)x * n1 + z;
#pragma unroll
        for (int k = 0; k < 2 * AR; k++)
            q[k] = grp ? __ldg(reinterpret_cast<const float4 *>(pp1 + (long long)(ya - AR + k) * s3))
                       : make_float4(0.f, 0.f, 0.f, 0.f);
        q[S3_Q - 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float *coef = a.coef;
    const int cofs = (warp + AR) * A_LZ + (4 * lane + A_ZH);  // this thread's float4 within a slab
    const int bofs = warp * A_TZ + 4 * lane;                  // ... within a p0 / vel box
    for (int yblk = ya; yblk < yb; yblk += S3_Q) {
#pragma unroll
        for (int u = 0; u < S3_Q; u++) {
            const int y = yblk + u;
            if (y >= yb) break;
            // slab y (x/z taps; landed before unless in the first slices),
            // slab y+5 (queue) and the p0/vel box of y
            const bool ok = slab_ok(y) && slab_ok(y + AR) && box_ok(y);
            if (__syncthreads_or(!ok)) {
                // record, let the copies in flight land (bounded) and stop
                if (threadIdx.x == 0) {
                    if (a.err) atomicExch(a.err, 1);
                    for (int s = y; s <= min(y + S3_LEAD - 1, slab_last); s++) slab_ok(s);
                    for (int s = y; s <= min(y + S3_NP - 2, yb - 1); s++) box_ok(s);
                }
                __syncthreads();
                return;
            }
            // every thread is past slice y-1: its slab slot takes slice y+7,
            // its box slot slice y+3
            if (threadIdx.x == 0) {
                if (y + S3_LEAD <= slab_last) issue_slab(y + S3_LEAD);
                if (y + S3_NP - 1 < yb) issue_box(y + S3_NP - 1);
            }
            q[(u + 2 * AR) % S3_Q] = *reinterpret_cast<const float4 *>(slab + ((y + AR - ya) & (S3_NS - 1)) * T3_SLICE + cofs);
            const int pk = (y - ya) & (S3_NP - 1);
            const float4 p0c = *reinterpret_cast<const float4 *>(p0b + pk * S3_BOX + bofs);
            const float4 velc = *reinterpret_cast<const float4 *>(velb + pk * S3_BOX + bofs);
            if (!grp) continue;
            float4 imgc = make_float4(0.f, 0.f, 0.f, 0.f), simgc = imgc;
            if (IMG) {
                imgc = *reinterpret_cast<const float4 *>(a.img + (long long)x * n1 + z + (long long)y * s3);
                simgc = __ldg(reinterpret_cast<const float4 *>(a.simg + (long long)x * n1 + z + (long long)y * s3));
            }
            const float *cz = slab + ((y - ya) & (S3_NS - 1)) * T3_SLICE + cofs;
            float w[20];  // rows z-8 .. z+11 of column x
#pragma unroll
            for (int i = 0; i < 20; i += 4) {
                const float4 t = *reinterpret_cast<const float4 *>(cz - 8 + i);
                w[i] = t.x; w[i + 1] = t.y; w[i + 2] = t.z; w[i + 3] = t.w;
            }
            const float4 pc = q[(u + AR) % S3_Q];
            float2 acc[2] = {mul2<PK>(bc2(coef[0]), lo2(pc)), mul2<PK>(bc2(coef[0]), hi2(pc))};
#pragma unroll
            for (int k = 1; k <= AR; k++) {
                const float4 xm = *reinterpret_cast<const float4 *>(cz - k * A_LZ);
                const float4 xp = *reinterpret_cast<const float4 *>(cz + k * A_LZ);
                const float4 ym = q[(u + AR - k) % S3_Q], yp = q[(u + AR + k) % S3_Q];
                const float2 cz2 = bc2(coef[1 + 3 * (k - 1)]), cx2 = bc2(coef[2 + 3 * (k - 1)]),
                             cy2 = bc2(coef[3 + 3 * (k - 1)]);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int j = 2 * h;
                    // z pairs are register pairs only for even k
                    const float2 zs = (k & 1) ? make_float2(__fadd_rn(w[8 + j + k], w[8 + j - k]),
                                                            __fadd_rn(w[9 + j + k], w[9 + j - k]))
                                              : add2<PK>(make_float2(w[8 + j + k], w[9 + j + k]),
                                                         make_float2(w[8 + j - k], w[9 + j - k]));
                    acc[h] = mac2<EXACT, PK>(acc[h], cz2, zs);
                    acc[h] = mac2<EXACT, PK>(acc[h], cx2, add2<PK>(h ? hi2(xp) : lo2(xp), h ? hi2(xm) : lo2(xm)));
                    acc[h] = mac2<EXACT, PK>(acc[h], cy2, add2<PK>(h ? hi2(yp) : lo2(yp), h ? hi2(ym) : lo2(ym)));
                }
            }
            // sponge factors of the 4 cells (uniform branch)
            const bool sp = damped && min(tile_e, edge_dist(y, n3)) < a.damp_a;
            float2 fac[2] = {bc2(1.f), bc2(1.f)};
            if (sp) {
                const int m = min(edge_dist(x, n2), edge_dist(y, n3));
                float f[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int e = min(edge_dist(z + j, n1), m);
                    f[j] = 1.f;
                    if (e >= 0 && e < a.damp_a) f[j] = fminf(__ldg(a.damp + e), 1.f);
                }
                fac[0] = make_float2(f[0], f[1]);
                fac[1] = make_float2(f[2], f[3]);
            }
            float2 v[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float2 p = h ? hi2(pc) : lo2(pc);
                const float2 p0d = sp ? mul2<PK>(fac[h], h ? hi2(p0c) : lo2(p0c)) : (h ? hi2(p0c) : lo2(p0c));
                const float2 vel = h ? hi2(velc) : lo2(velc);
                float2 t = EXACT ? add2<PK>(mul2<PK>(vel, acc[h]), p) : fma2<PK>(vel, acc[h], p);
                t = add2<PK>(t, p);
                v[h] = fma2<PK>(p0d, bc2(-1.f), t);  // t - p0d, one rounding
            }
            if (rj >= 0 || (sj >= 0 && y == ys)) {
                float vv[4] = {v[0].x, v[0].y, v[1].x, v[1].y};
                const long long ri = (long long)y * n2 + x;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (j == sj && y == ys) vv[j] = __fadd_rn(vv[j], a.src_val);
                    if (j == rj) {
                        if (a.rec_in) vv[j] = __fadd_rn(vv[j], a.rec_in[ri]);
                        if (a.rec_out) a.rec_out[ri] = vv[j];
                    }
                }
                v[0] = make_float2(vv[0], vv[1]);
                v[1] = make_float2(vv[2], vv[3]);
            }
            const long long o = (long long)y * s3;
            if (IMG) {
                float2 im[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const float2 t = mul2<PK>(bc2(1e-6f), v[h]);
                    const float2 ic = h ? hi2(imgc) : lo2(imgc), sc = h ? hi2(simgc) : lo2(simgc);
                    im[h] = EXACT ? add2<PK>(ic, mul2<PK>(t, sc)) : fma2<PK>(t, sc, ic);
                }
                float r[4] = {im[0].x, im[0].y, im[1].x, im[1].y};
                if (tile_rim) {
                    const float c[4] = {imgc.x, imgc.y, imgc.z, imgc.w};
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (z + j < AR || z + j >= n1 - AR) r[j] = c[j];
                }
                *reinterpret_cast<float4 *>(a.img + (long long)x * n1 + z + o) = make_float4(r[0], r[1], r[2], r[3]);
            }
            float2 out[2];
#pragma unroll
            for (int h = 0; h < 2; h++) out[h] = (sp && !a.raw_out) ? mul2<PK>(fac[h], v[h]) : v[h];
            float r[4] = {out[0].x, out[0].y, out[1].x, out[1].y};
            if (tile_rim) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (z + j < AR || z + j >= n1 - AR) r[j] = 0.f;
            }
            *reinterpret_cast<float4 *>(pp2 + o) = make_float4(r[0], r[1], r[2], r[3]);
        }
    }
}

// Step kernel where n1 % 4 == 0 and tensor maps are available:
// 0 slab (default), 1 ring, 2 cp.async pipelined, 3 slab with paired
// single-precision instructions in fast arithmetic
int g_ac_kind = 0;

// Tensor maps of a step: p1 with a box of the tile's 144 rows by 26 columns
// (ring and slab kernels), p0 and vel with a box of its 128 rows by 16
// columns (slab kernel).
int step_map(CUtensorMap *m, const float *p, const Ac3DArgs &a, bool slab)
{
    return make_map(m, p, false, a.n1, a.n2, a.n3, (long long)a.n1 * a.n2, slab ? A_LZ : A_TZ, slab ? T3_LX : T3_TX);
}

// Dynamic shared memory above 48 KB, set once per kernel and device.
template <typename K>
int smem_attr(K kern, int variant, size_t smem)
{
    static bool attr[RTM_MAX_DEVICES][16] = {};
    const int dev = rtm_current_device();
    std::lock_guard<std::mutex> lk(rtm_device_state_lock());
    if (!attr[dev][variant]) {
        RTM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr[dev][variant] = true;
    }
    return RTM_OK;
}

template <bool EXACT>
int launch_ac_tma(const Ac3DArgs &a0, int ychunks, cudaStream_t st)
{
    const bool img = a0.img != nullptr;
    const int v = (EXACT ? 8 : 0) + (img ? 4 : 0);
    const int ntz = (a0.n1 - 9 + A_TZ - 1) / A_TZ;
    const int ntx = (a0.n2 - 2 * AR + T3_TX - 1) / T3_TX;
    const int grid = ntz * ntx * ychunks;
    if (g_ac_kind == 1) {
        Ac3DTArgs t;
        memset(&t, 0, sizeof t);
        t.a = a0;
        t.a.ychunks = ychunks;
        TRY(step_map(&t.tm, a0.p1, a0, true));
        auto kern = img ? k_acoustic3d_t<EXACT, true> : k_acoustic3d_t<EXACT, false>;
        TRY(smem_attr(kern, v, T3_SMEM));
        kern<<<grid, T3_TX * 32, T3_SMEM, st>>>(t);
    } else {
        Ac3DSArgs t;
        memset(&t, 0, sizeof t);
        t.a = a0;
        t.a.ychunks = ychunks;
        TRY(step_map(&t.tm, a0.p1, a0, true));
        TRY(step_map(&t.tm0, a0.p0, a0, false));
        TRY(step_map(&t.tmv, a0.vel, a0, false));
        // paired instructions in fast arithmetic only (kind 3)
        auto kern = g_ac_kind != 3 ? (img ? k_acoustic3d_s<EXACT, true, false> : k_acoustic3d_s<EXACT, false, false>)
                                   : (img ? k_acoustic3d_s<EXACT, true, !EXACT> : k_acoustic3d_s<EXACT, false, !EXACT>);
        TRY(smem_attr(kern, v + (g_ac_kind != 3 ? 2 : 3), S3_SMEM));
        kern<<<grid, T3_TX * 32, S3_SMEM, st>>>(t);
    }
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

template <bool EXACT>
int launch_ac(const Ac3DArgs &a0, int tx, int ychunks, cudaStream_t st)
{
    if (a0.n1 % 4 == 0 && g_ac_kind != 2 && tensor_maps_available()) return launch_ac_tma<EXACT>(a0, ychunks, st);
    Ac3DArgs a = a0;
    a.ychunks = ychunks;
    const int ntx = (a.n2 - 2 * AR + tx - 1) / tx;
    if (a.n1 % 4 == 0) {
        const int ntz = (a.n1 - 9 + A_TZ - 1) / A_TZ;
        const int grid = ntz * ntx * ychunks;
        switch (tx) {
        case 8: k_acoustic3d_p<EXACT, 8><<<grid, 8 * 32, 0, st>>>(a); break;
        case 16: k_acoustic3d_p<EXACT, 16><<<grid, 16 * 32, 0, st>>>(a); break;
        default: rtm_set_error("unsupported 3D tile width %d", tx); return RTM_ERR_ARG;
        }
    } else {
        const int ntz = (a.n1 - 2 * AR + A_TZ - 1) / A_TZ;
        const int grid = ntz * ntx * ychunks;
        switch (tx) {
        case 8: k_acoustic3d<EXACT, 8><<<grid, 8 * 32, 0, st>>>(a); break;
        case 16: k_acoustic3d<EXACT, 16><<<grid, 16 * 32, 0, st>>>(a); break;
        default: rtm_set_error("unsupported 3D tile width %d", tx); return RTM_ERR_ARG;
        }
    }
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

struct Ac3D {
    int n1, n2, n3, nt;
    size_t vol;
    DevBuf<float> vel, buf, damp, rec, img;
    DevBuf<int> err;
    float coef[16];
    int damp_a = 0;
    int tx = 16, ych = 2;
    bool exact = false;
    cudaStream_t st = 0;

    int step(const float *p0, const float *p1, float *p2, bool damped, long long src_o, float src_val, int zr,
             float *rec_out, const float *rec_in, float *img, const float *simg, bool raw_out = false)
    {
        Ac3DArgs a;
        memset(&a, 0, sizeof a);
        a.p0 = p0; a.p1 = p1; a.p2 = p2; a.vel = vel.p;
        a.n1 = n1; a.n2 = n2; a.n3 = n3;
        memcpy(a.coef, coef, sizeof coef);
        a.damp = damped && damp_a > 0 ? damp.p : nullptr;
        a.damp_a = damp_a;
        a.src_o = src_o; a.src_val = src_val;
        a.zr = zr; a.rec_out = rec_out; a.rec_in = rec_in;
        a.img = img; a.simg = simg;
        a.err = err.p;
        a.raw_out = raw_out;
        return exact ? launch_ac<true>(a, tx, ych, st) : launch_ac<false>(a, tx, ych, st);
    }
    // status 4 when a kernel's bounded wait ran out during the run
    int check_waits()
    {
        int e = 0;
        RTM_CUDA(cudaMemcpy(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) {
            RTM_CUDA(cudaMemset(err.p, 0, sizeof(int)));
            rtm_set_error("a 3D step kernel's slice load did not complete within its time limit");
            return RTM_ERR_TIMEOUT;
        }
        return RTM_OK;
    }
};

void host_coeffs(double d1, double d2, double d3, float *coef)
{
    const double c[6] = {-5269.0 / 1800.0, 5.0 / 3.0, -5.0 / 21.0, 5.0 / 126.0, -5.0 / 1008.0, 1.0 / 3150.0};
    const double i1 = 1.0 / (d1 * d1), i2 = 1.0 / (d2 * d2), i3 = 1.0 / (d3 * d3);
    coef[0] = (float)(c[0] * (i1 + i2 + i3));
    for (int k = 1; k <= 5; k++) {
        coef[1 + 3 * (k - 1) + 0] = (float)(c[k] * i1);
        coef[1 + 3 * (k - 1) + 1] = (float)(c[k] * i2);
        coef[1 + 3 * (k - 1) + 2] = (float)(c[k] * i3);
    }
}

int ac_setup(Ac3D &m, int n1, int n2, int n3, int nt, float d1, float d2, float d3, const float *vel2, int vel_dev,
             int damp_a, float damp_b)
{
    RTM_CHECK_ARG(n1 >= 2 * AR + 1 && n2 >= 2 * AR + 1 && n3 >= 2 * AR + 1 && nt >= 2, "3D grid too small");
    TRY(ensure_device());
    m.n1 = n1; m.n2 = n2; m.n3 = n3; m.nt = nt;
    m.vol = (size_t)n1 * n2 * n3;
    host_coeffs(d1, d2, d3, m.coef);
    TRY(m.vel.alloc(m.vol));
    RTM_CUDA(cudaMemcpy(m.vel.p, vel2, m.vol * sizeof(float), vel_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    m.damp_a = damp_a;
    if (damp_a > 0) {
        std::vector<float> t(damp_a);
        for (int e = 0; e < damp_a; e++) t[e] = expf(-damp_b * (float)(damp_a - e));
        TRY(m.damp.alloc(damp_a));
        RTM_CUDA(cudaMemcpy(m.damp.p, t.data(), damp_a * sizeof(float), cudaMemcpyHostToDevice));
    }
    const char *e = getenv("ELASTIC_RTM_EXACT3D");
    m.exact = e && atoi(e) == 1;
    TRY(m.err.alloc(1));
    RTM_CUDA(cudaMemset(m.err.p, 0, sizeof(int)));
    return RTM_OK;
}

int g_ac_tx = 16, g_ac_ych = 0;  // tile width and y chunks (0: chosen from the SM count)
int g_ac_n3 = 512;                // n3 of the run being set up (y-chunk choice)
int n3_hint() { return g_ac_n3; }

int pick_ychunks(int n1, int n2, int tx)
{
    if (g_ac_ych > 0) return g_ac_ych;
    const int ntz = n1 % 4 == 0 ? (n1 - 9 + A_TZ - 1) / A_TZ : (n1 - 2 * AR + A_TZ - 1) / A_TZ;
    const int ntx = (n2 - 2 * AR + tx - 1) / tx;
    const bool tma = n1 % 4 == 0 && g_ac_kind != 2;
    const int nsm = device_sm_count() * (tx == 8 && !tma ? 2 : 1);
    int best = 1;
    double best_eff = 0;
    for (int c = 1; c <= 8; c++) {
        const int g = ntz * ntx * c;
        const double waves = (double)g / nsm;
        // each chunk reads the 10 slices of p1 around its y range once more
        // (the ring kernel all four arrays' worth of time, the slab kernel
        // one array of four)
        const double ylen = (double)(n3_hint() - 2 * AR) / c;
        const double extra = g_ac_kind == 1 ? 10.0 : 2.5;
        const double eff = waves / std::ceil(waves) * (tma ? ylen / (ylen + extra) : 1.0 - 0.01 * c);
        if (eff > best_eff) { best_eff = eff; best = c; }
    }
    return best;
}

// Forward modelling from rest (W/gpu_funcs_3d.cu:133-315 with the sponge of
// damp_kernel): returns the raw traces d[it][iy][ix] and the last two
// levels as the reference leaves them -- level nt-2 damped (by the last
// step's in-place damping), level nt-1 raw.
int ac_forward(Ac3D &m, bool damped, long long src_o, const float *wavelet, float dir, int zr, float *d_dev,
               float **last0, float **last1)
{
    m.tx = g_ac_kind != 2 && m.n1 % 4 == 0 ? T3_TX : g_ac_tx;
    g_ac_n3 = m.n3;
    m.ych = pick_ychunks(m.n1, m.n2, m.tx);
    TRY(m.buf.alloc(2 * m.vol));
    float *A = m.buf.p, *B = m.buf.p + m.vol;
    RTM_CUDA(cudaMemsetAsync(m.buf.p, 0, 2 * m.vol * sizeof(float), m.st));
    for (int it = 0; it < m.nt; it++) {
        // A = level it-2 (older), B = level it-1; the new level goes over A
        TRY(m.step(A, B, A, damped, src_o, dir * wavelet[it], zr, d_dev ? d_dev + (size_t)it * m.n2 * m.n3 : nullptr,
                   nullptr, nullptr, nullptr, damped && it == m.nt - 1));
        std::swap(A, B);
    }
    *last0 = A;  // level nt-2
    *last1 = B;  // level nt-1
    return RTM_OK;
}

}  // namespace

extern "C" int acoustic3d_set_kernel(int kind)
{
    RTM_CHECK_ARG(kind >= 0 && kind <= 3, "kind must be 0 (slab), 1 (ring), 2 (pipelined) or 3 (slab, paired)");
    g_ac_kind = kind;
    return RTM_OK;
}

extern "C" int acoustic3d_set(int tile_x, int ychunks)
{
    RTM_CHECK_ARG(tile_x == 8 || tile_x == 16, "tile_x must be 8 or 16");
    RTM_CHECK_ARG(ychunks >= 0 && ychunks <= 64, "ychunks must be 0..64");
    g_ac_tx = tile_x;
    g_ac_ych = ychunks;
    return RTM_OK;
}

extern "C" int acoustic3d_fwd_c_(int n1, int n2, int n3, int nt, float d1, float d2, float d3, const float *vel2,
                                 int damp_a, float damp_b, int zs, int xs, int ys, const float *wavelet, int zr,
                                 float *data, float *p_last0, float *p_last1, int on_device, double *ms)
{
    Ac3D m;
    TRY(ac_setup(m, n1, n2, n3, nt, d1, d2, d3, vel2, on_device, damp_a, damp_b));
    RTM_CHECK_ARG(zs >= 1 && zs <= n1 && xs >= 1 && xs <= n2 && ys >= 1 && ys <= n3, "source outside the grid");
    RTM_CHECK_ARG(zr == 0 || (zr >= 1 && zr <= n1), "receiver plane outside the grid");
    const long long so = ((long long)(ys - 1) * n2 + (xs - 1)) * n1 + (zs - 1);
    const size_t dn = (size_t)nt * n2 * n3;
    DevBuf<float> d;
    float *dd = nullptr;
    if (zr > 0 && data) {
        if (on_device) dd = data;
        else { TRY(d.alloc(dn)); dd = d.p; }
        RTM_CUDA(cudaMemsetAsync(dd, 0, dn * sizeof(float), m.st));
    }
    cudaEvent_t e0, e1;
    RTM_CUDA(cudaEventCreate(&e0));
    RTM_CUDA(cudaEventCreate(&e1));
    RTM_CUDA(cudaEventRecord(e0, m.st));
    float *l0, *l1;
    TRY(ac_forward(m, true, so, wavelet, 1.f, zr - 1, dd, &l0, &l1));
    RTM_CUDA(cudaEventRecord(e1, m.st));
    RTM_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    RTM_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (dd && !on_device) RTM_CUDA(cudaMemcpy(data, dd, dn * sizeof(float), k));
    if (p_last0) RTM_CUDA(cudaMemcpy(p_last0, l0, m.vol * sizeof(float), k));
    if (p_last1) RTM_CUDA(cudaMemcpy(p_last1, l1, m.vol * sizeof(float), k));
    RTM_CUDA(cudaDeviceSynchronize());
    return m.check_waits();
}

// 3D RTM (W/gpu_funcs_3d.cu:509-712): source propagated forward undamped,
// only its last two levels kept; backwards: the receiver field (damped) takes
// the traces at the receiver plane, the source field is rebuilt from its last
// two levels (reverse-time restart: S(t-2) = L-step(S(t-1), S(t) - w(t)
// delta)), and every jt-th level adds (1e-6*R)*S to the image.
extern "C" int acoustic3d_rtm_c_(int n1, int n2, int n3, int nt, float d1, float d2, float d3, const float *vel2,
                                 int damp_a, float damp_b, int zs, int xs, int ys, const float *wavelet, int zr,
                                 const float *data, int jt, float *img, int on_device, double *ms)
{
    Ac3D m;
    TRY(ac_setup(m, n1, n2, n3, nt, d1, d2, d3, vel2, on_device, damp_a, damp_b));
    RTM_CHECK_ARG(zs >= 1 && zs <= n1 && xs >= 1 && xs <= n2 && ys >= 1 && ys <= n3, "source outside the grid");
    RTM_CHECK_ARG(zr >= 1 && zr <= n1 && jt >= 1, "bad receiver plane or imaging interval");
    const long long so = ((long long)(ys - 1) * n2 + (xs - 1)) * n1 + (zs - 1);
    const size_t dn = (size_t)nt * n2 * n3;
    DevBuf<float> d, rbuf, ib;
    const float *dd = data;
    if (!on_device) {
        TRY(d.alloc(dn));
        RTM_CUDA(cudaMemcpy(d.p, data, dn * sizeof(float), cudaMemcpyHostToDevice));
        dd = d.p;
    }
    TRY(ib.alloc(m.vol));
    RTM_CUDA(cudaMemsetAsync(ib.p, 0, m.vol * sizeof(float), m.st));
    TRY(rbuf.alloc(2 * m.vol));
    RTM_CUDA(cudaMemsetAsync(rbuf.p, 0, 2 * m.vol * sizeof(float), m.st));
    cudaEvent_t e0, e1;
    RTM_CUDA(cudaEventCreate(&e0));
    RTM_CUDA(cudaEventCreate(&e1));
    RTM_CUDA(cudaEventRecord(e0, m.st));
    float *X, *Y;  // X = S(nt-2), Y = S(nt-1)
    TRY(ac_forward(m, false, so, wavelet, 1.f, -1, nullptr, &X, &Y));
    float *r0 = rbuf.p, *r1 = rbuf.p + m.vol;
    for (int it = nt - 1; it >= 0; it--) {
        // source level it: S(nt-1) = Y, S(nt-2) = X, else rebuilt
        const float *S;
        if (it == nt - 1) S = Y;
        else if (it == nt - 2) S = X;
        else {
            k_inject<<<1, 32, 0, m.st>>>(Y, so, -wavelet[it + 2]);
            RTM_CUDA(cudaGetLastError());
            TRY(m.step(Y, X, Y, false, -1, 0.f, -1, nullptr, nullptr, nullptr, nullptr));
            std::swap(X, Y);  // X = S(it), Y = S(it+1)
            S = X;
        }
        // receiver field level it (+ traces), imaging with S(it)
        TRY(m.step(r0, r1, r0, true, -1, 0.f, zr - 1, nullptr, dd + (size_t)it * n2 * n3,
                   it % jt == 0 ? ib.p : nullptr, S));
        std::swap(r0, r1);
    }
    RTM_CUDA(cudaEventRecord(e1, m.st));
    RTM_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    RTM_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    RTM_CUDA(cudaMemcpy(img, ib.p, m.vol * sizeof(float), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    RTM_CUDA(cudaDeviceSynchronize());
    return m.check_waits();
}
