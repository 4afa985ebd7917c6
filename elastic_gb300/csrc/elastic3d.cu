// One step of the 3D elastic kernel of the reference's kernel_3d_test (nine
// fields, six coefficient planes, 10th-order staggered differences along
// z, x and y), sm_103a.
//
// Reference: kernel_3d_test/rtmlib-modC.c:277-590 (the CPU step its main
// checks the GPU kernel against, cell by cell at 1e-13, :31-43, :697-705),
// kernel_3d_test/rtmlib-modC-gpu.cu:57-700 (its GPU kernel, which does not
// compile with current CUDA), host entry points rtm_gpu_init/func/final
// (kernel_3d_test/gpu.h:68-79, rtmlib-modC-gpu.cu:65,218,698).
//
// Layout: padded (ny+10)(nx+10)(nz+10) planes, z fastest, interior cells at
// padded index +5 on every axis (the halo is zero and is not written).
// Every output field is updated in place:
//   out = out + in1 + sum over its groups, in order, of the group's ten
//         taps in order, +/- (m[p'] * c_k) * f[p'],
// a group naming a coefficient plane m, an input field f (level `in`), an
// axis and a stagger (taps at offsets -5..4 or -4..5, the first five added
// with c1..c5, the last five subtracted with c5..c1).  Exact arithmetic
// rounds every product and sum separately in that order (bit-identical to
// the reference's CPU step); fast arithmetic lets the compiler fuse.
//
// Kernel: one thread per interior cell, blocks of 32 (z) x 4 (x) x 2 (y)
// threads so that a warp reads 32 consecutive z cells; every tap is a
// read-only load served by L1 and L2 (each input value is read by up to 31
// cells' taps), nothing is staged in shared memory.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/elastic_rtm.h"
#include "common.cuh"
#include "engine.h"

using namespace eg;

namespace {

enum { F_VY, F_VX, F_VZ, F_SYY, F_SXX, F_SZZ, F_SXY, F_SXZ, F_SYZ };
enum { C_M1Y, C_M1X, C_M1Z, C_M2, C_M3, C_M2M3 };
enum { AX_Z = 0, AX_X = 1, AX_Y = 2 };

// group: coefficient plane, field, axis, first tap offset (-5 or -4)
struct K3G {
    int coef, field, axis, first;
};
// per output field (the reference's argument order), its groups in the
// reference's summation order; unused entries have coef -1
__device__ constexpr K3G K3_GROUPS[9][5] = {
    // Vy (rtmlib-modC.c:350-413)
    {{C_M2M3, F_SYY, AX_Y, -5}, {C_M2, F_SZZ, AX_Y, -5}, {C_M2, F_SXX, AX_Y, -5}, {C_M3, F_SYZ, AX_Z, -4},
     {C_M3, F_SXY, AX_X, -4}},
    // Vx (:288-349)
    {{C_M2M3, F_SXX, AX_X, -5}, {C_M2, F_SYY, AX_X, -5}, {C_M2, F_SZZ, AX_X, -5}, {C_M3, F_SXY, AX_Y, -4},
     {C_M3, F_SXZ, AX_Z, -4}},
    // Vz (:414-472)
    {{C_M2M3, F_SZZ, AX_Z, -5}, {C_M2, F_SXX, AX_Z, -5}, {C_M2, F_SYY, AX_Z, -5}, {C_M3, F_SYZ, AX_Y, -4},
     {C_M3, F_SXZ, AX_X, -4}},
    // syy (:490-501)
    {{C_M1Y, F_VY, AX_Y, -4}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
    // sxx (:477-488)
    {{C_M1X, F_VX, AX_X, -4}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
    // szz (:503-514)
    {{C_M1Z, F_VZ, AX_Z, -4}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
    // sxy (:518-541)
    {{C_M1Y, F_VY, AX_X, -4}, {C_M1X, F_VX, AX_Y, -4}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
    // sxz (:543-564)
    {{C_M1X, F_VX, AX_Z, -4}, {C_M1Z, F_VZ, AX_X, -4}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
    // syz (:566-589)
    {{C_M1Y, F_VY, AX_Z, -4}, {C_M1Z, F_VZ, AX_Y, -4}, {-1, 0, 0, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
};
__device__ constexpr int K3_NG[9] = {5, 5, 5, 1, 1, 1, 2, 2, 2};

struct K3Args {
    const float *in[9];
    const float *in1[9];
    float *out[9];
    const float *m[6];
    int ny, nz, nx;
    float c[5];  // c1..c5 as the reference stores them
};

template <bool EXACT>
__device__ __forceinline__ float k3_term(float acc, float m, float c, float f, bool add)
{
    if (EXACT) {
        const float t = __fmul_rn(__fmul_rn(m, c), f);
        return add ? __fadd_rn(acc, t) : __fsub_rn(acc, t);
    }
    return add ? acc + m * c * f : acc - m * c * f;
}

template <bool EXACT, int O>
__device__ __forceinline__ void k3_field(const K3Args &a, long long p, const long long st[3])
{
    float acc = EXACT ? __fadd_rn(a.out[O][p], __ldg(a.in1[O] + p)) : a.out[O][p] + __ldg(a.in1[O] + p);
#pragma unroll
    for (int g = 0; g < K3_NG[O]; g++) {
        const K3G q = K3_GROUPS[O][g];
        const float *mm = a.m[q.coef], *ff = a.in[q.field];
        const long long s = st[q.axis];
#pragma unroll
        for (int t = 0; t < 10; t++) {
            const long long pp = p + (q.first + t) * s;
            acc = k3_term<EXACT>(acc, __ldg(mm + pp), a.c[t < 5 ? t : 9 - t], __ldg(ff + pp), t < 5);
        }
    }
    a.out[O][p] = acc;
}

template <bool EXACT>
__global__ void __launch_bounds__(256) k_k3_step(const __grid_constant__ K3Args a)
{
    const int iz = blockIdx.x * 32 + threadIdx.x, ix = blockIdx.y * 4 + threadIdx.y, iy = blockIdx.z * 2 + threadIdx.z;
    if (iz >= a.nz || ix >= a.nx || iy >= a.ny) return;
    const long long sx = a.nz + 10, sy = (long long)(a.nz + 10) * (a.nx + 10);
    const long long st[3] = {1, sx, sy};
    const long long p = (iy + 5) * sy + (ix + 5) * sx + (iz + 5);
    k3_field<EXACT, 0>(a, p, st);
    k3_field<EXACT, 1>(a, p, st);
    k3_field<EXACT, 2>(a, p, st);
    k3_field<EXACT, 3>(a, p, st);
    k3_field<EXACT, 4>(a, p, st);
    k3_field<EXACT, 5>(a, p, st);
    k3_field<EXACT, 6>(a, p, st);
    k3_field<EXACT, 7>(a, p, st);
    k3_field<EXACT, 8>(a, p, st);
}

// Paired form (nz even, 8-byte aligned planes): a thread owns the padded z
// positions 2m and 2m+1 (cells where they are interior) and reads every
// tap as an 8-byte pair -- the same offset serves both cells along x and y;
// along z the two cells' 10 taps fall in 11 consecutive positions, six
// aligned pairs.  Each cell's sum keeps the reference's order and
// roundings, so the results equal the scalar kernel's bit for bit.
template <bool EXACT, int O>
__device__ __forceinline__ void k3_field2(const K3Args &a, long long p, const long long st[3], bool ok0, bool ok1)
{
    const float2 o2 = *reinterpret_cast<const float2 *>(a.out[O] + p);
    const float2 i2 = __ldg(reinterpret_cast<const float2 *>(a.in1[O] + p));
    float acc0 = EXACT ? __fadd_rn(o2.x, i2.x) : o2.x + i2.x;
    float acc1 = EXACT ? __fadd_rn(o2.y, i2.y) : o2.y + i2.y;
#pragma unroll
    for (int g = 0; g < K3_NG[O]; g++) {
        const K3G q = K3_GROUPS[O][g];
        const float *mm = a.m[q.coef], *ff = a.in[q.field];
        if (q.axis == AX_Z) {
            // positions p + q.first - 1 .. p + q.first + 10 (6 aligned pairs
            // from the even position at or below p + q.first - 1)
            const int lo = q.first == -5 ? -6 : -4;
            float mv[12], fv[12];
#pragma unroll
            for (int i = 0; i < 6; i++) {
                const float2 m2 = __ldg(reinterpret_cast<const float2 *>(mm + p + lo + 2 * i));
                const float2 f2 = __ldg(reinterpret_cast<const float2 *>(ff + p + lo + 2 * i));
                mv[2 * i] = m2.x; mv[2 * i + 1] = m2.y;
                fv[2 * i] = f2.x; fv[2 * i + 1] = f2.y;
            }
            const int b0 = q.first - lo;  // index of cell 0's first tap
#pragma unroll
            for (int t = 0; t < 10; t++) {
                const float c = a.c[t < 5 ? t : 9 - t];
                acc0 = k3_term<EXACT>(acc0, mv[b0 + t], c, fv[b0 + t], t < 5);
                acc1 = k3_term<EXACT>(acc1, mv[b0 + t + 1], c, fv[b0 + t + 1], t < 5);
            }
        } else {
            const long long s = st[q.axis];
#pragma unroll
            for (int t = 0; t < 10; t++) {
                const long long pp = p + (q.first + t) * s;
                const float2 m2 = __ldg(reinterpret_cast<const float2 *>(mm + pp));
                const float2 f2 = __ldg(reinterpret_cast<const float2 *>(ff + pp));
                const float c = a.c[t < 5 ? t : 9 - t];
                acc0 = k3_term<EXACT>(acc0, m2.x, c, f2.x, t < 5);
                acc1 = k3_term<EXACT>(acc1, m2.y, c, f2.y, t < 5);
            }
        }
    }
    if (ok0 && ok1)
        *reinterpret_cast<float2 *>(a.out[O] + p) = make_float2(acc0, acc1);
    else if (ok0)
        a.out[O][p] = acc0;
    else if (ok1)
        a.out[O][p + 1] = acc1;
}

template <bool EXACT, bool PF>
__device__ __forceinline__ void k3_step2_body(const K3Args &a)
{
    // padded z pairs 2m, 2m+1 for m = 2 .. (nz + 10) / 2 - 3 cover the interior [5, nz + 5)
    const int m = 2 + blockIdx.x * 32 + threadIdx.x, ix = blockIdx.y * 4 + threadIdx.y,
              iy = blockIdx.z * 2 + threadIdx.z;
    const int zp = 2 * m;
    if (zp >= a.nz + 5 || ix >= a.nx || iy >= a.ny) return;
    const bool ok0 = zp >= 5, ok1 = zp + 1 < a.nz + 5;
    const long long sx = a.nz + 10, sy = (long long)(a.nz + 10) * (a.nx + 10);
    const long long st[3] = {1, sx, sy};
    const long long p = (iy + 5) * sy + (ix + 5) * sx + zp;
    if (PF) {
        // the lines of the thread's own cells, first touched here, requested
        // into L2 together before the taps
#pragma unroll
        for (int i = 0; i < 9; i++) {
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.in[i] + p));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.in1[i] + p));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a.out[i] + p));
        }
#pragma unroll
        for (int i = 0; i < 6; i++) asm volatile("prefetch.global.L2 [%0];" ::"l"(a.m[i] + p));
    }
    k3_field2<EXACT, 0>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 1>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 2>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 3>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 4>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 5>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 6>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 7>(a, p, st, ok0, ok1);
    k3_field2<EXACT, 8>(a, p, st, ok0, ok1);
}

template <bool EXACT, bool PF>
__global__ void __launch_bounds__(256) k_k3_step2(const __grid_constant__ K3Args a)
{
    k3_step2_body<EXACT, PF>(a);
}

// the same with a register bound of 4 blocks of 256 threads an SM (64
// registers)
template <bool EXACT, bool PF>
__global__ void __launch_bounds__(256, 4) k_k3_step2b(const __grid_constant__ K3Args a)
{
    k3_step2_body<EXACT, PF>(a);
}

// 0: one cell a thread; 1: the paired form where nz is even and planes are
// 8-byte aligned; + 2: L2 prefetch of the own cells' lines; + 4: register
// bound of 4 blocks an SM.  Default: paired, bounded (measured fastest at
// 384^3: 4.75 ms against 5.30 ms unbounded; the prefetch costs 35 %)
int g_k3_paired = 5;

void k3_coefs(float c[5])
{
    c[0] = (float)(35.0 / 294912.0);
    c[1] = (float)(-405.0 / 229376.0);
    c[2] = (float)(567.0 / 40960.0);
    c[3] = (float)(-735.0 / 8192.0);
    c[4] = (float)(19845.0 / 16384.0);
}

int k3_launch(int ny, int nz, int nx, const float *const *in, const float *const *in1, float *const *out,
              const float *const *m, bool exact, cudaStream_t st)
{
    K3Args a;
    memset(&a, 0, sizeof a);
    for (int i = 0; i < 9; i++) {
        a.in[i] = in[i];
        a.in1[i] = in1[i];
        a.out[i] = out[i];
    }
    for (int i = 0; i < 6; i++) a.m[i] = m[i];
    a.ny = ny;
    a.nz = nz;
    a.nx = nx;
    k3_coefs(a.c);
    bool paired = g_k3_paired && nz % 2 == 0;
    for (int i = 0; i < 9 && paired; i++) paired = !((uintptr_t)in[i] & 7) && !((uintptr_t)in1[i] & 7) && !((uintptr_t)out[i] & 7);
    for (int i = 0; i < 6 && paired; i++) paired = !((uintptr_t)m[i] & 7);
    const dim3 block(32, 4, 2);
    if (paired) {
        const int pairs = (nz + 10) / 2 - 4;  // m = 2 .. (nz + 10)/2 - 3
        const dim3 grid((pairs + 31) / 32, (nx + 3) / 4, (ny + 1) / 2);
        const bool pf = (g_k3_paired & 2) != 0, bound = (g_k3_paired & 4) != 0;
        if (bound) {
            if (exact && pf) k_k3_step2b<true, true><<<grid, block, 0, st>>>(a);
            else if (exact) k_k3_step2b<true, false><<<grid, block, 0, st>>>(a);
            else if (pf) k_k3_step2b<false, true><<<grid, block, 0, st>>>(a);
            else k_k3_step2b<false, false><<<grid, block, 0, st>>>(a);
        } else {
            if (exact && pf) k_k3_step2<true, true><<<grid, block, 0, st>>>(a);
            else if (exact) k_k3_step2<true, false><<<grid, block, 0, st>>>(a);
            else if (pf) k_k3_step2<false, true><<<grid, block, 0, st>>>(a);
            else k_k3_step2<false, false><<<grid, block, 0, st>>>(a);
        }
    } else {
        const dim3 grid((nz + 31) / 32, (nx + 3) / 4, (ny + 1) / 2);
        if (exact)
            k_k3_step<true><<<grid, block, 0, st>>>(a);
        else
            k_k3_step<false><<<grid, block, 0, st>>>(a);
    }
    RTM_CUDA(cudaGetLastError());
    return RTM_OK;
}

// device state of the drop-in (rtm_gpu_init .. rtm_gpu_final)
struct K3State {
    int ny = 0, nz = 0, nx = 0;
    DevBuf<float> buf;  // 33 padded planes: in 9, in1 9, out 9, m 6
};
K3State g_k3;
int g_k3_exact = 1;

}  // namespace

extern "C" int rtm3d_set_kernel(int kind)
{
    RTM_CHECK_ARG(kind == 0 || (kind & 1), "kernel kind %d", kind);
    RTM_CHECK_ARG(kind >= 0 && kind <= 7, "kernel kind %d", kind);
    g_k3_paired = kind;
    return RTM_OK;
}

extern "C" int rtm3d_set_exact(int exact)
{
    RTM_CHECK_ARG(exact == 0 || exact == 1, "exact must be 0 or 1");
    g_k3_exact = exact;
    return RTM_OK;
}

extern "C" int rtm3d_step_dev(int ny, int nz, int nx, const float *const *in, const float *const *in1, float *const *out,
                              const float *const *m, int exact)
{
    RTM_CHECK_ARG(ny > 0 && nz > 0 && nx > 0, "grid sizes must be positive");
    RTM_CHECK_ARG(in && in1 && out && m, "null argument");
    for (int i = 0; i < 9; i++) RTM_CHECK_ARG(in[i] && in1[i] && out[i], "null field plane");
    for (int i = 0; i < 6; i++) RTM_CHECK_ARG(m[i], "null coefficient plane");
    TRY(ensure_device());
    TRY(k3_launch(ny, nz, nx, in, in1, out, m, exact != 0, 0));
    return RTM_OK;
}

extern "C" void rtm3d_gpu_init(int ny, int nz, int nx)
{
    int s = RTM_OK;
    if (!(ny > 0 && nz > 0 && nx > 0)) {
        rtm_set_error("grid sizes must be positive");
        s = RTM_ERR_ARG;
    } else if ((s = ensure_device()) == RTM_OK) {
        const size_t vol = (size_t)(ny + 10) * (nx + 10) * (nz + 10);
        s = g_k3.buf.alloc(33 * vol);
        if (s == RTM_OK) {
            g_k3.ny = ny;
            g_k3.nz = nz;
            g_k3.nx = nx;
        }
    }
    rtm_set_status(s, "rtm3d_gpu_init");
}

extern "C" void rtm3d_gpu_func(int ny, int nz, int nx, float *vy0, float *vx0, float *vz0, float *syy0, float *sxx0,
                               float *szz0, float *sxy0, float *sxz0, float *syz0, float *vy1, float *vx1, float *vz1,
                               float *syy1, float *sxx1, float *szz1, float *sxy1, float *sxz1, float *syz1, float *vyo,
                               float *vxo, float *vzo, float *syyo, float *sxxo, float *szzo, float *sxyo, float *sxzo,
                               float *syzo, float *m1y, float *m1x, float *m1z, float *m2, float *m3, float *m2m3,
                               float *debug, float *gpu_kernel_time)
{
    (void)debug;
    auto run = [&]() -> int {
        RTM_CHECK_ARG(g_k3.buf.p && ny == g_k3.ny && nz == g_k3.nz && nx == g_k3.nx,
                      "rtm3d_gpu_init was not called for this grid");
        float *h[33] = {vy0, vx0, vz0, syy0, sxx0, szz0, sxy0, sxz0, syz0, vy1, vx1, vz1, syy1, sxx1, szz1, sxy1, sxz1,
                        syz1, vyo, vxo, vzo, syyo, sxxo, szzo, sxyo, sxzo, syzo, m1y, m1x, m1z, m2, m3, m2m3};
        for (int i = 0; i < 33; i++) RTM_CHECK_ARG(h[i], "null argument");
        const size_t vol = (size_t)(ny + 10) * (nx + 10) * (nz + 10);
        float *d[33];
        for (int i = 0; i < 33; i++) d[i] = g_k3.buf.p + i * vol;
        cudaEvent_t ev[4];
        for (int i = 0; i < 4; i++) RTM_CUDA(cudaEventCreate(&ev[i]));
        RTM_CUDA(cudaEventRecord(ev[0]));
        for (int i = 0; i < 33; i++) RTM_CUDA(cudaMemcpy(d[i], h[i], vol * sizeof(float), cudaMemcpyHostToDevice));
        RTM_CUDA(cudaEventRecord(ev[1]));
        TRY(k3_launch(ny, nz, nx, d, d + 9, d + 18, d + 27, g_k3_exact != 0, 0));
        RTM_CUDA(cudaEventRecord(ev[2]));
        for (int i = 18; i < 27; i++) RTM_CUDA(cudaMemcpy(h[i], d[i], vol * sizeof(float), cudaMemcpyDeviceToHost));
        RTM_CUDA(cudaEventRecord(ev[3]));
        RTM_CUDA(cudaEventSynchronize(ev[3]));
        if (gpu_kernel_time)
            for (int i = 0; i < 3; i++) {
                float ms = 0.f;
                RTM_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
                gpu_kernel_time[i] = ms / 1000.f;  // seconds, as the reference reports
            }
        for (int i = 0; i < 4; i++) cudaEventDestroy(ev[i]);
        return RTM_OK;
    };
    rtm_set_status(run(), "rtm3d_gpu_func");
}

extern "C" void rtm3d_gpu_final()
{
    g_k3.buf.release();
    g_k3.ny = g_k3.nz = g_k3.nx = 0;
    rtm_set_status(RTM_OK, "rtm3d_gpu_final");
}
