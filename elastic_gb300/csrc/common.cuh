// Shared helpers for the GB300 elastic RTM kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>

// Status codes returned by every int-returning entry point of the C-ABI.
enum RtmStatus {
    RTM_OK = 0,
    RTM_ERR_ARG = 1,      // bad size, index or pointer
    RTM_ERR_NOMEM = 2,    // device or pinned allocation failed
    RTM_ERR_CUDA = 3,     // a CUDA call failed (message in rtm_last_error)
    RTM_ERR_TIMEOUT = 4,  // a bounded device-side wait ran out
    RTM_ERR_STATE = 5,    // call order violated (e.g. no prior init)
};

void rtm_set_error(const char *fmt, ...);
void rtm_set_status(int s, const char *where);

// On failure the runtime's last-error slot is cleared as well, so that one
// failed call is reported once and not again by the next check.
#define RTM_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            rtm_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return RTM_ERR_CUDA;                                                           \
        }                                                                                  \
    } while (0)

#define RTM_CHECK_ARG(cond, ...)          \
    do {                                  \
        if (!(cond)) {                    \
            rtm_set_error(__VA_ARGS__);   \
            return RTM_ERR_ARG;           \
        }                                 \
    } while (0)

// Separately rounded multiply and add.  The intrinsics are never contracted
// into a fused multiply-add, which keeps "exact" kernels in the same
// arithmetic as the reference's CPU code.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

// 10th-order staggered-grid coefficients (lgan/elastic
// 2d_rtm_restart/Src_working/rtmlib-mod.f90:15).  c[0] = c1 ... c[4] = c5.
template <typename T>
struct StagCoef {
    static __host__ __device__ __forceinline__ T c(int k)
    {
        return k == 0 ? T(35.0 / 294912.0)
             : k == 1 ? T(-405.0 / 229376.0)
             : k == 2 ? T(567.0 / 40960.0)
             : k == 3 ? T(-735.0 / 8192.0)
                      : T(19845.0 / 16384.0);
    }
};

// One-time per-device settings (kernel attributes such as the dynamic
// shared-memory limit, occupancy-derived grid sizes, device attributes) are
// kept per CUDA device, indexed by the caller's current device, and set
// under one process-wide lock, so a process that launches on several
// devices, from several threads, sets each of them once on every device.
constexpr int RTM_MAX_DEVICES = 64;
static inline int rtm_current_device()
{
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= RTM_MAX_DEVICES) {
        cudaGetLastError();
        d = 0;
    }
    return d;
}
static inline std::mutex &rtm_device_state_lock()
{
    static std::mutex m;
    return m;
}

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Float max-abs accumulated with integer atomics on the bit pattern (valid
// for non-negative floats).
__device__ __forceinline__ void atomic_max_abs(float *addr, float v)
{
    atomicMax(reinterpret_cast<int *>(addr), __float_as_int(fabsf(v)));
}
