/* Build-time shim for compiling the reference's rtmlib-modC.c on the CPU
 * only (test infrastructure).  It pulls in the reference's own gpu.h (index
 * macros and tile sizes) and then sets the GPU hand-off step below zero, the
 * reference's documented switch for "CPU only computing"
 * (2d_rtm_restart/Src_working/rtmlib-modC.c:119). */
#include_next "gpu.h"
#undef GPU_start_step
#define GPU_start_step (-1)
