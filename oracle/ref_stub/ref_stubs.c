/* Empty stand-ins for the reference's CUDA glue (rtmlib-modC-gpu.cu:35,115,
 * 425), which rtmlib-modC.c calls even when the GPU hand-off is off (not
 * compiled into the GPU comparator build, REF_GPU_BUILD).  Test
 * infrastructure only.
 *
 * The reference reads the uninitialised halo of its padded copies
 * (rtmlib-modC.c:51-57, only the first plane is zeroed), multiplying it by
 * zero-padded coefficients.  Fresh mmap'd pages make that halo zero; fixing
 * the mmap threshold keeps every large malloc on fresh pages regardless of
 * what the calling process freed before, so repeated calls are
 * deterministic. */
#include <malloc.h>

__attribute__((constructor)) static void ref_fix_mmap_threshold(void)
{
    mallopt(M_MMAP_THRESHOLD, 128 * 1024);
}

#ifndef REF_GPU_BUILD  /* the GPU comparator links the reference's real ones */
void rtm_gpu_init(int nt, int nz, int nx) { (void)nt; (void)nz; (void)nx; }
void rtm_gpu_final(void) {}
void rtm_gpu_func(void) {}
#endif
