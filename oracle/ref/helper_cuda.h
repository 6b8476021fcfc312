/* Stand-in for the CUDA-samples header that the reference's gpu_err.h
 * includes (gpu_err.h:9).  The reference only needs a printable name for a
 * cufftResult (gpu_err.h:29); this header supplies one.  Test
 * infrastructure: used only to build the reference for golden vectors. */
#ifndef XCG_REF_HELPER_CUDA_SHIM_H
#define XCG_REF_HELPER_CUDA_SHIM_H
#include <cufft.h>
static inline const char *_cudaGetErrorEnum(cufftResult r)
{
    static char buf[32];
    snprintf(buf, sizeof buf, "cufftResult %d", (int)r);
    return buf;
}
#endif
