/* Minimal stand-in for the reference's vendored CUDA sample helper header, used
 * only when oracle/build_ref.sh compiles the reference's own sources.  The
 * vendored header reads cudaDeviceProp fields that CUDA 13 no longer has; the
 * reference code on the checked path needs just these two status checks. */
#ifndef ORACLE_REFSHIM_HELPER_CUDA_H
#define ORACLE_REFSHIM_HELPER_CUDA_H
#include <cstdio>
#include <cuda_runtime.h>
#define checkCudaErrors(val) refshim_check((val), #val, __FILE__, __LINE__)
#define getLastCudaError(msg) refshim_check(cudaGetLastError(), msg, __FILE__, __LINE__)
static inline void refshim_check(cudaError_t e, const char *what, const char *file, int line)
{
    if (e != cudaSuccess) std::fprintf(stderr, "refshim: %s failed at %s:%d: %s\n", what, file, line, cudaGetErrorString(e));
}
#endif
