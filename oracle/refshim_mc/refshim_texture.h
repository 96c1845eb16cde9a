/* Force-included when oracle/build_ref.sh compiles the reference's
 * MarchingCube.cu into a device-only cubin.  CUDA 13 no longer has texture
 * references; this header turns each of the file's `texture<T, 1, mode> name;`
 * declarations into a device-side holder of a plain pointer and its
 * tex1Dfetch(name, i) into a load through that pointer.  The host-side binding
 * calls of the file become no-ops: the checker (oracle/refgpu.py) sets the
 * pointers with the bind kernel of oracle/ref_mc_wrap.cu. */
#ifndef ORACLE_REFSHIM_TEXTURE_H
#define ORACLE_REFSHIM_TEXTURE_H
#include <cuda_runtime.h>
/* the reference file includes its vendored helper_cuda.h from its own folder;
 * that header reads cudaDeviceProp fields CUDA 13 no longer has, so the
 * checker's stand-in (refshim/) is taken first and its guard is set */
#include "isosurfaces_cuda/src/helper_cuda.h"
#define HELPER_CUDA_H

template <class T, int Dim, int Mode>
struct refshim_texture {
    const T *ptr;
};

template <class T, int D, int M>
__device__ __forceinline__ T tex1Dfetch(const refshim_texture<T, D, M> &t, int i)
{
    return t.ptr[i];
}

template <class T, int D, int M>
inline cudaError_t cudaBindTexture(size_t *, const refshim_texture<T, D, M> &, const void *, cudaChannelFormatDesc,
                                   size_t = ~(size_t)0)
{
    return cudaSuccess;
}

#define texture __device__ refshim_texture
#endif
