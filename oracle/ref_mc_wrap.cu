// Device code of the reference's marching cubes for the GPU checker
// (oracle/refgpu.py): the reference's MarchingCube.cu compiled from where it
// lies (with oracle/refshim_mc/refshim_texture.h force-included), its lookup
// tables compiled a second time from its tables.h as device arrays, and one
// kernel of this harness that points the file's texture holders at them and
// at the volume.  Test infrastructure only; nothing here copies reference code.
#include "isosurfaces_cuda/src/MarchingCube.cu"

namespace refdev {
#define uint __device__ unsigned int
#include "isosurfaces_cuda/src/tables.h"
#undef uint
}  // namespace refdev

extern "C" __global__ void refshim_mc_bind(const float *volume)
{
    edgeTex.ptr = refdev::edgeTable;
    triTex.ptr = &refdev::triTable[0][0];
    numVertsTex.ptr = refdev::numVertsTable;
    volumeTex.ptr = volume;
}
