// Device code of the reference's LBVH for the GPU checker (oracle/refgpu.py):
// the reference's BVH.cu compiled from where it lies, plus one kernel of this
// harness that reports the sizes of its node structs and where an internal
// node keeps its child ids, so that the host side allocates the node arrays
// as the reference does and can read the built tree back.  Test
// infrastructure only; nothing here copies reference code.
#include "isosurfaces_cuda/src/BVH.cu"

extern "C" __global__ void refshim_bvh_sizes(int *out)
{
    InternalNode n;
    out[0] = (int)sizeof(LeafNode);
    out[1] = (int)sizeof(InternalNode);
    out[2] = (int)sizeof(float3);
    out[3] = (int)((const char *)&n.leftChildId - (const char *)&n);
    out[4] = (int)((const char *)&n.rightChildId - (const char *)&n);
}
