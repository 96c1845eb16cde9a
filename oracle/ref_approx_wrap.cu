/* Harness around the reference's own voxel-approximation code
 * (isosurfaces_cuda/src/IsosurfaceApproximation.cu), compiled from the
 * reference sources by oracle/build_ref.sh into oracle/_ref/.  TEST
 * INFRASTRUCTURE.  calculate_approximation_CPU fills the (X-1)(Y-1)(Z-1) cell
 * array; the buffer starts as all-ones bytes like the GPU entry's cudaMemset
 * (IsosurfaceApproximation.cu:175) and is compacted stably as thrust::copy_if
 * does (thrustWrapper.h:47-54). */
#include "isosurfaces_cuda/src/IsosurfaceApproximation.cu"
#include <cstdlib>
#include <cstring>

extern "C" long ref_approximation_cpu(float *data, float iso, int X, int Y, int Z, int *out_xyz, long cap)
{
    const int scale = 1;
    unsigned long SIZE = (unsigned long)(X * Y * Z);
    unsigned long NUM_POINTS = ((X - scale) * (Y - scale) * (Z - scale)) / scale;
    int3 *cells = (int3 *)malloc(sizeof(int3) * NUM_POINTS);
    memset(cells, 0xff, sizeof(int3) * NUM_POINTS);
    calculate_approximation_CPU(data, iso, X, Y, Z, cells, (int)SIZE, 0, scale);
    long c = 0;
    for (unsigned long i = 0; i < NUM_POINTS; ++i) {
        if (cells[i].x >= 0) {
            if (c < cap) { out_xyz[3 * c] = cells[i].x; out_xyz[3 * c + 1] = cells[i].y; out_xyz[3 * c + 2] = cells[i].z; }
            ++c;
        }
    }
    free(cells);
    return c;
}
