// iso_internal.cuh -- shared internals of the GB300 isosurface-similarity engine:
// context, device arena, error reporting and the exact FP32 primitives every
// kernel uses.  All kernels are compiled with -fmad=false: no multiply-add is
// fused unless written as __fmaf_rn, so device results match the CPU rounding
// step for step.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>

#include "isosim.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
int iso_fail(int code, const char *fmt, ...);
void iso_clear_error();

#define ISO_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e__ = (call);                                                          \
        if (e__ != cudaSuccess)                                                            \
            return iso_fail(e__ == cudaErrorMemoryAllocation ? ISO_ERR_NOMEM : ISO_ERR_CUDA, \
                            "%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e__)); \
    } while (0)

#define ISO_TRY(expr)                 \
    do {                              \
        int s__ = (expr);             \
        if (s__ != ISO_OK) return s__; \
    } while (0)

#define ISO_LAUNCHED(ctx)                                                                  \
    do {                                                                                   \
        (ctx)->launches++;                                                                 \
        cudaError_t e__ = cudaGetLastError();                                              \
        if (e__ != cudaSuccess)                                                            \
            return iso_fail(ISO_ERR_CUDA, "%s:%d: launch failed: %s", __FILE__, __LINE__,   \
                            cudaGetErrorString(e__));                                      \
    } while (0)

constexpr int ISO_MAX_BINS = 256;
constexpr int64_t ISO_HIST_SEGMENT_VALUES = 2097152;  // segment-major above 2^21 values (226..256 bins)
constexpr int ISO_WIDE_MAX_BINS = 224;                // up to this many bins: 32-bit counters, one CTA per pair
constexpr size_t ISO_HIST_CHUNK_BYTES = (size_t)1 << 30;  // per-pair global histograms of one segment-major chunk
// LBVH surfaces are built and queried in groups of at most this many points
// (default of iso_ctx_set_limit(ISO_LIMIT_LBVH_GROUP_POINTS))
constexpr int64_t ISO_LBVH_GROUP_POINTS = (int64_t)1 << 27;
// marching cubes: default of the largest per-block count table kept between
// the count and write passes (256 isovalues of a 256^3 volume take 136 MB)
constexpr int64_t ISO_SURF_BLOCK_COUNT_BYTES = (int64_t)1 << 30;

// ---------------------------------------------------------------------------
// device arena: named grow-only buffers owned by a context
// ---------------------------------------------------------------------------
enum IsoBuf {
    BUF_VOLUME = 0,
    BUF_ISO_SORTED,
    BUF_ISO_ORDER,
    BUF_SURF_COUNTS,     // per sorted isovalue: [regular, corner candidates, active, total verts]
    BUF_SURF_CURSOR,
    BUF_POINTS_RAW,      // float4 raw positions (grid units), all isovalues
    BUF_POINTS_NORM,     // float4 normalised positions
    BUF_CORNER_KEYS,
    BUF_CORNER_KEYS_ALT,
    BUF_SEG_OFFSET,      // per segment: first point (int64)
    BUF_SEG_COUNT,       // per segment: point count (int64)
    BUF_SORT_KEYS,
    BUF_SORT_KEYS_ALT,
    BUF_SORT_VALS,
    BUF_SORT_VALS_ALT,
    BUF_BVH_NODES,
    BUF_BVH_PARENT,
    BUF_BVH_FLAGS,
    BUF_BVH_LEAVES,
    BUF_FIELDS,          // distance fields, m x field_stride floats
    BUF_FIELD_MINMAX,    // per field: uint32 bits of min and max
    BUF_PAIR_TASKS,
    BUF_HIST_SCRATCH,    // per CTA: bins*bins uint32
    BUF_ISM,
    BUF_TASK_COUNTER,
    BUF_HIST_DUMP,
    BUF_MISC,
    BUF_CUB_TEMP,
    BUF_STAGING_A,
    BUF_STAGING_B,
    BUF_CLNC,            // c*ln(c) for c < 65536, FP64
    BUF_HIST_DUMP_SEG,   // per-pair global histograms of the segment-major schedule
    BUF_SURF_BLOCK_COUNTS,  // marching cubes: per block and isovalue, the vertex versions it counted
    BUF_ROW_CODES,          // segment-major histograms: per field and value, its precomputed row bucket
    BUF_TC_OPERANDS,        // tensor-core distance: every surface's points as MMA operand rows
    BUF_REF32_SUMS,         // reference FP32 MI: column and row sums of every ordered pair
    BUF_LOGF_TABLE,         // reference FP32 MI: logf of every count below 65536
    BUF_ISO_INDEX,          // marching cubes: bucket edges and first sorted isovalue at or above each
    BUF_COUNT_
};

struct iso_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    void *buf[BUF_COUNT_] = {};
    size_t cap[BUF_COUNT_] = {};
    int64_t launches = 0;
    void *host_pinned = nullptr;
    size_t host_pinned_cap = 0;
    bool clnc_ready = false;
    // shape of the distance-field matrix left by the last iso_ism call
    int last_m = 0;
    int64_t last_F = 0, last_stride = 0;
    // admission hook: called by iso_ism once the surface counts fix the
    // request's device-memory need; a non-zero return aborts the request
    int64_t lbvh_group_points = ISO_LBVH_GROUP_POINTS;  // see iso_ctx_set_limit
    int64_t hist_segment_values = ISO_HIST_SEGMENT_VALUES;  // 0: one CTA per pair for every length
    int64_t surf_block_count_bytes = ISO_SURF_BLOCK_COUNT_BYTES;  // see iso_ctx_set_limit
    int mi_mode = ISO_MI_FP64;  // ISO_MI_*: precision and order of the mutual information
    int64_t device_bytes_cap = 0;  // ISO_LIMIT_DEVICE_BYTES (0: none)
    int query_run = 0;             // ISO_LIMIT_QUERY_RUN (0: by volume size)
    int hist_row_codes = 0;        // ISO_LIMIT_HIST_ROW_CODES
    // set while a caller-supplied interval leaves values of its field above
    // its maximum: the histogram kernels must then clamp buckets to the last bin
    bool hist_clamp_top = false;
    // joint histograms of all ordered pairs kept in BUF_HIST_DUMP by the last
    // ISO_MI_REF32 similarity run (0 = none)
    int joint_m = 0, joint_bins = 0;
    int (*admit)(void *user, size_t bytes) = nullptr;
    void *admit_user = nullptr;
    // request shape for the admission estimate (set by iso_ism)
    int64_t plan_V = 0, plan_stride = 0;
    int plan_bins = 0, plan_lbvh = 0, plan_volume_copy = 0;
};

// Frees every arena buffer of a context (the context stays usable).
void iso_ctx_release(iso_ctx *ctx);
// Frees every buffer except the ones a request holds between its surface count
// pass and its admission (staged volume, sorted isovalues, counts, offsets, the
// marching-cubes per-block counts that the write pass reads).
void iso_ctx_release_except_surfaces(iso_ctx *ctx);

// Ensures buffer `b` holds at least `bytes`; contents are not preserved.
int iso_buf(iso_ctx *ctx, IsoBuf b, size_t bytes, void **out);
// Pinned host scratch of at least `bytes`.
int iso_host_scratch(iso_ctx *ctx, size_t bytes, void **out);

// Process-wide context of the calling thread's current device, for the
// reference-named entry points (created on first use, reference FP32 MI).
iso_ctx *iso_default_ctx();

// True if `p` is a device (or managed) pointer.
bool iso_is_device_ptr(const void *p);

// ---------------------------------------------------------------------------
// exact FP32 primitives
// ---------------------------------------------------------------------------

// Canonical squared distance: fma(dz,dz, fma(dx,dx, dy*dy)), each step rounded
// once.  That is how nvcc, with its default contraction, compiles the
// reference's x2 + y2 + z2 (float3SquaredDistance2_d, isosurfaces_cuda/src/
// BVH.cu:410-416); its own traversal kernel, run on the GPU, gives the same
// fields bit for bit.  The CPU oracle uses the same expression with libm fmaf.
__device__ __forceinline__ float iso_dist2(float dx, float dy, float dz)
{
    return __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
}

// Bucket of isosurfaces_cuda/src/JointHistogram.cu:63-75 with IEEE division.
// Values below the interval (only possible with a caller-supplied interval that
// does not contain the data) go to bucket 0 instead of indexing out of bounds.
__device__ __forceinline__ int iso_bucket(float v, float mn, float step, int bins)
{
    if (step == 0.0f) return 0;
    int b = __float2int_rz(__fdiv_rn(__fsub_rn(v, mn), step));
    b = b >= bins ? bins - 1 : b;
    return b < 0 ? 0 : b;
}

// Distance-field sample grid: the sample of DF index idx (z fastest over the
// (X/ds, Y/ds, Z/ds) grid) is ((x*ds + ds/2)/X, (y*ds + ds/2)/Y, (z*ds + ds/2)/Z)
// (isosurfaces_cuda/src/BVH.cu:393-406).
struct IsoSampleGrid {
    int X, Y, Z, ds;
    int64_t Y10, Z10, F;
};

__device__ __forceinline__ float3 iso_sample_point(const IsoSampleGrid &g, int64_t idx)
{
    int64_t z = idx % g.Z10, y = (idx / g.Z10) % g.Y10, x = idx / (g.Y10 * g.Z10);
    float3 s;
    s.x = __fdiv_rn((float)(x * g.ds + g.ds / 2), (float)g.X);
    s.y = __fdiv_rn((float)(y * g.ds + g.ds / 2), (float)g.Y);
    s.z = __fdiv_rn((float)(z * g.ds + g.ds / 2), (float)g.Z);
    return s;
}

// Field value from the minimum canonical squared distance: its square root,
// except that a one-point surface keeps the squared distance (BVH.cu:604-611).
__device__ __forceinline__ float iso_df_finish(float best, int64_t P) { return P == 1 ? best : __fsqrt_rn(best); }

// The reference's initial upper bound of a nearest-point search (BVH.cu:639).
constexpr float ISO_DF_INIT_BOUND = 100000.0f;

// Point sets of a distance-field launch.
struct IsoSegments {
    const float4 *points;   // normalised points (w unused)
    const int64_t *offset;  // per segment: first point
    const int64_t *count;   // per segment: number of points
};

// Tensor-core distance fields (csrc/iso_distance_tc.cu): segment q's field
// into fields + q*stride, for q < m.
int iso_run_distance_tc(iso_ctx *ctx, const IsoSampleGrid &g, const IsoSegments &sg, const int64_t *h_seg_count, int m,
                        float *fields, int64_t stride);

// Host-side launch helpers implemented per stage.
int iso_run_surfaces(iso_ctx *ctx, const float *d_vol, int X, int Y, int Z, const float *h_iso, int n,
                     int surface, int frame, int64_t *h_counts, int64_t *h_offsets,
                     iso_surface_stats *h_stats, int64_t *total_points_out);
int iso_run_distance(iso_ctx *ctx, int X, int Y, int Z, int ds, int method, const int32_t *h_segments,
                     int num_segments, const int64_t *h_seg_offset, const int64_t *h_seg_count,
                     int64_t field_stride);
int iso_run_similarity(iso_ctx *ctx, const float *d_fields_a, const float *d_fields_b, int m,
                       int64_t n, int64_t stride, int bins, const uint32_t *d_minmax_a,
                       const uint32_t *d_minmax_b, float *d_ism, uint32_t *d_joint_dump,
                       uint32_t *d_colrow_dump);
// Same, over an explicit list of (i, j) tasks: i indexes fields_a, j fields_b;
// the result goes to ism[i*m + j] (and [j*m + i] when symmetric).
int iso_run_similarity_tasks(iso_ctx *ctx, const float *d_fields_a, const float *d_fields_b, int m, int64_t n,
                             int64_t stride, int bins, const uint32_t *d_minmax_a, const uint32_t *d_minmax_b,
                             float *d_ism, const int2 *h_tasks, int64_t num_tasks, bool symmetric,
                             uint32_t *d_joint_dump, uint32_t *d_colrow_dump);
int iso_run_minmax(iso_ctx *ctx, const float *d_fields, int m, int64_t n, int64_t stride, uint32_t *d_minmax);
// The reference's FP32 MI (calculateMutualInformation, summation order and
// contraction included) of all m*m ordered pairs whose joint histograms are at
// d_joint (pair i*m + j at d_joint + (i*m + j)*bins*bins) and whose column and
// row sums are at d_colrow ([2][m*m*bins], as the histogram kernels dump
// them), into d_ism[i*m + j].
int iso_run_mi_ref32(iso_ctx *ctx, const uint32_t *d_joint, const uint32_t *d_colrow, int m, int bins, int64_t n,
                     float *d_ism);

constexpr int ISO_MAX_ISOVALUES = 4096;
