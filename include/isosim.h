/*
 * isosim.h -- C ABI of the GB300 isosurface-similarity engine.
 *
 * Plain C types only (no CUDA, C++ or torch types).  Every entry point that can
 * fail returns an int status (ISO_OK == 0, negative on error) and never exits
 * the process; iso_last_error() returns the message of the calling thread's
 * most recent failure.  The reference instead terminates through
 * checkCudaErrors (isosurfaces_cuda/hdr/helper_cuda.h:968-996).
 *
 * Volumes are float32 in the reference's flattened "img" order (z fastest,
 * img[x*Y*Z + y*Z + z]; types/src/Isosurface.cpp:185-200).  Pointer arguments
 * documented as "host or device" are read with cudaMemcpyDefault, so both
 * pageable/pinned host memory and device memory are accepted.
 *
 * Paths in citations are relative to the reference's isosurfaces_lib/ folder.
 */
#ifndef ISOSIM_H
#define ISOSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C99 _Bool and C++ bool share size and ABI */
#ifdef __cplusplus
#define ISO_BOOL bool
#else
#define ISO_BOOL _Bool
#endif

#if defined(__GNUC__)
#define ISO_API __attribute__((visibility("default")))
#else
#define ISO_API
#endif

/* status codes */
#define ISO_OK 0
#define ISO_ERR_ARG (-1)      /* invalid argument */
#define ISO_ERR_CUDA (-2)     /* CUDA runtime error */
#define ISO_ERR_CAPACITY (-3) /* caller buffer or fixed-size structure too small */
#define ISO_ERR_NOMEM (-4)    /* device or host allocation failed */
#define ISO_ERR_INTERNAL (-5) /* a device-side consistency check failed */

/* surface extraction */
#define ISO_SURFACE_MC 0     /* marching cubes: cudaMarchingCube (isosurfaces_cuda/src/MarchingCube.cpp:588) */
#define ISO_SURFACE_APPROX 1 /* voxel approximation: approximate_isosurfaces_h (IsosurfaceApproximation.cu:160) */

/* marching-cubes coordinate frame */
#define ISO_FRAME_REF 0   /* the reference kernel's frame: the z-fastest volume indexed x-fastest (MarchingCube.cu:60-65) */
#define ISO_FRAME_CANON 1 /* geometric frame of the volume (x slowest, z fastest) */

/* distance-field method; all give bit-identical fields */
#define ISO_DF_BRUTE 0 /* every sample against every surface point, FP32 */
#define ISO_DF_LBVH 1  /* linear BVH (Morton codes, radix sort, Karras hierarchy, stack query) */
#define ISO_DF_TC 2    /* every sample against every point as a tensor-core contraction
                          |s-p|^2 = |s|^2 + |p|^2 - 2 s.p (split-f16 operands, FP32 accumulation)
                          that selects candidates; each candidate's distance is then
                          computed exactly in FP32 */

/* marching-cubes result flags (iso_surface_stats.flags) */
#define ISO_MC_REF_DROPPED 1 /* more than V-3 triangle vertices: the reference drops triangles here */

typedef struct iso_ctx iso_ctx;

typedef struct iso_opts {
    int surface;      /* ISO_SURFACE_* */
    int frame;        /* ISO_FRAME_* (marching cubes only) */
    int df_method;    /* ISO_DF_* */
    int df_downscale; /* >= 1; DF grid is (X/ds, Y/ds, Z/ds) */
    int bins;         /* joint-histogram bins per axis, 2..256 */
} iso_opts;

typedef struct iso_surface_stats {
    int64_t points;        /* unique surface points (0 = empty surface) */
    int64_t active_voxels; /* cells with a non-empty case (marching cubes) */
    int64_t total_verts;   /* sum of per-case triangle-vertex counts (marching cubes) */
    int32_t flags;         /* ISO_MC_* */
    int32_t reserved;
} iso_surface_stats;

typedef struct iso_rep {
    float isovalue; /* as the reference leaves it: the isovalue of the previously popped pick */
    float priority;
    int32_t id;     /* isovalue index */
    int32_t map_id; /* row of the similarity map */
} iso_rep;

typedef struct iso_timing {
    float surface_ms, distance_ms, histogram_ms, total_ms;
} iso_timing;

/* ---------------------------------------------------------------------- */
/* Context                                                                 */
/* ---------------------------------------------------------------------- */

/* Creates a context on `device` with its own CUDA stream and a grow-only
 * device arena reused by every call.  One context per host thread. */
ISO_API int iso_ctx_create(int device, iso_ctx **out);
ISO_API void iso_ctx_destroy(iso_ctx *ctx);
/* The context's cudaStream_t, as void*. */
ISO_API void *iso_ctx_stream(iso_ctx *ctx);
/* Bytes currently held by the context's device arena. */
ISO_API size_t iso_ctx_device_bytes(iso_ctx *ctx);
/* Thread-local message of the last failure ("" if none). */
ISO_API const char *iso_last_error(void);
/* Number of kernel launches issued by this context so far. */
ISO_API int64_t iso_ctx_launches(iso_ctx *ctx);

/* Tunable limits of a context. */
#define ISO_LIMIT_LBVH_GROUP_POINTS 1 /* LBVHs are built for groups of surfaces of at most this many
                                          points (default 2^27), bounding their device memory */
#define ISO_LIMIT_HIST_SEGMENT_VALUES 2 /* histograms of 226..256 bins over fields longer than this
                                            run segment by segment (all running pairs on the same
                                            slice of their fields; up to 1 GB of per-pair histograms);
                                            0 = never; otherwise a multiple of 4, at least 65536;
                                            default 2097152 */
#define ISO_LIMIT_SURF_BLOCK_COUNT_BYTES 3 /* marching cubes keeps each block's vertex counts between
                                               its count and write passes while that table takes at
                                               most this many bytes (default 2^30), else the write
                                               pass counts again; 0 = always count again */
#define ISO_LIMIT_DEVICE_BYTES 5 /* the context's arena may hold at most this many bytes (0 =
                                     no cap, the default); a call whose buffers would exceed it
                                     fails with ISO_ERR_NOMEM and leaves the context usable */
#define ISO_LIMIT_QUERY_RUN 6 /* LBVH query: samples each lane sweeps along x, 8, 16, 32 or 64
                                  (0 = by volume size, the default: 64 from 128 samples along x,
                                  else 8); results are identical for every value */
#define ISO_LIMIT_HIST_ROW_CODES 7 /* segment-major histograms: 1 computes each field's buckets
                                       once for the pairs in which it has the larger maximum,
                                       0 (default) computes both buckets in every pair; results
                                       are identical */
#define ISO_LIMIT_MI_MODE 4 /* ISO_MI_*: how the mutual information of a pair is computed
                                (default ISO_MI_FP64; the reference-named entry points use
                                ISO_MI_REF32) */
ISO_API int iso_ctx_set_limit(iso_ctx *ctx, int which, int64_t value);

/* Mutual-information modes (ISO_LIMIT_MI_MODE).  Both use the same exact
 * joint histograms and the reference's formula ISM = 2I/(hX+hY) on raw counts.
 *   ISO_MI_FP64:  FP64 sums, one value per unordered pair written to (i,j)
 *                 and (j,i): the map is symmetric and accurate to float
 *                 rounding of the FP64 result.
 *   ISO_MI_REF32: the reference's own FP32 evaluation
 *                 (isosurfaces_cuda/src/JointHistogram.cu:24-60, called once
 *                 per ordered pair at :156-160): same summation order, logf
 *                 and multiply-add contraction, so every entry equals the
 *                 reference's bit for bit and (i,j) may differ from (j,i).
 *                 Keeps all m*m joint histograms in device memory
 *                 (m*m*bins*bins*4 bytes).  Applies to iso_ism,
 *                 iso_similarity_map, iso_cross_map and calculate_histogram_h;
 *                 iso_pair_map and iso_similarity_map_noalloc are FP64 only. */
#define ISO_MI_FP64 0
#define ISO_MI_REF32 1

/* ---------------------------------------------------------------------- */
/* Whole-volume pipeline (replaces the per-isovalue loop of Single::run,   */
/* runtime/src/Single.cpp:193-243, and calculate_histogram_W,              */
/* isosurfaces_cuda/funcs.cpp:148-205)                                     */
/* ---------------------------------------------------------------------- */

/* volume: X*Y*Z floats (host or device).  isovalues: n floats (host).
 * Surfaces for all isovalues, distance fields of the non-empty ones, all-pairs
 * joint histograms and FP64 normalised mutual information.  Outputs (host or
 * device): ism_out m*m floats row-major, field_ids_out the isovalue index of
 * each row (n capacity), *m_out = number of non-empty surfaces.  stats_out
 * (n entries) and timing_out may be NULL. */
ISO_API int iso_ism(iso_ctx *ctx, const float *volume, int X, int Y, int Z,
                    const float *isovalues, int n, const iso_opts *opts,
                    float *ism_out, int32_t *field_ids_out, int32_t *m_out,
                    iso_surface_stats *stats_out, iso_timing *timing_out);

/* Cross map between two field sets of equal size m (the multi mode of
 * calculate_histogram_h, isosurfaces_cuda/src/JointHistogram.cu:309-318,
 * used by MultiVar::computeMultiMap, runtime/src/MultiVar.cpp:170-249):
 * out[i*m + j] = NMI(fields_a[i], fields_b[j]).  fields_*: m*n floats. */
ISO_API int iso_cross_map(iso_ctx *ctx, const float *fields_a, const float *fields_b, int m, int64_t n,
                          int bins, float *out);

/* Batched cross maps (the multi module over many volume pairs at once):
 * fields holds R rows of n values (row r at fields + r*stride, host or
 * device; aligned device rows are used in place).  For every pair
 * (pairs[2t], pairs[2t+1]) the NMI goes to out[a*R + b] and out[b*R + a]
 * (out: R*R floats, host or device; other entries are left as they are).
 * Each pair's histogram uses the union of its two fields' intervals, as
 * calculate_histogram_h's multi mode does (JointHistogram.cu:127-129). */
ISO_API int iso_pair_map(iso_ctx *ctx, const float *fields, int R, int64_t n, int64_t stride, int bins,
                         const int32_t *pairs, int64_t npairs, float *out);

/* Aggregates k x k blocks of a pair map (R x R, host or device) into one
 * similarity per block: for block (A, B) = (blocks[2q], blocks[2q+1]),
 * out[2q] = block mean, out[2q+1] = best-match score (mean of row maxima and
 * of column maxima, averaged).  With one block per (volume, volume) pair of
 * representative sets this gives the entries of timestep and variable
 * similarity matrices.  No reference counterpart: the reference stops at the
 * cross maps (runtime/src/MultiVar.cpp:222-227). */
ISO_API int iso_block_similarity(iso_ctx *ctx, const float *map, int64_t R, int k, const int32_t *blocks,
                                 int64_t nblocks, float *out);

/* ---------------------------------------------------------------------- */
/* Stage entry points                                                      */
/* ---------------------------------------------------------------------- */

/* Surface points of n isovalues.  counts_out[k] = unique points of isovalue k.
 * points_out (host or device, may be NULL to query counts): concatenated xyz
 * float triples in isovalue order, marching cubes vertices sorted
 * lexicographically per isovalue (the reference's sort + unique order),
 * approximation cells as float-converted integer triples in linear cell order.
 * Returns ISO_ERR_CAPACITY if cap_points < sum(counts). */
ISO_API int iso_surface_points(iso_ctx *ctx, const float *volume, int X, int Y, int Z,
                               const float *isovalues, int n, int surface, int frame,
                               int64_t *counts_out, float *points_out, int64_t cap_points,
                               iso_surface_stats *stats_out);

/* Distance field of one point set given in normalised coordinates (p / max(X,Y,Z),
 * isosurfaces_cuda/funcs.cpp:150-175): out[i] = sqrt(min_p |s_i - p|^2) over the
 * sample grid of isosurfaces_cuda/src/BVH.cu:393-406 (a single point gives the
 * squared distance, BVH.cu:604-611).  points: P xyz triples (host or device);
 * out: (X/ds)(Y/ds)(Z/ds) floats (host or device). */
ISO_API int iso_distance_field(iso_ctx *ctx, const float *points, int64_t P, int X, int Y, int Z,
                               int downscale, int method, float *out);

/* Similarity map of m fields of n values each (fields: m*n, host or device):
 * ism_out m*m (FP64 MI rounded to float).  joint_out (may be NULL): m*m*bins*bins
 * uint32 histograms of every ordered pair (row = bucket of field i). */
ISO_API int iso_similarity_map(iso_ctx *ctx, const float *fields, int m, int64_t n, int bins,
                               float *ism_out, uint32_t *joint_out);

/* Representative isovalues (types/src/SimilarityMap.cpp:88-227): Bruckner's
 * recursive prioritisation + greedy re-weighted selection; ties go to the lower
 * map index.  ism: m*m host floats; ids: isovalue index per row; isovalues:
 * indexed by id.  Writes min(cnt, m) entries, returns that count (or < 0). */
ISO_API int iso_select_representatives(const float *ism, int m, const int32_t *ids, const float *isovalues,
                                       int cnt, iso_rep *out);

/* Isovalues of runtime/src/Single.cpp:286-392: uniform != 0 equalises a
 * 65536-bin histogram of the volume (computed on the GPU) into n groups, else
 * min + i*(max-min)/n.  vmin/vmax: the volume's real range
 * (types/src/Isosurface.cpp:48-75, see iso_real_range). */
ISO_API int iso_isovalues(iso_ctx *ctx, const float *volume, int64_t V, float vmin, float vmax, int n,
                          int uniform, float *out);

/* Real min/max of values within [cfg_min, cfg_max] (types/src/Isosurface.cpp:48-75). */
ISO_API int iso_real_range(iso_ctx *ctx, const float *volume, int64_t V, float cfg_min, float cfg_max,
                           float *out_min, float *out_max);

/* Reorders a volume stored x-fastest (the .dat file layout read by
 * filehandler/src/BinaryFloatReader.cpp:29-48, element x + y*X + z*X*Y) into
 * the img order (z fastest, x*Y*Z + y*Z + z) on the GPU.  src and dst: host or
 * device, X*Y*Z floats each. */
ISO_API int iso_transpose_xfastest(iso_ctx *ctx, const float *src, int X, int Y, int Z, float *dst);

/* Copies row `row` of the distance-field matrix left by the context's last
 * iso_ism call (row = map index, i.e. field_ids_out[row]'s surface) to `out`
 * (host or device, (X/ds)(Y/ds)(Z/ds) floats) -- the representative
 * fields the single module writes as distancefield-<k>.df. */
ISO_API int iso_copy_field(iso_ctx *ctx, int row, float *out);

/* Autotuner: times the whole pipeline on this workload under candidate launch
 * shapes -- ISO_LIMIT_QUERY_RUN and ISO_LIMIT_LBVH_GROUP_POINTS for the
 * distance stage, ISO_LIMIT_HIST_SEGMENT_VALUES for the histogram stage --
 * each judged by the time of its own stage, and applies the best set to the
 * context (kept only if the whole pipeline is at least as fast as with the
 * context's previous settings).  Results do not depend on these settings.
 * cache_path (may be NULL): a text file of earlier choices; a hit applies the
 * cached set without trials, a miss appends the new choice.  Replaces the
 * reference's fixed launch shapes (isosurfaces_cuda/src/JointHistogram.cu:
 * 362-364, BVH.cu:667-673). */
typedef struct iso_tuning {
    int64_t hist_segment_values; /* chosen ISO_LIMIT_HIST_SEGMENT_VALUES */
    int64_t lbvh_group_points;   /* chosen ISO_LIMIT_LBVH_GROUP_POINTS */
    int32_t query_run;           /* chosen ISO_LIMIT_QUERY_RUN (0 = by volume size) */
    int32_t from_cache;          /* 1: read from cache_path, no trials run */
    float default_ms;            /* pipeline time with the previous settings */
    float tuned_ms;              /* pipeline time with the chosen settings */
    int32_t trials;              /* pipeline runs timed */
    int32_t reserved;
} iso_tuning;
ISO_API int iso_autotune(iso_ctx *ctx, const float *volume, int X, int Y, int Z, const float *isovalues, int n,
                         const iso_opts *opts, const char *cache_path, iso_tuning *out);

/* Copies the joint histogram of ordered pair (i, j) (row = bucket of field i)
 * kept by the context's last ISO_MI_REF32 similarity run (iso_ism,
 * iso_similarity_map or iso_cross_map) to out (host or device, bins*bins
 * uint32).  ISO_ERR_ARG when no histograms are kept. */
ISO_API int iso_copy_joint_histogram(iso_ctx *ctx, int i, int j, uint32_t *out);

/* Measures the peak rate of the joint-histogram kernel's counter update on
 * its own (packed 16-bit shared-memory atomic plus wrap check, random bins,
 * no bucket arithmetic or loads): the shared-memory-atomic roofline of the
 * histogram stage.  bins: a power of two in [2, 256]. */
ISO_API int iso_probe_counter_rate(iso_ctx *ctx, int bins, double *updates_per_s);

/* Failure-detection probe: runs the bounded barrier wait that the
 * tensor-core distance kernel uses (a wait that gives up after a time limit,
 * after which the kernel reports an error and returns) on a barrier that one
 * thread arrives at first (arrive != 0) or that nothing arrives at (arrive =
 * 0).  *timed_out is 1 when the wait gave up after limit_ns nanoseconds (at
 * most 1e10), 0 when it completed; the context stays usable either way. */
ISO_API int iso_probe_wait_timeout(iso_ctx *ctx, int arrive, int64_t limit_ns, int *timed_out);

/* ---------------------------------------------------------------------- */
/* Reference-named entry points (drop-in for isosurfaces_cuda/funcs.h)     */
/* ---------------------------------------------------------------------- */

typedef struct iso_int3 { int32_t x, y, z; } iso_int3;

/* isosurfaces_cuda/funcs.h:32-36, JointHistogram.cu:266-420.  Same arguments
 * and meaning: numFields fields (2*numFields with multi), similarity map
 * h_simMap (simMapSize x simMapSize), per-ordered-pair column and row sums
 * (numFields^2 * histogramSize each).  h_jointHist is left untouched, as the
 * reference leaves it (its copy-back is commented out, :397).  The map is the
 * reference's FP32 MI, bit for bit (ISO_MI_REF32).  Values above their
 * field's maxValue count in the last bucket, as in the reference; an interval
 * whose minValue lies above one of its field's values is refused (nothing is
 * written; iso_last_error names the field), since the reference would index
 * below its histogram there.  Runs on the calling thread's current CUDA
 * device, through a process-wide context per device. */
ISO_API void calculate_histogram_h(float **distanceFields, float *minValues, float *maxValues, const int fieldSize,
                                   const unsigned long numFields, const unsigned long histogramSize,
                                   unsigned int *h_jointHist, unsigned int *h_colSums, unsigned int *h_rowSums,
                                   float *h_simMap, const int simMapSize, const ISO_BOOL multi);

/* isosurfaces_cuda/funcs.h:23-24, IsosurfaceApproximation.cu:159-212: cells
 * crossing the isovalue as int triples in linear order; *h_points is
 * malloc'd by the callee and freed by the caller with free().  scale must be 1
 * (the only value the reference's callers use, types/src/Isosurface.cpp:284).
 * Returns the count, or a negative status. */
ISO_API long approximate_isosurfaces_h(float *h_data, float isovalue, const int dimX, const int dimY, const int dimZ,
                                       const int scale, iso_int3 **h_points);

/* C form of cudaMarchingCube (isosurfaces_cuda/hdr/MarchingCube.h:11-16,
 * MarchingCube.cpp:588-710): unique vertices (x,y,z,w=1) sorted
 * lexicographically, *out_xyzw malloc'd by the callee.  maxVerts as in the
 * reference (triangles whose first index is >= maxVerts-3 are dropped there;
 * here ISO_ERR_CAPACITY is returned in that case).  Reference frame. */
ISO_API int iso_marching_cube_h(float iso, int dimX, int dimY, int dimZ, const float *h_volume, int maxVerts,
                                float **out_xyzw, long *out_count);

/* C form of generateHierarchy_h (isosurfaces_cuda/funcs.h:43-44, BVH.cu:814-875)
 * for the non-sampleGiven case: points already normalised, distances written to
 * h_distances ((X/ds)(Y/ds)(Z/ds) floats).  numSamples (the reference's 1500
 * pre-sampled upper bound) does not change the result and is accepted for
 * signature parity. */
ISO_API int iso_generate_hierarchy_h(const float *points_xyz, long numPoints, int dimX, int dimY, int dimZ,
                                     float *h_distances, int numSamples, int dfDownscale);

/* ---------------------------------------------------------------------- */
/* Serving loop: device-resident request queue with continuous batching   */
/* (the reference's batch driver, runtime/src/Scripting.cpp:22-236, runs   */
/* one volume at a time; this is its concurrent form)                      */
/* ---------------------------------------------------------------------- */

typedef struct iso_server iso_server;

typedef struct iso_request {
    const float *volume;      /* X*Y*Z floats, img order, host or device; read while the request runs */
    int X, Y, Z;
    const float *isovalues;   /* n floats, host */
    int n;
    iso_opts opts;
    float *ism_out;           /* n*n floats capacity (m*m written), host or device */
    int32_t *field_ids_out;   /* n entries capacity */
    int32_t *m_out;           /* may be NULL */
} iso_request;

typedef struct iso_request_result {
    int status;
    int32_t m;
    double latency_ms;        /* submission to completion */
    double queue_ms;          /* submission to start */
    iso_timing timing;        /* GPU stage times */
} iso_request_result;

typedef struct iso_server_stats {
    int64_t completed, failed;
    double p50_ms, p99_ms;    /* request latency percentiles over completed requests */
    size_t peak_device_bytes; /* highest admitted total */
    size_t held_device_bytes; /* arenas currently held */
} iso_server_stats;

/* A pool of `slots` workers on `device`, each with its own stream and arena;
 * requests run concurrently as workers and device memory free up.  A request
 * is admitted once its surface count pass fixes its device-memory need and
 * that need fits the budget next to the running requests (idle arenas are
 * trimmed to make room; waiting requests go in submission order; a request
 * larger than the budget fails with ISO_ERR_NOMEM). */
ISO_API int iso_server_create(int device, int slots, size_t hbm_budget_bytes, iso_server **out);
/* Order in which workers take queued requests.  ISO_SERVE_FIFO (the default):
 * submission order.  ISO_SERVE_SHORTEST_FIRST: the request with the smallest
 * work estimate (samples x isovalues x (isovalues + 64)) first, unless the
 * oldest queued request has waited more than max_wait_ms, which then goes
 * first; a request smaller than one already running is issued on a
 * high-priority CUDA stream.  Results are the same under either policy. */
#define ISO_SERVE_FIFO 0
#define ISO_SERVE_SHORTEST_FIRST 1
ISO_API int iso_server_set_policy(iso_server *s, int policy, double max_wait_ms);
/* Applies iso_ctx_set_limit(which, value) to every worker context (for
 * example ISO_LIMIT_MI_MODE for the reference's own FP32 MI).  Only while no
 * request is queued or running; ISO_ERR_ARG otherwise. */
ISO_API int iso_server_set_limit(iso_server *s, int which, int64_t value);
/* Queues a request (the descriptor is copied; the buffers must stay valid
 * until iso_server_wait returns for its ticket). */
ISO_API int iso_server_submit(iso_server *s, const iso_request *req, int64_t *ticket);
/* Blocks until the request is done; returns its status. */
ISO_API int iso_server_wait(iso_server *s, int64_t ticket, iso_request_result *result);
ISO_API int iso_server_get_stats(iso_server *s, iso_server_stats *out);
/* Finishes queued requests, then stops the workers. */
ISO_API void iso_server_destroy(iso_server *s);

/* ---------------------------------------------------------------------- */
/* Allocation-free similarity map (no counterpart in the reference)        */
/* ---------------------------------------------------------------------- */

#define ISO_NOALLOC_MAX_FIELDS 256
#define ISO_NOALLOC_MAX_VALUES 16777216

/* The same similarity map as iso_similarity_map, for callers that must not
 * allocate GPU memory during the call: a process running under a fixed,
 * pre-committed device-memory budget, or code on a path where a call into the
 * allocator could block or fail.  Nothing is allocated: all scratch is a
 * fixed array of about 3.2 MB inside this library, which every device that
 * loads the library keeps until the process exits.
 *   d_fields: m rows of n float32 values in device memory, row i at
 *             d_fields + i*stride (16-byte aligned base, stride >= n and a
 *             multiple of 4);  d_ism_out: m*m floats of device memory;
 *   stream:   a cudaStream_t (NULL = legacy default stream); the call
 *             synchronises it before returning.
 * Limits: m <= ISO_NOALLOC_MAX_FIELDS and n <= ISO_NOALLOC_MAX_VALUES (larger
 * m or n return ISO_ERR_CAPACITY); bins even in [2, 256], a bad stride or
 * alignment, or host pointers return ISO_ERR_ARG.  The first call on a
 * device looks up the array's device address and fills a lookup table.  Every
 * call synchronises its stream, so no call can be captured into a CUDA graph.
 * All calls share the array: calls that overlap on the GPU race. */
ISO_API int iso_similarity_map_noalloc(const float *d_fields, int m, int64_t n, int64_t stride, int bins,
                                       float *d_ism_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
