/*
 * isooracle.c -- CPU oracle for the isosurface-similarity hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke check
 * and the CPU-baseline leg of bench.py load it; the product library never links,
 * loads or calls it, and no product code path falls back to it.
 *
 * Every routine restates the reference algorithm (mimre25/isosurface-analysis) in
 * plain C, citing the reference file:line it follows (paths relative to the
 * reference's isosurfaces_lib/ directory).  Pinning:
 *   - bucket selection, joint histograms, FP32 mutual information and the voxel
 *     approximation are checked against the reference's own CPU functions
 *     compiled from its sources (oracle/build_ref.sh -> oracle/_ref/) and against
 *     golden vectors those functions produced (tests/golden/);
 *   - the marching-cubes triangle-count table used here is derived from first
 *     principles and checked entry by entry against the reference's table;
 *   - marching cubes, distance fields and representative selection are
 *     restatements of the reference's GPU/host code (no runnable reference
 *     counterpart exists in this environment); the FP64 distance field is the
 *     exact nearest-surface distance they are compared against.
 *
 * Compile with -ffp-contract=off: every rounding step is written out explicitly
 * (fmaf where a fused multiply-add is meant), so x86-64 and aarch64 builds give
 * identical bits.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <time.h>
#include <string.h>

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* Joint histograms and mutual information                                    */
/* ------------------------------------------------------------------------- */

/* isosurfaces_cuda/src/JointHistogram.cu:63-75 (findBucket_d). */
ORC_API int orc_find_bucket(float val, float min_value, float step, int bins)
{
    if (step == 0.0f) return 0;
    int bucket = (int)((val - min_value) / step);
    return bucket >= bins ? bins - 1 : bucket;
}

/* types/src/DistanceField.cpp:159-200 (getInterval): min starts at FLT_MAX,
 * max starts at FLT_MIN (the smallest positive normal float). */
ORC_API void orc_field_interval(const float *f, long n, float *out_min, float *out_max)
{
    float mn = FLT_MAX, mx = FLT_MIN;
    for (long i = 0; i < n; ++i) {
        float v = f[i];
        if (v < mn) mn = v;
        if (v > mx) mx = v;
    }
    *out_min = mn;
    *out_max = mx;
}

/* isosurfaces_cuda/src/JointHistogram.cu:127-154 (calculate_histogram_g, one
 * task): pair interval = union of both field intervals, step = (max-min)/H,
 * row = bucket of field 1, column = bucket of field 2.  joint is H*H row-major;
 * col_sums / row_sums may be NULL. */
ORC_API void orc_pair_histogram(const float *f1, const float *f2, long n,
                                float min1, float max1, float min2, float max2, int bins,
                                uint32_t *joint, uint32_t *col_sums, uint32_t *row_sums)
{
    float mn = min1 < min2 ? min1 : min2;
    float mx = max1 > max2 ? max1 : max2;
    float step = (mx - mn) / (float)bins;
    memset(joint, 0, sizeof(uint32_t) * (size_t)bins * (size_t)bins);
    if (col_sums) memset(col_sums, 0, sizeof(uint32_t) * (size_t)bins);
    if (row_sums) memset(row_sums, 0, sizeof(uint32_t) * (size_t)bins);
    for (long j = 0; j < n; ++j) {
        int row = orc_find_bucket(f1[j], mn, step, bins);
        int col = orc_find_bucket(f2[j], mn, step, bins);
        ++joint[(size_t)row * bins + col];
        if (col_sums) ++col_sums[col];
        if (row_sums) ++row_sums[row];
    }
}

/* isosurfaces_cuda/src/JointHistogram.cu:24-60 (calculateMutualInformation),
 * restated in FP32 with the reference's summation order. */
ORC_API float orc_mi_f32(const uint32_t *hist, int bins, float num_values,
                         const uint32_t *col_sums, const uint32_t *row_sums)
{
    float hX = 0.0f, hY = 0.0f, hXY = 0.0f;
    for (int i = 0; i < bins; ++i) {
        for (int j = 0; j < bins; ++j) {
            uint32_t c = hist[(size_t)i * bins + j];
            if (c > 0) {
                float pxy = (float)c;
                hXY -= pxy * logf(pxy);
            }
        }
        if (col_sums[i] > 0) {
            float px = (float)col_sums[i];
            hX -= px * logf(px);
        }
        if (row_sums[i] > 0) {
            float py = (float)row_sums[i];
            hY -= py * logf(py);
        }
    }
    hXY = hXY / num_values + logf(num_values);
    hX = hX / num_values + logf(num_values);
    hY = hY / num_values + logf(num_values);
    float iXY = hX + hY - hXY;
    float val = 2.0f * iXY / (hX + hY);
    return val != val ? 0.0f : val;
}

/* The same normalised mutual information in FP64 (the engine's MI precision):
 * entropies of the raw counts, h = -sum(c ln c)/N + ln N, ISM = 2I/(hX+hY),
 * NaN -> 0.  Marginals are exact integer sums of the joint histogram. */
ORC_API double orc_mi_f64(const uint32_t *hist, int bins, double num_values)
{
    double hXY = 0.0, hX = 0.0, hY = 0.0;
    uint64_t *col = (uint64_t *)calloc((size_t)bins, sizeof(uint64_t));
    for (int i = 0; i < bins; ++i) {
        uint64_t row = 0;
        for (int j = 0; j < bins; ++j) {
            uint32_t c = hist[(size_t)i * bins + j];
            row += c;
            col[j] += c;
            if (c > 0) hXY -= (double)c * log((double)c);
        }
        if (row > 0) hY -= (double)row * log((double)row);
    }
    for (int j = 0; j < bins; ++j)
        if (col[j] > 0) hX -= (double)col[j] * log((double)col[j]);
    free(col);
    double lnN = log(num_values);
    hXY = hXY / num_values + lnN;
    hX = hX / num_values + lnN;
    hY = hY / num_values + lnN;
    double iXY = hX + hY - hXY;
    double val = 2.0 * iXY / (hX + hY);
    return val != val ? 0.0 : val;
}

/* Full similarity map over m fields (field k at fields + k*n).
 * mode 0: FP64 MI on unordered pairs, mirrored (the engine's contract);
 * mode 1: FP32 reference MI on every ordered pair (JointHistogram.cu:306-328,
 *         one task per ordered pair including the diagonal). */
ORC_API void orc_similarity_map(const float *fields, int m, long n, int bins, int mode, float *ism)
{
    float *mins = (float *)malloc(sizeof(float) * (size_t)m);
    float *maxs = (float *)malloc(sizeof(float) * (size_t)m);
    for (int k = 0; k < m; ++k) orc_field_interval(fields + (size_t)k * n, n, &mins[k], &maxs[k]);
    uint32_t *joint = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)bins * bins);
    uint32_t *cs = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)bins);
    uint32_t *rs = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)bins);
    for (int i = 0; i < m; ++i) {
        for (int j = (mode == 0 ? i : 0); j < m; ++j) {
            orc_pair_histogram(fields + (size_t)i * n, fields + (size_t)j * n, n,
                               mins[i], maxs[i], mins[j], maxs[j], bins, joint, cs, rs);
            if (mode == 0) {
                float v = (float)orc_mi_f64(joint, bins, (double)n);
                ism[(size_t)i * m + j] = v;
                ism[(size_t)j * m + i] = v;
            } else {
                ism[(size_t)i * m + j] = orc_mi_f32(joint, bins, (float)n, cs, rs);
            }
        }
    }
    free(joint); free(cs); free(rs); free(mins); free(maxs);
}

/* ------------------------------------------------------------------------- */
/* Surfaces                                                                   */
/* ------------------------------------------------------------------------- */

/* isosurfaces_cuda/src/IsosurfaceApproximation.cu:67-135 with scale 1, plus the
 * stable compaction of thrust::copy_if (isosurfaces_cuda/hdr/thrustWrapper.h:47-54):
 * cell (x,y,z) with x<X-1, y<Y-1, z<Z-1 (volume index x*Y*Z + y*Z + z) is kept iff
 * one of its 8 corners is > iso and one is < iso.  Output int triples in linear
 * order.  Returns the count (writes at most cap triples). */
ORC_API long orc_approximation(const float *img, int X, int Y, int Z, float iso, int32_t *out, long cap)
{
    long count = 0;
    long ZY = (long)Z * Y;
    for (int x = 0; x < X - 1; ++x)
        for (int y = 0; y < Y - 1; ++y)
            for (int z = 0; z < Z - 1; ++z) {
                long lu = (long)x * ZY + (long)y * Z + z;
                long id1 = lu + 1, id2 = lu + Z, id3 = id1 + Z;
                long c[8] = {lu, id1, id2, id3, lu + ZY, id1 + ZY, id2 + ZY, id3 + ZY};
                int above = 0, below = 0;
                for (int k = 0; k < 8; ++k) {
                    float v = img[c[k]];
                    above |= v > iso;
                    below |= v < iso;
                }
                if (above && below) {
                    if (count < cap) {
                        out[3 * count + 0] = x;
                        out[3 * count + 1] = y;
                        out[3 * count + 2] = z;
                    }
                    ++count;
                }
            }
    return count;
}

/* Marching-cubes triangle-vertex count per case code.  Derived here rather than
 * tabulated: on each cube face the crossing edges are joined into segments; a
 * face with four crossing edges (ambiguous) cuts off its two inside corners
 * (bit set = value < iso).  The segments close into polygons, a k-gon gives k-2
 * triangles.  This reproduces numVertsTable of isosurfaces_cuda/src/tables.h:320
 * for all 256 cases (checked by the test suite against that table). */
static const int MC_EDGE[12][2] = {{0,1},{1,2},{2,3},{3,0},{4,5},{5,6},{6,7},{7,4},{0,4},{1,5},{2,6},{3,7}};
static const int MC_FACE[6][4] = {{0,1,2,3},{4,5,6,7},{0,1,5,4},{3,2,6,7},{0,3,7,4},{1,2,6,5}};

static int mc_edge_of(int a, int b)
{
    for (int e = 0; e < 12; ++e)
        if ((MC_EDGE[e][0] == a && MC_EDGE[e][1] == b) || (MC_EDGE[e][0] == b && MC_EDGE[e][1] == a)) return e;
    return -1;
}

ORC_API void orc_mc_vertex_counts(uint32_t out[256])
{
    for (int cs = 0; cs < 256; ++cs) {
        int adj[12][2], deg[12];
        memset(deg, 0, sizeof deg);
        for (int f = 0; f < 6; ++f) {
            const int *q = MC_FACE[f];
            int ncross = 0, cross[4];
            for (int k = 0; k < 4; ++k) {
                int a = q[k], b = q[(k + 1) & 3];
                if (((cs >> a) & 1) != ((cs >> b) & 1)) cross[ncross++] = mc_edge_of(a, b);
            }
            if (ncross == 2) {
                adj[cross[0]][deg[cross[0]]++] = cross[1];
                adj[cross[1]][deg[cross[1]]++] = cross[0];
            } else if (ncross == 4) {
                for (int k = 0; k < 4; ++k) {
                    if (!((cs >> q[k]) & 1)) continue;
                    int e0 = mc_edge_of(q[(k + 3) & 3], q[k]);
                    int e1 = mc_edge_of(q[k], q[(k + 1) & 3]);
                    adj[e0][deg[e0]++] = e1;
                    adj[e1][deg[e1]++] = e0;
                }
            }
        }
        int seen[12] = {0}, tri = 0;
        for (int e = 0; e < 12; ++e) {
            if (!deg[e] || seen[e]) continue;
            int len = 0, stack[12], sp = 0;
            stack[sp++] = e;
            while (sp) {
                int x = stack[--sp];
                if (seen[x]) continue;
                seen[x] = 1; ++len;
                for (int d = 0; d < deg[x]; ++d) if (!seen[adj[x][d]]) stack[sp++] = adj[x][d];
            }
            tri += len - 2;
        }
        out[cs] = (uint32_t)(3 * tri);
    }
}

/* Number of voxels the reference's classifyVoxel launch covers
 * (isosurfaces_cuda/src/MarchingCube.cpp:594-608): 128-thread blocks,
 * grid.x = V/128 truncated, reshaped to 32768 x (grid.x/32768) above 65535. */
ORC_API long orc_mc_classified_voxels(long num_voxels)
{
    long gx = num_voxels / 128, gy = 1;
    if (gx > 65535) { gy = gx / 32768; gx = 32768; }
    long covered = gx * gy * 128;
    return covered < num_voxels ? covered : num_voxels;
}

static int cmp_vec3(const void *a, const void *b)
{
    const float *p = (const float *)a, *q = (const float *)b;
    for (int k = 0; k < 3; ++k) {
        if (p[k] < q[k]) return -1;
        if (p[k] > q[k]) return 1;
    }
    return 0;
}

/* GPU marching cubes of isosurfaces_cuda/src/MarchingCube.cu:59-124,159-331 and
 * MarchingCube.cpp:588-710, followed by the sort + unique of
 * isosurfaces_cuda/src/thrustWrapper.cu:44-56 (lexicographic order,
 * utils/typeOperation.h:1268).
 *   frame 0 ("reference frame"): cell (a,b,c) samples img[c*X*Y + b*X + a] with
 *     grid (X,Y,Z) -- the kernel's x-fastest indexing of the z-fastest volume;
 *   frame 1 ("canonical frame"): cell (a,b,c) samples img[a*Y*Z + b*Z + c].
 * Corners are clamped to grid-1, corner bit k = value < iso, vertices are
 * lerp(p0, p1, (iso-f0)/(f1-f0)) per cell edge direction.  Only the voxels the
 * reference launch covers are classified (frame 0).  Every crossing edge of an
 * active cell contributes its vertex (Bourke's triangulation uses every crossing
 * edge), so the vertex set equals the set of emitted triangle vertices.
 * Writes up to cap unique xyz triples sorted lexicographically; returns the
 * unique count.  stats (may be NULL): [0] active voxels, [1] total triangle
 * vertices (sum of per-case counts). */
ORC_API long orc_marching_cubes(const float *img, int X, int Y, int Z, float iso, int frame,
                                float *out, long cap, long *stats)
{
    static uint32_t nv[256];
    static int nv_ready = 0;
    if (!nv_ready) { orc_mc_vertex_counts(nv); nv_ready = 1; }
    long V = (long)X * Y * Z;
    long sa, sb, sc;
    if (frame == 0) { sa = 1; sb = X; sc = (long)X * Y; } else { sa = (long)Y * Z; sb = Z; sc = 1; }
    long limit = frame == 0 ? orc_mc_classified_voxels(V) : V;
    static const int corner[8][3] = {{0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1}};
    size_t rawcap = 1024, nraw = 0;
    float *raw = (float *)malloc(sizeof(float) * 3 * rawcap);
    long active = 0, total = 0;
    for (long i = 0; i < limit; ++i) {
        /* linear voxel index -> grid position in the kernel's own order */
        int a, b, c;
        if (frame == 0) { a = (int)(i % X); b = (int)((i / X) % Y); c = (int)(i / ((long)X * Y)); }
        else { c = (int)(i % Z); b = (int)((i / Z) % Y); a = (int)(i / ((long)Y * Z)); }
        int gA = frame == 0 ? X : X, gB = Y, gC = frame == 0 ? Z : Z;
        float f[8];
        unsigned cube = 0;
        for (int k = 0; k < 8; ++k) {
            int pa = a + corner[k][0], pb = b + corner[k][1], pc = c + corner[k][2];
            if (pa > gA - 1) pa = gA - 1;
            if (pb > gB - 1) pb = gB - 1;
            if (pc > gC - 1) pc = gC - 1;
            f[k] = img[pa * sa + pb * sb + pc * sc];
            cube |= (unsigned)(f[k] < iso) << k;
        }
        if (nv[cube] == 0) continue;
        ++active;
        total += nv[cube];
        for (int e = 0; e < 12; ++e) {
            int k0 = MC_EDGE[e][0], k1 = MC_EDGE[e][1];
            if ((((cube >> k0) & 1) == ((cube >> k1) & 1))) continue;
            float t = (iso - f[k0]) / (f[k1] - f[k0]);
            float v[3];
            for (int d = 0; d < 3; ++d) {
                float p0 = (float)((d == 0 ? a : d == 1 ? b : c) + corner[k0][d]);
                float p1 = (float)((d == 0 ? a : d == 1 ? b : c) + corner[k1][d]);
                float prod = t * (p1 - p0);
                v[d] = p0 + prod;
            }
            if (nraw == rawcap) { rawcap *= 2; raw = (float *)realloc(raw, sizeof(float) * 3 * rawcap); }
            memcpy(raw + 3 * nraw, v, sizeof v);
            ++nraw;
        }
    }
    qsort(raw, nraw, sizeof(float) * 3, cmp_vec3);
    long uniq = 0;
    for (size_t r = 0; r < nraw; ++r) {
        if (r > 0 && cmp_vec3(raw + 3 * r, raw + 3 * (r - 1)) == 0) continue;
        if (uniq < cap) memcpy(out + 3 * uniq, raw + 3 * r, sizeof(float) * 3);
        ++uniq;
    }
    free(raw);
    if (stats) { stats[0] = active; stats[1] = total; }
    return uniq;
}

/* ------------------------------------------------------------------------- */
/* Distance fields                                                            */
/* ------------------------------------------------------------------------- */

/* Host normalisation of isosurfaces_cuda/funcs.cpp:150-175: p / max(X,Y,Z). */
ORC_API void orc_normalize_points(const float *pts, long n, int X, int Y, int Z, float *out)
{
    int dmax = X > Y ? X : Y;
    if (Z > dmax) dmax = Z;
    for (long i = 0; i < 3 * n; ++i) out[i] = pts[i] / (float)dmax;
}

/* Sample point of DF index idx: isosurfaces_cuda/src/BVH.cu:393-406. */
static void df_sample(long idx, int X, int Y, int Z, int ds, float s[3])
{
    long Y10 = Y / ds, Z10 = Z / ds;
    long z = idx % Z10, y = (idx / Z10) % Y10, x = idx / (Y10 * Z10);
    s[0] = (float)(x * ds + ds / 2) / (float)X;
    s[1] = (float)(y * ds + ds / 2) / (float)Y;
    s[2] = (float)(z * ds + ds / 2) / (float)Z;
}

/* Brute-force FP32 distance field with the engine's canonical rounding:
 * d = s - p per axis, d2 = fma(dz,dz, fma(dx,dx, dy*dy)), DF = sqrt(min d2)
 * (the reference's x2 + y2 + z2 as nvcc contracts it, BVH.cu:410-416);
 * a single-point surface stores the squared distance, as the reference's
 * traversal does (isosurfaces_cuda/src/BVH.cu:599-611).  pts are normalised. */
ORC_API void orc_distance_field_f32(const float *pts, long P, int X, int Y, int Z, int ds, float *out)
{
    long F = (long)(X / ds) * (Y / ds) * (Z / ds);
    for (long idx = 0; idx < F; ++idx) {
        float s[3];
        df_sample(idx, X, Y, Z, ds, s);
        float best = 100000.0f;
        for (long p = 0; p < P; ++p) {
            float dx = s[0] - pts[3 * p], dy = s[1] - pts[3 * p + 1], dz = s[2] - pts[3 * p + 2];
            float d2 = fmaf(dz, dz, fmaf(dx, dx, dy * dy));
            if (d2 < best) best = d2;
        }
        out[idx] = P == 1 ? best : sqrtf(best);
    }
}

/* Exact (FP64) nearest distance from the same FP32 sample and point coordinates. */
ORC_API void orc_distance_field_f64(const float *pts, long P, int X, int Y, int Z, int ds, double *out)
{
    long F = (long)(X / ds) * (Y / ds) * (Z / ds);
    for (long idx = 0; idx < F; ++idx) {
        float s[3];
        df_sample(idx, X, Y, Z, ds, s);
        double best = 1e300;
        for (long p = 0; p < P; ++p) {
            double dx = (double)s[0] - pts[3 * p], dy = (double)s[1] - pts[3 * p + 1], dz = (double)s[2] - pts[3 * p + 2];
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < best) best = d2;
        }
        out[idx] = P == 1 ? best : sqrt(best);
    }
}

/* k-d tree nearest-point search with the same canonical distance: a subtree
 * is skipped only when the canonical distance to its box (fma chain over the
 * per-axis gaps, monotone in every gap) is >= the best so far, so the result
 * equals the brute-force minimum bit for bit.  Used for larger oracle cases
 * and for the CPU baseline. */
typedef struct { float lo[3], hi[3]; int left, right, start, count; } kd_node;
typedef struct { const float *pts; int *idx; kd_node *nodes; int nn; } kd_tree;

static int kd_build(kd_tree *t, int start, int count)
{
    int me = t->nn++;
    kd_node *n = &t->nodes[me];
    for (int d = 0; d < 3; ++d) { n->lo[d] = 3.4e38f; n->hi[d] = -3.4e38f; }
    for (int i = start; i < start + count; ++i)
        for (int d = 0; d < 3; ++d) {
            float v = t->pts[3 * t->idx[i] + d];
            if (v < n->lo[d]) n->lo[d] = v;
            if (v > n->hi[d]) n->hi[d] = v;
        }
    n->start = start; n->count = count; n->left = n->right = -1;
    if (count <= 8) return me;
    int axis = 0;
    for (int d = 1; d < 3; ++d)
        if (n->hi[d] - n->lo[d] > n->hi[axis] - n->lo[axis]) axis = d;
    /* quickselect the median on `axis` */
    int lo = start, hi = start + count - 1, k = start + count / 2;
    while (lo < hi) {
        float pivot = t->pts[3 * t->idx[(lo + hi) / 2] + axis];
        int i = lo, j = hi;
        while (i <= j) {
            while (t->pts[3 * t->idx[i] + axis] < pivot) ++i;
            while (t->pts[3 * t->idx[j] + axis] > pivot) --j;
            if (i <= j) { int tmp = t->idx[i]; t->idx[i] = t->idx[j]; t->idx[j] = tmp; ++i; --j; }
        }
        if (k <= j) hi = j; else if (k >= i) lo = i; else break;
    }
    int half = count / 2;
    int l = kd_build(t, start, half);
    int r = kd_build(t, start + half, count - half);
    t->nodes[me].left = l;
    t->nodes[me].right = r;
    return me;
}

static float kd_box_dist(const kd_node *n, const float s[3])
{
    float g[3];
    for (int d = 0; d < 3; ++d) {
        float a = n->lo[d] - s[d], b = s[d] - n->hi[d];
        float m = a > b ? a : b;
        g[d] = m > 0.0f ? m : 0.0f;
    }
    return fmaf(g[2], g[2], fmaf(g[0], g[0], g[1] * g[1]));
}

static float kd_query(const kd_tree *t, const float s[3])
{
    float best = 100000.0f;
    int stack[128], sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const kd_node *n = &t->nodes[stack[--sp]];
        if (!(kd_box_dist(n, s) < best)) continue;
        if (n->left < 0) {
            for (int i = n->start; i < n->start + n->count; ++i) {
                const float *p = t->pts + 3 * t->idx[i];
                float dx = s[0] - p[0], dy = s[1] - p[1], dz = s[2] - p[2];
                float d2 = fmaf(dz, dz, fmaf(dx, dx, dy * dy));
                if (d2 < best) best = d2;
            }
            continue;
        }
        float dl = kd_box_dist(&t->nodes[n->left], s), dr = kd_box_dist(&t->nodes[n->right], s);
        if (dl <= dr) { stack[sp++] = n->right; stack[sp++] = n->left; }
        else { stack[sp++] = n->left; stack[sp++] = n->right; }
    }
    return best;
}

/* Distance field through the k-d tree; idx (may be NULL for all samples)
 * selects sample indices, out gets one value per selected sample. */
static double orc_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* As orc_distance_field_kd; build_s and query_s (may be NULL) receive the
 * seconds spent building the tree and answering the queries. */
ORC_API void orc_distance_field_kd_timed(const float *pts, long P, int X, int Y, int Z, int ds, const long *idx,
                                         long cnt, float *out, double *build_s, double *query_s)
{
    kd_tree t;
    const double t0 = orc_now();
    t.pts = pts;
    t.idx = (int *)malloc(sizeof(int) * (size_t)P);
    t.nodes = (kd_node *)malloc(sizeof(kd_node) * (size_t)(2 * P + 1));
    t.nn = 0;
    for (long i = 0; i < P; ++i) t.idx[i] = (int)i;
    kd_build(&t, 0, (int)P);
    const double t1 = orc_now();
    long F = (long)(X / ds) * (Y / ds) * (Z / ds);
    long total = idx ? cnt : F;
    for (long q = 0; q < total; ++q) {
        float s[3];
        df_sample(idx ? idx[q] : q, X, Y, Z, ds, s);
        float best = kd_query(&t, s);
        out[q] = P == 1 ? best : sqrtf(best);
    }
    const double t2 = orc_now();
    if (build_s) *build_s = t1 - t0;
    if (query_s) *query_s = t2 - t1;
    free(t.idx);
    free(t.nodes);
}

ORC_API void orc_distance_field_kd(const float *pts, long P, int X, int Y, int Z, int ds, const long *idx, long cnt,
                                   float *out)
{
    orc_distance_field_kd_timed(pts, P, X, Y, Z, ds, idx, cnt, out, NULL, NULL);
}

/* ------------------------------------------------------------------------- */
/* Isovalues                                                                  */
/* ------------------------------------------------------------------------- */

/* types/src/Isosurface.cpp:48-75 (loadFile): real min/max among values inside
 * [cfg_min, cfg_max], starting from max=-100000, min=100000. */
ORC_API void orc_real_range(const float *img, long V, float cfg_min, float cfg_max, float *out_min, float *out_max)
{
    float mx = -100000.0f, mn = 100000.0f;
    for (long i = 0; i < V; ++i) {
        float v = img[i];
        if (v > mx && v <= cfg_max) mx = v;
        if (v < mn && v >= cfg_min) mn = v;
    }
    *out_min = mn;
    *out_max = mx;
}

/* runtime/src/Single.cpp:286-392 (compute_isovalues + get_uniform_histogram).
 * uniform != 0: 65536-bin histogram equalised into n groups; else linear. */
ORC_API void orc_isovalues(const float *img, long V, float mn, float mx, int n, int uniform, float *out)
{
    if (!uniform) {
        float step = (mx - mn) / (float)n;
        for (int i = 0; i < n; ++i) out[i] = mn + step * (float)i;
        return;
    }
    const int BINS = 65536;
    int *hist = (int *)calloc(BINS, sizeof(int));
    float gmin = mn, gmax = mx;
    float oneover = (float)(1.0 / (double)(gmax - gmin));
    float dataSize = (float)V;
    for (long i = 0; (float)i < dataSize && i < V; ++i) {
        float scaled = (float)BINS * (img[i] - gmin);
        int index = (int)(scaled * oneover);
        if (index > BINS - 1) index = BINS - 1;
        if (index < 0) index = 0;
        hist[index] += 1;
    }
    double sum = 0.0;
    for (int i = 0; i < BINS; ++i) sum += hist[i];
    double acc = 0.0, threshold = sum / (double)n;
    int index = 0;
    for (int i = 0; i < n; ++i) {
        while (((acc == 0.0) || ((acc + hist[index]) < threshold)) && (index < BINS - 1)) {
            acc += hist[index];
            hist[index] = i;
            index++;
        }
        sum -= acc;
        acc = 0.0;
        if (i < n - 1) threshold = sum / (double)(n - (i + 1));
    }
    int idx = 0, lastIdx = 0;
    float step = (mx - mn) / (float)BINS;
    for (int i = 0; i < n; ++i) {
        while (idx < BINS && hist[idx] <= i) ++idx;
        int range = idx - lastIdx;
        int mid = lastIdx + range / 2;
        out[i] = mn + step * (float)mid;
        lastIdx = idx;
    }
    free(hist);
}

/* ------------------------------------------------------------------------- */
/* Representative isovalues                                                   */
/* ------------------------------------------------------------------------- */

typedef struct { float isovalue; float priority; int id; int map_id; } orc_rep;

static void prioritize(const float *ism, int m, orc_rep *elems, int ne, orc_rep *heap, int *nh)
{
    if (ne == 0) return;
    float *dist = (float *)malloc(sizeof(float) * (size_t)m);
    for (int i = 0; i < ne; ++i) {
        float sum = 0.0f;
        for (int j = 0; j < ne; ++j) sum += ism[(size_t)elems[i].map_id * m + elems[j].map_id];
        dist[elems[i].map_id] = sum / (float)ne;
    }
    float best = -1.0f;
    int cur = -1;
    for (int i = 0; i < ne; ++i)
        if (dist[elems[i].map_id] > best) { best = dist[elems[i].map_id]; cur = i; }
    orc_rep c = elems[cur];
    float p = (float)ne * dist[c.map_id];
    free(dist);
    heap[(*nh)++] = (orc_rep){c.isovalue, p, c.id, c.map_id};
    orc_rep *smaller = (orc_rep *)malloc(sizeof(orc_rep) * (size_t)ne);
    orc_rep *bigger = (orc_rep *)malloc(sizeof(orc_rep) * (size_t)ne);
    int ns = 0, nb = 0;
    for (int i = 0; i < ne; ++i) {
        if (elems[i].map_id < c.map_id) smaller[ns++] = elems[i];
        else if (i != cur) bigger[nb++] = elems[i];
    }
    prioritize(ism, m, smaller, ns, heap, nh);
    prioritize(ism, m, bigger, nb, heap, nh);
    free(smaller);
    free(bigger);
}

/* types/src/SimilarityMap.cpp:88-227 (prioritize, selectValues,
 * findRepresentativeIsovalues).  The reference keeps the candidates in a
 * Boost Fibonacci heap whose tie order is unspecified; here ties go to the
 * lower map index.  The reference rewrites the isovalue field of every
 * remaining candidate with the popped one's; that is kept.  Returns the number
 * selected (min(cnt, m)). */
ORC_API int orc_select_representatives(const float *ism, int m, const int *ids, const float *isovalues,
                                       int cnt, orc_rep *out)
{
    orc_rep *elems = (orc_rep *)malloc(sizeof(orc_rep) * (size_t)m);
    orc_rep *heap = (orc_rep *)malloc(sizeof(orc_rep) * (size_t)m);
    for (int i = 0; i < m; ++i) elems[i] = (orc_rep){isovalues[ids[i]], -1.0f, ids[i], i};
    int nh = 0;
    prioritize(ism, m, elems, m, heap, &nh);
    int taken = 0;
    while (taken < cnt && nh > 0) {
        int top = 0;
        for (int h = 1; h < nh; ++h)
            if (heap[h].priority > heap[top].priority ||
                (heap[h].priority == heap[top].priority && heap[h].map_id < heap[top].map_id)) top = h;
        orc_rep e = heap[top];
        out[taken++] = e;
        for (int h = 0; h < nh; ++h) {
            if (h == top) continue;
            float p = heap[h].priority;
            p /= (1.0f + ism[(size_t)e.map_id * m + heap[h].map_id]);
            heap[h].priority = p;
            heap[h].isovalue = e.isovalue;
        }
        heap[top] = heap[--nh];
    }
    free(elems);
    free(heap);
    return taken;
}

/* ------------------------------------------------------------------------
 * The reference's LBVH construction, restated so that the GPU checker
 * (oracle/refgpu.py) can verify, before it runs the reference's own BVH
 * kernels on an input, that the tree they build is a tree: every node but the
 * root has exactly one parent, every node is reachable from the root, and the
 * depth stays below the traversal's fixed 64-entry stack
 * (isosurfaces_cuda/src/BVH.cu:515).  A duplicate-code run takes the
 * reference's own branch (BVH.cu:202-216), so the check follows the
 * reference's rules, not the engine's index-augmented ones.
 * ------------------------------------------------------------------------ */

static int clz32(uint32_t x)
{
    int n = 0;
    if (x == 0) return 32;
    while (!(x & 0x80000000u)) { x <<= 1; ++n; }
    return n;
}

/* morton3D_d and expandBits_d (BVH.cu:86-106) on packed float3 points */
ORC_API void orc_ref_morton(const float *pts, long n, uint32_t *codes)
{
    for (long i = 0; i < n; ++i) {
        uint32_t c[3];
        for (int a = 0; a < 3; ++a) {
            float v = pts[3 * i + a] * 1024.0f;
            v = v > 0.0f ? v : 0.0f;
            v = v < 1023.0f ? v : 1023.0f;
            uint32_t b = (uint32_t)v;
            b = (b * 0x00010001u) & 0xFF0000FFu;
            b = (b * 0x00000101u) & 0x0F00F00Fu;
            b = (b * 0x00000011u) & 0xC30C30C3u;
            b = (b * 0x00000005u) & 0x49249249u;
            c[a] = b;
        }
        codes[i] = c[0] * 4u + c[1] * 2u + c[2];
    }
}

/* delta_d (BVH.cu:170-193): common prefix length, index-extended for equal codes */
static int ref_delta(const uint32_t *c, long n, long i, long j)
{
    if (j >= n || j < 0) return -1;
    if (c[i] == c[j]) return 32 + clz32((uint32_t)(i ^ j));
    return clz32(c[i] ^ c[j]);
}

/* determineRange_d (BVH.cu:195-244) */
static void ref_range(const uint32_t *c, long n, long idx, long *first, long *last)
{
    if (idx == 0) { *first = 0; *last = n - 1; return; }
    if (idx != n - 1 && c[idx] == c[idx + 1] && c[idx] == c[idx - 1]) {
        long index = idx;
        for (;;) {
            index += 1;
            if (index >= n - 1) break;
            if (c[index] != c[index + 1]) break;
        }
        *first = idx;
        *last = index;
        return;
    }
    int dd = ref_delta(c, n, idx, idx + 1) - ref_delta(c, n, idx, idx - 1);
    long d = dd == 0 ? 0 : (dd < 0 ? -1 : 1);
    int dmin = ref_delta(c, n, idx, idx - d);
    long lmax = 2;
    while (ref_delta(c, n, idx, idx + lmax * d) > dmin) lmax *= 2;
    long l = 0;
    for (long t = lmax / 2; t >= 1; t /= 2)
        if (ref_delta(c, n, idx, idx + (l + t) * d) > dmin) l += t;
    long j = idx + l * d;
    if (d < 0) { *first = j; *last = idx; } else { *first = idx; *last = j; }
}

/* findSplit_d (BVH.cu:122-166) */
static long ref_split(const uint32_t *c, long first, long last)
{
    uint32_t fc = c[first], lc = c[last];
    if (fc == lc) return first;
    int common = clz32(fc ^ lc);
    long split = first, step = last - first;
    do {
        step = (step + 1) >> 1;
        long ns = split + step;
        if (ns < last && clz32(fc ^ c[ns]) > common) split = ns;
    } while (step > 1);
    return split;
}

/* The reference's tree over n sorted codes (generateInternalNodes_g,
 * BVH.cu:273-345): child ids of internal node i in left[i], right[i], with
 * leaves as -(index) - 1 (calcId_d, BVH.cu:23-26).  Returns the tree's depth
 * (edges on the longest root-to-leaf path), or -1 when it is not a tree (a
 * node with no or several parents, one unreachable, or a cycle). */
ORC_API long orc_ref_lbvh(const uint32_t *c, long n, int32_t *left, int32_t *right)
{
    if (n < 2) return 0;
    long ni = n - 1;
    for (long i = 0; i < ni; ++i) {
        long f, l;
        ref_range(c, n, i, &f, &l);
        long s = ref_split(c, f, l);
        left[i] = s != f ? (int32_t)s : (int32_t)(-s - 1);
        right[i] = s + 1 != l ? (int32_t)(s + 1) : (int32_t)(-(s + 1) - 1);
    }
    /* parents: internal nodes 0..ni-1, leaves ni..ni+n-1 */
    int32_t *parents = (int32_t *)calloc((size_t)(ni + n), sizeof(int32_t));
    long bad = 0;
    for (long i = 0; i < ni; ++i) {
        int32_t ch[2] = {left[i], right[i]};
        for (int k = 0; k < 2; ++k) {
            long v = ch[k] >= 0 ? ch[k] : ni + (-(long)ch[k] - 1);
            if (ch[k] == 0 || v >= ni + n) { bad = 1; continue; }
            parents[v]++;
        }
    }
    for (long v = 1; v < ni + n && !bad; ++v) if (parents[v] != 1) bad = 1;
    if (parents[0] != 0) bad = 1;
    long depth = -1;
    if (!bad) {
        /* iterative walk from the root; with one parent per node a revisit
         * cannot happen, so the visit count proves reachability */
        long *stack = (long *)malloc(sizeof(long) * (size_t)(ni + n));
        long *dep = (long *)malloc(sizeof(long) * (size_t)(ni + n));
        long sp = 0, seen = 0, maxd = 0;
        stack[sp] = 0;
        dep[sp++] = 0;
        while (sp > 0) {
            long v = stack[--sp], dv = dep[sp];
            ++seen;
            if (dv > maxd) maxd = dv;
            if (seen > ni + n) break;
            if (v < ni) {
                int32_t ch[2] = {left[v], right[v]};
                for (int k = 0; k < 2; ++k) {
                    stack[sp] = ch[k] >= 0 ? ch[k] : ni + (-(long)ch[k] - 1);
                    dep[sp++] = dv + 1;
                }
            }
        }
        if (seen == ni + n) depth = maxd;
        free(stack);
        free(dep);
    }
    free(parents);
    return depth;
}
