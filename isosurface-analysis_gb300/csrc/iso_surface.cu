// iso_surface.cu -- surface points of many isovalues in one pass over the volume.
//
// Marching cubes (replaces classifyVoxel / generateTriangles / removeDuplicates,
// isosurfaces_cuda/src/MarchingCube.cu:84-331, MarchingCube.cpp:588-710,
// thrustWrapper.cu:44-56).  The reference emits, per active cell, one vertex per
// triangle corner, computed along the cell's own edge direction, then sorts and
// de-duplicates bit-exactly.  Every crossing edge of a case is used by its
// triangles, so the unique vertex set is the set of (edge, direction) vertices
// over all classified cells that contain the edge.  Here each thread owns the
// three grid edges leaving one grid point (virtual edges on the max faces
// included, their samples clamped like the reference's), finds the isovalues
// that cross each edge by binary search over the sorted isovalues
// (min(f0,f1) < iso <= max(f0,f1)), and emits the forward and/or reverse vertex
// once each.  Only vertices that land exactly on a grid point can coincide
// across edges; those go to a corner list that is radix-sorted and
// de-duplicated.  The same thread classifies its cell for every isovalue in
// (min corner, max corner] to count active cells and triangle vertices.
//
// Voxel approximation (replaces calculate_approximation_g + copy_if,
// IsosurfaceApproximation.cu:67-135,160-212): a cell is kept for every isovalue
// strictly inside its corner range.
//
// Both kernels run twice per block (count, then write at reserved offsets) so
// no per-block staging is needed; a first count-only launch sizes the outputs.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "iso_internal.cuh"

namespace {

constexpr int SURF_THREADS = 256;

__constant__ uint8_t c_mc_verts[256];  // triangle-vertex count per case code

// Derivation of the per-case triangle-vertex counts (same rule as the
// reference's numVertsTable, isosurfaces_cuda/src/tables.h:320): crossing
// edges on each face are joined into segments, a face with four crossing edges
// cuts off its inside corners (bit set = value < iso), the segments close into
// polygons and a k-gon gives k-2 triangles.
const int MC_EDGE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
const int MC_FACE[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};

int edge_of(int a, int b)
{
    for (int e = 0; e < 12; ++e)
        if ((MC_EDGE[e][0] == a && MC_EDGE[e][1] == b) || (MC_EDGE[e][0] == b && MC_EDGE[e][1] == a)) return e;
    return -1;
}

void derive_case_vertex_counts(uint8_t out[256])
{
    for (int cs = 0; cs < 256; ++cs) {
        int adj[12][2], deg[12] = {0};
        for (int f = 0; f < 6; ++f) {
            const int *q = MC_FACE[f];
            int nc = 0, cross[4];
            for (int k = 0; k < 4; ++k) {
                int a = q[k], b = q[(k + 1) & 3];
                if (((cs >> a) & 1) != ((cs >> b) & 1)) cross[nc++] = edge_of(a, b);
            }
            if (nc == 2) {
                adj[cross[0]][deg[cross[0]]++] = cross[1];
                adj[cross[1]][deg[cross[1]]++] = cross[0];
            } else if (nc == 4) {
                for (int k = 0; k < 4; ++k) {
                    if (!((cs >> q[k]) & 1)) continue;
                    int e0 = edge_of(q[(k + 3) & 3], q[k]), e1 = edge_of(q[k], q[(k + 1) & 3]);
                    adj[e0][deg[e0]++] = e1;
                    adj[e1][deg[e1]++] = e0;
                }
            }
        }
        bool seen[12] = {false};
        int tri = 0;
        for (int e = 0; e < 12; ++e) {
            if (!deg[e] || seen[e]) continue;
            int len = 0, stack[12], sp = 0;
            stack[sp++] = e;
            while (sp) {
                int x = stack[--sp];
                if (seen[x]) continue;
                seen[x] = true;
                ++len;
                for (int d = 0; d < deg[x]; ++d)
                    if (!seen[adj[x][d]]) stack[sp++] = adj[x][d];
            }
            tri += len - 2;
        }
        out[cs] = (uint8_t)(3 * tri);
    }
}

struct Grid {
    const float *vol;
    int gA, gB, gC;      // cell grid in the kernel's (a,b,c) coordinates
    int64_t sa, sb, sc;  // volume strides of a, b, c
    int64_t limit;       // cells with kernel-linear index < limit are classified
    int frame;
};

__device__ __forceinline__ float sample(const Grid &g, int a, int b, int c)
{
    a = a < g.gA - 1 ? a : g.gA - 1;
    b = b < g.gB - 1 ? b : g.gB - 1;
    c = c < g.gC - 1 ? c : g.gC - 1;
    return __ldg(g.vol + a * g.sa + b * g.sb + c * g.sc);
}

__device__ __forceinline__ bool cell_valid(const Grid &g, int a, int b, int c)
{
    if (a < 0 || b < 0 || c < 0 || a >= g.gA || b >= g.gB || c >= g.gC) return false;
    int64_t lin = g.frame == ISO_FRAME_REF ? (int64_t)a + (int64_t)b * g.gA + (int64_t)c * g.gA * g.gB
                                           : ((int64_t)a * g.gB + b) * g.gC + c;
    return lin < g.limit;
}

// first index with s[k] > v
__device__ __forceinline__ int upper_bound(const float *s, int n, float v)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (s[mid] > v) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// first index with s[k] >= v
__device__ __forceinline__ int lower_bound(const float *s, int n, float v)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (s[mid] >= v) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// Bucket index over the sorted isovalues, for the searches of every grid
// point: bucket b of [s[0], s[n-1]] has a float edge e_b and start[b] =
// #{k : s[k] < e_b}.  For v >= e_b, upper_bound(v) >= start[b], so a search
// finds v's bucket, steps down while e_b > v (rounding puts it at most one
// bucket high), and scans forward from start[b]: the exact first index with
// s[k] > v, in one or two steps where the binary search takes log2(n).
constexpr int ISO_INDEX_BUCKETS = 1024;

struct IsoIndex {
    const int *start;    // per bucket (shared memory in the kernel)
    const float *edge;
    float base, scale;   // bucket of v: (v - base) * scale; scale 0: binary search
};

__device__ __forceinline__ int iso_upper(const float *s, int n, float v, const IsoIndex &ix)
{
    if (ix.scale == 0.0f) return upper_bound(s, n, v);
    const float t = __fmul_rn(__fsub_rn(v, ix.base), ix.scale);
    int b = t >= 1.0f ? (t < (float)ISO_INDEX_BUCKETS ? (int)t : ISO_INDEX_BUCKETS - 1) : 0;
    while (b > 0 && ix.edge[b] > v) --b;
    int k = ix.start[b];
    while (k < n && !(s[k] > v)) ++k;
    return k;
}

struct SurfOut {
    unsigned long long *counts;   // per sorted k: [4] regular, corner candidates, active cells, triangle vertices
    const int64_t *reg_offset;    // per k: first slot of its regular vertices in points
    const int64_t *cor_offset;    // per k: first slot of its corner candidates in corner_keys
    unsigned long long *cursor;   // per k: [2] reserved regular / corner slots
    float4 *points;
    unsigned long long *corner_keys;
    int64_t corner_stride;        // (gA+1)(gB+1)(gC+1)
    unsigned int *block_counts;   // marching cubes: per block and k, [2] regular / corner versions counted
};

// Emits one vertex version.  phase 0: count; phase 1: write.
__device__ __forceinline__ void put_vertex(int phase, int k, float x, float y, float z, const Grid &g,
                                           unsigned int *s_reg, unsigned int *s_cor, const unsigned long long *s_base,
                                           const SurfOut &o, int axis, float pos)
{
    const bool corner = pos == truncf(pos);
    if (phase == 0) {
        atomicAdd(corner ? &s_cor[k] : &s_reg[k], 1u);
        return;
    }
    if (!corner) {
        unsigned int slot = atomicAdd(&s_reg[k], 1u);
        o.points[o.reg_offset[k] + s_base[2 * k] + slot] = make_float4(x, y, z, 1.0f);
    } else {
        unsigned int slot = atomicAdd(&s_cor[k], 1u);
        int64_t ia = (int64_t)x, ib = (int64_t)y, ic = (int64_t)z;
        unsigned long long key = ((unsigned long long)k << 40) |
                                 (unsigned long long)((ia * (g.gB + 1) + ib) * (g.gC + 1) + ic);
        o.corner_keys[o.cor_offset[k] + s_base[2 * k + 1] + slot] = key;
    }
}

// PHASE 0: count vertex versions; PHASE 1: write them.  CLASSIFY: also count
// the cell's active isovalues and triangle vertices (the count launch only).
template <int PHASE, bool CLASSIFY>
__device__ void mc_point(const Grid &g, int a, int b, int c, const float *s_iso, int n, const IsoIndex &ix,
                         unsigned int *s_reg, unsigned int *s_cor, const unsigned long long *s_base, const SurfOut &o,
                         unsigned int *s_active, unsigned int *s_total)
{
    const float f0 = sample(g, a, b, c);
    // ---- x edge (a,b,c)-(a+1,b,c): forward users e0/e4, reverse users e2/e6
    if (a < g.gA) {
        bool fw = cell_valid(g, a, b, c) || cell_valid(g, a, b, c - 1);
        bool rv = cell_valid(g, a, b - 1, c) || cell_valid(g, a, b - 1, c - 1);
        if (fw || rv) {
            const float f1 = sample(g, a + 1, b, c);
            const float lo = fminf(f0, f1), hi = fmaxf(f0, f1);
            if (lo < hi) {
                int k0 = iso_upper(s_iso, n, lo, ix), k1 = iso_upper(s_iso, n, hi, ix);
                for (int k = k0; k < k1; ++k) {
                    const float iso = s_iso[k];
                    float pf = 0.f, pr = 0.f;
                    if (fw) pf = __fadd_rn((float)a, __fdiv_rn(__fsub_rn(iso, f0), __fsub_rn(f1, f0)));
                    if (rv) pr = __fsub_rn((float)(a + 1), __fdiv_rn(__fsub_rn(iso, f1), __fsub_rn(f0, f1)));
                    if (fw) put_vertex(PHASE, k, pf, (float)b, (float)c, g, s_reg, s_cor, s_base, o, 0, pf);
                    if (rv && !(fw && __float_as_uint(pf) == __float_as_uint(pr)))
                        put_vertex(PHASE, k, pr, (float)b, (float)c, g, s_reg, s_cor, s_base, o, 0, pr);
                }
            }
        }
    }
    // ---- y edge (a,b,c)-(a,b+1,c): forward users e1/e5, reverse users e3/e7
    if (b < g.gB) {
        bool fw = cell_valid(g, a - 1, b, c) || cell_valid(g, a - 1, b, c - 1);
        bool rv = cell_valid(g, a, b, c) || cell_valid(g, a, b, c - 1);
        if (fw || rv) {
            const float f1 = sample(g, a, b + 1, c);
            const float lo = fminf(f0, f1), hi = fmaxf(f0, f1);
            if (lo < hi) {
                int k0 = iso_upper(s_iso, n, lo, ix), k1 = iso_upper(s_iso, n, hi, ix);
                for (int k = k0; k < k1; ++k) {
                    const float iso = s_iso[k];
                    float pf = 0.f, pr = 0.f;
                    if (fw) pf = __fadd_rn((float)b, __fdiv_rn(__fsub_rn(iso, f0), __fsub_rn(f1, f0)));
                    if (rv) pr = __fsub_rn((float)(b + 1), __fdiv_rn(__fsub_rn(iso, f1), __fsub_rn(f0, f1)));
                    if (fw) put_vertex(PHASE, k, (float)a, pf, (float)c, g, s_reg, s_cor, s_base, o, 1, pf);
                    if (rv && !(fw && __float_as_uint(pf) == __float_as_uint(pr)))
                        put_vertex(PHASE, k, (float)a, pr, (float)c, g, s_reg, s_cor, s_base, o, 1, pr);
                }
            }
        }
    }
    // ---- z edge (a,b,c)-(a,b,c+1): forward users e8/e9/e10/e11 (no reverse user)
    if (c < g.gC) {
        bool fw = cell_valid(g, a, b, c) || cell_valid(g, a - 1, b, c) || cell_valid(g, a - 1, b - 1, c) ||
                  cell_valid(g, a, b - 1, c);
        if (fw) {
            const float f1 = sample(g, a, b, c + 1);
            const float lo = fminf(f0, f1), hi = fmaxf(f0, f1);
            if (lo < hi) {
                int k0 = iso_upper(s_iso, n, lo, ix), k1 = iso_upper(s_iso, n, hi, ix);
                for (int k = k0; k < k1; ++k) {
                    const float iso = s_iso[k];
                    float pf = __fadd_rn((float)c, __fdiv_rn(__fsub_rn(iso, f0), __fsub_rn(f1, f0)));
                    put_vertex(PHASE, k, (float)a, (float)b, pf, g, s_reg, s_cor, s_base, o, 2, pf);
                }
            }
        }
    }
    // ---- case codes of cell (a,b,c) for every isovalue in (min, max]
    if (CLASSIFY && cell_valid(g, a, b, c)) {
        float f[8];
        f[0] = f0;
        f[1] = sample(g, a + 1, b, c);
        f[2] = sample(g, a + 1, b + 1, c);
        f[3] = sample(g, a, b + 1, c);
        f[4] = sample(g, a, b, c + 1);
        f[5] = sample(g, a + 1, b, c + 1);
        f[6] = sample(g, a + 1, b + 1, c + 1);
        f[7] = sample(g, a, b + 1, c + 1);
        float lo = f[0], hi = f[0];
#pragma unroll
        for (int q = 1; q < 8; ++q) {
            lo = fminf(lo, f[q]);
            hi = fmaxf(hi, f[q]);
        }
        if (lo < hi) {
            int k0 = iso_upper(s_iso, n, lo, ix), k1 = iso_upper(s_iso, n, hi, ix);
            for (int k = k0; k < k1; ++k) {
                const float iso = s_iso[k];
                unsigned cube = 0;
#pragma unroll
                for (int q = 0; q < 8; ++q) cube |= (unsigned)(f[q] < iso) << q;
                unsigned nv = c_mc_verts[cube];
                if (nv) {
                    atomicAdd(&s_active[k], 1u);
                    atomicAdd(&s_total[k], nv);
                }
            }
        }
    }
}

// Grid points are visited in the volume's memory order (stride-1 axis fastest).
__device__ __forceinline__ void point_of(const Grid &g, int64_t id, int &a, int &b, int &c)
{
    if (g.frame == ISO_FRAME_REF) {  // a has stride 1
        a = (int)(id % (g.gA + 1));
        int64_t r = id / (g.gA + 1);
        b = (int)(r % (g.gB + 1));
        c = (int)(r / (g.gB + 1));
    } else {  // c has stride 1
        c = (int)(id % (g.gC + 1));
        int64_t r = id / (g.gC + 1);
        b = (int)(r % (g.gB + 1));
        a = (int)(r / (g.gB + 1));
    }
}

// mode 0: accumulate per-isovalue counts and keep the block's own counts;
// mode 1: reserve the block's slots from those counts and write vertices.
__global__ void __launch_bounds__(SURF_THREADS) mc_kernel(Grid g, const float *iso_sorted, int n, IsoIndex gix,
                                                          SurfOut o, int mode)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ int s_start[ISO_INDEX_BUCKETS];
    __shared__ float s_edge[ISO_INDEX_BUCKETS];
    const IsoIndex ix{s_start, s_edge, gix.base, gix.scale};
    if (gix.scale != 0.0f)
        for (int q = threadIdx.x; q < ISO_INDEX_BUCKETS; q += blockDim.x) {
            s_start[q] = gix.start[q];
            s_edge[q] = gix.edge[q];
        }
    float *s_iso = reinterpret_cast<float *>(smem_raw);
    unsigned long long *s_base = reinterpret_cast<unsigned long long *>(s_iso + ((n + 1) & ~1));
    // per-block counts fit 32 bits (at most 15 triangle vertices per cell):
    // native shared-memory atomics, widened when added to the global counts
    unsigned int *s_reg = reinterpret_cast<unsigned int *>(s_base + 2 * n);
    unsigned int *s_cor = s_reg + n;
    unsigned int *s_active = s_cor + n;
    unsigned int *s_total = s_active + n;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        s_iso[k] = iso_sorted[k];
        s_reg[k] = 0;
        s_cor[k] = 0;
        s_active[k] = 0;
        s_total[k] = 0;
    }
    __syncthreads();
    const int64_t total = (int64_t)(g.gA + 1) * (g.gB + 1) * (g.gC + 1);
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int a = 0, b = 0, c = 0;
    const bool live = id < total;
    if (live) point_of(g, id, a, b, c);
    uint2 *own = o.block_counts ? reinterpret_cast<uint2 *>(o.block_counts) + (size_t)blockIdx.x * n : nullptr;
    if (mode == 0) {
        if (live) mc_point<0, true>(g, a, b, c, s_iso, n, ix, s_reg, s_cor, s_base, o, s_active, s_total);
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            if (own) own[k] = make_uint2(s_reg[k], s_cor[k]);
            if (s_reg[k]) atomicAdd(&o.counts[4 * k + 0], (unsigned long long)s_reg[k]);
            if (s_cor[k]) atomicAdd(&o.counts[4 * k + 1], (unsigned long long)s_cor[k]);
            if (s_active[k]) atomicAdd(&o.counts[4 * k + 2], (unsigned long long)s_active[k]);
            if (s_total[k]) atomicAdd(&o.counts[4 * k + 3], (unsigned long long)s_total[k]);
        }
        return;
    }
    if (!own) {  // no room was kept for the block counts: count again
        if (live) mc_point<0, false>(g, a, b, c, s_iso, n, ix, s_reg, s_cor, s_base, o, s_active, s_total);
        __syncthreads();
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const uint2 cnt = own ? own[k] : make_uint2(s_reg[k], s_cor[k]);
        s_base[2 * k] = cnt.x ? atomicAdd(&o.cursor[2 * k], (unsigned long long)cnt.x) : 0;
        s_base[2 * k + 1] = cnt.y ? atomicAdd(&o.cursor[2 * k + 1], (unsigned long long)cnt.y) : 0;
        s_reg[k] = 0;
        s_cor[k] = 0;
    }
    __syncthreads();
    if (live) mc_point<1, false>(g, a, b, c, s_iso, n, ix, s_reg, s_cor, s_base, o, s_active, s_total);
}

// Voxel approximation, host frame, scale 1.
template <int PHASE>
__device__ void approx_cell(const float *vol, int X, int Y, int Z, int x, int y, int z, const float *s_iso, int n,
                            unsigned int *s_cnt, const unsigned long long *s_base, const SurfOut &o)
{
    const int64_t ZY = (int64_t)Z * Y;
    const int64_t lu = (int64_t)x * ZY + (int64_t)y * Z + z;
    const int64_t id1 = lu + 1, id2 = lu + Z, id3 = id1 + Z;
    float f[8] = {__ldg(vol + lu), __ldg(vol + id1), __ldg(vol + id2), __ldg(vol + id3),
                  __ldg(vol + lu + ZY), __ldg(vol + id1 + ZY), __ldg(vol + id2 + ZY), __ldg(vol + id3 + ZY)};
    float lo = f[0], hi = f[0];
#pragma unroll
    for (int q = 1; q < 8; ++q) {
        lo = fminf(lo, f[q]);
        hi = fmaxf(hi, f[q]);
    }
    if (!(lo < hi)) return;
    const int k0 = upper_bound(s_iso, n, lo), k1 = lower_bound(s_iso, n, hi);
    for (int k = k0; k < k1; ++k) {
        unsigned int slot = atomicAdd(&s_cnt[k], 1u);
        if (PHASE == 1) o.points[o.reg_offset[k] + s_base[2 * k] + slot] = make_float4((float)x, (float)y, (float)z, 1.0f);
    }
}

__global__ void __launch_bounds__(SURF_THREADS) approx_kernel(const float *vol, int X, int Y, int Z,
                                                              const float *iso_sorted, int n, SurfOut o, int mode)
{
    extern __shared__ unsigned char smem_raw[];
    float *s_iso = reinterpret_cast<float *>(smem_raw);
    unsigned long long *s_base = reinterpret_cast<unsigned long long *>(s_iso + ((n + 1) & ~1));
    unsigned int *s_cnt = reinterpret_cast<unsigned int *>(s_base + 2 * n);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        s_iso[k] = iso_sorted[k];
        s_cnt[k] = 0;
    }
    __syncthreads();
    const int64_t total = (int64_t)(X - 1) * (Y - 1) * (Z - 1);
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int x = 0, y = 0, z = 0;
    const bool live = id < total;
    if (live) {
        z = (int)(id % (Z - 1));
        int64_t r = id / (Z - 1);
        y = (int)(r % (Y - 1));
        x = (int)(r / (Y - 1));
        approx_cell<0>(vol, X, Y, Z, x, y, z, s_iso, n, s_cnt, s_base, o);
    }
    __syncthreads();
    if (mode == 0) {
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            if (s_cnt[k]) atomicAdd(&o.counts[4 * k + 0], (unsigned long long)s_cnt[k]);
        return;
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        s_base[2 * k] = s_cnt[k] ? atomicAdd(&o.cursor[2 * k], (unsigned long long)s_cnt[k]) : 0;
        s_cnt[k] = 0;
    }
    __syncthreads();
    if (live) approx_cell<1>(vol, X, Y, Z, x, y, z, s_iso, n, s_cnt, s_base, o);
}

// Sorted corner keys -> unique corner vertices appended after each isovalue's
// regular vertices.
__global__ void corner_unique_kernel(const unsigned long long *keys, int64_t count, int gB, int gC,
                                     const int64_t *reg_offset, unsigned long long *cursor, float4 *points)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    unsigned long long key = keys[i];
    if (i > 0 && keys[i - 1] == key) return;
    int k = (int)(key >> 40);
    int64_t lin = (int64_t)(key & ((1ull << 40) - 1));
    int64_t c = lin % (gC + 1), r = lin / (gC + 1);
    int64_t b = r % (gB + 1), a = r / (gB + 1);
    unsigned long long slot = atomicAdd(&cursor[2 * k], 1ull);
    points[reg_offset[k] + slot] = make_float4((float)a, (float)b, (float)c, 1.0f);
}

__global__ void normalize_kernel(const float4 *raw, float4 *norm, int64_t count, float dmax)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float4 p = raw[i];
    norm[i] = make_float4(__fdiv_rn(p.x, dmax), __fdiv_rn(p.y, dmax), __fdiv_rn(p.z, dmax), 0.0f);
}

}  // namespace

static int upload_case_table(iso_ctx *ctx)
{
    static int uploaded_device_mask = 0;
    if (ctx->device < 31 && (uploaded_device_mask >> ctx->device) & 1) return ISO_OK;
    uint8_t table[256];
    derive_case_vertex_counts(table);
    ISO_CUDA(cudaMemcpyToSymbol(c_mc_verts, table, sizeof table));
    if (ctx->device < 31) uploaded_device_mask |= 1 << ctx->device;
    return ISO_OK;
}

// Number of voxels the reference's classification launch covers
// (MarchingCube.cpp:594-608): 128-thread blocks, V/128 blocks truncated,
// reshaped to 32768 x (blocks/32768) above 65535 blocks.
static int64_t reference_classified_voxels(int64_t V)
{
    int64_t gx = V / 128, gy = 1;
    if (gx > 65535) {
        gy = gx / 32768;
        gx = 32768;
    }
    int64_t covered = gx * gy * 128;
    return covered < V ? covered : V;
}

// Runs surface extraction for n isovalues on a device volume.  On return the
// arena's BUF_POINTS_RAW (grid units) and BUF_POINTS_NORM (divided by
// max(X,Y,Z)) hold float4 points; isovalue k (original order) owns
// h_counts[k] points starting at h_offsets[k].  h_stats (may be NULL) gets per-isovalue statistics.
int iso_run_surfaces(iso_ctx *ctx, const float *d_vol, int X, int Y, int Z, const float *h_iso, int n,
                     int surface, int frame, int64_t *h_counts, int64_t *h_offsets, iso_surface_stats *h_stats,
                     int64_t *total_points_out)
{
    if (n <= 0 || n > ISO_MAX_ISOVALUES) return iso_fail(ISO_ERR_ARG, "isovalue count %d out of range", n);
    if (X < 2 || Y < 2 || Z < 2) return iso_fail(ISO_ERR_ARG, "volume must be at least 2x2x2");
    if (surface != ISO_SURFACE_MC && surface != ISO_SURFACE_APPROX) return iso_fail(ISO_ERR_ARG, "bad surface mode");
    if (frame != ISO_FRAME_REF && frame != ISO_FRAME_CANON) return iso_fail(ISO_ERR_ARG, "bad frame");
    ISO_TRY(upload_case_table(ctx));

    // sort isovalues, remember the permutation (sorted slot -> original index)
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return h_iso[p] < h_iso[q]; });
    std::vector<float> sorted(n);
    for (int k = 0; k < n; ++k) sorted[k] = h_iso[order[k]];

    void *d_iso, *d_counts, *d_cursor, *d_reg_off, *d_cor_off;
    ISO_TRY(iso_buf(ctx, BUF_ISO_SORTED, n * sizeof(float), &d_iso));
    ISO_TRY(iso_buf(ctx, BUF_SURF_COUNTS, (size_t)n * 4 * sizeof(unsigned long long), &d_counts));
    ISO_TRY(iso_buf(ctx, BUF_SURF_CURSOR, (size_t)n * 2 * sizeof(unsigned long long), &d_cursor));
    ISO_TRY(iso_buf(ctx, BUF_SEG_OFFSET, (size_t)n * sizeof(int64_t), &d_reg_off));
    ISO_TRY(iso_buf(ctx, BUF_SEG_COUNT, (size_t)n * sizeof(int64_t), &d_cor_off));
    ISO_CUDA(cudaMemcpyAsync(d_iso, sorted.data(), n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    // bucket index of the sorted isovalues (marching cubes' searches); the
    // write pass reads it after the admission hook, so it is one of the
    // buffers iso_ctx_release_except_surfaces keeps
    IsoIndex gix{nullptr, nullptr, sorted[0], 0.0f};
    {
        const float range = sorted[n - 1] - sorted[0];
        const float width = range / (float)ISO_INDEX_BUCKETS;
        const float scale = 1.0f / width;
        // below 64 isovalues each block's table load costs more than the
        // binary searches it saves (64^3 with 32 isovalues: 0.12 against 0.09 ms)
        if (n >= 64 && range > 0.0f && std::isfinite(range) && width > 0.0f && std::isfinite(scale)) {
            std::vector<int> start(ISO_INDEX_BUCKETS);
            std::vector<float> edge(ISO_INDEX_BUCKETS);
            for (int q = 0; q < ISO_INDEX_BUCKETS; ++q) {
                edge[q] = sorted[0] + (float)q * width;
                start[q] = (int)(std::lower_bound(sorted.begin(), sorted.end(), edge[q]) - sorted.begin());
            }
            start[0] = 0;  // bucket 0 also serves values below its edge
            void *d_ix;
            ISO_TRY(iso_buf(ctx, BUF_ISO_INDEX, (size_t)ISO_INDEX_BUCKETS * 2 * sizeof(int), &d_ix));
            ISO_CUDA(cudaMemcpyAsync(d_ix, start.data(), ISO_INDEX_BUCKETS * sizeof(int), cudaMemcpyHostToDevice,
                                     ctx->stream));
            ISO_CUDA(cudaMemcpyAsync((int *)d_ix + ISO_INDEX_BUCKETS, edge.data(), ISO_INDEX_BUCKETS * sizeof(float),
                                     cudaMemcpyHostToDevice, ctx->stream));
            gix.start = (const int *)d_ix;
            gix.edge = (const float *)((const int *)d_ix + ISO_INDEX_BUCKETS);
            gix.scale = scale;
        }
    }
    ISO_CUDA(cudaMemsetAsync(d_counts, 0, (size_t)n * 4 * sizeof(unsigned long long), ctx->stream));
    ISO_CUDA(cudaMemsetAsync(d_cursor, 0, (size_t)n * 2 * sizeof(unsigned long long), ctx->stream));

    Grid g;
    g.vol = d_vol;
    g.gA = X;
    g.gB = Y;
    g.gC = Z;
    g.frame = frame;
    if (frame == ISO_FRAME_REF) {
        g.sa = 1;
        g.sb = X;
        g.sc = (int64_t)X * Y;
        g.limit = reference_classified_voxels((int64_t)X * Y * Z);
    } else {
        g.sa = (int64_t)Y * Z;
        g.sb = Z;
        g.sc = 1;
        g.limit = (int64_t)X * Y * Z;
    }
    SurfOut o;
    o.counts = (unsigned long long *)d_counts;
    o.cursor = (unsigned long long *)d_cursor;
    o.reg_offset = (const int64_t *)d_reg_off;
    o.cor_offset = (const int64_t *)d_cor_off;
    o.points = nullptr;
    o.corner_keys = nullptr;
    o.corner_stride = (int64_t)(X + 1) * (Y + 1) * (Z + 1);
    o.block_counts = nullptr;

    const bool mc = surface == ISO_SURFACE_MC;
    const size_t iso_bytes = (size_t)((n + 1) & ~1) * sizeof(float);
    const size_t smem = mc ? iso_bytes + (size_t)n * (2 * sizeof(unsigned long long) + 4 * sizeof(unsigned int))
                           : iso_bytes + (size_t)n * (2 * sizeof(unsigned long long) + sizeof(unsigned int));
    const int64_t items = mc ? (int64_t)(X + 1) * (Y + 1) * (Z + 1) : (int64_t)(X - 1) * (Y - 1) * (Z - 1);
    const int64_t blocks = (items + SURF_THREADS - 1) / SURF_THREADS;
    if (blocks > 0x7fffffffLL) return iso_fail(ISO_ERR_ARG, "volume too large");
    // marching cubes keeps each block's counts for the write pass (which then
    // does not count again) while they fit the context's limit
    const size_t bc_bytes = (size_t)blocks * n * 2 * sizeof(unsigned int);
    if (mc && (int64_t)bc_bytes <= ctx->surf_block_count_bytes) {
        void *d_bc;
        ISO_TRY(iso_buf(ctx, BUF_SURF_BLOCK_COUNTS, bc_bytes, &d_bc));
        o.block_counts = (unsigned int *)d_bc;
    }
    if (smem > 48 * 1024) {
        ISO_CUDA(cudaFuncSetAttribute(mc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ISO_CUDA(cudaFuncSetAttribute(approx_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }

    // pass 1: counts
    if (mc) mc_kernel<<<(unsigned)blocks, SURF_THREADS, smem, ctx->stream>>>(g, (const float *)d_iso, n, gix, o, 0);
    else approx_kernel<<<(unsigned)blocks, SURF_THREADS, smem, ctx->stream>>>(d_vol, X, Y, Z, (const float *)d_iso, n, o, 0);
    ISO_LAUNCHED(ctx);
    std::vector<unsigned long long> cnt((size_t)n * 4);
    ISO_CUDA(cudaMemcpyAsync(cnt.data(), d_counts, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));

    // regions in sorted order: regular + corner candidates per isovalue
    std::vector<int64_t> reg_off(n), cor_off(n);
    int64_t tot_pts = 0, tot_cor = 0;
    int nonempty = 0;
    for (int k = 0; k < n; ++k) {
        reg_off[k] = tot_pts;
        cor_off[k] = tot_cor;
        tot_pts += (int64_t)(cnt[4 * k] + cnt[4 * k + 1]);
        tot_cor += (int64_t)cnt[4 * k + 1];
        nonempty += (cnt[4 * k] + cnt[4 * k + 1]) > 0;
    }
    if (ctx->admit) {
        // device bytes the rest of the request needs, from the exact counts:
        // points (raw + normalised), corner keys, LBVH arrays (keys, values,
        // gathered and sorted points, 64-byte nodes, links, flags, sort
        // temporaries), distance fields, histogram scratch and the map
        const double P = (double)tot_pts, m = (double)nonempty;
        double need = 4.0 * ctx->plan_V * ctx->plan_volume_copy + 32.0 * P + 16.0 * tot_cor +
                      (o.block_counts ? (double)bc_bytes : 0.0) +
                      (ctx->plan_lbvh ? 180.0 * std::min(P, (double)ctx->lbvh_group_points) : 0.0) +
                      4.0 * m * ctx->plan_stride + 12.0 * m * m +
                      8.0 * 65536 + 16.0 * (1 << 20);
        // segment-major histograms keep one chunk of per-pair global histograms
        if (ctx->hist_segment_values > 0 && ctx->plan_stride > ctx->hist_segment_values &&
            ctx->plan_bins > ISO_WIDE_MAX_BINS) {
            const double hist = 4.0 * ctx->plan_bins * ctx->plan_bins;
            need += std::min(m * (m + 1) / 2 * hist, (double)ISO_HIST_CHUNK_BYTES);
            need += 4.0 * m * ctx->plan_stride;  // the fields' precomputed row buckets
        }
        // the reference's FP32 MI keeps every ordered pair's histogram
        if (ctx->mi_mode == ISO_MI_REF32)
            need += 4.0 * m * m * ctx->plan_bins * ctx->plan_bins + 8.0 * m * m * ctx->plan_bins;
        need *= 1.15;  // arena growth slack
        if (ctx->admit(ctx->admit_user, (size_t)need) != 0)
            return iso_fail(ISO_ERR_NOMEM, "request needs %.0f bytes of device memory; over the budget", need);
    }
    void *d_raw, *d_norm, *d_ck = nullptr, *d_ck2 = nullptr;
    ISO_TRY(iso_buf(ctx, BUF_POINTS_RAW, (size_t)(tot_pts + 1) * sizeof(float4), &d_raw));
    ISO_TRY(iso_buf(ctx, BUF_POINTS_NORM, (size_t)(tot_pts + 1) * sizeof(float4), &d_norm));
    ISO_TRY(iso_buf(ctx, BUF_CORNER_KEYS, (size_t)(tot_cor + 1) * sizeof(unsigned long long), &d_ck));
    ISO_TRY(iso_buf(ctx, BUF_CORNER_KEYS_ALT, (size_t)(tot_cor + 1) * sizeof(unsigned long long), &d_ck2));
    ISO_CUDA(cudaMemcpyAsync(d_reg_off, reg_off.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    ISO_CUDA(cudaMemcpyAsync(d_cor_off, cor_off.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    o.points = (float4 *)d_raw;
    o.corner_keys = (unsigned long long *)d_ck;

    // pass 2: write
    if (tot_pts > 0) {
        if (mc) mc_kernel<<<(unsigned)blocks, SURF_THREADS, smem, ctx->stream>>>(g, (const float *)d_iso, n, gix, o, 1);
        else approx_kernel<<<(unsigned)blocks, SURF_THREADS, smem, ctx->stream>>>(d_vol, X, Y, Z, (const float *)d_iso, n, o, 1);
        ISO_LAUNCHED(ctx);
    }
    std::vector<int64_t> final_cnt(n);
    for (int k = 0; k < n; ++k) final_cnt[k] = (int64_t)cnt[4 * k];
    if (tot_cor > 0) {
        // corner vertices: radix sort (isovalue, grid point) keys, keep the first of each run
        int end_bit = 40;
        while ((1 << (end_bit - 40)) < n && end_bit < 64) ++end_bit;
        size_t temp_bytes = 0;
        cub::DoubleBuffer<unsigned long long> keys((unsigned long long *)d_ck, (unsigned long long *)d_ck2);
        ISO_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, temp_bytes, keys, (int)tot_cor, 0, end_bit, ctx->stream));
        void *d_temp;
        ISO_TRY(iso_buf(ctx, BUF_CUB_TEMP, temp_bytes, &d_temp));
        ISO_CUDA(cub::DeviceRadixSort::SortKeys(d_temp, temp_bytes, keys, (int)tot_cor, 0, end_bit, ctx->stream));
        ctx->launches += 4;
        // cursor[2k] already equals the regular count of k after pass 2
        corner_unique_kernel<<<(unsigned)((tot_cor + 255) / 256), 256, 0, ctx->stream>>>(
            keys.Current(), tot_cor, Y, Z, (const int64_t *)d_reg_off, (unsigned long long *)d_cursor, (float4 *)d_raw);
        ISO_LAUNCHED(ctx);
        std::vector<unsigned long long> cur((size_t)n * 2);
        ISO_CUDA(cudaMemcpyAsync(cur.data(), d_cursor, cur.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
        ISO_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int k = 0; k < n; ++k) final_cnt[k] = (int64_t)cur[2 * k];
    }
    const int dmax = std::max(X, std::max(Y, Z));
    if (tot_pts > 0) {
        normalize_kernel<<<(unsigned)((tot_pts + 255) / 256), 256, 0, ctx->stream>>>((const float4 *)d_raw, (float4 *)d_norm,
                                                                                   tot_pts, (float)dmax);
        ISO_LAUNCHED(ctx);
    }
    // per original isovalue: offset and count of its points in the arena
    for (int k = 0; k < n; ++k) {
        int orig = order[k];
        h_counts[orig] = final_cnt[k];
        h_offsets[orig] = reg_off[k];
        if (h_stats) {
            h_stats[orig].points = final_cnt[k];
            h_stats[orig].active_voxels = mc ? (int64_t)cnt[4 * k + 2] : 0;
            h_stats[orig].total_verts = mc ? (int64_t)cnt[4 * k + 3] : 0;
            h_stats[orig].flags = (mc && frame == ISO_FRAME_REF && (int64_t)cnt[4 * k + 3] > (int64_t)X * Y * Z - 3)
                                      ? ISO_MC_REF_DROPPED : 0;
            h_stats[orig].reserved = 0;
        }
    }
    if (total_points_out) *total_points_out = tot_pts;
    return ISO_OK;
}
