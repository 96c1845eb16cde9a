// iso_distance.cu -- nearest-surface distance fields for many point sets.
//
// Replaces generateHierarchy_h / traverse_h and their kernels
// (isosurfaces_cuda/src/BVH.cu:108-383, 393-706, 814-875).  The sample point of
// DF index idx (z fastest over the (X/ds, Y/ds, Z/ds) grid) is
// ((x*ds + ds/2)/X, (y*ds + ds/2)/Y, (z*ds + ds/2)/Z) (BVH.cu:393-406); surface
// points are normalised by max(X,Y,Z) (funcs.cpp:150-175).  The field value is
// sqrt(min over points of the canonical squared distance); a one-point surface
// stores the squared distance, as the reference does (BVH.cu:604-611).
//
// Two methods with bit-identical output:
//  * brute force: each thread owns four samples, points stream through shared
//    memory in tiles (plain FP32 comparator path);
//  * LBVH: all point sets at once -- 30-bit Morton codes (BVH.cu:84-117), one
//    radix sort of (set, code) keys, Karras hierarchy per set with ties broken
//    by index (exact for duplicate codes), bottom-up boxes (acquire-release
//    arrival counts), then warp packet traversals (four samples per lane).  A
//    child box is skipped only if its canonical box distance is >= the best
//    squared distance so far; the box distance is the same fma chain over
//    per-axis gaps, which never exceeds the
//    canonical distance of any point inside (rounding is monotone), so the
//    minimum equals the brute-force minimum bit for bit.
#include <cub/cub.cuh>

#include <vector>

#include "iso_internal.cuh"

namespace {

constexpr int BRUTE_THREADS = 256;
constexpr int BRUTE_SAMPLES = 4;  // per thread
constexpr int BRUTE_TILE = 1024;  // points per shared-memory tile
constexpr int QUERY_THREADS = 128;
constexpr int STACK_DEPTH = 64;
constexpr float INIT_BOUND = 100000.0f;  // the reference's initial upper bound (BVH.cu:639)

using SampleGrid = IsoSampleGrid;
using Segments = IsoSegments;

__device__ __forceinline__ float3 sample_point(const SampleGrid &g, int64_t idx) { return iso_sample_point(g, idx); }
__device__ __forceinline__ float finish(float best, int64_t P) { return iso_df_finish(best, P); }

__global__ void __launch_bounds__(BRUTE_THREADS) df_brute_kernel(Segments sg, SampleGrid g, float *fields,
                                                                   int64_t stride, int seg_base)
{
    __shared__ float4 tile[BRUTE_TILE];
    const int seg = seg_base + blockIdx.y;
    const int64_t off = sg.offset[seg], P = sg.count[seg];
    const int64_t first = (int64_t)blockIdx.x * BRUTE_THREADS * BRUTE_SAMPLES + threadIdx.x;
    float sx[BRUTE_SAMPLES], sy[BRUTE_SAMPLES], sz[BRUTE_SAMPLES], best[BRUTE_SAMPLES];
#pragma unroll
    for (int q = 0; q < BRUTE_SAMPLES; ++q) {
        int64_t idx = first + (int64_t)q * BRUTE_THREADS;
        float3 s = sample_point(g, idx < g.F ? idx : g.F - 1);
        sx[q] = s.x;
        sy[q] = s.y;
        sz[q] = s.z;
        best[q] = INIT_BOUND;
    }
    for (int64_t base = 0; base < P; base += BRUTE_TILE) {
        const int len = (int)(P - base < BRUTE_TILE ? P - base : BRUTE_TILE);
        __syncthreads();
        for (int t = threadIdx.x; t < len; t += BRUTE_THREADS) tile[t] = sg.points[off + base + t];
        __syncthreads();
#pragma unroll 4
        for (int t = 0; t < len; ++t) {
            const float4 p = tile[t];
#pragma unroll
            for (int q = 0; q < BRUTE_SAMPLES; ++q) {
                float d = iso_dist2(__fsub_rn(sx[q], p.x), __fsub_rn(sy[q], p.y), __fsub_rn(sz[q], p.z));
                best[q] = fminf(best[q], d);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < BRUTE_SAMPLES; ++q) {
        int64_t idx = first + (int64_t)q * BRUTE_THREADS;
        if (idx < g.F) fields[(size_t)blockIdx.y * stride + idx] = finish(best[q], P);
    }
}

// ---------------------------------------------------------------------------
// LBVH
// ---------------------------------------------------------------------------

// 64-byte node holding both children's boxes pairwise (left, right) so one
// visit evaluates both box distances with packed float2 arithmetic; the max
// corner is stored negated (s - hi becomes s + (-hi)).
struct BvhNode {
    float4 a;  // lo.x (l, r), lo.y (l, r)
    float4 b;  // lo.z (l, r), -hi.x (l, r)
    float4 c;  // -hi.y (l, r), -hi.z (l, r)
    int4 d;    // left child, right child, unused, unused
};
constexpr int LEAF_BIT = (int)0x80000000;

// Expands a 10-bit integer into 30 bits with two zeros between bits, and the
// Morton code of a point in the unit cube with `bits` bits per axis (at most
// 10; with 10 it is the 30-bit code of BVH.cu:84-117).
__device__ __forceinline__ unsigned int expand_bits(unsigned int v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ unsigned int morton_code(float x, float y, float z, int bits)
{
    const float cells = (float)(1u << bits), top = cells - 1.0f;
    x = fminf(fmaxf(__fmul_rn(x, cells), 0.0f), top);
    y = fminf(fmaxf(__fmul_rn(y, cells), 0.0f), top);
    z = fminf(fmaxf(__fmul_rn(z, cells), 0.0f), top);
    return expand_bits((unsigned int)x) * 4 + expand_bits((unsigned int)y) * 2 + expand_bits((unsigned int)z);
}

// Sort keys of one LBVH group: the surface index in the top seg_bits bits and
// the point's Morton code below, with as many bits per axis as fit in 32 (10
// for up to 4 surfaces, 8 for up to 256, the most a group holds).  Coarser
// codes only loosen the lowest boxes; the queries' minima are exact whatever
// the tree.
constexpr int LBVH_MAX_GROUP_SURFACES = 256;
inline int lbvh_seg_bits(int m)
{
    int b = 0;
    while ((1 << b) < m) ++b;
    return b;
}
inline int lbvh_axis_bits(int m)
{
    const int a = (32 - lbvh_seg_bits(m)) / 3;
    return a < 10 ? a : 10;
}

__device__ __forceinline__ int find_segment(const int64_t *starts, int m, int64_t i)
{
    int lo = 0, hi = m - 1;  // last s with starts[s] <= i
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct Bvh {
    const int64_t *cstart;   // per segment: first sorted leaf (compact numbering)
    const int64_t *ccount;   // per segment: leaves
    int m;
    int64_t total;           // all leaves
    unsigned int *keys;      // surface index above the Morton code (lbvh_axis_bits)
    int axis_bits;
    unsigned int *vals;
    float4 *compact;         // gathered points, compact numbering
    float4 *leaves;          // sorted points
    BvhNode *nodes;          // segment s owns nodes [cstart[s]-s, cstart[s]-s+count-1)
    int *parent_node;        // per internal node: parent (group-wide index)*4 + side*2 + parent local, -1 at the root
    unsigned int *flags;     // per internal node: leaf children (count | left << 8 | right << 9), then arrivals
    int *error;
};

__global__ void bvh_keys_kernel(Segments sg, Bvh b)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.total) return;
    int s = find_segment(b.cstart, b.m, i);
    float4 p = sg.points[sg.offset[s] + (i - b.cstart[s])];
    b.compact[i] = p;
    b.keys[i] = ((unsigned int)s << (3 * b.axis_bits)) | morton_code(p.x, p.y, p.z, b.axis_bits);
    b.vals[i] = (unsigned int)i;
}

__global__ void bvh_gather_kernel(Bvh b, const unsigned int *sorted_vals)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.total) return;
    b.leaves[i] = b.compact[sorted_vals[i]];
}

// delta of the Karras construction over index-augmented keys
__device__ __forceinline__ int karras_delta(const unsigned int *codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const unsigned int ci = codes[i], cj = codes[j];
    if (ci == cj) return 32 + __clz(i ^ j);
    return __clz(ci ^ cj);
}

__device__ __forceinline__ void store_box(BvhNode *node, int side, float3 lo, float3 hi)
{
    float *a = &node->a.x, *b = &node->b.x, *c = &node->c.x;
    __stcg(a + side, lo.x);
    __stcg(a + 2 + side, lo.y);
    __stcg(b + side, lo.z);
    __stcg(b + 2 + side, -hi.x);
    __stcg(c + side, -hi.y);
    __stcg(c + 2 + side, -hi.z);
}

// Block size of the build and box kernels, one thread per internal node.  A
// node whose subtree's internal nodes all fall into one block of BOX_THREADS
// node indices is "local": every arrival at it comes from that block.  The
// internal nodes of a subtree over leaves [first, last] have indices in
// [first, last] (each node's index is an end of its own range), so a node is
// local when nbase + first and nbase + last fall into one block.
constexpr int BOX_THREADS = 256;
// Points of one LBVH build (the parent links hold group-wide node indices * 4).
constexpr int64_t LBVH_MAX_GROUP_POINTS = (int64_t)1 << 29;

// Arrival count with release (this thread's box stores before it) and
// acquire (the sibling's box stores visible after it) at device scope: one
// ordered atomic instead of a fence on either side.
__device__ __forceinline__ unsigned int arrive_acq_rel(unsigned int *p)
{
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// The same at block scope, on a flag in shared memory.
__device__ __forceinline__ unsigned int arrive_acq_rel_cta(unsigned int *p)
{
    unsigned int old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], 1;"
                 : "=r"(old)
                 : "r"((uint32_t)__cvta_generic_to_shared(p))
                 : "memory");
    return old;
}

// The box of a node from its children's halves (a, b, c as in BvhNode).
__device__ __forceinline__ void union_of_halves(const float4 &a, const float4 &b, const float4 &c, float3 &lo,
                                                float3 &hi)
{
    lo = make_float3(fminf(a.x, a.y), fminf(a.z, a.w), fminf(b.x, b.y));
    hi = make_float3(-fminf(b.z, b.w), -fminf(c.x, c.y), -fminf(c.z, c.w));
}

// One thread per internal node: the node's Karras split, then the boxes.
// Each node's arrival flag starts at its number of leaf children (count | left
// leaf << 8 | right leaf << 9), so the climbs start at the nodes with two
// leaves: a thread writes its node's box into the parent's half and arrives
// there, and the thread that brings the flag to 2 carries on upwards with the
// union of both halves.  The block builds its nodes into shared memory; once
// all are built, the climbs through local parents run there (block-scope
// acquire-release on the shared flag, no global access), and the block writes
// every node once.  The climbs through parents that span blocks are left to
// bvh_boxes_kernel.
__global__ void __launch_bounds__(BOX_THREADS) bvh_build_kernel(Bvh b, const unsigned int *sorted_keys)
{
    __shared__ unsigned int s_flag[BOX_THREADS];
    __shared__ int s_link[BOX_THREADS];        // link to a local parent; -1 at a root, -2 otherwise
    __shared__ float4 s_node[BOX_THREADS][3];  // a, b, c of the block's nodes
    const int64_t total_nodes = b.total - b.m;
    const int64_t base = (int64_t)blockIdx.x * BOX_THREADS;
    const int64_t g = base + threadIdx.x;
    s_link[threadIdx.x] = -2;
    __syncthreads();
    bool climbing = false;
    if (g < total_nodes) {
        // segment s owns internal nodes [cstart[s] - s, cstart[s] - s + count[s] - 1)
        int lo = 0, hi = b.m - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (b.cstart[mid] - mid <= g) lo = mid; else hi = mid - 1;
        }
        // one-point segments own no node and share the next segment's base; the
        // last segment whose base is <= g owns node g
        const int s = lo;
        const int64_t nbase = b.cstart[s] - s;
        const int n = (int)b.ccount[s];
        const int i = (int)(g - nbase);
        const unsigned int *codes = sorted_keys + b.cstart[s];

        int d = karras_delta(codes, n, i, i + 1) - karras_delta(codes, n, i, i - 1) > 0 ? 1 : -1;
        if (i == 0) d = 1;
        int dmin = karras_delta(codes, n, i, i - d);
        int lmax = 2;
        while (karras_delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (karras_delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = karras_delta(codes, n, i, j);
        int sp = 0;
        int t = l;
        do {
            t = (t + 1) >> 1;
            if (karras_delta(codes, n, i, i + (sp + t) * d) > dnode) sp += t;
        } while (t > 1);
        const int split = i + sp * d + (d < 0 ? -1 : 0);
        const int first = i < j ? i : j, last = i < j ? j : i;
        const int left = (first == split) ? (split | LEAF_BIT) : split;
        const int right = (last == split + 1) ? ((split + 1) | LEAF_BIT) : split + 1;
        const bool ll = (left & LEAF_BIT) != 0, rl = (right & LEAF_BIT) != 0;

        // leaf children's boxes (their points); an internal child's half is
        // written when that child's box is complete
        const float4 *lv = b.leaves + b.cstart[s];
        float *half = &s_node[threadIdx.x][0].x;
        if (ll) {
            const float4 p = lv[left & ~LEAF_BIT];
            half[0] = p.x, half[2] = p.y, half[4] = p.z, half[6] = -p.x, half[8] = -p.y, half[10] = -p.z;
        }
        if (rl) {
            const float4 q = lv[right & ~LEAF_BIT];
            half[1] = q.x, half[3] = q.y, half[5] = q.z, half[7] = -q.x, half[9] = -q.y, half[11] = -q.z;
        }
        const int local = (nbase + first) / BOX_THREADS == (nbase + last) / BOX_THREADS ? 1 : 0;
        b.nodes[g].d = make_int4(left, right, local, 0);
        const unsigned int flag = ((unsigned int)ll + (unsigned int)rl) | ((unsigned int)ll << 8) | ((unsigned int)rl << 9);
        s_flag[threadIdx.x] = flag;
        b.flags[g] = flag;
        const int self = (int)g * 4 + local;  // group-wide index: below 2^29
        // a local node's children are inside the block; a child index outside
        // it would be a build error and is reported, not stored
        auto link_child = [&](int child, int side) {
            b.parent_node[nbase + child] = self + 2 * side;
            if (!local) return;
            const int64_t ct = nbase + child - base;
            if (ct >= 0 && ct < BOX_THREADS) s_link[ct] = self + 2 * side;
            else atomicExch(b.error, 1);
        };
        if (!ll) link_child(left, 0);
        if (!rl) link_child(right, 1);
        if (i == 0) {
            b.parent_node[g] = -1;
            s_link[threadIdx.x] = -1;
        }
        climbing = ll && rl && local;
    }
    __syncthreads();
    float3 lo = make_float3(0.f, 0.f, 0.f), hi = lo;
    int link = -2;
    if (climbing) {
        union_of_halves(s_node[threadIdx.x][0], s_node[threadIdx.x][1], s_node[threadIdx.x][2], lo, hi);
        link = s_link[threadIdx.x];
    }
    // depth is bounded by the 62-bit augmented key, the loop by the node count
    for (int guard = 0; climbing && link >= 0 && guard < 4096; ++guard) {
        const int t = (link >> 2) - (int)base, side = (link >> 1) & 1;  // parent inside this block
        if ((unsigned int)t >= (unsigned int)BOX_THREADS) {  // a local parent outside the block: a build error
            atomicExch(b.error, 1);
            break;
        }
        float *half = &s_node[t][0].x;
        half[side] = lo.x, half[2 + side] = lo.y, half[4 + side] = lo.z;
        half[6 + side] = -hi.x, half[8 + side] = -hi.y, half[10 + side] = -hi.z;
        if ((arrive_acq_rel_cta(&s_flag[t]) & 0xffu) == 0) break;  // sibling not done yet
        union_of_halves(s_node[t][0], s_node[t][1], s_node[t][2], lo, hi);
        link = s_link[t];
    }
    __syncthreads();
    if (g < total_nodes) {  // every node once; spanning nodes' internal halves follow in bvh_boxes_kernel
        __stcg(&b.nodes[g].a, s_node[threadIdx.x][0]);
        __stcg(&b.nodes[g].b, s_node[threadIdx.x][1]);
        __stcg(&b.nodes[g].c, s_node[threadIdx.x][2]);
    }
}

// The climbs through parents that span blocks, one thread per internal node:
// they start at the local nodes whose parent spans blocks (their boxes are
// complete after bvh_build_kernel) and at the spanning nodes with two leaf
// children, and go through the nodes' flags and halves in global memory,
// ordered at device scope.  Every ancestor of a spanning node spans blocks too.
__global__ void __launch_bounds__(BOX_THREADS) bvh_boxes_kernel(Bvh b)
{
    const int64_t g = (int64_t)blockIdx.x * BOX_THREADS + threadIdx.x;
    if (g >= b.total - b.m) return;
    const int4 cd = b.nodes[g].d;
    int link = b.parent_node[g];
    const bool two_leaves = (cd.x & LEAF_BIT) && (cd.y & LEAF_BIT);
    if (!(cd.z ? (link >= 0 && !(link & 1)) : two_leaves)) return;
    float3 lo, hi;
    union_of_halves(__ldcg(&b.nodes[g].a), __ldcg(&b.nodes[g].b), __ldcg(&b.nodes[g].c), lo, hi);
    for (int guard = 0; guard < 4096 && link >= 0; ++guard) {
        const int64_t pg = link >> 2;
        const int side = (link >> 1) & 1;
        BvhNode *node = b.nodes + pg;
        store_box(node, side, lo, hi);
        if ((arrive_acq_rel(&b.flags[pg]) & 0xffu) == 0) return;  // sibling not done yet
        float3 plo, phi;
        union_of_halves(__ldcg(&node->a), __ldcg(&node->b), __ldcg(&node->c), plo, phi);
        lo = plo;
        hi = phi;
        link = b.parent_node[pg];
    }
    if (link >= 0) atomicExch(b.error, 1);
}

__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Sample point prepared for packed box tests.
struct Query {
    float2 sx, sy, sz;  // (s, s) per axis
};

__device__ __forceinline__ Query make_query(float3 s)
{
    Query q;
    q.sx = make_float2(s.x, s.x);
    q.sy = make_float2(s.y, s.y);
    q.sz = make_float2(s.z, s.z);
    return q;
}

// Canonical squared distances from the sample to both child boxes (0 inside):
// per-axis gap max(lo - s, s - hi, 0), then fma(gz,gz, fma(gx,gx, gy*gy)) --
// the same expression as the point distance, so a leaf (lo = hi = p) gives
// exactly its canonical distance.
__device__ __forceinline__ float2 child_dist2(const Query &q, const float4 &a, const float4 &b, const float4 &c)
{
    // lo - s as fma(s, -1, lo): one rounding of the exact difference
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 ux = __ffma2_rn(q.sx, m1, make_float2(a.x, a.y)), vx = __fadd2_rn(q.sx, make_float2(b.z, b.w));
    const float2 uy = __ffma2_rn(q.sy, m1, make_float2(a.z, a.w)), vy = __fadd2_rn(q.sy, make_float2(c.x, c.y));
    const float2 uz = __ffma2_rn(q.sz, m1, make_float2(b.x, b.y)), vz = __fadd2_rn(q.sz, make_float2(c.z, c.w));
    const float2 gx = make_float2(max3f(ux.x, vx.x, 0.0f), max3f(ux.y, vx.y, 0.0f));
    const float2 gy = make_float2(max3f(uy.x, vy.x, 0.0f), max3f(uy.y, vy.y, 0.0f));
    const float2 gz = make_float2(max3f(uz.x, vz.x, 0.0f), max3f(uz.y, vz.y, 0.0f));
    return __ffma2_rn(gz, gz, __ffma2_rn(gx, gx, __fmul2_rn(gy, gy)));
}

// Query layout: a warp owns an 8 (z) x 4 (y) patch of sample columns and each
// thread sweeps RUN_X consecutive samples along x, two at a time (x, x+1):
// one node load serves both samples of a lane, which halves the L1 traffic
// per sample (the broadcast node loads' register writeback is what bounds
// the query kernel).  A block stacks four warps in y, covering 16 (y) x 8 (z)
// x RUN_X (x) samples.  The nearest points of one pair seed the next pair's
// bounds (canonical distances to those real points), which keeps the
// traversal exact and prunes almost everything but the nearest region.
constexpr int PATCH_Z = 8, PATCH_Y = 4, WARPS_Y = QUERY_THREADS / 32;
// samples per lane along x: long runs amortise the first pair's greedy bound;
// short runs keep enough blocks in flight for small volumes
constexpr int RUN_X_LONG = 64, RUN_X_SHORT = 8;
constexpr int QUERY_GROUP = 4;  // samples per lane traversed together
// neighbour lanes whose last nearest point is a further candidate bound:
// z +- 1, y +- 1 and z +- 2 (lane xor 1, xor 8, xor 2; 256^3 distance stage
// 291 ms with the first two, 287 ms with three, 289 ms adding y +- 2)
constexpr int NEIGHBOURS = 3;

__device__ __forceinline__ void load_node(const BvhNode *nodes, int cur, float4 &a, float4 &b, float4 &c, int4 &d)
{
    a = __ldg(&nodes[cur].a);
    b = __ldg(&nodes[cur].b);
    c = __ldg(&nodes[cur].c);
    d = __ldg(&nodes[cur].d);
}

// Exact nearest canonical squared distances for the 32*K samples of a warp (K
// per lane), traversed as one packet: every lane evaluates every visited node
// against all its samples and bounds, and a subtree is skipped only when no
// sample's bound admits it (bounds only decrease, so skipping is safe for
// every sample).  Node addresses are warp-uniform (one broadcast load per
// node) and no lane idles.  Each best starts as the canonical distance to a
// real point bp; on return it is the minimum and bp its point.
template <int K>
__device__ __forceinline__ void traverse_packet(const BvhNode *nodes, const Query (&q)[K], float (&best)[K],
                                                float3 (&bp)[K], int *error)
{
    int stack[STACK_DEPTH];      // warp-uniform node ids
    float sd[STACK_DEPTH];       // the lane's nearest sample distance to each postponed node
    int top = 0;
    int cur = 0;
    for (;;) {
        float4 a, b, c;
        int4 d;
        load_node(nodes, cur, a, b, c, d);
        float2 dd[K];
#pragma unroll
        for (int k = 0; k < K; ++k) dd[k] = child_dist2(q[k], a, b, c);
        const int left = d.x, right = d.y;
        bool gl = false, gr = false;
        if (left & LEAF_BIT) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (dd[k].x < best[k]) {
                    best[k] = dd[k].x;
                    bp[k] = make_float3(a.x, a.z, b.x);
                }
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) gl |= dd[k].x < best[k];
        }
        if (right & LEAF_BIT) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (dd[k].y < best[k]) {
                    best[k] = dd[k].y;
                    bp[k] = make_float3(a.y, a.w, b.y);
                }
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) gr |= dd[k].y < best[k];
        }
        const bool any_l = __any_sync(0xffffffffu, gl), any_r = __any_sync(0xffffffffu, gr);
        if (any_l && any_r) {
            // most lanes' nearer child (for the first sample) first
            const bool lfirst = __popc(__ballot_sync(0xffffffffu, dd[0].x <= dd[0].y)) >= 16;
            if (top == STACK_DEPTH) {
                atomicExch(error, 2);
                break;
            }
            stack[top] = lfirst ? right : left;
#pragma unroll
            float near = lfirst ? dd[0].y : dd[0].x;
#pragma unroll
            for (int k = 1; k < K; ++k) near = fminf(near, lfirst ? dd[k].y : dd[k].x);
            sd[top] = near;
            ++top;
            cur = lfirst ? left : right;
        } else if (any_l) {
            cur = left;
        } else if (any_r) {
            cur = right;
        } else {
            for (;;) {
                if (top == 0) break;
                float loosest = best[0];
#pragma unroll
                for (int k = 1; k < K; ++k) loosest = fmaxf(loosest, best[k]);
                const bool keep = sd[top - 1] < loosest;  // skipped only where no sample's bound admits it
                if (__any_sync(0xffffffffu, keep)) break;
                --top;
            }
            if (top == 0) break;
            cur = stack[--top];
        }
    }
}

template <int RUN_X, int K>
__global__ void __launch_bounds__(QUERY_THREADS, 8) bvh_query_kernel(Bvh b, SampleGrid g, float *fields, int64_t stride)
{
    static_assert(RUN_X % K == 0 && K >= 2, "samples go in groups of K along x");
    const int s = blockIdx.y;
    const int64_t X10 = g.F / (g.Y10 * g.Z10);
    const int64_t nbz = (g.Z10 + PATCH_Z - 1) / PATCH_Z;
    const int64_t nby = (g.Y10 + PATCH_Y * WARPS_Y - 1) / (PATCH_Y * WARPS_Y);
    const int64_t tile = blockIdx.x;
    const int64_t tz = tile % nbz, ty = (tile / nbz) % nby, tx = tile / (nbz * nby);
    const int lz = threadIdx.x % PATCH_Z, ly = threadIdx.x / PATCH_Z;  // ly in [0, 16)
    const int64_t z = tz * PATCH_Z + lz, y = ty * PATCH_Y * WARPS_Y + ly, x0 = tx * RUN_X;
    const bool col_valid = z < g.Z10 && y < g.Y10;
    const int64_t n = b.ccount[s];
    const float4 *leaves = b.leaves + b.cstart[s];
    float *out = fields + (size_t)s * stride;

    if (n == 1) {
        const float4 p = __ldg(leaves);
        for (int k = 0; k < RUN_X; ++k) {
            const int64_t x = x0 + k;
            if (!col_valid || x >= X10) break;
            const int64_t idx = (x * g.Y10 + y) * g.Z10 + z;
            const float3 sp = sample_point(g, idx);
            out[idx] = fminf(INIT_BOUND, iso_dist2(__fsub_rn(sp.x, p.x), __fsub_rn(sp.y, p.y), __fsub_rn(sp.z, p.z)));
        }
        return;
    }
    const BvhNode *nodes = b.nodes + (b.cstart[s] - s);

    // first sample of the run: greedy descent to a leaf, then the greedy points
    // of five warp neighbours as further candidates (all lanes take part)
    // lanes outside the grid follow the nearest in-grid sample (coherent packet)
    const int64_t yc = y < g.Y10 ? y : g.Y10 - 1, zc = z < g.Z10 ? z : g.Z10 - 1;
    const int64_t idx0 = ((x0 < X10 ? x0 : X10 - 1) * g.Y10 + yc) * g.Z10 + zc;
    float3 sp = sample_point(g, idx0);
    Query qy = make_query(sp);
    int cur = 0, leaf = 0;
    for (int depth = 0; depth < STACK_DEPTH; ++depth) {
        float4 a, b, c;
        int4 d;
        load_node(nodes, cur, a, b, c, d);
        const float2 dd = child_dist2(qy, a, b, c);
        const int next = dd.x <= dd.y ? d.x : d.y;
        if (next & LEAF_BIT) {
            leaf = next & ~LEAF_BIT;
            break;
        }
        cur = next;
    }
    const float4 gp = __ldg(leaves + leaf);
    float best = INIT_BOUND;
    float3 bp = make_float3(gp.x, gp.y, gp.z);
#pragma unroll
    for (int o = 0; o < 6; ++o) {
        const int mask = o == 0 ? 0 : (1 << (o - 1));
        const float px = __shfl_xor_sync(0xffffffffu, gp.x, mask);
        const float py = __shfl_xor_sync(0xffffffffu, gp.y, mask);
        const float pz = __shfl_xor_sync(0xffffffffu, gp.z, mask);
        const float dv = iso_dist2(__fsub_rn(sp.x, px), __fsub_rn(sp.y, py), __fsub_rn(sp.z, pz));
        if (dv < best) {
            best = dv;
            bp = make_float3(px, py, pz);
        }
    }
    // every lane runs every step (the packet traversal needs the whole warp);
    // lanes past the grid edge repeat a valid sample and do not store
    // nearest points of the previous group's last two samples
    float3 p_last = bp, p_prev = bp;
    // y and z coordinates are fixed per lane (the sample-grid formula of
    // BVH.cu:393-406, as sample_point computes it)
    const float sy = __fdiv_rn((float)(yc * g.ds + g.ds / 2), (float)g.Y);
    const float sz = __fdiv_rn((float)(zc * g.ds + g.ds / 2), (float)g.Z);
    for (int k0 = 0; k0 < RUN_X; k0 += K) {
        if (!__any_sync(0xffffffffu, col_valid && x0 + k0 < X10)) break;
        // candidates (all real points, so every bound is a true distance):
        // the previous group's last two nearest points and the last one of
        // the neighbour lanes z +- 1, y +- 1, z +- 2 (for the first group, the
        // greedy points)
        float3 cand[2 + NEIGHBOURS];
        cand[0] = p_last;
        cand[1] = p_prev;
#pragma unroll
        for (int o = 0; o < NEIGHBOURS; ++o) {
            const int mask = o == 0 ? 1 : (o == 1 ? PATCH_Z : (o == 2 ? 2 : 2 * PATCH_Z));
            cand[2 + o].x = __shfl_xor_sync(0xffffffffu, p_last.x, mask);
            cand[2 + o].y = __shfl_xor_sync(0xffffffffu, p_last.y, mask);
            cand[2 + o].z = __shfl_xor_sync(0xffffffffu, p_last.z, mask);
        }
        Query q[K];
        float bst[K];
        float3 pts[K];
        int64_t idx[K];
        bool val[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int64_t x = x0 + k0 + k;
            val[k] = col_valid && x < X10;
            const int64_t xc = x < X10 ? x : X10 - 1;
            idx[k] = (xc * g.Y10 + yc) * g.Z10 + zc;
            const float3 sk = make_float3(__fdiv_rn((float)(xc * g.ds + g.ds / 2), (float)g.X), sy, sz);
            q[k] = make_query(sk);
            bst[k] = iso_dist2(__fsub_rn(sk.x, cand[0].x), __fsub_rn(sk.y, cand[0].y), __fsub_rn(sk.z, cand[0].z));
            pts[k] = cand[0];
            if (k0 == 0 && k == 0) {
                bst[k] = best;  // the greedy bound of this very sample
                pts[k] = bp;
            }
#pragma unroll
            for (int o = 1; o < 2 + NEIGHBOURS; ++o) {
                const float cd = iso_dist2(__fsub_rn(sk.x, cand[o].x), __fsub_rn(sk.y, cand[o].y),
                                           __fsub_rn(sk.z, cand[o].z));
                if (cd < bst[k]) {
                    bst[k] = cd;
                    pts[k] = cand[o];
                }
            }
        }
        traverse_packet<K>(nodes, q, bst, pts, b.error);
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (val[k]) out[idx[k]] = __fsqrt_rn(bst[k]);
        p_last = pts[K - 1];
        p_prev = pts[K - 2];
    }
}

}  // namespace

// One group of surfaces: segments [seg0, seg0 + m) of sg (absolute indices)
// with counts h_count[0..m), fields written from `fields` (row 0 = seg0).
static int lbvh_group(iso_ctx *ctx, const SampleGrid &g, Segments sg, const int64_t *h_count, int m, int seg0,
                      float *fields, int64_t field_stride)
{
    std::vector<int64_t> cstart(m);
    int64_t total = 0;
    for (int q = 0; q < m; ++q) {
        cstart[q] = total;
        total += h_count[q];
    }
    if (total >= LBVH_MAX_GROUP_POINTS)  // parent links hold the node index * 4
        return iso_fail(ISO_ERR_CAPACITY, "surface %d has too many points (%lld)", seg0, (long long)total);
    if (total >= (int64_t)0x7fffffff) return iso_fail(ISO_ERR_CAPACITY, "too many surface points (%lld)", (long long)total);
    void *d_cstart, *d_keys, *d_keys2, *d_vals, *d_vals2, *d_compact, *d_leaves, *d_nodes, *d_pn, *d_flags, *d_misc;
    ISO_TRY(iso_buf(ctx, BUF_STAGING_A, (size_t)m * 2 * sizeof(int64_t), &d_cstart));
    ISO_TRY(iso_buf(ctx, BUF_SORT_KEYS, (size_t)total * 4, &d_keys));
    ISO_TRY(iso_buf(ctx, BUF_SORT_KEYS_ALT, (size_t)total * 4, &d_keys2));
    ISO_TRY(iso_buf(ctx, BUF_SORT_VALS, (size_t)total * 4, &d_vals));
    ISO_TRY(iso_buf(ctx, BUF_SORT_VALS_ALT, (size_t)total * 4, &d_vals2));
    ISO_TRY(iso_buf(ctx, BUF_STAGING_B, (size_t)total * sizeof(float4), &d_compact));
    ISO_TRY(iso_buf(ctx, BUF_BVH_LEAVES, (size_t)total * sizeof(float4), &d_leaves));
    ISO_TRY(iso_buf(ctx, BUF_BVH_NODES, (size_t)total * sizeof(BvhNode), &d_nodes));
    ISO_TRY(iso_buf(ctx, BUF_BVH_PARENT, (size_t)total * sizeof(int), &d_pn));
    ISO_TRY(iso_buf(ctx, BUF_BVH_FLAGS, (size_t)total * sizeof(unsigned int), &d_flags));
    ISO_TRY(iso_buf(ctx, BUF_MISC, 256, &d_misc));
    std::vector<int64_t> cs2(2 * (size_t)m);
    for (int q = 0; q < m; ++q) {
        cs2[q] = cstart[q];
        cs2[m + q] = h_count[q];
    }
    ISO_CUDA(cudaMemcpyAsync(d_cstart, cs2.data(), cs2.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    ISO_CUDA(cudaMemsetAsync(d_misc, 0, sizeof(int), ctx->stream));
    Segments gs = sg;  // segment offsets of this group
    gs.offset = sg.offset + seg0;
    gs.count = sg.count + seg0;
    Bvh b;
    b.cstart = (const int64_t *)d_cstart;
    b.ccount = (const int64_t *)d_cstart + m;
    b.m = m;
    b.total = total;
    b.keys = (unsigned int *)d_keys;
    b.axis_bits = lbvh_axis_bits(m);
    b.vals = (unsigned int *)d_vals;
    b.compact = (float4 *)d_compact;
    b.leaves = (float4 *)d_leaves;
    b.nodes = (BvhNode *)d_nodes;
    b.parent_node = (int *)d_pn;
    b.flags = (unsigned int *)d_flags;
    b.error = (int *)d_misc;
    const unsigned tb = (unsigned)((total + 255) / 256);
    bvh_keys_kernel<<<tb, 256, 0, ctx->stream>>>(gs, b);
    ISO_LAUNCHED(ctx);
    const int end_bit = lbvh_seg_bits(m) + 3 * b.axis_bits;
    cub::DoubleBuffer<unsigned int> kb((unsigned int *)d_keys, (unsigned int *)d_keys2);
    cub::DoubleBuffer<unsigned int> vb((unsigned int *)d_vals, (unsigned int *)d_vals2);
    size_t temp_bytes = 0;
    ISO_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, kb, vb, (int)total, 0, end_bit, ctx->stream));
    void *d_temp;
    ISO_TRY(iso_buf(ctx, BUF_CUB_TEMP, temp_bytes, &d_temp));
    ISO_CUDA(cub::DeviceRadixSort::SortPairs(d_temp, temp_bytes, kb, vb, (int)total, 0, end_bit, ctx->stream));
    ctx->launches += 4;
    bvh_gather_kernel<<<tb, 256, 0, ctx->stream>>>(b, vb.Current());
    ISO_LAUNCHED(ctx);
    const int64_t total_nodes = total - m;
    if (total_nodes > 0) {
        bvh_build_kernel<<<(unsigned)((total_nodes + BOX_THREADS - 1) / BOX_THREADS), BOX_THREADS, 0, ctx->stream>>>(
            b, kb.Current());
        ISO_LAUNCHED(ctx);
        bvh_boxes_kernel<<<(unsigned)((total_nodes + BOX_THREADS - 1) / BOX_THREADS), BOX_THREADS, 0, ctx->stream>>>(b);
        ISO_LAUNCHED(ctx);
    }
    for (int base = 0; base < m; base += 65535) {
        const int cnt = m - base < 65535 ? m - base : 65535;
        Bvh bb = b;
        bb.cstart = b.cstart + base;
        bb.ccount = b.ccount + base;
        // node bases are cstart[s] - s with the group-local s: shift nodes accordingly
        bb.nodes = b.nodes - base;
        const int64_t X10 = g.F / (g.Y10 * g.Z10);
        const int64_t cols = ((g.Y10 + PATCH_Y * WARPS_Y - 1) / (PATCH_Y * WARPS_Y)) * ((g.Z10 + PATCH_Z - 1) / PATCH_Z);
        // samples per lane along x: the context's choice (autotuner), else
        // 64 for volumes of 128 and more along x, 8 below
        const int run = ctx->query_run > 0 ? ctx->query_run : (X10 >= 128 ? RUN_X_LONG : RUN_X_SHORT);
        const int64_t bricks = ((X10 + run - 1) / run) * cols;
        const dim3 grid((unsigned)bricks, cnt);
        float *out = fields + (size_t)base * field_stride;
        switch (run) {
        case 8: bvh_query_kernel<8, QUERY_GROUP><<<grid, QUERY_THREADS, 0, ctx->stream>>>(bb, g, out, field_stride); break;
        case 16: bvh_query_kernel<16, QUERY_GROUP><<<grid, QUERY_THREADS, 0, ctx->stream>>>(bb, g, out, field_stride); break;
        case 32: bvh_query_kernel<32, QUERY_GROUP><<<grid, QUERY_THREADS, 0, ctx->stream>>>(bb, g, out, field_stride); break;
        default: bvh_query_kernel<64, QUERY_GROUP><<<grid, QUERY_THREADS, 0, ctx->stream>>>(bb, g, out, field_stride); break;
        }
        ISO_LAUNCHED(ctx);
    }
    int err = 0;
    ISO_CUDA(cudaMemcpyAsync(&err, d_misc, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (err) return iso_fail(ISO_ERR_INTERNAL, "LBVH consistency check failed (code %d)", err);
    return ISO_OK;
}

// Distance fields of `num_segments` point sets (normalised points in
// BUF_POINTS_NORM; segment q has h_seg_count[q] points at h_seg_offset[q]) into
// BUF_FIELDS rows q (stride field_stride floats), then per-field min/max into
// BUF_FIELD_MINMAX.
int iso_run_distance(iso_ctx *ctx, int X, int Y, int Z, int ds, int method, const int32_t * /*h_segments*/,
                     int num_segments, const int64_t *h_seg_offset, const int64_t *h_seg_count, int64_t field_stride)
{
    const int m = num_segments;
    if (m <= 0) return ISO_OK;
    if (ds < 1 || X / ds < 1 || Y / ds < 1 || Z / ds < 1) return iso_fail(ISO_ERR_ARG, "bad downscale %d", ds);
    SampleGrid g;
    g.X = X;
    g.Y = Y;
    g.Z = Z;
    g.ds = ds;
    g.Y10 = Y / ds;
    g.Z10 = Z / ds;
    g.F = (int64_t)(X / ds) * g.Y10 * g.Z10;
    for (int q = 0; q < m; ++q)
        if (h_seg_count[q] < 1) return iso_fail(ISO_ERR_ARG, "distance field of an empty surface");

    void *d_off, *d_cnt, *d_fields, *d_minmax;
    ISO_TRY(iso_buf(ctx, BUF_SEG_OFFSET, (size_t)m * sizeof(int64_t), &d_off));
    ISO_TRY(iso_buf(ctx, BUF_SEG_COUNT, (size_t)m * sizeof(int64_t), &d_cnt));
    ISO_TRY(iso_buf(ctx, BUF_FIELDS, (size_t)m * field_stride * sizeof(float), &d_fields));
    ISO_TRY(iso_buf(ctx, BUF_FIELD_MINMAX, (size_t)m * 2 * sizeof(uint32_t), &d_minmax));
    ISO_CUDA(cudaMemcpyAsync(d_off, h_seg_offset, m * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    ISO_CUDA(cudaMemcpyAsync(d_cnt, h_seg_count, m * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    Segments sg;
    sg.points = (const float4 *)ctx->buf[BUF_POINTS_NORM];
    sg.offset = (const int64_t *)d_off;
    sg.count = (const int64_t *)d_cnt;
    float *fields = (float *)d_fields;

    if (method == ISO_DF_BRUTE) {
        const int64_t per_block = (int64_t)BRUTE_THREADS * BRUTE_SAMPLES;
        const unsigned bx = (unsigned)((g.F + per_block - 1) / per_block);
        for (int base = 0; base < m; base += 65535) {
            int cnt = m - base < 65535 ? m - base : 65535;
            df_brute_kernel<<<dim3(bx, cnt), BRUTE_THREADS, 0, ctx->stream>>>(sg, g, fields + (size_t)base * field_stride,
                                                                             field_stride, base);
            ISO_LAUNCHED(ctx);
        }
    } else if (method == ISO_DF_TC) {
        ISO_TRY(iso_run_distance_tc(ctx, g, sg, h_seg_count, m, fields, field_stride));
    } else if (method == ISO_DF_LBVH) {
        // surfaces are processed in groups of at most ctx->lbvh_group_points
        // points (one surface may exceed it alone), which bounds the LBVH
        // arrays' memory independently of the number of isovalues
        for (int q0 = 0; q0 < m;) {
            int q1 = q0;
            int64_t pts = 0;
            const int64_t cap = ctx->lbvh_group_points < LBVH_MAX_GROUP_POINTS - 1 ? ctx->lbvh_group_points
                                                                                   : LBVH_MAX_GROUP_POINTS - 1;
            while (q1 < m && q1 - q0 < LBVH_MAX_GROUP_SURFACES && (q1 == q0 || pts + h_seg_count[q1] <= cap))
                pts += h_seg_count[q1++];
            ISO_TRY(lbvh_group(ctx, g, sg, h_seg_count + q0, q1 - q0, q0, fields + (size_t)q0 * field_stride,
                               field_stride));
            q0 = q1;
        }
    } else {
        return iso_fail(ISO_ERR_ARG, "unknown distance-field method %d", method);
    }
    return iso_run_minmax(ctx, fields, m, g.F, field_stride, (uint32_t *)d_minmax);
}
