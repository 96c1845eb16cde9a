// iso_distance_tc.cu -- distance fields by brute force on the tensor cores
// (ISO_DF_TC): every sample against every surface point, recast as the
// contraction |s - p|^2 = |s|^2 + |p|^2 - 2 s.p, with an exact FP32 pass over
// the candidates it selects.  Same output as the other methods, bit for bit:
// sqrt of the minimum canonical squared distance (the brute-force comparator
// of isosurfaces_cuda/src/DistanceField.cu:49-65 and the nearest query of
// isosurfaces_cuda/src/BVH.cu:577-613).
//
// One CTA owns a brick of 128 samples (8 z x 4 y x 4 x) of one field and
// streams the surface's points in blocks of 128:
//  * both sides are centred on the brick: sigma = s - c per sample, pi = p - c
//    per point (FP32), so the terms of the contraction shrink with the
//    distance instead of being O(1), and split into f16 hi + lo parts;
//  * A (128 x 16, one row per sample):  [sh, sh, sl, 1 1 1, 0...]
//    B (128 x 16, one row per point):   [-2 ph, -2 pl, -2 ph, q_hi q_mid q_lo, 0...]
//    so that A.B = |pi|^2 - 2 sigma.pi (the sl*pl products are dropped);
//    one tcgen05.mma (M = 128, N = 128, K = 16, f16 in, FP32 out) per block
//    writes a 128 x 128 FP32 tile to tensor memory;
//  * each thread reads its sample's 128 values back (tcgen05.ld) and keeps the
//    smallest, B; every point whose value is within tau of B is a candidate,
//    and its canonical FP32 distance (the fma chain every method uses) is
//    computed from the original coordinates; the field value is the minimum
//    over candidates.
//
// Exactness: the canonical winner w (smallest canonical FP32 distance) is
// always a candidate, because a(w) - B_final <= |e(w)| + |e(j)| + 1e-6 * D,
// where a = A.B, e is a's error against the exact |sigma - pi|^2 - |sigma|^2
// and j the point giving B.  tau bounds that: with D ~ B + |sigma|^2 (the
// squared distance) and R = |sigma| + sqrt(D) (the radius within which both
// points lie, measured from the brick centre), the error of a is at most
// kappa * R^2 (f16 split residuals, the dropped sl*pl terms and FP32
// accumulation of at most 12 terms of magnitude <= R^2; kappa = 2^-14 is about
// ten times the bound) plus the rounding of the centring (<= 1e-6 * sqrt(D))
// and of the f16 parts of |pi|^2 (< 1e-7).  Any other point within tau is
// also rechecked, so a loose tau costs time, never exactness.
#include <cuda_fp16.h>

#include "iso_internal.cuh"
#include "iso_tc.cuh"

using namespace isotc;

namespace {

// Warp roles: warps 0-3 own one sample each per thread (A rows, read-back and
// candidates); warps 4-5 convert the next block of points into the B operand
// while the tensor cores and the first four warps work on the current one.
// Two operand stages and two accumulators (2 x 128 TMEM columns) alternate;
// full[s] completes when the MMA of stage s is done (tcgen05.commit), empty[s]
// when the four sample warps have read its accumulator and points.
constexpr int EPI_WARPS = 4;
constexpr int PROD_WARPS = 2;
constexpr int TC_THREADS = 32 * (EPI_WARPS + PROD_WARPS);
constexpr int TC_POINTS = 128;        // points per MMA (N)
constexpr uint32_t TC_COLS = 256;     // two accumulators of TC_POINTS columns
constexpr int BRICK_Z = 8, BRICK_Y = 4, BRICK_X = 4;
// shared memory: A tile, two B stages, two point stages, barriers and the
// TMEM slot; the dynamic size is padded so that at most two CTAs share an SM
// (2 x 256 TMEM columns = all 512)
constexpr int SM_A = 0;
constexpr int SM_B0 = 4096;                          // 128 rows x 32 B per stage
constexpr int SM_P0 = SM_B0 + 2 * TC_POINTS * 32;    // 128 float4 per stage
constexpr int SM_BAR = SM_P0 + 2 * TC_POINTS * 16;   // full[2], empty[2], slot
constexpr int SM_USED = SM_BAR + 64;
constexpr int SM_ALLOC = 80 * 1024;
constexpr float KAPPA = 6.103515625e-05f;      // 2^-14
constexpr float SENTINEL_Q = 30000.0f;         // |pi|^2 of padding rows: never within tau
constexpr uint32_t WAIT_LIMIT = 1u << 26;      // polls of one barrier wait before giving up

__device__ __forceinline__ void split_f16(float v, __half &hi, __half &lo)
{
    hi = __float2half_rn(v);
    lo = __float2half_rn(__fsub_rn(v, __half2float(hi)));
}

// Two f16 values as one 32-bit word, the first in the low half (the lower K index).
__device__ __forceinline__ uint32_t pack_h2(__half lo, __half hi)
{
    return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}

__device__ __forceinline__ int64_t clamp_hi(int64_t v, int64_t hi) { return v < hi ? v : hi; }

__device__ __forceinline__ float tau_of(float best, float s2, float sn)
{
    const float D = fmaxf(best + s2, 0.0f) + 1e-6f;
    const float sd = sqrtf(D);
    const float R = sn + sd;
    return 1e-6f * D + 2.0f * KAPPA * R * R + 1e-6f * sd + 4e-7f;
}

// B row of one point (or of padding when `valid` is false) and its FP32 copy.
__device__ __forceinline__ void write_row(unsigned char *sB, float4 *sP, int r, bool valid, float4 p, float3 c)
{
    uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
    if (valid) {
        const float px = __fsub_rn(p.x, c.x), py = __fsub_rn(p.y, c.y), pz = __fsub_rn(p.z, c.z);
        __half hx, lx, hy, ly, hz, lz;
        split_f16(px, hx, lx);
        split_f16(py, hy, ly);
        split_f16(pz, hz, lz);
        const __half m2 = __float2half_rn(-2.0f);
        hx = __hmul(m2, hx);
        hy = __hmul(m2, hy);
        hz = __hmul(m2, hz);
        lx = __hmul(m2, lx);
        ly = __hmul(m2, ly);
        lz = __hmul(m2, lz);
        const float q = __fmaf_rn(pz, pz, __fmaf_rn(py, py, __fmul_rn(px, px)));
        const __half qh = __float2half_rn(q);
        const float q1 = __fsub_rn(q, __half2float(qh));
        const __half qm = __float2half_rn(q1);
        const __half ql = __float2half_rn(__fsub_rn(q1, __half2float(qm)));
        w0 = make_uint4(pack_h2(hx, hy), pack_h2(hz, lx), pack_h2(ly, lz), pack_h2(hx, hy));
        w1 = make_uint4(pack_h2(hz, qh), pack_h2(qm, ql), 0u, 0u);
    } else {
        w1.x = pack_h2(__float2half_rn(0.0f), __float2half_rn(SENTINEL_Q));
    }
    *reinterpret_cast<uint4 *>(sB + tc_offset(r, 0)) = w0;
    *reinterpret_cast<uint4 *>(sB + tc_offset(r, 8)) = w1;
    sP[r] = p;
}

struct TcArgs {
    IsoSampleGrid g;
    IsoSegments sg;
    float *fields;
    int64_t stride;
    int bx, by, bz;  // bricks per axis
    int *error;
};

__global__ void __launch_bounds__(TC_THREADS, 2) df_tc_kernel(TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *sA = sm + SM_A;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + SM_BAR);
    uint64_t *empty = full + 2;
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + SM_BAR + 32);
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const int seg = blockIdx.y;
    const int64_t off = a.sg.offset[seg], P = a.sg.count[seg];
    const IsoSampleGrid &g = a.g;
    const int64_t X10 = g.F / (g.Y10 * g.Z10);

    // the brick and its centre
    const int brick = blockIdx.x;
    const int bz = brick % a.bz, by = (brick / a.bz) % a.by, bxi = brick / (a.bz * a.by);
    const int64_t cx = clamp_hi((int64_t)bxi * BRICK_X + 2, X10 - 1),
                  cy = clamp_hi((int64_t)by * BRICK_Y + 2, g.Y10 - 1), cz = clamp_hi((int64_t)bz * BRICK_Z + 4, g.Z10 - 1);
    const float3 c = iso_sample_point(g, (cx * g.Y10 + cy) * g.Z10 + cz);

    // sample warps: this thread's sample and its A row
    const int ts = t & 127;
    const int64_t z = (int64_t)bz * BRICK_Z + (ts & 7), y = (int64_t)by * BRICK_Y + ((ts >> 3) & 3),
                  x = (int64_t)bxi * BRICK_X + (ts >> 5);
    const bool inside = w < EPI_WARPS && z < g.Z10 && y < g.Y10 && x < X10;
    const int64_t idx = inside ? (x * g.Y10 + y) * g.Z10 + z : 0;
    const float3 s = iso_sample_point(g, idx);
    const float3 sig = make_float3(__fsub_rn(s.x, c.x), __fsub_rn(s.y, c.y), __fsub_rn(s.z, c.z));
    const float s2 = __fmaf_rn(sig.z, sig.z, __fmaf_rn(sig.y, sig.y, __fmul_rn(sig.x, sig.x)));
    const float sn = sqrtf(s2);
    if (w < EPI_WARPS) {
        __half hx, lx, hy, ly, hz, lz;
        split_f16(sig.x, hx, lx);
        split_f16(sig.y, hy, ly);
        split_f16(sig.z, hz, lz);
        const __half one = __float2half_rn(1.0f);
        *reinterpret_cast<uint4 *>(sA + tc_offset(ts, 0)) =
            make_uint4(pack_h2(hx, hy), pack_h2(hz, hx), pack_h2(hy, hz), pack_h2(lx, ly));
        *reinterpret_cast<uint4 *>(sA + tc_offset(ts, 8)) = make_uint4(pack_h2(lz, one), pack_h2(one, one), 0u, 0u);
    }
    if (t == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&empty[0], EPI_WARPS);
        mbar_init(&empty[1], EPI_WARPS);
    }
    if (w == 0) {
        tmem_alloc(slot, TC_COLS);
        tmem_relinquish();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *slot;
    const int64_t nblocks = (P + TC_POINTS - 1) / TC_POINTS;
    bool ok = true;

    if (w >= EPI_WARPS) {
        // producers: 64 rows per warp, two per lane; the next block's points
        // are loaded while the current one is converted
        const int pw = w - EPI_WARPS;
        const uint64_t adesc = tc_desc(sA);
        const uint32_t idesc = tc_idesc_f16_f32(128, TC_POINTS);
        const int r0 = pw * 64 + lane, r1 = r0 + 32;
        float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f), p1 = p0;
        if (r0 < P) p0 = a.sg.points[off + r0];
        if (r1 < P) p1 = a.sg.points[off + r1];
        for (int64_t b = 0; b < nblocks; ++b) {
            const int st = (int)(b & 1);
            const int64_t base = b * TC_POINTS;
            float4 n0 = make_float4(0.f, 0.f, 0.f, 0.f), n1 = n0;
            if (base + TC_POINTS + r0 < P) n0 = a.sg.points[off + base + TC_POINTS + r0];
            if (base + TC_POINTS + r1 < P) n1 = a.sg.points[off + base + TC_POINTS + r1];
            // stage st was last used by block b - 2: wait until it was read
            if (b >= 2) ok = __all_sync(0xffffffffu, mbar_wait(&empty[st], (uint32_t)(((b >> 1) - 1) & 1), WAIT_LIMIT));
            if (!ok) break;
            unsigned char *sB = sm + SM_B0 + st * TC_POINTS * 32;
            float4 *sP = reinterpret_cast<float4 *>(sm + SM_P0) + st * TC_POINTS;
            write_row(sB, sP, r0, base + r0 < P, p0, c);
            write_row(sB, sP, r1, base + r1 < P, p1, c);
            fence_async_smem();
            named_bar(1, 32 * PROD_WARPS);
            if (t == 32 * EPI_WARPS) {
                tc_fence_after();
                tc_mma_f16(tbase + st * TC_POINTS, adesc, tc_desc(sB), idesc, 0);
                tc_commit(&full[st]);
            }
            p0 = n0;
            p1 = n1;
        }
    } else {
        float best = ISO_DF_INIT_BOUND;  // exact canonical minimum
        float bapprox = __int_as_float(0x7f800000), thr = bapprox;
        const uint32_t lane_addr = tbase + ((uint32_t)(32 * w) << 16);
        for (int64_t b = 0; b < nblocks; ++b) {
            const int st = (int)(b & 1);
            ok = __all_sync(0xffffffffu, mbar_wait(&full[st], (uint32_t)((b >> 1) & 1), WAIT_LIMIT));
            if (!ok) break;
            tc_fence_after();
            const float4 *sP = reinterpret_cast<const float4 *>(sm + SM_P0) + st * TC_POINTS;
            // all 128 accumulators of the block in one round trip
            uint32_t r[TC_POINTS];
#pragma unroll
            for (int ch = 0; ch < TC_POINTS / 32; ++ch) tmem_ld32_async(lane_addr + st * TC_POINTS + 32 * ch, r + 32 * ch);
            tmem_wait_ld128(r);
            float m[43];
#pragma unroll
            for (int k = 0; k < 42; ++k)
                m[k] = fmin3(__uint_as_float(r[3 * k]), __uint_as_float(r[3 * k + 1]), __uint_as_float(r[3 * k + 2]));
            m[42] = fminf(__uint_as_float(r[126]), __uint_as_float(r[127]));
#pragma unroll
            for (int k = 0; k < 14; ++k) m[k] = fmin3(m[3 * k], m[3 * k + 1], m[3 * k + 2]);
            m[14] = m[42];
#pragma unroll
            for (int k = 0; k < 5; ++k) m[k] = fmin3(m[3 * k], m[3 * k + 1], m[3 * k + 2]);
            const float cm = fminf(fmin3(m[0], m[1], m[2]), fminf(m[3], m[4]));
            if (cm <= thr) {
                bapprox = fminf(bapprox, cm);
                thr = bapprox + tau_of(bapprox, s2, sn);
#pragma unroll
                for (int j = 0; j < TC_POINTS; ++j) {
                    if (__uint_as_float(r[j]) <= thr) {
                        const float4 p = sP[j];
                        best = fminf(best, iso_dist2(__fsub_rn(s.x, p.x), __fsub_rn(s.y, p.y), __fsub_rn(s.z, p.z)));
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
        }
        if (ok && inside) a.fields[(size_t)seg * a.stride + idx] = iso_df_finish(best, P);
    }
    if (!ok && (t & 31) == 0) atomicExch(a.error, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (w == 0) tmem_dealloc(tbase, TC_COLS);
}

}  // namespace

int iso_run_distance_tc(iso_ctx *ctx, const IsoSampleGrid &g, const IsoSegments &sg, const int64_t *h_seg_count, int m,
                        float *fields, int64_t stride)
{
    (void)h_seg_count;
    static_assert(SM_USED <= SM_ALLOC, "shared memory layout");
    const int64_t X10 = g.F / (g.Y10 * g.Z10);
    TcArgs a;
    a.g = g;
    a.sg = sg;
    a.fields = fields;
    a.stride = stride;
    a.bz = (int)((g.Z10 + BRICK_Z - 1) / BRICK_Z);
    a.by = (int)((g.Y10 + BRICK_Y - 1) / BRICK_Y);
    a.bx = (int)((X10 + BRICK_X - 1) / BRICK_X);
    const int64_t bricks = (int64_t)a.bx * a.by * a.bz;
    if (bricks > 0x7fffffff) return iso_fail(ISO_ERR_ARG, "tensor-core distance: grid too large");
    void *d_err;
    ISO_TRY(iso_buf(ctx, BUF_TASK_COUNTER, 256, &d_err));
    a.error = (int *)d_err + 2;
    ISO_CUDA(cudaMemsetAsync(a.error, 0, sizeof(int), ctx->stream));
    ISO_CUDA(cudaFuncSetAttribute(df_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_ALLOC));
    for (int base = 0; base < m; base += 65535) {
        const int cnt = m - base < 65535 ? m - base : 65535;
        IsoSegments s2 = sg;
        s2.offset = sg.offset + base;
        s2.count = sg.count + base;
        a.sg = s2;
        a.fields = fields + (size_t)base * stride;
        df_tc_kernel<<<dim3((unsigned)bricks, cnt), TC_THREADS, SM_ALLOC, ctx->stream>>>(a);
        ISO_LAUNCHED(ctx);
    }
    int err = 0;
    ISO_CUDA(cudaMemcpyAsync(&err, a.error, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (err) return iso_fail(ISO_ERR_INTERNAL, "tensor-core distance: an MMA did not complete");
    return ISO_OK;
}
