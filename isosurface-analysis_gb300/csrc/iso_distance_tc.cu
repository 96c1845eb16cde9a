// iso_distance_tc.cu -- distance fields by brute force on the tensor cores
// (ISO_DF_TC): every sample against every surface point, recast as the
// contraction |s - p|^2 = |s|^2 + |p|^2 - 2 s.p, with an exact FP32 pass over
// the candidates it selects.  Same output as the other methods, bit for bit:
// sqrt of the minimum canonical squared distance (the brute-force comparator
// of isosurfaces_cuda/src/DistanceField.cu:49-65 and the nearest query of
// isosurfaces_cuda/src/BVH.cu:577-613).
//
// One CTA (4 warps, 128 threads) owns a brick of 128 samples (8 z x 4 y x 4 x)
// of one field and streams the surface's points in blocks of 256:
//  * both sides are centred on the brick: sigma = s - c per sample, pi = p - c
//    per point (FP32), so the terms of the contraction shrink with the
//    distance instead of being O(1), and split into f16 hi + lo parts;
//  * A (128 x 16, one row per sample):  [sh, sh, sl, 1 1 1, 0...]
//    B (256 x 16, one row per point):   [-2 ph, -2 pl, -2 ph, q_hi q_mid q_lo, 0...]
//    so that A.B = |pi|^2 - 2 sigma.pi (the sl*pl products are dropped);
//    one tcgen05.mma (M = 128, N = 256, K = 16, f16 in, FP32 out) per block
//    writes a 128 x 256 FP32 tile to tensor memory;
//  * each thread reads its sample's 256 values back (tcgen05.ld) and keeps the
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

constexpr int TC_THREADS = 128;       // one sample per thread
constexpr int TC_POINTS = 256;        // points per MMA (N)
constexpr uint32_t TC_COLS = 256;     // tensor-memory columns per CTA
constexpr int BRICK_Z = 8, BRICK_Y = 4, BRICK_X = 4;
// shared memory: A tile, B tile, block points, barrier and TMEM slot; the
// dynamic size is padded so that at most two CTAs share an SM (2 x 256 TMEM
// columns = all 512)
constexpr int SM_A = 0;
constexpr int SM_B = 4096;
constexpr int SM_P = SM_B + 8192;
constexpr int SM_BAR = SM_P + TC_POINTS * 16;
constexpr int SM_USED = SM_BAR + 64;
constexpr int SM_ALLOC = 80 * 1024;
constexpr float KAPPA = 6.103515625e-05f;      // 2^-14
constexpr float SENTINEL_Q = 30000.0f;         // |pi|^2 of padding rows: never within tau
constexpr uint32_t WAIT_LIMIT = 1u << 26;      // polls of an MMA-completion wait before giving up

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

struct TcArgs {
    IsoSampleGrid g;
    IsoSegments sg;
    float *fields;
    int64_t stride;
    int bx, by, bz;  // bricks per axis
    int *error;
};

__global__ void __launch_bounds__(TC_THREADS) df_tc_kernel(TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *sA = sm + SM_A, *sB = sm + SM_B;
    float4 *sP = reinterpret_cast<float4 *>(sm + SM_P);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + SM_BAR);
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + SM_BAR + 8);
    const int t = threadIdx.x, w = t >> 5;
    const int seg = blockIdx.y;
    const int64_t off = a.sg.offset[seg], P = a.sg.count[seg];
    const IsoSampleGrid &g = a.g;
    const int64_t X10 = g.F / (g.Y10 * g.Z10);

    // this thread's sample and the brick centre
    const int brick = blockIdx.x;
    const int bz = brick % a.bz, by = (brick / a.bz) % a.by, bxi = brick / (a.bz * a.by);
    const int64_t z = (int64_t)bz * BRICK_Z + (t & 7), y = (int64_t)by * BRICK_Y + ((t >> 3) & 3),
                  x = (int64_t)bxi * BRICK_X + (t >> 5);
    const bool inside = z < g.Z10 && y < g.Y10 && x < X10;
    const int64_t idx = ((inside ? x : 0) * g.Y10 + (inside ? y : 0)) * g.Z10 + (inside ? z : 0);
    const float3 s = iso_sample_point(g, idx);
    const int64_t cx = clamp_hi((int64_t)bxi * BRICK_X + 2, X10 - 1), cy = clamp_hi((int64_t)by * BRICK_Y + 2, g.Y10 - 1),
                  cz = clamp_hi((int64_t)bz * BRICK_Z + 4, g.Z10 - 1);
    const float3 c = iso_sample_point(g, (cx * g.Y10 + cy) * g.Z10 + cz);
    const float3 sig = make_float3(__fsub_rn(s.x, c.x), __fsub_rn(s.y, c.y), __fsub_rn(s.z, c.z));
    const float s2 = __fmaf_rn(sig.z, sig.z, __fmaf_rn(sig.y, sig.y, __fmul_rn(sig.x, sig.x)));
    const float sn = sqrtf(s2);

    // A row t: sh (3), sh (3), sl (3), 1 x 3, 0 x 4
    {
        __half hx, lx, hy, ly, hz, lz;
        split_f16(sig.x, hx, lx);
        split_f16(sig.y, hy, ly);
        split_f16(sig.z, hz, lz);
        const __half one = __float2half_rn(1.0f);
        *reinterpret_cast<uint4 *>(sA + tc_offset(t, 0)) =
            make_uint4(pack_h2(hx, hy), pack_h2(hz, hx), pack_h2(hy, hz), pack_h2(lx, ly));
        *reinterpret_cast<uint4 *>(sA + tc_offset(t, 8)) =
            make_uint4(pack_h2(lz, one), pack_h2(one, one), 0u, 0u);
    }
    if (t == 0) mbar_init(mbar, 1);
    if (w == 0) {
        tmem_alloc(slot, TC_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *slot;
    const uint64_t adesc = tc_desc(sA), bdesc = tc_desc(sB);
    const uint32_t idesc = tc_idesc_f16_f32(128, TC_POINTS);
    const uint32_t lane_addr = tbase + ((uint32_t)(32 * w) << 16);

    float best = ISO_DF_INIT_BOUND;  // exact canonical minimum
    float bapprox = __int_as_float(0x7f800000), thr = bapprox;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t base = 0; base < P && ok; base += TC_POINTS) {
        // B rows and FP32 copies of this block's points (two per thread)
#pragma unroll
        for (int r2 = 0; r2 < 2; ++r2) {
            const int r = 2 * t + r2;
            // row halves: -2 ph (3), -2 pl (3), -2 ph (3), q_hi, q_mid, q_lo, 0 x 4
            uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
            float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
            if (base + r < P) {
                p = a.sg.points[off + base + r];
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
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (t == 0) {
            tc_mma_f16(tbase, adesc, bdesc, idesc, 0);
            tc_commit(mbar);
        }
        // every lane of a warp takes the same path (the tensor-memory loads are
        // warp-collective); the CTA agrees at the barrier below
        const bool done = __all_sync(0xffffffffu, mbar_wait(mbar, phase, WAIT_LIMIT));
        phase ^= 1u;
        tc_fence_after();
        if (done) {
#pragma unroll 1
            for (int ch = 0; ch < TC_POINTS / 32; ++ch) {
                float v[32];
                tmem_ld32(lane_addr + 32 * ch, v);
                float cm = v[0];
#pragma unroll
                for (int j = 1; j < 32; ++j) cm = fminf(cm, v[j]);
                if (cm <= thr) {
                    bapprox = fminf(bapprox, cm);
                    thr = bapprox + tau_of(bapprox, s2, sn);
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        if (v[j] <= thr) {
                            const float4 p = sP[32 * ch + j];
                            best = fminf(best, iso_dist2(__fsub_rn(s.x, p.x), __fsub_rn(s.y, p.y), __fsub_rn(s.z, p.z)));
                        }
                    }
                }
            }
        }
        tc_fence_before();
        ok = __syncthreads_and(done) != 0;
    }
    if (!ok && t == 0) atomicExch(a.error, 1);
    tc_fence_after();
    if (w == 0) tmem_dealloc(tbase, TC_COLS);
    if (ok && inside) a.fields[(size_t)seg * a.stride + idx] = iso_df_finish(best, P);
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
