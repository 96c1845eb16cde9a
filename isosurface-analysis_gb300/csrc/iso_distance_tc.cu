// iso_distance_tc.cu -- distance fields by brute force on the tensor cores
// (ISO_DF_TC): every sample against every surface point, recast as the
// contraction |s - p|^2 = |s|^2 + |p|^2 - 2 s.p, with an exact FP32 pass over
// the candidates it selects.  Same output as the other methods, bit for bit:
// sqrt of the minimum canonical squared distance (the brute-force comparator
// of isosurfaces_cuda/src/DistanceField.cu:49-65 and the nearest query of
// isosurfaces_cuda/src/BVH.cu:577-613).
//
// Operands, built once per surface (tc_prepare_kernel) and per CTA:
//  * B (one row of 16 f16 per point, in blocks of 128 rows laid out as the
//    MMA reads them, padding rows of each surface's last block marked):
//      [-2 ph (3), -2 pl (3), -2 ph (3), q_hi, q_mid, q_lo, 0 x 4]
//    with p = ph + pl split into f16 parts and q = |p|^2 (FP32) in three;
//  * A (one row per sample s of the CTA's 8 x 4 x 4 brick):
//      [sh (3), sh (3), sl (3), 1, 1, 1, 0 x 4]
//    so that A.B = |p|^2 - 2 s.p = |s - p|^2 - |s|^2 (the sl*pl products are
//    dropped).  One tcgen05.mma (M 128, N 128, K 16, f16 in, FP32 out) per
//    block of points writes a 128 x 128 tile to tensor memory.
//  * One warp streams the blocks: bulk copies (TMA) bring a block's B rows and
//    FP32 points into one of six shared-memory stages (four blocks in
//    flight), and one thread issues the block's MMA into one of two
//    accumulators once its copy has landed and the block two before it has
//    been read back.  Each CTA sweeps the blocks from the one holding the
//    first point at or beyond its brick's middle in x, wrapping around: with
//    points ordered by x the samples' running minima settle within the first
//    blocks, so the later blocks rarely hold a candidate to recheck.
//    Eight warps read the accumulators back (tcgen05.ld): warp w takes the 32
//    samples of TMEM lane quarter w % 4 and columns 64 (w / 4) .. +63, keeps
//    the smallest value B of its columns and recomputes the canonical FP32
//    distance of every point within tau of B; the two halves' minima are
//    merged at the end.
//  * Every barrier wait gives up after 2 s of the global timer.  A CTA whose
//    wait gave up waits (with the same limit) for its copies still in flight
//    and its last MMA, frees its tensor memory and raises the launch's error
//    flag, which the host returns as ISO_ERR_INTERNAL; iso_probe_wait_timeout
//    exercises the same wait on a barrier that nothing arrives at.
//
// Exactness: the canonical winner w (smallest canonical FP32 distance) is
// always a candidate: with e the error of A.B against the exact
// |s - p|^2 - |s|^2 and j the point giving B, A.B(w) - B <= |e(w)| + |e(j)|
// + the rounding of the canonical distances (<= 6e-7 of the squared
// distance).  |e| <= 12 * 2^-23 * (|s| + |p|)^2 (FP32 accumulation of 12 exact
// f16 products, allowing truncation) + 2^-20 (|s| + |p|)^2 (f16 split
// residuals and the dropped terms) + 5e-7 (f16 parts in the subnormal range);
// tau is twice the sum of two such bounds and the canonical rounding, for the
// largest |s| of the brick and |p| of the surface.  For coordinates in [0, 1]
// tau ~ 1.3e-4 in squared normalised units; any other point within tau is
// also rechecked, so a loose tau costs rechecks (a few dozen per sample),
// never exactness.
#include <cuda_fp16.h>

#include <vector>

#include "iso_internal.cuh"
#include "iso_tc.cuh"

using namespace isotc;

namespace {

constexpr int READ_WARPS = 8;                 // two per TMEM lane quarter
constexpr int TC_THREADS = 32 * (READ_WARPS + 1);
constexpr int TC_POINTS = 128;                // points per MMA (N), rows per B block
constexpr uint32_t TC_COLS = 256;             // two accumulators of TC_POINTS columns
constexpr int HALF = TC_POINTS / 2;           // columns read back per thread and block
constexpr int BLOCK_BYTES = TC_POINTS * 32;   // one B block (4 KB)
constexpr int BRICK_Z = 8, BRICK_Y = 4, BRICK_X = 4;
// shared memory: A tile, two B stages, two point stages, the halves' minima,
// barriers and the TMEM slot; padded so that at most two CTAs share an SM
// (2 x 256 TMEM columns = all 512)
constexpr int STAGES = 6;                             // operand stages (copies in flight: STAGES - 2)
constexpr int SM_A = 0;
constexpr int SM_B0 = 4096;
constexpr int SM_P0 = SM_B0 + STAGES * BLOCK_BYTES;        // 128 float4 per stage
constexpr int SM_BEST = SM_P0 + STAGES * TC_POINTS * 16;   // 128 floats
constexpr int SM_BAR = SM_BEST + 128 * 4;  // loaded[STAGES], consumed[STAGES], full[2], slot
constexpr int SM_USED = SM_BAR + (2 * STAGES + 2) * 8 + 16;
constexpr int SM_ALLOC = 80 * 1024;
constexpr float SENTINEL_Q = 30000.0f;        // |p|^2 of padding rows: never within tau
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // one barrier wait gives up after 2 s

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

// B rows of every surface in blocks of TC_POINTS (surface q's first block at
// block_base[q]); the largest |p| of each surface as float bits in pmax.
__global__ void tc_prepare_kernel(IsoSegments sg, const int64_t *block_base, int m, unsigned char *bops,
                                  uint32_t *pmax)
{
    const int q = blockIdx.y;
    const int64_t P = sg.count[q], padded = (P + TC_POINTS - 1) / TC_POINTS * TC_POINTS;
    unsigned char *dst = bops + (size_t)block_base[q] * BLOCK_BYTES;
    float mx = 0.0f;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < padded; r += (int64_t)gridDim.x * blockDim.x) {
        uint4 w0 = make_uint4(0u, 0u, 0u, 0u), w1 = w0;
        if (r < P) {
            const float4 p = sg.points[sg.offset[q] + r];
            __half hx, lx, hy, ly, hz, lz;
            split_f16(p.x, hx, lx);
            split_f16(p.y, hy, ly);
            split_f16(p.z, hz, lz);
            const __half m2 = __float2half_rn(-2.0f);
            hx = __hmul(m2, hx);
            hy = __hmul(m2, hy);
            hz = __hmul(m2, hz);
            lx = __hmul(m2, lx);
            ly = __hmul(m2, ly);
            lz = __hmul(m2, lz);
            const float qq = __fmaf_rn(p.z, p.z, __fmaf_rn(p.y, p.y, __fmul_rn(p.x, p.x)));
            const __half qh = __float2half_rn(qq);
            const float q1 = __fsub_rn(qq, __half2float(qh));
            const __half qm = __float2half_rn(q1);
            const __half ql = __float2half_rn(__fsub_rn(q1, __half2float(qm)));
            w0 = make_uint4(pack_h2(hx, hy), pack_h2(hz, lx), pack_h2(ly, lz), pack_h2(hx, hy));
            w1 = make_uint4(pack_h2(hz, qh), pack_h2(qm, ql), 0u, 0u);
            mx = fmaxf(mx, qq);
        } else {
            w1.x = pack_h2(__float2half_rn(0.0f), __float2half_rn(SENTINEL_Q));
        }
        unsigned char *blk = dst + (size_t)(r / TC_POINTS) * BLOCK_BYTES;
        const uint32_t row = (uint32_t)(r % TC_POINTS);
        *reinterpret_cast<uint4 *>(blk + tc_offset(row, 0)) = w0;
        *reinterpret_cast<uint4 *>(blk + tc_offset(row, 8)) = w1;
    }
    // |p|^2 >= 0: float bits order like values
    mx = sqrtf(mx);
    atomicMax(&pmax[q], __float_as_uint(mx));
}

struct TcArgs {
    IsoSampleGrid g;
    IsoSegments sg;
    const unsigned char *bops;    // prepared B blocks
    const int64_t *block_base;    // per segment: first B block
    const uint32_t *pmax;         // per segment: largest |p| (float bits)
    float *fields;
    int64_t stride;
    int bx, by, bz;  // bricks per axis
    int *error;
};

__global__ void __launch_bounds__(TC_THREADS, 2) df_tc_kernel(TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *sA = sm + SM_A;
    float *sBest = reinterpret_cast<float *>(sm + SM_BEST);
    uint64_t *loaded = reinterpret_cast<uint64_t *>(sm + SM_BAR);  // stage's copies landed
    uint64_t *consumed = loaded + STAGES;                            // stage's block read back
    uint64_t *full = consumed + STAGES;                              // accumulator's MMA done
    uint32_t *slot = reinterpret_cast<uint32_t *>(full + 2);
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    const int seg = blockIdx.y;
    const int64_t off = a.sg.offset[seg], P = a.sg.count[seg];
    const IsoSampleGrid &g = a.g;
    const int64_t X10 = g.F / (g.Y10 * g.Z10);

    // this thread's sample: warp w % 4 covers samples 32 (w % 4) .. + 31
    const int brick = blockIdx.x;
    const int bz = brick % a.bz, by = (brick / a.bz) % a.by, bxi = brick / (a.bz * a.by);
    const int ts = (32 * (w & 3) + lane) & 127;
    const int64_t z = (int64_t)bz * BRICK_Z + (ts & 7), y = (int64_t)by * BRICK_Y + ((ts >> 3) & 3),
                  x = (int64_t)bxi * BRICK_X + (ts >> 5);
    const bool inside = z < g.Z10 && y < g.Y10 && x < X10;
    const int64_t idx = inside ? (x * g.Y10 + y) * g.Z10 + z : 0;
    const float3 s = iso_sample_point(g, idx);
    if (w < 4) {
        __half hx, lx, hy, ly, hz, lz;
        split_f16(s.x, hx, lx);
        split_f16(s.y, hy, ly);
        split_f16(s.z, hz, lz);
        const __half one = __float2half_rn(1.0f);
        *reinterpret_cast<uint4 *>(sA + tc_offset(ts, 0)) =
            make_uint4(pack_h2(hx, hy), pack_h2(hz, hx), pack_h2(hy, hz), pack_h2(lx, ly));
        *reinterpret_cast<uint4 *>(sA + tc_offset(ts, 8)) = make_uint4(pack_h2(lz, one), pack_h2(one, one), 0u, 0u);
    }
    // tau from the largest |s| of the brick (its far corner from the origin)
    // and the surface's largest |p|
    float tau, corner_x;
    {
        const int64_t xc = clamp_hi((int64_t)bxi * BRICK_X + BRICK_X - 1, X10 - 1),
                      yc = clamp_hi((int64_t)by * BRICK_Y + BRICK_Y - 1, g.Y10 - 1),
                      zc = clamp_hi((int64_t)bz * BRICK_Z + BRICK_Z - 1, g.Z10 - 1);
        const float3 corner = iso_sample_point(g, (xc * g.Y10 + yc) * g.Z10 + zc);
        corner_x = corner.x;
        const float smax = sqrtf(corner.x * corner.x + corner.y * corner.y + corner.z * corner.z) * 1.0001f;
        const float R = smax + __uint_as_float(a.pmax[seg]) * 1.0001f;
        // twice (the error bound of two values plus the canonical rounding)
        tau = 2.0f * (2.0f * ((12.0f * 1.1920929e-7f + 9.5367432e-7f) * R * R + 5e-7f) + 6e-7f * R * R);
    }
    if (t == 0) {
        for (int k = 0; k < STAGES; ++k) {
            mbar_init(&loaded[k], 1);
            mbar_init(&consumed[k], READ_WARPS);
        }
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
    }
    if (w == 0) {
        tmem_alloc(slot, TC_COLS);
        tmem_relinquish();
    }
    const int nb = (int)((P + TC_POINTS - 1) / TC_POINTS);  // blocks of the surface (< 2^31, checked on the host)
    if (w == READ_WARPS && lane == 0) {
        // The sweep over the blocks starts at the block holding the first
        // point at or beyond the brick's middle in x and wraps around.  The
        // minimum does not depend on the order; starting near the brick
        // brings each sample's running minimum close to its final value
        // within the first blocks when the points are ordered by x (as
        // marching cubes emits them), so later blocks rarely hold a
        // candidate.  This lane's sample is the brick's first (ts = 0).
        const float sx = 0.5f * (s.x + corner_x);
        int64_t lo = 0, hi = P;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (a.sg.points[off + mid].x < sx) lo = mid + 1;
            else hi = mid;
        }
        const int64_t first = lo / TC_POINTS;
        slot[1] = (uint32_t)(first < nb ? first : (nb > 0 ? nb - 1 : 0));
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = slot[0];
    const int start = (int)slot[1];
    const unsigned char *bsrc = a.bops + (size_t)a.block_base[seg] * BLOCK_BYTES;
    bool ok = true;

    if (w == READ_WARPS) {
        // the streaming warp: one thread copies blocks and issues the MMAs
        if (lane == 0) {
            const uint64_t adesc = tc_desc(sA);
            const uint32_t idesc = tc_idesc_f16_f32(128, TC_POINTS);
            // sweep position i holds block (start + i) mod nb, in stage
            // i mod STAGES (phase (i / STAGES) & 1) and accumulator i & 1
            int fetched = 0, landed = 0, issued = 0;  // positions copied, waited for, contracted
            auto fetch = [&](int i, int st) {
                ++fetched;
                int blk = start + i;
                if (blk >= nb) blk -= nb;
                const int64_t rest = P - (int64_t)blk * TC_POINTS;
                const int64_t cnt = rest < TC_POINTS ? rest : TC_POINTS;
                mbar_expect_tx(&loaded[st], (uint32_t)(BLOCK_BYTES + cnt * 16));
                bulk_g2s(sm + SM_B0 + st * BLOCK_BYTES, bsrc + (size_t)blk * BLOCK_BYTES, BLOCK_BYTES, &loaded[st]);
                bulk_g2s(sm + SM_P0 + st * TC_POINTS * 16, a.sg.points + off + (int64_t)blk * TC_POINTS,
                         (uint32_t)(cnt * 16), &loaded[st]);
            };
            for (int i = 0; i < STAGES && i < nb; ++i) fetch(i, i);
            int st = 0;
            uint32_t ph = 0;
            for (int i = 0; i < nb && ok; ++i) {
                ok = mbar_wait(&loaded[st], ph, WAIT_LIMIT_NS);
                if (!ok) break;
                ++landed;
                if (i >= 2) {
                    // position i - 2 read back: its accumulator (i % 2) and
                    // its stage are free; the stage takes position
                    // i - 2 + STAGES
                    const int sd = st >= 2 ? st - 2 : st + STAGES - 2;
                    ok = mbar_wait(&consumed[sd], st >= 2 ? ph : ph ^ 1u, WAIT_LIMIT_NS);
                    if (!ok) break;
                    if (i - 2 + STAGES < nb) fetch(i - 2 + STAGES, sd);
                }
                tc_fence_after();
                tc_mma_f16(tbase + (uint32_t)(i & 1) * TC_POINTS, adesc, tc_desc(sm + SM_B0 + st * BLOCK_BYTES), idesc,
                           0);
                tc_commit(&full[i & 1]);
                ++issued;
                if (++st == STAGES) {
                    st = 0;
                    ph ^= 1u;
                }
            }
            if (!ok) {
                // before the CTA gives its shared and tensor memory back: the
                // copies still in flight and the last MMA, each with a limit
                for (int q = landed; q < fetched; ++q)
                    mbar_wait(&loaded[q % STAGES], (uint32_t)((q / STAGES) & 1), WAIT_LIMIT_NS);
                if (issued > 0) mbar_wait(&full[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1), WAIT_LIMIT_NS);
            }
        }
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    } else {
        float best = ISO_DF_INIT_BOUND;  // exact canonical minimum over this thread's columns
        float bapprox = __int_as_float(0x7f800000), thr = bapprox;
        const int col0 = HALF * (w >> 2);
        const uint32_t lane_addr = tbase + ((uint32_t)(32 * (w & 3)) << 16) + col0;
        int st = 0, blk = start;
        for (int i = 0; i < nb; ++i) {
            const int acc = i & 1;
            ok = __all_sync(0xffffffffu, mbar_wait(&full[acc], (uint32_t)((i >> 1) & 1), WAIT_LIMIT_NS));
            if (!ok) break;
            tc_fence_after();
            uint32_t r[HALF];
            tmem_ld32_async(lane_addr + acc * TC_POINTS, r);
            tmem_ld32_async(lane_addr + acc * TC_POINTS + 32, r + 32);
            tmem_wait_ld64(r);
            float mm[22];
#pragma unroll
            for (int k = 0; k < 21; ++k)
                mm[k] = fmin3(__uint_as_float(r[3 * k]), __uint_as_float(r[3 * k + 1]), __uint_as_float(r[3 * k + 2]));
            mm[21] = __uint_as_float(r[63]);
#pragma unroll
            for (int k = 0; k < 7; ++k) mm[k] = fmin3(mm[3 * k], mm[3 * k + 1], mm[3 * k + 2]);
            const float cm = fminf(fmin3(fmin3(mm[0], mm[1], mm[2]), fmin3(mm[3], mm[4], mm[5]), mm[6]), mm[21]);
            if (cm <= thr) {
                bapprox = fminf(bapprox, cm);
                thr = bapprox + tau;
                const float4 *sP = reinterpret_cast<const float4 *>(sm + SM_P0) + st * TC_POINTS + col0;
                // padding rows of the last block have no point behind them
                const int64_t valid = P - (int64_t)blk * TC_POINTS - col0;
#pragma unroll
                for (int j = 0; j < HALF; ++j) {
                    if (__uint_as_float(r[j]) <= thr && j < valid) {
                        const float4 p = sP[j];
                        best = fminf(best, iso_dist2(__fsub_rn(s.x, p.x), __fsub_rn(s.y, p.y), __fsub_rn(s.z, p.z)));
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&consumed[st]);
            if (++st == STAGES) st = 0;
            if (++blk == nb) blk = 0;
        }
        if (w >= 4) sBest[ts] = best;
        named_bar(1, 32 * READ_WARPS);
        if (w < 4 && ok && inside)
            a.fields[(size_t)seg * a.stride + idx] = iso_df_finish(fminf(best, sBest[ts]), P);
    }
    if (!ok && lane == 0) atomicExch(a.error, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (w == 0) tmem_dealloc(tbase, TC_COLS);
}

// Failure-detection probe: the kernels' bounded barrier wait on a barrier
// that one thread arrives at first (arrive != 0) or that nothing arrives at;
// the wait gives up after limit_ns and the kernel returns normally.
__global__ void wait_probe_kernel(int arrive, uint64_t limit_ns, int *timed_out)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (arrive && threadIdx.x == 0) mbar_arrive(&bar);
    __syncthreads();
    const bool ok = __all_sync(0xffffffffu, mbar_wait(&bar, 0, limit_ns));
    if (threadIdx.x == 0) *timed_out = ok ? 0 : 1;
}

}  // namespace

extern "C" int iso_probe_wait_timeout(iso_ctx *ctx, int arrive, int64_t limit_ns, int *timed_out)
{
    iso_clear_error();
    if (!ctx || !timed_out || limit_ns < 0 || limit_ns > 10000000000ll)
        return iso_fail(ISO_ERR_ARG, "iso_probe_wait_timeout: limit_ns must be in [0, 1e10]");
    ISO_CUDA(cudaSetDevice(ctx->device));
    void *d;
    ISO_TRY(iso_buf(ctx, BUF_MISC, 256, &d));
    int *flag = (int *)d;
    ISO_CUDA(cudaMemsetAsync(flag, 0xff, sizeof(int), ctx->stream));
    wait_probe_kernel<<<1, 32, 0, ctx->stream>>>(arrive, (uint64_t)limit_ns, flag);
    ISO_LAUNCHED(ctx);
    int h = -1;
    ISO_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h != 0 && h != 1) return iso_fail(ISO_ERR_INTERNAL, "iso_probe_wait_timeout: the probe did not report");
    *timed_out = h;
    return ISO_OK;
}

int iso_run_distance_tc(iso_ctx *ctx, const IsoSampleGrid &g, const IsoSegments &sg, const int64_t *h_seg_count, int m,
                        float *fields, int64_t stride)
{
    static_assert(SM_USED <= SM_ALLOC, "shared memory layout");
    const int64_t X10 = g.F / (g.Y10 * g.Z10);
    // prepared B blocks of every surface
    std::vector<int64_t> base((size_t)m + 1, 0);
    for (int q = 0; q < m; ++q) {
        const int64_t nb = (h_seg_count[q] + TC_POINTS - 1) / TC_POINTS;
        if (nb > 0x7fffffff) return iso_fail(ISO_ERR_ARG, "tensor-core distance: more than 2^31 point blocks");
        base[q + 1] = base[q] + nb;
    }
    void *d_bops, *d_base, *d_pmax, *d_err;
    ISO_TRY(iso_buf(ctx, BUF_TC_OPERANDS, (size_t)base[m] * BLOCK_BYTES, &d_bops));
    ISO_TRY(iso_buf(ctx, BUF_STAGING_A, (size_t)(m + 1) * sizeof(int64_t) + (size_t)m * sizeof(uint32_t) + 256,
                    &d_base));
    d_pmax = (char *)d_base + ((size_t)(m + 1) * sizeof(int64_t) + 255) / 256 * 256;
    ISO_CUDA(cudaMemcpyAsync(d_base, base.data(), (size_t)(m + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                             ctx->stream));
    ISO_CUDA(cudaMemsetAsync(d_pmax, 0, (size_t)m * sizeof(uint32_t), ctx->stream));
    ISO_TRY(iso_buf(ctx, BUF_TASK_COUNTER, 256, &d_err));
    int *err_flag = (int *)d_err + 2;
    ISO_CUDA(cudaMemsetAsync(err_flag, 0, sizeof(int), ctx->stream));
    ISO_CUDA(cudaFuncSetAttribute(df_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_ALLOC));
    TcArgs a;
    a.g = g;
    a.stride = stride;
    a.bz = (int)((g.Z10 + BRICK_Z - 1) / BRICK_Z);
    a.by = (int)((g.Y10 + BRICK_Y - 1) / BRICK_Y);
    a.bx = (int)((X10 + BRICK_X - 1) / BRICK_X);
    a.error = err_flag;
    const int64_t bricks = (int64_t)a.bx * a.by * a.bz;
    if (bricks > 0x7fffffff) return iso_fail(ISO_ERR_ARG, "tensor-core distance: grid too large");
    for (int q0 = 0; q0 < m; q0 += 65535) {
        const int cnt = m - q0 < 65535 ? m - q0 : 65535;
        IsoSegments s2 = sg;
        s2.offset = sg.offset + q0;
        s2.count = sg.count + q0;
        tc_prepare_kernel<<<dim3(64, cnt), 256, 0, ctx->stream>>>(s2, (const int64_t *)d_base + q0, cnt,
                                                                  (unsigned char *)d_bops, (uint32_t *)d_pmax + q0);
        ISO_LAUNCHED(ctx);
        a.sg = s2;
        a.bops = (const unsigned char *)d_bops;
        a.block_base = (const int64_t *)d_base + q0;
        a.pmax = (const uint32_t *)d_pmax + q0;
        a.fields = fields + (size_t)q0 * stride;
        df_tc_kernel<<<dim3((unsigned)bricks, cnt), TC_THREADS, SM_ALLOC, ctx->stream>>>(a);
        ISO_LAUNCHED(ctx);
    }
    int err = 0;
    ISO_CUDA(cudaMemcpyAsync(&err, err_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (err) return iso_fail(ISO_ERR_INTERNAL, "tensor-core distance: a copy or an MMA did not complete");
    return ISO_OK;
}
