// iso_multi.cu -- batched cross maps over many volumes and their aggregation
// into timestep / variable similarity matrices.
//
// The reference computes one 16 x 16 cross map per (volume, volume) pair, each
// through its own calculate_histogram_h call with host staging
// (runtime/src/MultiVar.cpp:170-249).  Here the representative fields of all
// volumes sit in one device matrix and every requested field pair of every
// volume pair runs in one launch of the joint-histogram kernel.  The reference
// stops at the cross maps; the block aggregation below turns each 16 x 16 block
// into one similarity per volume pair (the inputs of a TSM/VSM).
#include <vector>

#include "iso_internal.cuh"

namespace {

int64_t round_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// One block (A, B) of the pair map: rows A*k.., columns B*k.. (k x k).
// out[2q]   = mean of the block,
// out[2q+1] = best-match score: (mean over rows of the row maximum + mean over
//             columns of the column maximum) / 2.
__global__ void block_similarity_kernel(const float *map, int64_t R, int k, const int2 *blocks, int64_t nb, float *out)
{
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (q >= nb) return;
    const int lane = threadIdx.x & 31;
    const int2 bl = blocks[q];
    const int64_t r0 = (int64_t)bl.x * k, c0 = (int64_t)bl.y * k;
    float sum = 0.0f, rowmax_sum = 0.0f, colmax_sum = 0.0f;
    for (int i = lane; i < k; i += 32) {
        float rmax = -1e30f, cmax = -1e30f;
        for (int j = 0; j < k; ++j) {
            const float v = map[(r0 + i) * R + c0 + j];
            const float w = map[(r0 + j) * R + c0 + i];
            sum += v;
            rmax = fmaxf(rmax, v);
            cmax = fmaxf(cmax, w);
        }
        rowmax_sum += rmax;
        colmax_sum += cmax;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        rowmax_sum += __shfl_xor_sync(0xffffffffu, rowmax_sum, o);
        colmax_sum += __shfl_xor_sync(0xffffffffu, colmax_sum, o);
    }
    if (lane == 0) {
        out[2 * q] = sum / (float)(k * k);
        out[2 * q + 1] = 0.5f * (rowmax_sum + colmax_sum) / (float)k;
    }
}

}  // namespace

extern "C" int iso_pair_map(iso_ctx *ctx, const float *fields, int R, int64_t n, int64_t stride, int bins,
                            const int32_t *pairs, int64_t npairs, float *out)
{
    iso_clear_error();
    if (!ctx || !fields || !pairs || !out || R <= 0 || n <= 0 || npairs < 0 || stride < n)
        return iso_fail(ISO_ERR_ARG, "iso_pair_map: bad argument");
    ISO_CUDA(cudaSetDevice(ctx->device));
    ctx->last_m = 0;
    std::vector<int2> tasks((size_t)npairs);
    for (int64_t t = 0; t < npairs; ++t) {
        const int a = pairs[2 * t], b = pairs[2 * t + 1];
        if (a < 0 || b < 0 || a >= R || b >= R) return iso_fail(ISO_ERR_ARG, "iso_pair_map: pair %lld out of range", (long long)t);
        tasks[t] = make_int2(a, b);
    }
    // fields are used in place when they are aligned device rows, else staged
    const float *d_fields = fields;
    int64_t st = stride;
    if (!iso_is_device_ptr(fields) || stride % 4 != 0 || ((uintptr_t)fields & 15)) {
        st = round_up(n, 64);
        void *d;
        ISO_TRY(iso_buf(ctx, BUF_FIELDS, (size_t)R * st * sizeof(float), &d));
        ISO_CUDA(cudaMemcpy2DAsync(d, st * sizeof(float), fields, stride * sizeof(float), n * sizeof(float), R,
                                   cudaMemcpyDefault, ctx->stream));
        d_fields = (const float *)d;
    }
    void *d_mm, *d_map;
    ISO_TRY(iso_buf(ctx, BUF_FIELD_MINMAX, (size_t)2 * R * sizeof(uint32_t), &d_mm));
    const bool out_dev = iso_is_device_ptr(out);
    float *d_out = out;
    if (!out_dev) {
        ISO_TRY(iso_buf(ctx, BUF_ISM, (size_t)R * R * sizeof(float), &d_map));
        d_out = (float *)d_map;
    }
    ISO_TRY(iso_run_minmax(ctx, d_fields, R, n, st, (uint32_t *)d_mm));
    ISO_TRY(iso_run_similarity_tasks(ctx, d_fields, d_fields, R, n, st, bins, (const uint32_t *)d_mm,
                                     (const uint32_t *)d_mm, d_out, tasks.data(), npairs, true, nullptr, nullptr));
    if (!out_dev)
        ISO_CUDA(cudaMemcpyAsync(out, d_out, (size_t)R * R * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

extern "C" int iso_block_similarity(iso_ctx *ctx, const float *map, int64_t R, int k, const int32_t *blocks,
                                    int64_t nblocks, float *out)
{
    iso_clear_error();
    if (!ctx || !map || !blocks || !out || R <= 0 || k <= 0 || nblocks < 0)
        return iso_fail(ISO_ERR_ARG, "iso_block_similarity: bad argument");
    if (nblocks == 0) return ISO_OK;
    ISO_CUDA(cudaSetDevice(ctx->device));
    const float *d_map = map;
    if (!iso_is_device_ptr(map)) {
        void *d;
        ISO_TRY(iso_buf(ctx, BUF_ISM, (size_t)R * R * sizeof(float), &d));
        ISO_CUDA(cudaMemcpyAsync(d, map, (size_t)R * R * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        d_map = (const float *)d;
    }
    void *d_blocks, *d_out;
    ISO_TRY(iso_buf(ctx, BUF_PAIR_TASKS, (size_t)nblocks * sizeof(int2), &d_blocks));
    ISO_TRY(iso_buf(ctx, BUF_STAGING_B, (size_t)nblocks * 2 * sizeof(float), &d_out));
    ISO_CUDA(cudaMemcpyAsync(d_blocks, blocks, (size_t)nblocks * sizeof(int2), cudaMemcpyDefault, ctx->stream));
    const int warps = 8;
    block_similarity_kernel<<<(unsigned)((nblocks + warps - 1) / warps), warps * 32, 0, ctx->stream>>>(
        d_map, R, k, (const int2 *)d_blocks, nblocks, (float *)d_out);
    ISO_LAUNCHED(ctx);
    ISO_CUDA(cudaMemcpyAsync(out, d_out, (size_t)nblocks * 2 * sizeof(float), cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}
