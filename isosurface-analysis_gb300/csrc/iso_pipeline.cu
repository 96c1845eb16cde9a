// iso_pipeline.cu -- the public C ABI: the whole-volume pipeline, stage entry
// points, isovalue selection and the reference-named drop-in functions.
#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "iso_internal.cuh"

namespace {

int64_t round_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// Makes `volume` (host or device) available on the device.
int device_volume(iso_ctx *ctx, const float *volume, int64_t V, const float **out)
{
    if (iso_is_device_ptr(volume)) {
        *out = volume;
        return ISO_OK;
    }
    void *d;
    ISO_TRY(iso_buf(ctx, BUF_VOLUME, (size_t)V * sizeof(float), &d));
    ISO_CUDA(cudaMemcpyAsync(d, volume, (size_t)V * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    *out = (const float *)d;
    return ISO_OK;
}

__global__ void repack_xyz_kernel(const float *xyz, float4 *out, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.0f);
}

__global__ void bits_kernel(const float *mins, const float *maxs, uint32_t *mm, int m)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m) {
        mm[2 * f] = __float_as_uint(mins[f]);
        mm[2 * f + 1] = __float_as_uint(maxs[f]);
    }
}

// Real range of types/src/Isosurface.cpp:48-75: max of {-100000} and values <=
// cfg_max, min of {100000} and values >= cfg_min.  Result as float bits with a
// sign-aware order key so atomicMin/atomicMax on uint32 work for any sign.
__device__ __forceinline__ uint32_t order_key(float f)
{
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ __forceinline__ float from_order_key(uint32_t k)
{
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
}

__global__ void real_range_kernel(const float *vol, int64_t V, float cmin, float cmax, uint32_t *out)
{
    float mn = 100000.0f, mx = -100000.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < V; i += (int64_t)gridDim.x * blockDim.x) {
        float v = vol[i];
        if (v > mx && v <= cmax) mx = v;
        if (v < mn && v >= cmin) mn = v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&out[0], order_key(mn));
        atomicMax(&out[1], order_key(mx));
    }
}

// 65536-bin histogram of runtime/src/Single.cpp:350-359:
// index = int((65536 * (v - gmin)) * oneover), clamped to [0, 65535].
__global__ void uniform_hist_kernel(const float *vol, int64_t count, float gmin, float oneover, unsigned int *hist)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        float scaled = __fmul_rn(65536.0f, __fsub_rn(vol[i], gmin));
        float q = __fmul_rn(scaled, oneover);
        int index;
        if (q != q) index = (int)0x80000000;  // x86/C conversion of NaN; clamps to 0 below
        else if (q >= 2147483648.0f) index = 0x7fffffff;
        else if (q < -2147483648.0f) index = (int)0x80000000;
        else index = __float2int_rz(q);
        if (index > 65535) index = 65535;
        if (index < 0) index = 0;
        atomicAdd(&hist[index], 1u);
    }
}

// dst[x*Y*Z + y*Z + z] = src[x + y*X + z*X*Y], through a 32x32 shared tile over
// the (x, z) plane of each y slice so both sides are coalesced.
__global__ void transpose_xz_kernel(const float *src, float *dst, int X, int Y, int Z)
{
    __shared__ float tile[32][33];
    const int y = blockIdx.z;
    const int x0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int x = x0 + threadIdx.x, z = z0 + k;
        if (x < X && z < Z) tile[k][threadIdx.x] = src[(size_t)x + (size_t)y * X + (size_t)z * X * Y];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int z = z0 + threadIdx.x, x = x0 + k;
        if (x < X && z < Z) dst[(size_t)x * Y * Z + (size_t)y * Z + z] = tile[threadIdx.x][k];
    }
}

void sort_points_host(std::vector<float> &xyz)
{
    const size_t n = xyz.size() / 3;
    std::vector<size_t> idx(n);
    for (size_t i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
        for (int d = 0; d < 3; ++d) {
            float p = xyz[3 * a + d], q = xyz[3 * b + d];
            if (p < q) return true;
            if (p > q) return false;
        }
        return false;
    });
    std::vector<float> out(xyz.size());
    for (size_t i = 0; i < n; ++i) memcpy(&out[3 * i], &xyz[3 * idx[i]], 3 * sizeof(float));
    xyz.swap(out);
}

}  // namespace

// ---------------------------------------------------------------------------
// whole-volume pipeline
// ---------------------------------------------------------------------------

extern "C" int iso_ism(iso_ctx *ctx, const float *volume, int X, int Y, int Z, const float *isovalues, int n,
                       const iso_opts *opts, float *ism_out, int32_t *field_ids_out, int32_t *m_out,
                       iso_surface_stats *stats_out, iso_timing *timing_out)
{
    iso_clear_error();
    if (!ctx || !volume || !isovalues || !opts || !ism_out || !field_ids_out || !m_out)
        return iso_fail(ISO_ERR_ARG, "iso_ism: NULL argument");
    if (opts->bins < 2 || opts->bins > ISO_MAX_BINS || (opts->bins & 1))
        return iso_fail(ISO_ERR_ARG, "iso_ism: bins must be even and in [2, %d]", ISO_MAX_BINS);
    ISO_CUDA(cudaSetDevice(ctx->device));
    const int64_t V = (int64_t)X * Y * Z;
    cudaEvent_t ev[4];
    for (auto &e : ev) ISO_CUDA(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() { for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]); }
    } guard{ev};
    ISO_CUDA(cudaEventRecord(ev[0], ctx->stream));
    const bool dev_vol = iso_is_device_ptr(volume);
    const float *d_vol;
    ISO_TRY(device_volume(ctx, volume, V, &d_vol));
    {
        const int ds0 = opts->df_downscale < 1 ? 1 : opts->df_downscale;
        ctx->plan_V = V;
        ctx->plan_stride = round_up((int64_t)(X / ds0) * (Y / ds0) * (Z / ds0), 64);
        ctx->plan_bins = opts->bins;
        ctx->plan_lbvh = opts->df_method == ISO_DF_LBVH;
        ctx->plan_volume_copy = dev_vol ? 0 : 1;
    }

    std::vector<int64_t> counts(n), offsets(n);
    std::vector<iso_surface_stats> stats(n);
    int64_t total_pts = 0;
    ISO_TRY(iso_run_surfaces(ctx, d_vol, X, Y, Z, isovalues, n, opts->surface, opts->frame, counts.data(),
                             offsets.data(), stats.data(), &total_pts));
    ISO_CUDA(cudaEventRecord(ev[1], ctx->stream));

    std::vector<int32_t> ids;
    std::vector<int64_t> seg_off, seg_cnt;
    for (int k = 0; k < n; ++k)
        if (counts[k] > 0) {
            ids.push_back(k);
            seg_off.push_back(offsets[k]);
            seg_cnt.push_back(counts[k]);
        }
    const int m = (int)ids.size();
    const int ds = opts->df_downscale < 1 ? 1 : opts->df_downscale;
    const int64_t F = (int64_t)(X / ds) * (Y / ds) * (Z / ds);
    const int64_t stride = round_up(F, 64);
    if (m > 0)
        ISO_TRY(iso_run_distance(ctx, X, Y, Z, ds, opts->df_method, ids.data(), m, seg_off.data(), seg_cnt.data(),
                                 stride));
    ISO_CUDA(cudaEventRecord(ev[2], ctx->stream));
    if (m > 0) {
        void *d_ism;
        ISO_TRY(iso_buf(ctx, BUF_ISM, (size_t)m * m * sizeof(float), &d_ism));
        ISO_TRY(iso_run_similarity(ctx, (const float *)ctx->buf[BUF_FIELDS], nullptr, m, F, stride, opts->bins,
                                   (const uint32_t *)ctx->buf[BUF_FIELD_MINMAX], nullptr, (float *)d_ism, nullptr,
                                   nullptr));
        ISO_CUDA(cudaMemcpyAsync(ism_out, d_ism, (size_t)m * m * sizeof(float), cudaMemcpyDefault, ctx->stream));
    }
    ISO_CUDA(cudaEventRecord(ev[3], ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    ISO_CUDA(cudaMemcpy(field_ids_out, ids.data(), (size_t)m * sizeof(int32_t), cudaMemcpyDefault));
    *m_out = m;
    ctx->last_m = m;
    ctx->last_F = F;
    ctx->last_stride = stride;
    if (stats_out) memcpy(stats_out, stats.data(), (size_t)n * sizeof(iso_surface_stats));
    if (timing_out) {
        cudaEventElapsedTime(&timing_out->surface_ms, ev[0], ev[1]);
        cudaEventElapsedTime(&timing_out->distance_ms, ev[1], ev[2]);
        cudaEventElapsedTime(&timing_out->histogram_ms, ev[2], ev[3]);
        cudaEventElapsedTime(&timing_out->total_ms, ev[0], ev[3]);
    }
    return ISO_OK;
}

extern "C" int iso_cross_map(iso_ctx *ctx, const float *fields_a, const float *fields_b, int m, int64_t n, int bins,
                             float *out)
{
    iso_clear_error();
    if (!ctx || !fields_a || !fields_b || !out || m <= 0 || n <= 0) return iso_fail(ISO_ERR_ARG, "iso_cross_map: bad argument");
    ISO_CUDA(cudaSetDevice(ctx->device));
    ctx->last_m = 0;
    const int64_t stride = round_up(n, 64);
    void *d_fields, *d_mm, *d_ism;
    ISO_TRY(iso_buf(ctx, BUF_FIELDS, (size_t)2 * m * stride * sizeof(float), &d_fields));
    ISO_TRY(iso_buf(ctx, BUF_FIELD_MINMAX, (size_t)4 * m * sizeof(uint32_t), &d_mm));
    ISO_TRY(iso_buf(ctx, BUF_ISM, (size_t)m * m * sizeof(float), &d_ism));
    float *f = (float *)d_fields;
    ISO_CUDA(cudaMemcpy2DAsync(f, stride * sizeof(float), fields_a, n * sizeof(float), n * sizeof(float), m,
                               cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaMemcpy2DAsync(f + (size_t)m * stride, stride * sizeof(float), fields_b, n * sizeof(float),
                               n * sizeof(float), m, cudaMemcpyDefault, ctx->stream));
    ISO_TRY(iso_run_minmax(ctx, f, 2 * m, n, stride, (uint32_t *)d_mm));
    ISO_TRY(iso_run_similarity(ctx, f, f + (size_t)m * stride, m, n, stride, bins, (const uint32_t *)d_mm,
                               (const uint32_t *)d_mm + 2 * m, (float *)d_ism, nullptr, nullptr));
    ISO_CUDA(cudaMemcpyAsync(out, d_ism, (size_t)m * m * sizeof(float), cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

// ---------------------------------------------------------------------------
// stage entry points
// ---------------------------------------------------------------------------

extern "C" int iso_surface_points(iso_ctx *ctx, const float *volume, int X, int Y, int Z, const float *isovalues,
                                  int n, int surface, int frame, int64_t *counts_out, float *points_out,
                                  int64_t cap_points, iso_surface_stats *stats_out)
{
    iso_clear_error();
    if (!ctx || !volume || !isovalues || !counts_out) return iso_fail(ISO_ERR_ARG, "iso_surface_points: NULL argument");
    ISO_CUDA(cudaSetDevice(ctx->device));
    const float *d_vol;
    ISO_TRY(device_volume(ctx, volume, (int64_t)X * Y * Z, &d_vol));
    std::vector<int64_t> offsets(n);
    std::vector<iso_surface_stats> stats(n);
    int64_t total = 0;
    ISO_TRY(iso_run_surfaces(ctx, d_vol, X, Y, Z, isovalues, n, surface, frame, counts_out, offsets.data(),
                             stats.data(), &total));
    if (stats_out) memcpy(stats_out, stats.data(), (size_t)n * sizeof(iso_surface_stats));
    int64_t sum = 0;
    for (int k = 0; k < n; ++k) sum += counts_out[k];
    if (!points_out) {
        ISO_CUDA(cudaStreamSynchronize(ctx->stream));
        return ISO_OK;
    }
    if (cap_points < sum) return iso_fail(ISO_ERR_CAPACITY, "iso_surface_points: need %lld points", (long long)sum);
    std::vector<float4> raw(total > 0 ? total : 1);
    if (total > 0)
        ISO_CUDA(cudaMemcpyAsync(raw.data(), ctx->buf[BUF_POINTS_RAW], (size_t)total * sizeof(float4),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<float> all;
    all.reserve((size_t)sum * 3);
    for (int k = 0; k < n; ++k) {
        std::vector<float> xyz((size_t)counts_out[k] * 3);
        for (int64_t i = 0; i < counts_out[k]; ++i) {
            float4 p = raw[offsets[k] + i];
            xyz[3 * i] = p.x;
            xyz[3 * i + 1] = p.y;
            xyz[3 * i + 2] = p.z;
        }
        sort_points_host(xyz);  // lexicographic == linear cell order for integer cells
        all.insert(all.end(), xyz.begin(), xyz.end());
    }
    if (sum > 0) ISO_CUDA(cudaMemcpy(points_out, all.data(), (size_t)sum * 3 * sizeof(float), cudaMemcpyDefault));
    return ISO_OK;
}

extern "C" int iso_distance_field(iso_ctx *ctx, const float *points, int64_t P, int X, int Y, int Z, int downscale,
                                  int method, float *out)
{
    iso_clear_error();
    if (!ctx || !points || !out || P < 1) return iso_fail(ISO_ERR_ARG, "iso_distance_field: bad argument");
    ISO_CUDA(cudaSetDevice(ctx->device));
    ctx->last_m = 0;
    const int ds = downscale < 1 ? 1 : downscale;
    void *d_xyz, *d_norm;
    ISO_TRY(iso_buf(ctx, BUF_STAGING_A, (size_t)P * 3 * sizeof(float), &d_xyz));
    ISO_TRY(iso_buf(ctx, BUF_POINTS_NORM, (size_t)P * sizeof(float4), &d_norm));
    ISO_CUDA(cudaMemcpyAsync(d_xyz, points, (size_t)P * 3 * sizeof(float), cudaMemcpyDefault, ctx->stream));
    repack_xyz_kernel<<<(unsigned)((P + 255) / 256), 256, 0, ctx->stream>>>((const float *)d_xyz, (float4 *)d_norm, P);
    ISO_LAUNCHED(ctx);
    const int64_t F = (int64_t)(X / ds) * (Y / ds) * (Z / ds);
    const int64_t off = 0;
    const int32_t id = 0;
    ISO_TRY(iso_run_distance(ctx, X, Y, Z, ds, method, &id, 1, &off, &P, round_up(F, 64)));
    ISO_CUDA(cudaMemcpyAsync(out, ctx->buf[BUF_FIELDS], (size_t)F * sizeof(float), cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

static int similarity_impl(iso_ctx *ctx, const float *const *field_ptrs, const float *fields, int m, int64_t n,
                           int bins, const float *mins, const float *maxs, float *ism_out, int64_t ism_ld,
                           uint32_t *joint_out, uint32_t *col_out, uint32_t *row_out, bool multi)
{
    ISO_CUDA(cudaSetDevice(ctx->device));
    ctx->last_m = 0;  // the field matrix is reused below
    const int nf = multi ? 2 * m : m;
    const int64_t stride = round_up(n, 64);
    void *d_fields, *d_mm, *d_ism;
    ISO_TRY(iso_buf(ctx, BUF_FIELDS, (size_t)nf * stride * sizeof(float), &d_fields));
    ISO_TRY(iso_buf(ctx, BUF_FIELD_MINMAX, (size_t)2 * nf * sizeof(uint32_t), &d_mm));
    ISO_TRY(iso_buf(ctx, BUF_ISM, (size_t)m * m * sizeof(float), &d_ism));
    float *f = (float *)d_fields;
    bool clamp_top = false;  // a caller's interval leaves values above its maximum
    if (field_ptrs) {
        for (int k = 0; k < nf; ++k)
            ISO_CUDA(cudaMemcpyAsync(f + (size_t)k * stride, field_ptrs[k], (size_t)n * sizeof(float), cudaMemcpyDefault,
                                     ctx->stream));
    } else {
        ISO_CUDA(cudaMemcpy2DAsync(f, stride * sizeof(float), fields, n * sizeof(float), n * sizeof(float), nf,
                                   cudaMemcpyDefault, ctx->stream));
    }
    if (mins && maxs) {
        // caller-supplied intervals (the reference's getInterval values): a
        // value above its field's maximum counts in the last bucket, as the
        // reference clamps it (JointHistogram.cu:74); a value below the
        // minimum is refused, since the reference would index below its
        // histogram there (JointHistogram.cu:69-73)
        ISO_TRY(iso_run_minmax(ctx, f, nf, n, stride, (uint32_t *)d_mm));
        std::vector<uint32_t> mm((size_t)2 * nf);
        std::vector<float> hmin(nf), hmax(nf);
        ISO_CUDA(cudaMemcpyAsync(mm.data(), d_mm, mm.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        ISO_CUDA(cudaMemcpy(hmin.data(), mins, nf * sizeof(float), cudaMemcpyDefault));
        ISO_CUDA(cudaMemcpy(hmax.data(), maxs, nf * sizeof(float), cudaMemcpyDefault));
        ISO_CUDA(cudaStreamSynchronize(ctx->stream));
        clamp_top = false;
        for (int k = 0; k < nf; ++k) {
            float lo, hi;
            memcpy(&lo, &mm[2 * k], sizeof lo);
            memcpy(&hi, &mm[2 * k + 1], sizeof hi);
            if (!(hmin[k] <= lo) || !(hmax[k] >= hmin[k]))
                return iso_fail(ISO_ERR_ARG, "field %d: interval [%g, %g] is empty or above its smallest value %g", k,
                                hmin[k], hmax[k], lo);
            if (hi > hmax[k]) clamp_top = true;
        }
        void *d_tmp;
        ISO_TRY(iso_buf(ctx, BUF_STAGING_B, (size_t)2 * nf * sizeof(float), &d_tmp));
        float *t = (float *)d_tmp;
        ISO_CUDA(cudaMemcpyAsync(t, mins, nf * sizeof(float), cudaMemcpyDefault, ctx->stream));
        ISO_CUDA(cudaMemcpyAsync(t + nf, maxs, nf * sizeof(float), cudaMemcpyDefault, ctx->stream));
        bits_kernel<<<(nf + 255) / 256, 256, 0, ctx->stream>>>(t, t + nf, (uint32_t *)d_mm, nf);
        ISO_LAUNCHED(ctx);
    } else {
        ISO_TRY(iso_run_minmax(ctx, f, nf, n, stride, (uint32_t *)d_mm));
    }
    uint32_t *d_joint = nullptr, *d_cr = nullptr;
    struct ClampScope {  // the histogram kernels clamp only for this call
        iso_ctx *c;
        ~ClampScope() { c->hist_clamp_top = false; }
    } clamp_scope{ctx};
    ctx->hist_clamp_top = clamp_top;
    if (joint_out) {
        void *p;
        ISO_TRY(iso_buf(ctx, BUF_HIST_DUMP, (size_t)m * m * bins * bins * sizeof(uint32_t), &p));
        d_joint = (uint32_t *)p;
    }
    if (col_out || row_out) {
        void *p;
        ISO_TRY(iso_buf(ctx, BUF_STAGING_A, (size_t)2 * m * m * bins * sizeof(uint32_t), &p));
        d_cr = (uint32_t *)p;
    }
    ISO_TRY(iso_run_similarity(ctx, f, multi ? f + (size_t)m * stride : nullptr, m, n, stride, bins,
                               (const uint32_t *)d_mm, multi ? (const uint32_t *)d_mm + 2 * m : nullptr,
                               (float *)d_ism, d_joint, d_cr));
    ISO_CUDA(cudaMemcpy2DAsync(ism_out, ism_ld * sizeof(float), d_ism, m * sizeof(float), m * sizeof(float), m,
                               cudaMemcpyDefault, ctx->stream));
    if (joint_out)
        ISO_CUDA(cudaMemcpyAsync(joint_out, d_joint, (size_t)m * m * bins * bins * sizeof(uint32_t), cudaMemcpyDefault,
                                 ctx->stream));
    if (col_out)
        ISO_CUDA(cudaMemcpyAsync(col_out, d_cr, (size_t)m * m * bins * sizeof(uint32_t), cudaMemcpyDefault, ctx->stream));
    if (row_out)
        ISO_CUDA(cudaMemcpyAsync(row_out, d_cr + (size_t)m * m * bins, (size_t)m * m * bins * sizeof(uint32_t),
                                 cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

extern "C" int iso_similarity_map(iso_ctx *ctx, const float *fields, int m, int64_t n, int bins, float *ism_out,
                                  uint32_t *joint_out)
{
    iso_clear_error();
    if (!ctx || !fields || !ism_out || m <= 0 || n <= 0) return iso_fail(ISO_ERR_ARG, "iso_similarity_map: bad argument");
    return similarity_impl(ctx, nullptr, fields, m, n, bins, nullptr, nullptr, ism_out, m, joint_out, nullptr, nullptr,
                           false);
}

extern "C" int iso_real_range(iso_ctx *ctx, const float *volume, int64_t V, float cfg_min, float cfg_max,
                              float *out_min, float *out_max)
{
    iso_clear_error();
    if (!ctx || !volume || !out_min || !out_max || V <= 0) return iso_fail(ISO_ERR_ARG, "iso_real_range: bad argument");
    ISO_CUDA(cudaSetDevice(ctx->device));
    const float *d_vol;
    ISO_TRY(device_volume(ctx, volume, V, &d_vol));
    void *d;
    ISO_TRY(iso_buf(ctx, BUF_MISC, 256, &d));
    uint32_t init[2] = {0xffffffffu, 0u};
    ISO_CUDA(cudaMemcpyAsync(d, init, sizeof init, cudaMemcpyHostToDevice, ctx->stream));
    int blocks = ctx->num_sms * 4;
    real_range_kernel<<<blocks, 256, 0, ctx->stream>>>(d_vol, V, cfg_min, cfg_max, (uint32_t *)d);
    ISO_LAUNCHED(ctx);
    uint32_t res[2];
    ISO_CUDA(cudaMemcpyAsync(res, d, sizeof res, cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    *out_min = from_order_key(res[0]);
    *out_max = from_order_key(res[1]);
    return ISO_OK;
}

extern "C" int iso_isovalues(iso_ctx *ctx, const float *volume, int64_t V, float vmin, float vmax, int n, int uniform,
                             float *out)
{
    iso_clear_error();
    if (!ctx || !out || n <= 0) return iso_fail(ISO_ERR_ARG, "iso_isovalues: bad argument");
    if (!uniform) {
        // runtime/src/Single.cpp:325-329
        float step = (vmax - vmin) / (float)n;
        for (int i = 0; i < n; ++i) out[i] = vmin + step * (float)i;
        return ISO_OK;
    }
    if (!volume || V <= 0) return iso_fail(ISO_ERR_ARG, "iso_isovalues: volume required");
    ISO_CUDA(cudaSetDevice(ctx->device));
    const float *d_vol;
    ISO_TRY(device_volume(ctx, volume, V, &d_vol));
    const int BINS = 65536;
    void *d_hist;
    ISO_TRY(iso_buf(ctx, BUF_STAGING_B, BINS * sizeof(unsigned int), &d_hist));
    ISO_CUDA(cudaMemsetAsync(d_hist, 0, BINS * sizeof(unsigned int), ctx->stream));
    // the reference loops while (float)i < (float)V (its dataSize parameter is a float)
    const float dataSize = (float)V;
    int64_t count = V;
    while (count > 0 && !((float)(count - 1) < dataSize)) --count;
    const float oneover = (float)(1.0 / (double)(vmax - vmin));
    uniform_hist_kernel<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(d_vol, count, vmin, oneover, (unsigned int *)d_hist);
    ISO_LAUNCHED(ctx);
    std::vector<int> hist(BINS);
    ISO_CUDA(cudaMemcpyAsync(hist.data(), d_hist, BINS * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    // runtime/src/Single.cpp:362-390: equalise into n groups (bins are relabelled with their group)
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
    // runtime/src/Single.cpp:306-320: group midpoints back to values
    int idx = 0, last = 0;
    float step = (vmax - vmin) / (float)BINS;
    for (int i = 0; i < n; ++i) {
        while (idx < BINS && hist[idx] <= i) ++idx;
        int range = idx - last;
        int mid = last + range / 2;
        out[i] = vmin + step * (float)mid;
        last = idx;
    }
    return ISO_OK;
}

extern "C" int iso_transpose_xfastest(iso_ctx *ctx, const float *src, int X, int Y, int Z, float *dst)
{
    iso_clear_error();
    if (!ctx || !src || !dst || X < 1 || Y < 1 || Z < 1) return iso_fail(ISO_ERR_ARG, "iso_transpose_xfastest: bad argument");
    if (Y > 65535) return iso_fail(ISO_ERR_ARG, "iso_transpose_xfastest: Y above 65535");
    ISO_CUDA(cudaSetDevice(ctx->device));
    const size_t V = (size_t)X * Y * Z;
    void *a, *b;
    ISO_TRY(iso_buf(ctx, BUF_STAGING_A, V * sizeof(float), &a));
    ISO_TRY(iso_buf(ctx, BUF_STAGING_B, V * sizeof(float), &b));
    ISO_CUDA(cudaMemcpyAsync(a, src, V * sizeof(float), cudaMemcpyDefault, ctx->stream));
    dim3 grid((X + 31) / 32, (Z + 31) / 32, Y);
    transpose_xz_kernel<<<grid, dim3(32, 8), 0, ctx->stream>>>((const float *)a, (float *)b, X, Y, Z);
    ISO_LAUNCHED(ctx);
    ISO_CUDA(cudaMemcpyAsync(dst, b, V * sizeof(float), cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

extern "C" int iso_copy_field(iso_ctx *ctx, int row, float *out)
{
    iso_clear_error();
    if (!ctx || !out || row < 0 || row >= ctx->last_m)
        return iso_fail(ISO_ERR_ARG, "iso_copy_field: row %d outside the last map (%d rows)", row, ctx ? ctx->last_m : 0);
    ISO_CUDA(cudaSetDevice(ctx->device));
    ISO_CUDA(cudaMemcpyAsync(out, (const float *)ctx->buf[BUF_FIELDS] + (size_t)row * ctx->last_stride,
                             (size_t)ctx->last_F * sizeof(float), cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

extern "C" int iso_copy_joint_histogram(iso_ctx *ctx, int i, int j, uint32_t *out)
{
    iso_clear_error();
    if (!ctx || !out) return iso_fail(ISO_ERR_ARG, "iso_copy_joint_histogram: bad argument");
    const int m = ctx->joint_m, bins = ctx->joint_bins;
    if (m <= 0 || !ctx->buf[BUF_HIST_DUMP])
        return iso_fail(ISO_ERR_ARG, "iso_copy_joint_histogram: no histograms kept (run a map in ISO_MI_REF32 mode)");
    if (i < 0 || j < 0 || i >= m || j >= m)
        return iso_fail(ISO_ERR_ARG, "iso_copy_joint_histogram: pair (%d, %d) outside %d x %d", i, j, m, m);
    ISO_CUDA(cudaSetDevice(ctx->device));
    const size_t h = (size_t)bins * bins;
    ISO_CUDA(cudaMemcpyAsync(out, (const uint32_t *)ctx->buf[BUF_HIST_DUMP] + ((size_t)i * m + j) * h,
                             h * sizeof(uint32_t), cudaMemcpyDefault, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    return ISO_OK;
}

// ---------------------------------------------------------------------------
// reference-named drop-in functions
// ---------------------------------------------------------------------------

extern "C" void calculate_histogram_h(float **distanceFields, float *minValues, float *maxValues, const int fieldSize,
                                      const unsigned long numFields, const unsigned long histogramSize,
                                      unsigned int *h_jointHist, unsigned int *h_colSums, unsigned int *h_rowSums,
                                      float *h_simMap, const int simMapSize, const ISO_BOOL multi)
{
    (void)h_jointHist;  // the reference never fills it (JointHistogram.cu:397)
    iso_clear_error();
    iso_ctx *ctx = iso_default_ctx();
    if (!ctx) return;
    if (!distanceFields || !minValues || !maxValues || !h_simMap || numFields == 0 || fieldSize <= 0 ||
        (int)numFields > simMapSize) {
        iso_fail(ISO_ERR_ARG, "calculate_histogram_h: bad argument");
        return;
    }
    similarity_impl(ctx, distanceFields, nullptr, (int)numFields, fieldSize, (int)histogramSize, minValues, maxValues,
                    h_simMap, simMapSize, nullptr, h_colSums, h_rowSums, multi);
}

extern "C" long approximate_isosurfaces_h(float *h_data, float isovalue, const int dimX, const int dimY, const int dimZ,
                                          const int scale, iso_int3 **h_points)
{
    iso_clear_error();
    if (!h_data || !h_points) return iso_fail(ISO_ERR_ARG, "approximate_isosurfaces_h: NULL argument");
    if (scale != 1) return iso_fail(ISO_ERR_ARG, "approximate_isosurfaces_h: only scale 1 is supported");
    iso_ctx *ctx = iso_default_ctx();
    if (!ctx) return ISO_ERR_CUDA;
    int64_t count = 0;
    ISO_TRY(iso_surface_points(ctx, h_data, dimX, dimY, dimZ, &isovalue, 1, ISO_SURFACE_APPROX, ISO_FRAME_CANON,
                               &count, nullptr, 0, nullptr));
    std::vector<float> xyz((size_t)count * 3 + 3);
    ISO_TRY(iso_surface_points(ctx, h_data, dimX, dimY, dimZ, &isovalue, 1, ISO_SURFACE_APPROX, ISO_FRAME_CANON,
                               &count, xyz.data(), count, nullptr));
    iso_int3 *out = (iso_int3 *)malloc(sizeof(iso_int3) * (size_t)(count > 0 ? count : 1));
    if (!out) return iso_fail(ISO_ERR_NOMEM, "approximate_isosurfaces_h: host allocation failed");
    for (int64_t i = 0; i < count; ++i) out[i] = iso_int3{(int32_t)xyz[3 * i], (int32_t)xyz[3 * i + 1], (int32_t)xyz[3 * i + 2]};
    *h_points = out;
    return (long)count;
}

extern "C" int iso_marching_cube_h(float iso, int dimX, int dimY, int dimZ, const float *h_volume, int maxVerts,
                                   float **out_xyzw, long *out_count)
{
    iso_clear_error();
    if (!h_volume || !out_xyzw || !out_count) return iso_fail(ISO_ERR_ARG, "iso_marching_cube_h: NULL argument");
    iso_ctx *ctx = iso_default_ctx();
    if (!ctx) return ISO_ERR_CUDA;
    int64_t count = 0;
    iso_surface_stats st;
    ISO_TRY(iso_surface_points(ctx, h_volume, dimX, dimY, dimZ, &iso, 1, ISO_SURFACE_MC, ISO_FRAME_REF, &count, nullptr,
                               0, &st));
    if (st.total_verts > (int64_t)maxVerts - 3)
        return iso_fail(ISO_ERR_CAPACITY, "iso_marching_cube_h: %lld triangle vertices exceed maxVerts-3",
                        (long long)st.total_verts);
    std::vector<float> xyz((size_t)count * 3 + 3);
    ISO_TRY(iso_surface_points(ctx, h_volume, dimX, dimY, dimZ, &iso, 1, ISO_SURFACE_MC, ISO_FRAME_REF, &count,
                               xyz.data(), count, nullptr));
    float *out = (float *)malloc(sizeof(float) * 4 * (size_t)(count > 0 ? count : 1));
    if (!out) return iso_fail(ISO_ERR_NOMEM, "iso_marching_cube_h: host allocation failed");
    for (int64_t i = 0; i < count; ++i) {
        out[4 * i] = xyz[3 * i];
        out[4 * i + 1] = xyz[3 * i + 1];
        out[4 * i + 2] = xyz[3 * i + 2];
        out[4 * i + 3] = 1.0f;
    }
    *out_xyzw = out;
    *out_count = (long)count;
    return ISO_OK;
}

extern "C" int iso_generate_hierarchy_h(const float *points_xyz, long numPoints, int dimX, int dimY, int dimZ,
                                        float *h_distances, int numSamples, int dfDownscale)
{
    (void)numSamples;
    iso_ctx *ctx = iso_default_ctx();
    if (!ctx) return ISO_ERR_CUDA;
    return iso_distance_field(ctx, points_xyz, numPoints, dimX, dimY, dimZ, dfDownscale, ISO_DF_LBVH, h_distances);
}
