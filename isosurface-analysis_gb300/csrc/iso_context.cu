// iso_context.cu -- contexts, the device arena and error reporting.
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "iso_internal.cuh"

static thread_local char g_last_error[1024] = "";

int iso_fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
    return code;
}

void iso_clear_error() { g_last_error[0] = '\0'; }

extern "C" const char *iso_last_error(void) { return g_last_error; }

extern "C" int iso_ctx_create(int device, iso_ctx **out)
{
    if (!out) return iso_fail(ISO_ERR_ARG, "iso_ctx_create: out is NULL");
    *out = nullptr;
    int count = 0;
    ISO_CUDA(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count)
        return iso_fail(ISO_ERR_ARG, "iso_ctx_create: device %d out of range (%d devices)", device, count);
    ISO_CUDA(cudaSetDevice(device));
    iso_ctx *ctx = new iso_ctx();
    ctx->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return iso_fail(ISO_ERR_CUDA, "iso_ctx_create: %s", cudaGetErrorString(e));
    }
    *out = ctx;
    return ISO_OK;
}

extern "C" void iso_ctx_destroy(iso_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int b = 0; b < BUF_COUNT_; ++b)
        if (ctx->buf[b]) cudaFree(ctx->buf[b]);
    if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

void iso_ctx_release(iso_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (int b = 0; b < BUF_COUNT_; ++b) {
        if (ctx->buf[b]) cudaFree(ctx->buf[b]);
        ctx->buf[b] = nullptr;
        ctx->cap[b] = 0;
    }
    ctx->clnc_ready = false;
    ctx->last_m = 0;
    ctx->joint_m = 0;
}

void iso_ctx_release_except_surfaces(iso_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (int b = 0; b < BUF_COUNT_; ++b) {
        // everything the surface stage's write pass reads (iso_surface.cu)
        if (b == BUF_VOLUME || b == BUF_ISO_SORTED || b == BUF_ISO_INDEX || b == BUF_SURF_COUNTS ||
            b == BUF_SURF_CURSOR || b == BUF_SEG_OFFSET || b == BUF_SEG_COUNT || b == BUF_SURF_BLOCK_COUNTS)
            continue;
        if (ctx->buf[b]) cudaFree(ctx->buf[b]);
        ctx->buf[b] = nullptr;
        ctx->cap[b] = 0;
    }
    ctx->clnc_ready = false;
    ctx->last_m = 0;
    ctx->joint_m = 0;
}

extern "C" int iso_ctx_set_limit(iso_ctx *ctx, int which, int64_t value)
{
    if (!ctx) return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: NULL context");
    switch (which) {
    case ISO_LIMIT_LBVH_GROUP_POINTS:
        if (value < 1) return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: group size must be positive");
        ctx->lbvh_group_points = value;
        return ISO_OK;
    case ISO_LIMIT_HIST_SEGMENT_VALUES:
        if (value != 0 && (value < 65536 || value % 4 != 0))
            return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: segment length must be 0 or a multiple of 4 >= 65536");
        ctx->hist_segment_values = value;
        return ISO_OK;
    case ISO_LIMIT_SURF_BLOCK_COUNT_BYTES:
        if (value < 0) return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: byte limit must be >= 0");
        ctx->surf_block_count_bytes = value;
        return ISO_OK;
    case ISO_LIMIT_DEVICE_BYTES:
        if (value < 0) return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: byte cap must be >= 0");
        ctx->device_bytes_cap = value;
        return ISO_OK;
    case ISO_LIMIT_QUERY_RUN:
        if (value != 0 && value != 8 && value != 16 && value != 32 && value != 64)
            return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: query run must be 0, 8, 16, 32 or 64");
        ctx->query_run = (int)value;
        return ISO_OK;
    case ISO_LIMIT_HIST_ROW_CODES:
        if (value != 0 && value != 1) return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: row codes must be 0 or 1");
        ctx->hist_row_codes = (int)value;
        return ISO_OK;
    case ISO_LIMIT_MI_MODE:
        if (value != ISO_MI_FP64 && value != ISO_MI_REF32)
            return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: unknown MI mode %lld", (long long)value);
        ctx->mi_mode = (int)value;
        return ISO_OK;
    default:
        return iso_fail(ISO_ERR_ARG, "iso_ctx_set_limit: unknown limit %d", which);
    }
}

extern "C" void *iso_ctx_stream(iso_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int64_t iso_ctx_launches(iso_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" size_t iso_ctx_device_bytes(iso_ctx *ctx)
{
    size_t s = 0;
    if (ctx)
        for (int b = 0; b < BUF_COUNT_; ++b) s += ctx->cap[b];
    return s;
}

int iso_buf(iso_ctx *ctx, IsoBuf b, size_t bytes, void **out)
{
    if (bytes == 0) bytes = 256;
    if (ctx->cap[b] < bytes) {
        size_t want = bytes + bytes / 8;
        want = (want + 4095) & ~size_t(4095);
        if (ctx->device_bytes_cap > 0) {
            size_t held = 0;
            for (int k = 0; k < BUF_COUNT_; ++k) held += ctx->cap[k];
            if (held - ctx->cap[b] + want > (size_t)ctx->device_bytes_cap)
                return iso_fail(ISO_ERR_NOMEM, "device allocation of %zu bytes would exceed the context's cap of %lld "
                                "bytes (%zu held)", want, (long long)ctx->device_bytes_cap, held);
        }
        if (ctx->buf[b]) {
            // the old buffer may still be read by queued work on this stream
            ISO_CUDA(cudaStreamSynchronize(ctx->stream));
            ISO_CUDA(cudaFree(ctx->buf[b]));
            ctx->buf[b] = nullptr;
            ctx->cap[b] = 0;
        }
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return iso_fail(ISO_ERR_NOMEM, "device allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
        }
        ctx->buf[b] = p;
        ctx->cap[b] = want;
    }
    *out = ctx->buf[b];
    return ISO_OK;
}

int iso_host_scratch(iso_ctx *ctx, size_t bytes, void **out)
{
    if (ctx->host_pinned_cap < bytes) {
        if (ctx->host_pinned) {
            ISO_CUDA(cudaStreamSynchronize(ctx->stream));
            cudaFreeHost(ctx->host_pinned);
            ctx->host_pinned = nullptr;
            ctx->host_pinned_cap = 0;
        }
        size_t want = (bytes + bytes / 4 + 4095) & ~size_t(4095);
        void *p = nullptr;
        if (cudaMallocHost(&p, want) != cudaSuccess) {
            cudaGetLastError();
            return iso_fail(ISO_ERR_NOMEM, "pinned host allocation of %zu bytes failed", want);
        }
        ctx->host_pinned = p;
        ctx->host_pinned_cap = want;
    }
    *out = ctx->host_pinned;
    return ISO_OK;
}

bool iso_is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static std::mutex g_default_mu;
static std::map<int, iso_ctx *> g_default_ctx;  // one per device, kept until exit

iso_ctx *iso_default_ctx()
{
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        iso_fail(ISO_ERR_CUDA, "no current CUDA device");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_default_mu);
    iso_ctx *&c = g_default_ctx[device];
    if (!c) {
        if (iso_ctx_create(device, &c) != ISO_OK) {
            c = nullptr;
            return nullptr;
        }
        // the reference-named entry points return the reference's own numbers
        c->mi_mode = ISO_MI_REF32;
    }
    return c;
}
