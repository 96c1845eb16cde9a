// iso_histogram.cu -- all-pairs joint histograms and FP64 normalised mutual
// information (the ISM).  Replaces calculate_histogram_g + calculateMutualInformation
// (isosurfaces_cuda/src/JointHistogram.cu:24-162).
//
// Layout: fields are rows of a [m x stride] float matrix (stride a multiple of 4,
// rows 16-byte aligned).  Per-field interval (min, max) as uint32 float bits
// (all distance values are >= 0, so bit order is value order).
//
// Kernel: persistent CTAs pull unordered pair tasks (i <= j) from a counter.
// A CTA owns one pair at a time and streams both fields with 128-bit loads.
// Each voxel's two buckets (exact IEEE division, the reference's binning) form
// one bin; the bin is counted in shared memory as a 16-bit half of a 32-bit
// word (bins*bins/2 words: 128 KB at 256 bins).  Every 63488 voxels (fewer than
// 2^16, so no half can overflow) the packed counts are added into the CTA's
// private uint32 histogram in global memory (L2-resident).  After the last voxel
// the CTA reduces that histogram: FP64 sum of c*ln(c) over bins and over the
// exact integer row and column sums, then NMI = 2I/(hX+hY), written to both
// (i,j) and (j,i).
#include <vector>

#include "iso_internal.cuh"

namespace {

constexpr int HIST_THREADS = 512;
constexpr int HIST_ITERS_PER_FLUSH = 31;  // 31 * 512 threads * 4 voxels = 63488 < 65536

__device__ __forceinline__ float bits_to_float(uint32_t b) { return __uint_as_float(b); }

struct PairArgs {
    const float *fa;      // field set for the row side
    const float *fb;      // field set for the column side
    int64_t n;            // values per field
    int64_t stride;       // floats between consecutive fields
    const uint32_t *mma;  // min/max bits of fa fields (2 per field)
    const uint32_t *mmb;  // min/max bits of fb fields
    const int2 *tasks;
    int num_tasks;
    int m;                // ISM row length
    int bins;
    int symmetric;        // write (j,i) too
    float *ism;
    uint32_t *scratch;    // per CTA bins*bins uint32 (zero on entry, left zero)
    unsigned int *counter;
    uint32_t *joint_dump; // optional: m*m*bins*bins
    uint32_t *colrow_dump;// optional: [2][m*m*bins] (col sums, row sums) per ordered pair
};

__device__ __forceinline__ void count_bin(uint32_t *hist_words, int bin)
{
    atomicAdd(&hist_words[bin >> 1], 1u << ((bin & 1) << 4));
}

__device__ void flush_packed(uint32_t *hist_words, int words, uint32_t *global_hist)
{
    uint2 *g2 = reinterpret_cast<uint2 *>(global_hist);
    for (int w = threadIdx.x; w < words; w += blockDim.x) {
        uint32_t v = hist_words[w];
        if (v) {
            uint2 g = g2[w];
            g.x += v & 0xffffu;
            g.y += v >> 16;
            g2[w] = g;
            hist_words[w] = 0;
        }
    }
}

__global__ void __launch_bounds__(HIST_THREADS, 1) joint_histogram_mi_kernel(PairArgs a)
{
    extern __shared__ uint32_t hist_words[];
    __shared__ int s_task;
    __shared__ double s_red[3][HIST_THREADS / 32];
    __shared__ unsigned long long s_colsum[ISO_MAX_BINS];

    const int bins = a.bins;
    const int words = bins * bins / 2;
    uint32_t *ghist = a.scratch + (size_t)blockIdx.x * bins * bins;

    for (int w = threadIdx.x; w < words; w += blockDim.x) hist_words[w] = 0;

    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int t = s_task;
        if (t >= a.num_tasks) break;
        const int2 task = a.tasks[t];
        const int i = task.x, j = task.y;

        float mn_i = bits_to_float(a.mma[2 * i]), mx_i = bits_to_float(a.mma[2 * i + 1]);
        float mn_j = bits_to_float(a.mmb[2 * j]), mx_j = bits_to_float(a.mmb[2 * j + 1]);
        const float mn = mn_i < mn_j ? mn_i : mn_j;
        const float mx = mx_i > mx_j ? mx_i : mx_j;
        const float step = __fdiv_rn(__fsub_rn(mx, mn), (float)bins);

        const float *f1 = a.fa + (size_t)i * a.stride;
        const float *f2 = a.fb + (size_t)j * a.stride;
        const float4 *v1 = reinterpret_cast<const float4 *>(f1);
        const float4 *v2 = reinterpret_cast<const float4 *>(f2);
        const int64_t n4 = a.n >> 2;

        // block-uniform chunks of at most 63488 voxels: no 16-bit half overflows
        const int64_t chunk = (int64_t)HIST_ITERS_PER_FLUSH * blockDim.x;
        for (int64_t base = 0; base < n4; base += chunk) {
            const int64_t end = base + chunk < n4 ? base + chunk : n4;
            for (int64_t q = base + threadIdx.x; q < end; q += blockDim.x) {
                float4 x = __ldg(v1 + q);
                float4 y = __ldg(v2 + q);
                count_bin(hist_words, iso_bucket(x.x, mn, step, bins) * bins + iso_bucket(y.x, mn, step, bins));
                count_bin(hist_words, iso_bucket(x.y, mn, step, bins) * bins + iso_bucket(y.y, mn, step, bins));
                count_bin(hist_words, iso_bucket(x.z, mn, step, bins) * bins + iso_bucket(y.z, mn, step, bins));
                count_bin(hist_words, iso_bucket(x.w, mn, step, bins) * bins + iso_bucket(y.w, mn, step, bins));
            }
            __syncthreads();
            flush_packed(hist_words, words, ghist);
            __syncthreads();
        }
        // tail (n not a multiple of 4)
        for (int64_t v = (n4 << 2) + threadIdx.x; v < a.n; v += blockDim.x)
            count_bin(hist_words, iso_bucket(f1[v], mn, step, bins) * bins + iso_bucket(f2[v], mn, step, bins));
        __syncthreads();
        flush_packed(hist_words, words, ghist);
        __syncthreads();

        // ---- reduction: row sums, column sums, sum c ln c; clears ghist ----
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
        for (int c = threadIdx.x; c < bins; c += blockDim.x) s_colsum[c] = 0;
        __syncthreads();
        double hxy = 0.0, hy = 0.0;
        unsigned long long colpart[ISO_MAX_BINS / 32];
#pragma unroll
        for (int k = 0; k < ISO_MAX_BINS / 32; ++k) colpart[k] = 0;
        const bool dump = a.joint_dump != nullptr;
        const bool dumpcr = a.colrow_dump != nullptr;
        for (int r = warp; r < bins; r += nwarps) {
            unsigned long long rowsum = 0;
            uint32_t *row = ghist + (size_t)r * bins;
#pragma unroll
            for (int k = 0; k < ISO_MAX_BINS / 32; ++k) {
                int c = lane + 32 * k;
                if (c < bins) {
                    uint32_t cnt = row[c];
                    row[c] = 0;
                    if (dump) {
                        a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + c] = cnt;
                        if (a.symmetric && i != j) a.joint_dump[(((size_t)j * a.m + i) * bins + c) * bins + r] = cnt;
                    }
                    rowsum += cnt;
                    colpart[k] += cnt;
                    if (cnt) hxy -= (double)cnt * log((double)cnt);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) rowsum += __shfl_xor_sync(0xffffffffu, rowsum, o);
            if (lane == 0 && rowsum) hy -= (double)rowsum * log((double)rowsum);
            if (lane == 0 && dumpcr) {
                size_t base = ((size_t)i * a.m + j) * bins;
                a.colrow_dump[(size_t)a.m * a.m * bins + base + r] = (uint32_t)rowsum;  // row sums of (i,j)
                if (a.symmetric && i != j) a.colrow_dump[((size_t)j * a.m + i) * bins + r] = (uint32_t)rowsum;  // col sums of (j,i)
            }
        }
#pragma unroll
        for (int k = 0; k < ISO_MAX_BINS / 32; ++k) {
            int c = lane + 32 * k;
            if (c < bins && colpart[k]) atomicAdd(&s_colsum[c], colpart[k]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            hxy += __shfl_xor_sync(0xffffffffu, hxy, o);
            hy += __shfl_xor_sync(0xffffffffu, hy, o);
        }
        if (lane == 0) {
            s_red[0][warp] = hxy;
            s_red[1][warp] = hy;
        }
        __syncthreads();
        double hx = 0.0;
        for (int c = threadIdx.x; c < bins; c += blockDim.x) {
            unsigned long long cs = s_colsum[c];
            if (cs) hx -= (double)cs * log((double)cs);
            if (dumpcr) {
                size_t base = ((size_t)i * a.m + j) * bins;
                a.colrow_dump[base + c] = (uint32_t)cs;  // col sums of (i,j)
                if (a.symmetric && i != j)
                    a.colrow_dump[(size_t)a.m * a.m * bins + ((size_t)j * a.m + i) * bins + c] = (uint32_t)cs;  // row sums of (j,i)
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) hx += __shfl_xor_sync(0xffffffffu, hx, o);
        if (lane == 0) s_red[2][warp] = hx;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sxy = 0.0, sy = 0.0, sx = 0.0;
            for (int w = 0; w < nwarps; ++w) {
                sxy += s_red[0][w];
                sy += s_red[1][w];
                sx += s_red[2][w];
            }
            const double N = (double)a.n;
            const double lnN = log(N);
            sxy = sxy / N + lnN;
            sx = sx / N + lnN;
            sy = sy / N + lnN;
            double iXY = sx + sy - sxy;
            double val = 2.0 * iXY / (sx + sy);
            float out = val != val ? 0.0f : (float)val;
            a.ism[(size_t)i * a.m + j] = out;
            if (a.symmetric) a.ism[(size_t)j * a.m + i] = out;
        }
        __syncthreads();
    }
}

// Per-field min/max over the first n values: min starts at FLT_MAX and max at
// FLT_MIN as in types/src/DistanceField.cpp:159-200.  Values are >= 0, so
// unsigned comparison of the bit patterns orders them.
__global__ void field_minmax_kernel(const float *fields, int64_t n, int64_t stride, uint32_t *minmax)
{
    const int f = blockIdx.y;
    const float *row = fields + (size_t)f * stride;
    uint32_t lo = 0x7f7fffffu, hi = 0x00800000u;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        uint32_t b = __float_as_uint(row[v]);
        lo = b < lo ? b : lo;
        hi = b > hi ? b : hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        uint32_t l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&minmax[2 * f], lo);
        atomicMax(&minmax[2 * f + 1], hi);
    }
}

__global__ void minmax_init_kernel(uint32_t *minmax, int m)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m) {
        minmax[2 * f] = 0x7f7fffffu;
        minmax[2 * f + 1] = 0x00800000u;
    }
}

}  // namespace

int iso_run_minmax(iso_ctx *ctx, const float *d_fields, int m, int64_t n, int64_t stride, uint32_t *d_minmax)
{
    if (m <= 0) return ISO_OK;
    minmax_init_kernel<<<(m + 255) / 256, 256, 0, ctx->stream>>>(d_minmax, m);
    ISO_LAUNCHED(ctx);
    int64_t per = (n + 255) / 256;
    int bx = (int)(per < 64 ? per : 64);
    if (bx < 1) bx = 1;
    field_minmax_kernel<<<dim3(bx, m), 256, 0, ctx->stream>>>(d_fields, n, stride, d_minmax);
    ISO_LAUNCHED(ctx);
    return ISO_OK;
}

// Pair tasks ordered in 16-field tiles so concurrently running CTAs share fields
// in L2.  symmetric: i <= j over one set; otherwise all (i, j) of two sets.
static void build_tasks(int m, bool symmetric, int2 *out, int *count)
{
    const int T = 16;
    int c = 0;
    for (int bi = 0; bi < m; bi += T)
        for (int bj = symmetric ? bi : 0; bj < m; bj += T)
            for (int i = bi; i < bi + T && i < m; ++i)
                for (int j = bj; j < bj + T && j < m; ++j)
                    if (!symmetric || j >= i) out[c++] = make_int2(i, j);
    *count = c;
}

int iso_run_similarity(iso_ctx *ctx, const float *d_fields_a, const float *d_fields_b, int m, int64_t n,
                       int64_t stride, int bins, const uint32_t *d_minmax_a, const uint32_t *d_minmax_b,
                       float *d_ism, uint32_t *d_joint_dump, uint32_t *d_colrow_dump)
{
    if (m <= 0) return ISO_OK;
    if (bins < 2 || bins > ISO_MAX_BINS || (bins & 1))
        return iso_fail(ISO_ERR_ARG, "bins must be even and in [2, %d], got %d", ISO_MAX_BINS, bins);
    if (stride % 4 != 0 || ((uintptr_t)d_fields_a & 15) || ((uintptr_t)d_fields_b & 15))
        return iso_fail(ISO_ERR_ARG, "field rows must be 16-byte aligned with a stride multiple of 4");
    const bool symmetric = d_fields_b == nullptr;
    const float *fb = symmetric ? d_fields_a : d_fields_b;
    const uint32_t *mmb = symmetric ? d_minmax_a : d_minmax_b;

    const size_t max_tasks = symmetric ? (size_t)m * (m + 1) / 2 : (size_t)m * m;
    std::vector<int2> h_tasks(max_tasks);
    int num_tasks = 0;
    build_tasks(m, symmetric, h_tasks.data(), &num_tasks);

    void *d_tasks = nullptr, *d_counter = nullptr, *d_scratch = nullptr;
    ISO_TRY(iso_buf(ctx, BUF_PAIR_TASKS, max_tasks * sizeof(int2), &d_tasks));
    ISO_TRY(iso_buf(ctx, BUF_TASK_COUNTER, 256, &d_counter));
    ISO_CUDA(cudaMemcpyAsync(d_tasks, h_tasks.data(), num_tasks * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
    ISO_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), ctx->stream));

    const size_t smem = (size_t)bins * bins / 2 * sizeof(uint32_t);
    ISO_CUDA(cudaFuncSetAttribute(joint_histogram_mi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(ISO_MAX_BINS * ISO_MAX_BINS / 2 * sizeof(uint32_t))));
    int per_sm = 0;
    ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, joint_histogram_mi_kernel, HIST_THREADS, smem));
    if (per_sm < 1) per_sm = 1;
    int grid = ctx->num_sms * per_sm;
    if (grid > num_tasks) grid = num_tasks;
    ISO_TRY(iso_buf(ctx, BUF_HIST_SCRATCH, (size_t)grid * bins * bins * sizeof(uint32_t), &d_scratch));
    // scratch must start zero; the kernel leaves it zero after every task
    ISO_CUDA(cudaMemsetAsync(d_scratch, 0, (size_t)grid * bins * bins * sizeof(uint32_t), ctx->stream));

    PairArgs a;
    a.fa = d_fields_a;
    a.fb = fb;
    a.n = n;
    a.stride = stride;
    a.mma = d_minmax_a;
    a.mmb = mmb;
    a.tasks = (const int2 *)d_tasks;
    a.num_tasks = num_tasks;
    a.m = m;
    a.bins = bins;
    a.symmetric = symmetric ? 1 : 0;
    a.ism = d_ism;
    a.scratch = (uint32_t *)d_scratch;
    a.counter = (unsigned int *)d_counter;
    a.joint_dump = d_joint_dump;
    a.colrow_dump = d_colrow_dump;
    joint_histogram_mi_kernel<<<grid, HIST_THREADS, smem, ctx->stream>>>(a);
    ISO_LAUNCHED(ctx);
    return ISO_OK;
}
