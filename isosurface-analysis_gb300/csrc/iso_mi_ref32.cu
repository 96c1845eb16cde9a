// iso_mi_ref32.cu -- the reference's FP32 mutual information, reproduced bit for
// bit on the GPU (opt-in: ISO_MI_REF32; the default of the reference-named
// entry points).
//
// The reference evaluates calculateMutualInformation
// (isosurfaces_cuda/src/JointHistogram.cu:24-60) on the device, inside
// calculate_histogram_g (:156-160), once per ORDERED pair (i, j): one thread
// walks the pair's joint histogram row by row in FP32, with logf and the
// compiler's default multiply-add contraction.  Its map is therefore not
// symmetric, and it differs from an accurate MI by its own rounding (about
// 7e-5 on 64^3 fields at 128 bins).  A caller who needs the reference's numbers
// (the drop-in calculate_histogram_h) gets them from this kernel.
//
// This file is compiled WITHOUT -fmad=false (nvcc's default contraction, as
// the reference's build uses), so that each accumulation below compiles to the
// same fused operation as the reference's; every other file of the engine
// forbids contraction.
//
// Layout: joint histograms of all m*m ordered pairs, pair q = i*m + j at
// joint + q*bins*bins, row = bucket of field i (the histogram kernels' dump),
// and their column and row sums (colrow: [2][m*m*bins]; exact integers, so
// the histogram kernels' sums are the reference's).  One warp walks 32
// pairs, one lane per pair: it stages 32 consecutive bins of each of its
// pairs in shared memory by asynchronous copies several steps ahead, and each
// lane continues its pair's serial sum over the staged bins.  The row entropy is the sum over the
// row sums in row order (the reference adds each at its row's end), the column
// entropy over the column sums in column order.  The logarithm of a count
// below 65536 is read from a table that logf_table_kernel fills with the
// device's own logf, so the serial chains carry only the fused
// multiply-subtract, and a zero count's step leaves the sum unchanged, so the
// walks have no branch per bin.  The order of every summation chain is the reference's.
#include "iso_async.cuh"
#include "iso_internal.cuh"

namespace {

constexpr int R32_PAIRS = 32;        // ordered pairs per CTA (one warp, one lane per pair)
constexpr int R32_TILE = 32;         // bins of each pair staged per step
constexpr int R32_LOG_TABLE = 65536; // counts whose logarithm is tabulated

// Entry 0 holds 0 rather than logf(0) = -inf: a zero count's step h - 0 * 0
// then returns h unchanged (h is never -0: it starts at +0 and only falls),
// which is what the reference's skip of zero counts does, and the walks below
// need no branch per bin.
__global__ void logf_table_kernel(float *t)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < R32_LOG_TABLE) t[c] = c == 0 ? 0.0f : logf((float)c);
}

__device__ __forceinline__ float log_count(const float *__restrict__ tab, uint32_t c)
{
    return c < (uint32_t)R32_LOG_TABLE ? __ldg(tab + c) : logf((float)c);
}

// The table entry of a count, clamped into the table (counts past it are
// corrected by the caller).
__device__ __forceinline__ float log_small(const float *__restrict__ tab, uint32_t c)
{
    return __ldg(tab + (c < (uint32_t)R32_LOG_TABLE ? c : (uint32_t)R32_LOG_TABLE - 1));
}

// The reference's per-bin term h -= c * logf(c) for a nonzero count, with
// lg = logf(c).  Kept as one expression so that the compiler fuses the
// product into the subtraction exactly as it does in the reference's kernel.
__device__ __forceinline__ float entropy_step(float h, uint32_t count, float lg)
{
    float c = (float)count;
    h -= c * lg;
    return h;
}

// Each step stages 32 bins of each of the CTA's 32 pairs (one 128-byte row
// per pair, 4 KB) by asynchronous copies, R32_STAGES steps ahead of the walk,
// so that the walk does not wait on memory.  A row's eight 16-byte chunks are
// stored at chunk position c ^ (pair % 8), which lets the 32 lanes read their
// own rows 16 bytes at a time without bank conflicts.  Bins past the
// histogram's end are zero-filled: the walk skips zero counts, as the
// reference does.
constexpr int R32_STAGES = 6;

__global__ void __launch_bounds__(R32_PAIRS) mi_ref32_kernel(const uint32_t *__restrict__ joint,
                                                            const uint32_t *__restrict__ colrow, int64_t num_pairs,
                                                            int bins, float num_values,
                                                            const float *__restrict__ logtab, float *__restrict__ ism)
{
    static_assert(R32_TILE == 32 && R32_PAIRS == 32, "one 128-byte row per lane and step");
    __shared__ __align__(16) uint32_t tiles[R32_STAGES][R32_PAIRS * R32_TILE];
    const int lane = threadIdx.x;
    const int64_t first = (int64_t)blockIdx.x * R32_PAIRS;
    const int64_t hist = (int64_t)bins * bins;  // a multiple of 4: bins is even
    const int64_t steps = (hist + R32_TILE - 1) / R32_TILE;

    // lane l copies chunk l % 8 of the rows of pairs 4 j + l / 8, j = 0..7
    auto issue = [&](int64_t step, int st) {
        if (step < steps) {
            const int c = lane & 7;
            const int64_t bin = step * R32_TILE + 4 * c;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int p = 4 * j + (lane >> 3);
                const bool valid = first + p < num_pairs && bin < hist;
                const uint32_t *src = valid ? joint + (first + p) * hist + bin : joint;
                const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tiles[st][p * R32_TILE + ((c ^ (p & 7)) << 2)]);
                cp_async16(dst, src, valid ? 16u : 0u);
            }
        }
        cp_async_commit();  // one group per step, empty past the end
    };
#pragma unroll
    for (int s0 = 0; s0 < R32_STAGES - 1; ++s0) issue(s0, s0);

    float hXY = 0.0f;
    for (int64_t step = 0; step < steps; ++step) {
        const int st = (int)(step % R32_STAGES);
        cp_async_wait<R32_STAGES - 2>();  // this step's copies (and every lane's: next line) have landed
        __syncwarp();
        // the stage read in the previous step takes step + R32_STAGES - 1
        issue(step + R32_STAGES - 1, (int)((step + R32_STAGES - 1) % R32_STAGES));
        // this lane's pair: the reference's row-major walk over the staged
        // bins.  Counts and logarithms of all 32 bins are fetched before the
        // chain, with no branch between them; zero counts step through the
        // chain unchanged (table entry 0).
        const uint32_t *own = tiles[st] + lane * R32_TILE;
        uint32_t v[R32_TILE];
#pragma unroll
        for (int q = 0; q < R32_TILE / 4; ++q) {
            const uint4 v4 = *reinterpret_cast<const uint4 *>(own + ((q ^ (lane & 7)) << 2));
            v[4 * q] = v4.x;
            v[4 * q + 1] = v4.y;
            v[4 * q + 2] = v4.z;
            v[4 * q + 3] = v4.w;
        }
        __syncwarp();  // every lane is done with stage st before it is refilled
        float lg[R32_TILE];
        uint32_t any = 0;
#pragma unroll
        for (int k = 0; k < R32_TILE; ++k) {
            lg[k] = log_small(logtab, v[k]);
            any |= v[k];
        }
        if (any >= (uint32_t)R32_LOG_TABLE) {
#pragma unroll
            for (int k = 0; k < R32_TILE; ++k)
                if (v[k] >= (uint32_t)R32_LOG_TABLE) lg[k] = logf((float)v[k]);
        }
#pragma unroll
        for (int k = 0; k < R32_TILE; ++k) hXY = entropy_step(hXY, v[k], lg[k]);
    }
    cp_async_wait<0>();
    if (first + lane >= num_pairs) return;
    const uint32_t *cs = colrow + (first + lane) * bins;
    const uint32_t *rs = colrow + num_pairs * bins + (first + lane) * bins;
    float hX = 0.0f, hY = 0.0f;  // zero sums step through unchanged, as above
#pragma unroll 8
    for (int c = 0; c < bins; ++c) {
        const uint32_t v = __ldg(cs + c);
        hX = entropy_step(hX, v, log_count(logtab, v));
    }
#pragma unroll 8
    for (int r = 0; r < bins; ++r) {
        const uint32_t v = __ldg(rs + r);
        hY = entropy_step(hY, v, log_count(logtab, v));
    }
    // JointHistogram.cu:53-59, operation for operation
    hXY = hXY / num_values + logf(num_values);
    hX = hX / num_values + logf(num_values);
    hY = hY / num_values + logf(num_values);
    float iXY = hX + hY - hXY;
    float val = 2 * iXY / (hX + hY);
    ism[first + lane] = val != val ? 0.0f : val;
}

}  // namespace

// Reference-order FP32 MI of all m*m ordered pairs whose joint histograms are
// at d_joint (pair i*m + j, row = bucket of field i) and column and row sums at
// d_colrow; n = values per field.
int iso_run_mi_ref32(iso_ctx *ctx, const uint32_t *d_joint, const uint32_t *d_colrow, int m, int bins, int64_t n,
                     float *d_ism)
{
    if (m <= 0) return ISO_OK;
    const int64_t pairs = (int64_t)m * m;
    const int64_t ctas = (pairs + R32_PAIRS - 1) / R32_PAIRS;
    if (ctas > 0x7fffffff) return iso_fail(ISO_ERR_ARG, "reference FP32 MI: too many pairs");
    void *tab;
    ISO_TRY(iso_buf(ctx, BUF_LOGF_TABLE, (size_t)R32_LOG_TABLE * sizeof(float), &tab));
    logf_table_kernel<<<R32_LOG_TABLE / 256, 256, 0, ctx->stream>>>((float *)tab);
    ISO_LAUNCHED(ctx);
    // the reference converts its int field size to float (JointHistogram.cu:24, :159)
    const float nv = (float)n;
    mi_ref32_kernel<<<(unsigned)ctas, R32_PAIRS, 0, ctx->stream>>>(d_joint, d_colrow, pairs, bins, nv,
                                                                   (const float *)tab, d_ism);
    ISO_LAUNCHED(ctx);
    return ISO_OK;
}
