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
#include <mutex>
#include <vector>

#include "iso_internal.cuh"

namespace {

constexpr int HIST_THREADS = 1024;
constexpr float BUCKET_TOL = 1.220703125e-4f;  // 2^-13, see fast_bucket

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
    int4 *events;         // per CTA: event_cap wrap events {bin, delta, c16, corr}
    int event_cap;
    const double *clnc;   // c*ln(c) for c < 65536
    unsigned int *counter;
    int *error;
    uint32_t *joint_dump; // optional: m*m*bins*bins
    uint32_t *colrow_dump;// optional: [2][m*m*bins] (col sums, row sums) per ordered pair
};

struct Binner {
    float mn, step, r;
    int bins;
    int mode;  // 0: reciprocal with exact fallback, 1: exact division only, 2: step == 0
};

// Exact bucket of JointHistogram.cu:63-75 (IEEE division), clamped to [0, bins).
__device__ __forceinline__ int exact_bucket(const Binner &b, float v) { return iso_bucket(v, b.mn, b.step, b.bins); }

// Out of line: the exact path is rare and would otherwise cost registers in the
// streaming loop.
__device__ __noinline__ int2 exact_bucket_pair(float mn, float step, int bins, float va, float vb)
{
    return make_int2(iso_bucket(va, mn, step, bins), iso_bucket(vb, mn, step, bins));
}

// Both buckets of one voxel through a reciprocal, the two fields as one packed
// float2.  q' = RN(RN(v-mn) * RN(1/step)) is within 257 * 2^-23 + 2^-15 <
// 2^-13.5 of RN((v-mn)/step) for q < 257, so floor(q') is the exact bucket
// unless q' lies within 2^-13 of an integer boundary that matters; then both
// values take the exact division.  floor(q') comes from adding 1.5 * 2^23 to
// q' - 0.5 (exact): the integer part lands in the low mantissa bits.  Exact
// integers q' round to an even neighbour there, but their fraction (0 or 1)
// sends them to the exact path, except q' = 0, whose floor 0 is right.  Values
// lie inside the pair interval, so q' < 2^22; anything beyond clamps to the
// last bucket.
__device__ __forceinline__ void fast_bucket_pair(const Binner &b, float va, float vb, int &ka, int &kb)
{
    constexpr float MAGIC = 12582912.0f;  // 1.5 * 2^23
    constexpr int MAGIC_BITS = 0x4B400000;
    const float2 d = __fadd2_rn(make_float2(va, vb), make_float2(-b.mn, -b.mn));
    const float2 q = __fmul2_rn(d, make_float2(b.r, b.r));
    const float2 m = __fadd2_rn(__fadd2_rn(q, make_float2(-0.5f, -0.5f)), make_float2(MAGIC, MAGIC));
    const float2 f = __fadd2_rn(m, make_float2(-MAGIC, -MAGIC));               // floor(q')
    const float2 fr = __ffma2_rn(f, make_float2(-1.0f, -1.0f), q);             // q' - floor(q'), exact
    const unsigned inner = (unsigned)(b.bins - 1);
    const bool slow = fr.x > 1.0f - BUCKET_TOL || (fr.x < BUCKET_TOL && f.x != 0.0f) ||
                      fr.y > 1.0f - BUCKET_TOL || (fr.y < BUCKET_TOL && f.y != 0.0f);
    ka = (int)min((unsigned)(__float_as_int(m.x) - MAGIC_BITS), inner);
    kb = (int)min((unsigned)(__float_as_int(m.y) - MAGIC_BITS), inner);
    if (slow) {
        const int2 e = exact_bucket_pair(b.mn, b.step, b.bins, va, vb);
        ka = e.x;
        kb = e.y;
    }
}

// Counts one bin as a 16-bit half of a shared 32-bit word.  The returned old
// word tells this thread exactly when a half wraps: the low half's 16 bits
// advance only by its own increments, the high half's by its increments plus
// the low half's carries.  Wraps are logged as corrections:
//   low half wraps  -> low bin +65536, high bin -1 (the carry it received)
//   high half wraps -> high bin +65536
__device__ __noinline__ void log_wrap(int bin, uint32_t sh, uint32_t old, int4 *ev, int cap, unsigned int *nev,
                                     int *error)
{
    const int lo = bin & ~1, hi = bin | 1;
    const bool both = sh == 0 && (old >> 16) == 0xffffu;
    const unsigned int ne = sh == 0 ? (both ? 3u : 2u) : 1u;
    const unsigned int slot = atomicAdd(nev, ne);
    if (slot + ne > (unsigned int)cap) {
        atomicExch(error, 3);
        return;
    }
    if (sh == 0) {
        ev[slot] = make_int4(lo, 65536, 0, 0);
        ev[slot + 1] = make_int4(hi, -1, 0, 0);
        if (both) ev[slot + 2] = make_int4(hi, 65536, 0, 0);
    } else {
        ev[slot] = make_int4(hi, 65536, 0, 0);
    }
}

__device__ __forceinline__ void count_bin(uint32_t *words, int bin, int4 *ev, int cap, unsigned int *nev, int *error)
{
    // odd bins live in the high half: increment 0x10000 and wrap mask
    // 0xFFFF0000, even bins 1 and 0xFFFF (integer multiply-adds instead of
    // shifts keep the ALU pipe free)
    const uint32_t odd = (uint32_t)bin & 1u;
    const uint32_t inc = odd * 0xFFFFu + 1u;
    const uint32_t mask = inc * 0xFFFFu;
    const uint32_t old = atomicAdd(&words[bin >> 1], inc);
    if (__builtin_expect((old & mask) == mask, 0)) log_wrap(bin, odd << 4, old, ev, cap, nev, error);
}

__device__ __forceinline__ double clnc_of(const double *table, unsigned long long c)
{
    if (c < 65536ull) return __ldg(table + c);
    const double x = (double)c;
    return x * log(x);
}

template <int MODE>
__device__ __forceinline__ void bucket_pair(const Binner &b, float va, float vb, int &ka, int &kb)
{
    if (MODE == 0) {
        fast_bucket_pair(b, va, vb, ka, kb);
    } else {
        ka = b.mode == 2 ? 0 : exact_bucket(b, va);
        kb = b.mode == 2 ? 0 : exact_bucket(b, vb);
    }
}

template <int MODE>
__device__ __forceinline__ void stream_pair(const Binner &bn, const float *f1, const float *f2, int64_t n,
                                            uint32_t *words, int4 *ev, int cap, unsigned int *nev, int *error)
{
    const float4 *v1 = reinterpret_cast<const float4 *>(f1);
    const float4 *v2 = reinterpret_cast<const float4 *>(f2);
    const int64_t n4 = n >> 2;
    const int bins = bn.bins;
    int64_t q = threadIdx.x;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f), y = x;
    if (q < n4) {
        x = __ldg(v1 + q);
        y = __ldg(v2 + q);
    }
    while (q < n4) {
        const int64_t qn = q + blockDim.x;
        float4 xn = x, yn = y;
        if (qn < n4) {
            xn = __ldg(v1 + qn);
            yn = __ldg(v2 + qn);
        }
        int a0, b0, a1, b1, a2, b2, a3, b3;
        bucket_pair<MODE>(bn, x.x, y.x, a0, b0);
        bucket_pair<MODE>(bn, x.y, y.y, a1, b1);
        bucket_pair<MODE>(bn, x.z, y.z, a2, b2);
        bucket_pair<MODE>(bn, x.w, y.w, a3, b3);
        count_bin(words, a0 * bins + b0, ev, cap, nev, error);
        count_bin(words, a1 * bins + b1, ev, cap, nev, error);
        count_bin(words, a2 * bins + b2, ev, cap, nev, error);
        count_bin(words, a3 * bins + b3, ev, cap, nev, error);
        x = xn;
        y = yn;
        q = qn;
    }
    for (int64_t v = (n4 << 2) + threadIdx.x; v < n; v += blockDim.x) {
        int ka, kb;
        bucket_pair<MODE>(bn, f1[v], f2[v], ka, kb);
        count_bin(words, ka * bins + kb, ev, cap, nev, error);
    }
}

__global__ void __launch_bounds__(HIST_THREADS, 1) joint_histogram_mi_kernel(PairArgs a)
{
    extern __shared__ uint32_t words[];
    __shared__ int s_task;
    __shared__ unsigned int s_nev;
    __shared__ double s_red[3][HIST_THREADS / 32];
    __shared__ unsigned long long s_colsum[ISO_MAX_BINS];
    __shared__ unsigned long long s_rowsum[ISO_MAX_BINS];

    const int bins = a.bins;
    const int nwords = bins * bins / 2;
    const int wpr = bins / 2;  // words per histogram row
    int4 *ev = a.events + (size_t)blockIdx.x * a.event_cap;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;

    for (int w = threadIdx.x; w < nwords; w += blockDim.x) words[w] = 0;

    for (;;) {
        if (threadIdx.x == 0) {
            s_task = (int)atomicAdd(a.counter, 1u);
            s_nev = 0;
        }
        for (int c = threadIdx.x; c < bins; c += blockDim.x) {
            s_colsum[c] = 0;
            s_rowsum[c] = 0;
        }
        __syncthreads();
        const int t = s_task;
        if (t >= a.num_tasks) break;
        const int2 task = a.tasks[t];
        const int i = task.x, j = task.y;

        Binner bn;
        {
            const float mn_i = bits_to_float(a.mma[2 * i]), mx_i = bits_to_float(a.mma[2 * i + 1]);
            const float mn_j = bits_to_float(a.mmb[2 * j]), mx_j = bits_to_float(a.mmb[2 * j + 1]);
            bn.mn = mn_i < mn_j ? mn_i : mn_j;
            const float mx = mx_i > mx_j ? mx_i : mx_j;
            bn.step = __fdiv_rn(__fsub_rn(mx, bn.mn), (float)bins);
            bn.bins = bins;
            bn.r = __frcp_rn(bn.step);
            bn.mode = bn.step == 0.0f ? 2 : (isfinite(bn.r) && bn.step >= 1.17549435e-38f ? 0 : 1);
        }

        const float *f1 = a.fa + (size_t)i * a.stride;
        const float *f2 = a.fb + (size_t)j * a.stride;
        const float4 *v1 = reinterpret_cast<const float4 *>(f1);
        const float4 *v2 = reinterpret_cast<const float4 *>(f2);
        const int64_t n4 = a.n >> 2;

        // streaming loop, one load pair in flight ahead of the one being binned
        if (bn.mode == 0) stream_pair<0>(bn, f1, f2, a.n, words, ev, a.event_cap, &s_nev, a.error);
        else stream_pair<1>(bn, f1, f2, a.n, words, ev, a.event_cap, &s_nev, a.error);
        __syncthreads();

        // ---- wrap corrections: per distinct bin, total correction and its
        // effect on sum(c ln c) and the marginals (events are rare: at most
        // about 2n/65536 per pair)
        const int nev = (int)(s_nev < (unsigned int)a.event_cap ? s_nev : (unsigned int)a.event_cap);
        double hxy = 0.0;
        for (int e = threadIdx.x; e < nev; e += blockDim.x) {
            const int bin = ev[e].x;
            bool first = true;
            long long corr = 0;
            for (int g = 0; g < nev; ++g) {
                if (ev[g].x != bin) continue;
                if (g < e) {
                    first = false;
                    break;
                }
                corr += ev[g].y;
            }
            if (!first) continue;
            const uint32_t c16 = (words[bin >> 1] >> ((bin & 1) << 4)) & 0xffffu;
            const unsigned long long ctrue = (unsigned long long)((long long)c16 + corr);
            hxy -= clnc_of(a.clnc, ctrue) - clnc_of(a.clnc, c16);
            atomicAdd(&s_rowsum[bin / bins], (unsigned long long)corr);
            atomicAdd(&s_colsum[bin % bins], (unsigned long long)corr);
            ev[e].z = (int)c16;
            ev[e].w = (int)ctrue;  // only read back for histogram dumps
        }
        __syncthreads();  // the bin pass below clears the words read above

        // ---- bin pass: 16-bit counts, marginals, sum(c ln c); clears the bins.
        // Thread (g, w) reads word column w of rows g, g+groups, ...
        const bool dump = a.joint_dump != nullptr;
        {
            const int groups = blockDim.x / wpr;
            const int w = threadIdx.x % wpr, g = threadIdx.x / wpr;
            if (g < groups) {
                uint32_t cs0 = 0, cs1 = 0;
                for (int r = g; r < bins; r += groups) {
                    const uint32_t word = words[r * wpr + w];
                    if (!word && !dump) continue;
                    words[r * wpr + w] = 0;
                    const uint32_t c0 = word & 0xffffu, c1 = word >> 16;
                    cs0 += c0;
                    cs1 += c1;
                    atomicAdd(&s_rowsum[r], (unsigned long long)(c0 + c1));
                    if (c0) hxy -= __ldg(a.clnc + c0);
                    if (c1) hxy -= __ldg(a.clnc + c1);
                    if (dump) {
                        const int c = 2 * w;
                        a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + c] = c0;
                        a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + c + 1] = c1;
                        if (a.symmetric && i != j) {
                            a.joint_dump[(((size_t)j * a.m + i) * bins + c) * bins + r] = c0;
                            a.joint_dump[(((size_t)j * a.m + i) * bins + c + 1) * bins + r] = c1;
                        }
                    }
                }
                if (cs0) atomicAdd(&s_colsum[2 * w], (unsigned long long)cs0);
                if (cs1) atomicAdd(&s_colsum[2 * w + 1], (unsigned long long)cs1);
            }
        }
        __syncthreads();
        if (dump && nev > 0) {
            // overwrite the corrected bins (distinct events carry c16 != or corr)
            for (int e = threadIdx.x; e < nev; e += blockDim.x) {
                const int bin = ev[e].x;
                bool first = true;
                for (int g = 0; g < e; ++g)
                    if (ev[g].x == bin) {
                        first = false;
                        break;
                    }
                if (!first) continue;
                const int r = bin / bins, c = bin % bins;
                const uint32_t val = (uint32_t)ev[e].w;
                a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + c] = val;
                if (a.symmetric && i != j) a.joint_dump[(((size_t)j * a.m + i) * bins + c) * bins + r] = val;
            }
        }
        double hx = 0.0, hy = 0.0;
        for (int c = threadIdx.x; c < bins; c += blockDim.x) {
            const unsigned long long cs = s_colsum[c], rs = s_rowsum[c];
            if (cs) hx -= clnc_of(a.clnc, cs);
            if (rs) hy -= clnc_of(a.clnc, rs);
            if (a.colrow_dump) {
                const size_t mm = (size_t)a.m * a.m * bins;
                const size_t bij = ((size_t)i * a.m + j) * bins, bji = ((size_t)j * a.m + i) * bins;
                a.colrow_dump[bij + c] = (uint32_t)cs;        // column sums of (i,j)
                a.colrow_dump[mm + bij + c] = (uint32_t)rs;   // row sums of (i,j)
                if (a.symmetric && i != j) {
                    a.colrow_dump[bji + c] = (uint32_t)rs;
                    a.colrow_dump[mm + bji + c] = (uint32_t)cs;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            hxy += __shfl_xor_sync(0xffffffffu, hxy, o);
            hx += __shfl_xor_sync(0xffffffffu, hx, o);
            hy += __shfl_xor_sync(0xffffffffu, hy, o);
        }
        if (lane == 0) {
            s_red[0][warp] = hxy;
            s_red[1][warp] = hy;
            s_red[2][warp] = hx;
        }
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
            const double iXY = sx + sy - sxy;
            const double val = 2.0 * iXY / (sx + sy);
            const float out = val != val ? 0.0f : (float)val;
            a.ism[(size_t)i * a.m + j] = out;
            if (a.symmetric) a.ism[(size_t)j * a.m + i] = out;
        }
        __syncthreads();
    }
}

__global__ void clnc_table_kernel(double *table)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < 65536) table[c] = c < 2 ? 0.0 : (double)c * log((double)c);
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
    const bool symmetric = d_fields_b == nullptr;
    const size_t max_tasks = symmetric ? (size_t)m * (m + 1) / 2 : (size_t)m * m;
    std::vector<int2> h_tasks(max_tasks);
    int num_tasks = 0;
    build_tasks(m, symmetric, h_tasks.data(), &num_tasks);
    return iso_run_similarity_tasks(ctx, d_fields_a, symmetric ? d_fields_a : d_fields_b, m, n, stride, bins, d_minmax_a,
                                    symmetric ? d_minmax_a : d_minmax_b, d_ism, h_tasks.data(), num_tasks,
                                    symmetric, d_joint_dump, d_colrow_dump);
}

int iso_run_similarity_tasks(iso_ctx *ctx, const float *d_fields_a, const float *d_fields_b, int m, int64_t n,
                             int64_t stride, int bins, const uint32_t *d_minmax_a, const uint32_t *d_minmax_b,
                             float *d_ism, const int2 *h_tasks, int64_t num_tasks_in, bool symmetric,
                             uint32_t *d_joint_dump, uint32_t *d_colrow_dump)
{
    if (num_tasks_in <= 0) return ISO_OK;
    if (num_tasks_in > 0x7fffffff) return iso_fail(ISO_ERR_ARG, "too many pair tasks");
    if (bins < 2 || bins > ISO_MAX_BINS || (bins & 1))
        return iso_fail(ISO_ERR_ARG, "bins must be even and in [2, %d], got %d", ISO_MAX_BINS, bins);
    if (stride % 4 != 0 || ((uintptr_t)d_fields_a & 15) || ((uintptr_t)d_fields_b & 15))
        return iso_fail(ISO_ERR_ARG, "field rows must be 16-byte aligned with a stride multiple of 4");
    const float *fb = d_fields_b;
    const uint32_t *mmb = d_minmax_b;
    const int num_tasks = (int)num_tasks_in;
    const size_t max_tasks = (size_t)num_tasks;

    void *d_tasks = nullptr, *d_counter = nullptr, *d_events = nullptr, *d_clnc = nullptr;
    ISO_TRY(iso_buf(ctx, BUF_PAIR_TASKS, max_tasks * sizeof(int2), &d_tasks));
    ISO_TRY(iso_buf(ctx, BUF_TASK_COUNTER, 256, &d_counter));
    ISO_CUDA(cudaMemcpyAsync(d_tasks, h_tasks, (size_t)num_tasks * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
    ISO_CUDA(cudaMemsetAsync(d_counter, 0, 2 * sizeof(unsigned int), ctx->stream));
    if (!ctx->clnc_ready) {
        ISO_TRY(iso_buf(ctx, BUF_CLNC, 65536 * sizeof(double), &d_clnc));
        clnc_table_kernel<<<256, 256, 0, ctx->stream>>>((double *)d_clnc);
        ISO_LAUNCHED(ctx);
        ctx->clnc_ready = true;
    }
    d_clnc = ctx->buf[BUF_CLNC];

    const size_t smem = (size_t)bins * bins / 2 * sizeof(uint32_t);
    ISO_CUDA(cudaFuncSetAttribute(joint_histogram_mi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(ISO_MAX_BINS * ISO_MAX_BINS / 2 * sizeof(uint32_t))));
    int per_sm = 0;
    ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, joint_histogram_mi_kernel, HIST_THREADS, smem));
    if (per_sm < 1) per_sm = 1;
    int grid = ctx->num_sms * per_sm;
    if (grid > num_tasks) grid = num_tasks;
    // wrap events per pair: each needs 65536 increments of one 16-bit half
    const int64_t event_cap = 2 * (n / 65536 + 1) + 64;
    if (event_cap > 0x7fffffff / 2) return iso_fail(ISO_ERR_ARG, "fields too long (%lld values)", (long long)n);
    ISO_TRY(iso_buf(ctx, BUF_HIST_SCRATCH, (size_t)grid * event_cap * sizeof(int4), &d_events));

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
    a.events = (int4 *)d_events;
    a.event_cap = (int)event_cap;
    a.clnc = (const double *)d_clnc;
    a.counter = (unsigned int *)d_counter;
    a.error = (int *)d_counter + 1;
    a.joint_dump = d_joint_dump;
    a.colrow_dump = d_colrow_dump;
    joint_histogram_mi_kernel<<<grid, HIST_THREADS, smem, ctx->stream>>>(a);
    ISO_LAUNCHED(ctx);
    int err = 0;
    ISO_CUDA(cudaMemcpyAsync(&err, a.error, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ISO_CUDA(cudaStreamSynchronize(ctx->stream));
    if (err) return iso_fail(ISO_ERR_INTERNAL, "joint histogram: wrap-event list overflow (code %d)", err);
    return ISO_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free similarity map
//
// For callers that must not allocate device memory while they run, for
// example a host process that hands the GPU a fixed memory budget up front,
// or code that runs where allocating would stall or fail (an allocator
// callback, a tight service loop that must not touch the driver's allocator).
// All scratch lives in one file-scope device array of fixed size, loaded with
// this library and kept by every device until the process exits.  The
// caller's fields and output are device memory the caller owns.
//
// Limits: at most ISO_NOALLOC_MAX_FIELDS fields of at most
// ISO_NOALLOC_MAX_VALUES values each, 2..256 bins (even).
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current) and fills the c*ln(c)
// table; make that first call before any stream capture.  Every call reuses
// the same array: calls that overlap on the GPU (different streams, or
// concurrent host threads on one device) race and corrupt each other.
// ---------------------------------------------------------------------------

namespace {

constexpr int NOALLOC_MAX_CTAS = 256;
constexpr int64_t NOALLOC_EVENT_CAP = 2 * (ISO_NOALLOC_MAX_VALUES / 65536 + 1) + 64;
constexpr size_t NA_OFF_CLNC = 0;
constexpr size_t NA_OFF_TASKS = NA_OFF_CLNC + 65536 * sizeof(double);
constexpr size_t NA_MAX_TASKS = (size_t)ISO_NOALLOC_MAX_FIELDS * (ISO_NOALLOC_MAX_FIELDS + 1) / 2;
constexpr size_t NA_OFF_MINMAX = (NA_OFF_TASKS + NA_MAX_TASKS * sizeof(int2) + 255) / 256 * 256;
constexpr size_t NA_OFF_CTRL = NA_OFF_MINMAX + (2 * ISO_NOALLOC_MAX_FIELDS * sizeof(uint32_t) + 255) / 256 * 256;
constexpr size_t NA_OFF_EVENTS = NA_OFF_CTRL + 256;
constexpr size_t NA_BYTES = NA_OFF_EVENTS + (size_t)NOALLOC_MAX_CTAS * NOALLOC_EVENT_CAP * sizeof(int4);

// The scratch array (about 3.2 MB).  Host code may not use this name as an
// address: it refers to a host-side stand-in; the device address comes from
// cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
struct NoAllocDevice {
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int grid = 0;
};
NoAllocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mu;

// Upper-triangle pair list, row-major (i <= j).
__global__ void noalloc_tasks_kernel(int2 *tasks, int m)
{
    const int i = blockIdx.x;
    for (int j = i + threadIdx.x; j < m; j += blockDim.x) {
        const int64_t idx = (int64_t)i * m - (int64_t)i * (i - 1) / 2 + (j - i);
        tasks[idx] = make_int2(i, j);
    }
}

int noalloc_setup(int device, NoAllocDevice **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[device];
    if (!d.scratch) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return iso_fail(ISO_ERR_CUDA, "iso_similarity_map_noalloc: cudaGetSymbolAddress failed: %s",
                            cudaGetErrorString(e));
        ISO_CUDA(cudaFuncSetAttribute(joint_histogram_mi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(ISO_MAX_BINS * ISO_MAX_BINS / 2 * sizeof(uint32_t))));
        int sms = 0, per_sm = 0;
        ISO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, joint_histogram_mi_kernel, HIST_THREADS,
                                                               ISO_MAX_BINS * ISO_MAX_BINS / 2 * sizeof(uint32_t)));
        int grid = sms * (per_sm < 1 ? 1 : per_sm);
        d.grid = grid < NOALLOC_MAX_CTAS ? grid : NOALLOC_MAX_CTAS;
        clnc_table_kernel<<<256, 256>>>((double *)((unsigned char *)p + NA_OFF_CLNC));
        ISO_CUDA(cudaGetLastError());
        ISO_CUDA(cudaDeviceSynchronize());
        d.scratch = (unsigned char *)p;
    }
    *out = &d;
    return ISO_OK;
}

}  // namespace

extern "C" int iso_similarity_map_noalloc(const float *d_fields, int m, int64_t n, int64_t stride, int bins,
                                          float *d_ism_out, void *stream)
{
    iso_clear_error();
    if (!d_fields || !d_ism_out) return iso_fail(ISO_ERR_ARG, "iso_similarity_map_noalloc: NULL pointer");
    if (m < 1 || m > ISO_NOALLOC_MAX_FIELDS)
        return iso_fail(ISO_ERR_CAPACITY, "iso_similarity_map_noalloc: %d fields; the limit is %d", m,
                        ISO_NOALLOC_MAX_FIELDS);
    if (n < 1 || n > ISO_NOALLOC_MAX_VALUES)
        return iso_fail(ISO_ERR_CAPACITY, "iso_similarity_map_noalloc: %lld values per field; the limit is %d",
                        (long long)n, ISO_NOALLOC_MAX_VALUES);
    if (bins < 2 || bins > ISO_MAX_BINS || (bins & 1))
        return iso_fail(ISO_ERR_ARG, "iso_similarity_map_noalloc: bins must be even and in [2, %d]", ISO_MAX_BINS);
    if (stride < n || stride % 4 != 0 || ((uintptr_t)d_fields & 15))
        return iso_fail(ISO_ERR_ARG,
                        "iso_similarity_map_noalloc: rows need a 16-byte aligned base and a stride >= n, multiple of 4");
    if (!iso_is_device_ptr(d_fields) || !iso_is_device_ptr(d_ism_out))
        return iso_fail(ISO_ERR_ARG, "iso_similarity_map_noalloc: fields and output must be device memory");
    int device = 0;
    ISO_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return iso_fail(ISO_ERR_ARG, "iso_similarity_map_noalloc: device %d out of range", device);
    NoAllocDevice *d = nullptr;
    ISO_TRY(noalloc_setup(device, &d));
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *base = d->scratch;
    int2 *tasks = (int2 *)(base + NA_OFF_TASKS);
    uint32_t *minmax = (uint32_t *)(base + NA_OFF_MINMAX);
    unsigned int *ctrl = (unsigned int *)(base + NA_OFF_CTRL);
    const int num_tasks = (int)((int64_t)m * (m + 1) / 2);

    // the counter and error word must start at zero; the rest is overwritten
    ISO_CUDA(cudaMemsetAsync(ctrl, 0, 2 * sizeof(unsigned int), st));
    noalloc_tasks_kernel<<<m, 256, 0, st>>>(tasks, m);
    ISO_CUDA(cudaGetLastError());
    minmax_init_kernel<<<(m + 255) / 256, 256, 0, st>>>(minmax, m);
    ISO_CUDA(cudaGetLastError());
    {
        const int64_t per = (n + 255) / 256;
        const int bx = (int)(per < 64 ? (per < 1 ? 1 : per) : 64);
        field_minmax_kernel<<<dim3(bx, m), 256, 0, st>>>(d_fields, n, stride, minmax);
        ISO_CUDA(cudaGetLastError());
    }
    PairArgs a;
    a.fa = d_fields;
    a.fb = d_fields;
    a.n = n;
    a.stride = stride;
    a.mma = minmax;
    a.mmb = minmax;
    a.tasks = tasks;
    a.num_tasks = num_tasks;
    a.m = m;
    a.bins = bins;
    a.symmetric = 1;
    a.ism = d_ism_out;
    a.events = (int4 *)(base + NA_OFF_EVENTS);
    a.event_cap = (int)NOALLOC_EVENT_CAP;
    a.clnc = (const double *)(base + NA_OFF_CLNC);
    a.counter = ctrl;
    a.error = (int *)(ctrl + 1);
    a.joint_dump = nullptr;
    a.colrow_dump = nullptr;
    const int grid = d->grid < num_tasks ? d->grid : num_tasks;
    const size_t smem = (size_t)bins * bins / 2 * sizeof(uint32_t);
    joint_histogram_mi_kernel<<<grid, HIST_THREADS, smem, st>>>(a);
    ISO_CUDA(cudaGetLastError());
    int err = 0;
    ISO_CUDA(cudaMemcpyAsync(&err, ctrl + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    ISO_CUDA(cudaStreamSynchronize(st));
    if (err) return iso_fail(ISO_ERR_INTERNAL, "iso_similarity_map_noalloc: wrap-event list overflow (code %d)", err);
    return ISO_OK;
}
