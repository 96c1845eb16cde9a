// iso_histogram.cu -- all-pairs joint histograms and FP64 normalised mutual
// information (the ISM).  Replaces calculate_histogram_g + calculateMutualInformation
// (isosurfaces_cuda/src/JointHistogram.cu:24-162).
//
// Layout: fields are rows of a [m x stride] float matrix (stride a multiple of 4,
// rows 16-byte aligned).  Per-field interval (min, max) as uint32 float bits
// (all distance values are >= 0, so bit order is value order).
//
// Kernels: persistent CTAs pull unordered pair tasks (i <= j) from a counter and
// stream both fields with 128-bit loads.  Each voxel's two buckets (the
// reference's binning: floors of the products with two widened reciprocals,
// exact IEEE division where they disagree) form one bin, counted in shared
// memory as a 16-bit half of a 32-bit word (rows of bins/2 words plus 3 pad
// words: 131 KB at 256 bins).  A half that
// wraps is seen by the thread whose atomic returned 0xFFFF, which records the
// exact correction.  Short fields: one CTA per pair, FP64 NMI in the same CTA
// (joint_histogram_mi_kernel).  Long fields: (segment, pair) tasks add into
// per-pair global histograms, reduced by joint_mi_kernel.  NMI = 2I/(hX+hY)
// from FP64 sums of c*ln(c) over the bins and over the exact row and column
// sums, written to both (i,j) and (j,i).
#include <algorithm>
#include <mutex>
#include <vector>

#include "iso_internal.cuh"

namespace {

constexpr int HIST_THREADS = 1024;

// Shared histograms pad every row, so that the same column of rows r and r + 1
// lies in different banks.  Without it a row of 256 packed counters (128
// words) or of 32 * k 32-bit counters starts in the same bank as the row
// before, and the atomics of a warp whose voxels differ only in their row bin
// (common for two similar fields) all hit one bank.
//   packed 16-bit counters: counter index row * (bins + 2 * PACKED_PAD) + col,
//                           word = index / 2 (PACKED_PAD pad words per row)
//   32-bit counters:        counter index row * (bins + 1) + col
// Three pad words rather than one: 4 % fewer shared-memory wavefronts per
// atomic on the distance fields of a 128^3 volume (a CPU model of the bank
// conflicts over 28 field pairs: 4.88 unpadded, 3.54 with one, 3.39 with three).
constexpr int PACKED_PAD = 3;
__host__ __device__ constexpr int packed_stride(int bins) { return bins + 2 * PACKED_PAD; }
__host__ __device__ constexpr int packed_row_words(int bins) { return bins / 2 + PACKED_PAD; }
__host__ __device__ constexpr int packed_words(int bins) { return bins * (bins / 2 + PACKED_PAD); }
__host__ __device__ constexpr int wide_stride(int bins) { return bins + 1; }
__host__ __device__ constexpr int wide_words(int bins) { return bins * (bins + 1); }

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
    float mn, step;
    float rlo, rhi;  // RN(1/step) widened down and up (mode 0)
    int bins;
    int rstride;     // counter index of (row, col) = row * rstride + col (padded rows)
    int mode;  // 0: bracketed reciprocal with exact fallback, 1: exact division only, 2: step == 0
};



// Exact bucket of JointHistogram.cu:63-75 (IEEE division), clamped to [0, bins).
__device__ __forceinline__ int exact_bucket(const Binner &b, float v) { return iso_bucket(v, b.mn, b.step, b.bins); }

// Bins of four voxels by IEEE division.  Out of line: the exact path is rare
// in mode 0 and would otherwise cost registers in the streaming loop.
__device__ __noinline__ int4 exact_bins4(float mn, float step, int bins, int rs, float4 x, float4 y)
{
    return make_int4(iso_bucket(x.x, mn, step, bins) * rs + iso_bucket(y.x, mn, step, bins),
                     iso_bucket(x.y, mn, step, bins) * rs + iso_bucket(y.y, mn, step, bins),
                     iso_bucket(x.z, mn, step, bins) * rs + iso_bucket(y.z, mn, step, bins),
                     iso_bucket(x.w, mn, step, bins) * rs + iso_bucket(y.w, mn, step, bins));
}

// ---- bracketed floor bucket ----------------------------------------------
// With d = RN(v - mn) >= 0, r = RN(1/step), rlo = RD(r * (1 - 2^-22)) and
// rhi = RU(r * (1 + 2^-22)): r lies within a relative 2^-24 of 1/step and the
// reference's quotient q = RN(d / step) within a relative 2^-24 of d / step,
// so d * rlo <= q <= d * rhi and floor(d * rlo) <= floor(q) <= floor(d * rhi).
// Two packed FMAs give both floors exactly:
//   lo = RD(d * rlo + 2^23)   = 2^23 + floor(d * rlo)  (ulp 1 in [2^23, 2^24)),
//   hi = RU(d * -rhi - 2^23)  = -(2^23 + floor(d * rhi)),
// and lo + hi = floor(d * rlo) - floor(d * rhi) <= 0 is exact.  Where it is 0
// (+0.0, all bits clear) the bucket is bits(lo) - bits(2^23).  One OR over the
// bits of the eight sums of four voxels is 0 exactly when every pair of floors
// agrees; a NaN value gives a NaN sum, whose bits are not 0.  Otherwise the
// four voxels take the division, which happens for about 2^-21 * q of the
// values.  Near q = bins the bucket is clamped to the last bin on both paths.
constexpr float FLOOR_BASE = 8388608.0f;  // 2^23
constexpr uint32_t FLOOR_BASE_BITS = 0x4B000000u;

// The same four voxels, loaded again from p1[q], p2[q]: the rare exact path
// reloads them, so the streaming loop does not keep x and y alive across the
// bucket arithmetic.
__device__ __noinline__ int4 exact_bins4_at(float mn, float step, int bins, int rs, const float4 *p1, const float4 *p2,
                                            int q)
{
    return exact_bins4(mn, step, bins, rs, __ldg(p1 + q), __ldg(p2 + q));
}

// Bins (row = field-1 bucket, column = field-2 bucket) of the four voxels in
// x = p1[q], y = p2[q].  FB / FRS: bins and row stride as compile-time
// constants (0: read from the binner), which keeps them out of registers in
// the streaming loop.  RELOAD: the exact path loads the voxels again instead
// of keeping x and y.
template <int MODE, int FB, int FRS, bool RELOAD>
__device__ __forceinline__ void bins4(const Binner &bn, const float4 &x, const float4 &y, const float4 *p1,
                                      const float4 *p2, int q, int &b0, int &b1, int &b2, int &b3)
{
    const int bins = FB ? FB : bn.bins;
    const int rstride = FRS ? FRS : bn.rstride;
    if (MODE == 0) {
        const float2 nm = make_float2(-bn.mn, -bn.mn);
        const float2 rl = make_float2(bn.rlo, bn.rlo), nrh = make_float2(-bn.rhi, -bn.rhi);
        const float2 pb = make_float2(FLOOR_BASE, FLOOR_BASE), nb = make_float2(-FLOOR_BASE, -FLOOR_BASE);
        const float2 dx01 = __fadd2_rn(make_float2(x.x, x.y), nm), dx23 = __fadd2_rn(make_float2(x.z, x.w), nm);
        const float2 dy01 = __fadd2_rn(make_float2(y.x, y.y), nm), dy23 = __fadd2_rn(make_float2(y.z, y.w), nm);
        const float2 lx01 = __ffma2_rd(dx01, rl, pb), lx23 = __ffma2_rd(dx23, rl, pb);
        const float2 ly01 = __ffma2_rd(dy01, rl, pb), ly23 = __ffma2_rd(dy23, rl, pb);
        const float2 hx01 = __ffma2_ru(dx01, nrh, nb), hx23 = __ffma2_ru(dx23, nrh, nb);
        const float2 hy01 = __ffma2_ru(dy01, nrh, nb), hy23 = __ffma2_ru(dy23, nrh, nb);
        const float2 zx01 = __fadd2_rn(lx01, hx01), zx23 = __fadd2_rn(lx23, hx23);
        const float2 zy01 = __fadd2_rn(ly01, hy01), zy23 = __fadd2_rn(ly23, hy23);
        // bucket = bits(lo) - bits(2^23).  The generic instance (FB == 0)
        // clamps it to bins - 1 as unsigned, so that any input (also one above
        // a caller's interval) stays inside the histogram.  The specialised
        // instances run only where every value v lies in its pair's interval
        // (the dispatch picks the generic one otherwise), and there no clamp
        // is needed: d = RN(v - mn) <= RN(mx - mn) = range, and with
        // step = RN(range / bins) >= (range / bins)(1 - 2^-24) and
        // r <= (1 / step)(1 + 2^-24), range * rlo <= bins (1 + 2^-24)
        // (1 - 2^-22) / (1 - 2^-24) < bins, so lo < 2^23 + bins.
        const uint32_t top = (uint32_t)(bins - 1);
        const uint32_t ub = (uint32_t)rstride;
        auto bucket = [&](float lo) {
            const uint32_t b = __float_as_uint(lo) - FLOOR_BASE_BITS;
            return FB ? b : min(b, top);
        };
        b0 = (int)(bucket(lx01.x) * ub + bucket(ly01.x));
        b1 = (int)(bucket(lx01.y) * ub + bucket(ly01.y));
        b2 = (int)(bucket(lx23.x) * ub + bucket(ly23.x));
        b3 = (int)(bucket(lx23.y) * ub + bucket(ly23.y));
        const bool slow = ((__float_as_uint(zx01.x) | __float_as_uint(zx01.y) | __float_as_uint(zx23.x) |
                            __float_as_uint(zx23.y) | __float_as_uint(zy01.x) | __float_as_uint(zy01.y) |
                            __float_as_uint(zy23.x) | __float_as_uint(zy23.y)) != 0u);
        if (__builtin_expect(slow, 0)) {
            const int4 e = RELOAD ? exact_bins4_at(bn.mn, bn.step, bins, rstride, p1, p2, q)
                                  : exact_bins4(bn.mn, bn.step, bins, rstride, x, y);
            b0 = e.x;
            b1 = e.y;
            b2 = e.z;
            b3 = e.w;
        }
    } else {
        b0 = exact_bucket(bn, x.x) * rstride + exact_bucket(bn, y.x);
        b1 = exact_bucket(bn, x.y) * rstride + exact_bucket(bn, y.y);
        b2 = exact_bucket(bn, x.z) * rstride + exact_bucket(bn, y.z);
        b3 = exact_bucket(bn, x.w) * rstride + exact_bucket(bn, y.w);
    }
}

// A bin is counted as a 16-bit half of a shared 32-bit word.  The old word an
// atomic returns tells its thread exactly when a half wraps: the low half's 16 bits
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

// Counts four bins.  A bin is a 16-bit half of word bin/2 (odd bins in the
// high half); its increment is 1 or 65536.  old * (increment ^ 0x10001), i.e.
// old * 65536 for the low half and old * 1 for the high half, moves the
// counted half of the old word to the top 16 bits, so the half wrapped exactly
// when that product is >= 0xFFFF0000; one test covers the four updates, and
// the rare wraps go to wrap(bin, odd, old).
template <class Wrap>
__device__ __forceinline__ void count4(uint32_t *words, int b0, int b1, int b2, int b3, const Wrap &wrap)
{
    const uint32_t o0 = (uint32_t)b0 & 1u, o1 = (uint32_t)b1 & 1u, o2 = (uint32_t)b2 & 1u, o3 = (uint32_t)b3 & 1u;
    const uint32_t i0 = o0 * 0xFFFFu + 1u, i1 = o1 * 0xFFFFu + 1u, i2 = o2 * 0xFFFFu + 1u, i3 = o3 * 0xFFFFu + 1u;
    const uint32_t old0 = atomicAdd(&words[b0 >> 1], i0);
    const uint32_t old1 = atomicAdd(&words[b1 >> 1], i1);
    const uint32_t old2 = atomicAdd(&words[b2 >> 1], i2);
    const uint32_t old3 = atomicAdd(&words[b3 >> 1], i3);
    const uint32_t t0 = old0 * (i0 ^ 0x10001u), t1 = old1 * (i1 ^ 0x10001u);
    const uint32_t t2 = old2 * (i2 ^ 0x10001u), t3 = old3 * (i3 ^ 0x10001u);
    if (__builtin_expect(max(max(t0, t1), max(t2, t3)) >= 0xFFFF0000u, 0)) {
        if (t0 >= 0xFFFF0000u) wrap(b0, o0, old0);
        if (t1 >= 0xFFFF0000u) wrap(b1, o1, old1);
        if (t2 >= 0xFFFF0000u) wrap(b2, o2, old2);
        if (t3 >= 0xFFFF0000u) wrap(b3, o3, old3);
    }
}

template <class Wrap>
__device__ __forceinline__ void count1(uint32_t *words, int bin, const Wrap &wrap)
{
    const uint32_t odd = (uint32_t)bin & 1u;
    const uint32_t old = atomicAdd(&words[bin >> 1], odd * 0xFFFFu + 1u);
    if (old * (65536u - odd * 65535u) >= 0xFFFF0000u) wrap(bin, odd, old);
}

__device__ __forceinline__ double clnc_of(const double *table, unsigned long long c)
{
    if (c < 65536ull) return __ldg(table + c);
    const double x = (double)c;
    return x * log(x);
}

// Streams values [v0, v1) of one field pair (v0 a multiple of 4, rows 16-byte
// aligned) into a shared histogram through count.add4 / count.add1.  Two load
// pairs alternate so that one is in flight while the other is binned.  Blocks
// of HIST_THREADS threads; CSTEP: that block size as a constant instead of
// blockDim.x (the compiler's register allocation in this loop, and with it the
// kernel's speed, depends on the choice: each kernel uses the faster one).
template <int MODE, int FB, int FRS, bool CSTEP, bool RELOAD, class Count>
__device__ __forceinline__ void stream_values(const Binner &bn, const float *f1, const float *f2, int64_t v0,
                                              int64_t v1, const Count &count)
{
    const float4 *p1 = reinterpret_cast<const float4 *>(f1 + v0);
    const float4 *p2 = reinterpret_cast<const float4 *>(f2 + v0);
    const int n4 = (int)((v1 - v0) >> 2);
    const int step = CSTEP ? HIST_THREADS : (int)blockDim.x;
    int q = (int)threadIdx.x;
    float4 xa = make_float4(0.f, 0.f, 0.f, 0.f), ya = xa, xb = xa, yb = xa;
    if (q < n4) {
        xa = __ldg(p1 + q);
        ya = __ldg(p2 + q);
    }
    while (q < n4) {
        const int qb = q + step;
        if (qb < n4) {
            xb = __ldg(p1 + qb);
            yb = __ldg(p2 + qb);
        }
        int c0, c1, c2, c3;
        bins4<MODE, FB, FRS, RELOAD>(bn, xa, ya, p1, p2, q, c0, c1, c2, c3);
        count.add4(c0, c1, c2, c3);
        if (qb >= n4) break;
        const int qa = qb + step;
        if (qa < n4) {
            xa = __ldg(p1 + qa);
            ya = __ldg(p2 + qa);
        }
        bins4<MODE, FB, FRS, RELOAD>(bn, xb, yb, p1, p2, qb, c0, c1, c2, c3);
        count.add4(c0, c1, c2, c3);
        q = qa;
    }
    for (int64_t v = v0 + ((int64_t)n4 << 2) + threadIdx.x; v < v1; v += step) {
        const int bin = bn.mode == 2 ? 0 : exact_bucket(bn, f1[v]) * bn.rstride + exact_bucket(bn, f2[v]);
        count.add1(bin);
    }
}

// Wraps logged as per-CTA events (fused kernel).
struct EventWrap {
    int4 *ev;
    int cap;
    unsigned int *nev;
    int *error;
    __device__ __forceinline__ void operator()(int bin, uint32_t odd, uint32_t old) const
    {
        log_wrap(bin, odd << 4, old, ev, cap, nev, error);
    }
};

// Packed 16-bit counters (two bins per word) with exact wrap handling.
template <class Wrap>
struct Counter {
    uint32_t *words;
    Wrap wrap;
    __device__ __forceinline__ void add4(int b0, int b1, int b2, int b3) const { count4(words, b0, b1, b2, b3, wrap); }
    __device__ __forceinline__ void add1(int bin) const { count1(words, bin, wrap); }
};

// One 32-bit counter per bin (histograms of up to WIDE_MAX_BINS^2 bins): no
// halves, no wraps (a pair has fewer than 2^32 values), and the atomics'
// results are unused.
struct WideCounter {
    uint32_t *words;
    __device__ __forceinline__ void add4(int b0, int b1, int b2, int b3) const
    {
        atomicAdd(&words[b0], 1u);
        atomicAdd(&words[b1], 1u);
        atomicAdd(&words[b2], 1u);
        atomicAdd(&words[b3], 1u);
    }
    __device__ __forceinline__ void add1(int bin) const { atomicAdd(&words[bin], 1u); }
};

// Interval of one pair: the union of both fields' intervals; step, reciprocal
// and the bucket mode (JointHistogram.cu:100-120).
__device__ __forceinline__ Binner make_binner(const uint32_t *mma, const uint32_t *mmb, int i, int j, int bins,
                                              int rstride)
{
    Binner bn;
    bn.rstride = rstride;
    const float mn_i = bits_to_float(mma[2 * i]), mx_i = bits_to_float(mma[2 * i + 1]);
    const float mn_j = bits_to_float(mmb[2 * j]), mx_j = bits_to_float(mmb[2 * j + 1]);
    bn.mn = mn_i < mn_j ? mn_i : mn_j;
    const float mx = mx_i > mx_j ? mx_i : mx_j;
    bn.step = __fdiv_rn(__fsub_rn(mx, bn.mn), (float)bins);
    bn.bins = bins;
    const float r = __frcp_rn(bn.step);
    bn.rlo = __fmul_rd(r, 0.99999976158142089844f);  // 1 - 2^-22
    bn.rhi = __fmul_ru(r, 1.00000023841857910156f);  // 1 + 2^-22
    // mode 0 needs a finite interval (every non-NaN value then lies in it) and
    // a normal, finite step with finite nonzero reciprocals
    bn.mode = bn.step == 0.0f ? 2
              : (isfinite(bn.step) && bn.step >= 1.17549435e-38f && isfinite(r) && r >= 1.17549435e-38f &&
                         isfinite(bn.rhi)
                     ? 0
                     : 1);
    return bn;
}

template <int FB, bool CSTEP, bool RELOAD>
__global__ void __launch_bounds__(HIST_THREADS, 1) joint_histogram_mi_kernel(PairArgs a)
{
    constexpr int FRS = FB ? packed_stride(FB) : 0;
    extern __shared__ uint32_t words[];
    __shared__ int s_task;
    __shared__ unsigned int s_nev;
    __shared__ double s_red[3][HIST_THREADS / 32];
    __shared__ uint32_t s_colsum[ISO_MAX_BINS];  // marginals (n < 2^32)
    __shared__ uint32_t s_rowsum[ISO_MAX_BINS];

    const int bins = a.bins;
    const int nwords = packed_words(bins);
    const int wpr = bins / 2;                   // counter words per histogram row
    const int wps = packed_row_words(bins);     // words per padded row
    const int rs = packed_stride(bins);
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

        const Binner bn = make_binner(a.mma, a.mmb, i, j, bins, rs);

        const float *f1 = a.fa + (size_t)i * a.stride;
        const float *f2 = a.fb + (size_t)j * a.stride;

        // streaming loop, one load pair in flight ahead of the one being binned
        const Counter<EventWrap> cnt{words, EventWrap{ev, a.event_cap, &s_nev, a.error}};
        if (bn.mode == 0) stream_values<0, FB, FRS, CSTEP, RELOAD>(bn, f1, f2, 0, a.n, cnt);
        else stream_values<1, FB, FRS, CSTEP, RELOAD>(bn, f1, f2, 0, a.n, cnt);
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
            atomicAdd(&s_rowsum[bin / rs], (uint32_t)corr);  // modular: corr may be negative
            atomicAdd(&s_colsum[bin % rs], (uint32_t)corr);
            ev[e].z = (int)c16;
            ev[e].w = (int)ctrue;  // only read back for histogram dumps
        }
        __syncthreads();  // the bin pass below clears the words read above

        // ---- bin pass: 16-bit counts, marginals, sum(c ln c); clears the bins.
        // Thread (g, w) reads word column w of rows g, g+groups, ...  With a
        // multiple of 32 words per row a warp covers part of one row, and a
        // warp sum replaces the per-thread row-sum atomics.
        const bool dump = a.joint_dump != nullptr;
        // the transposed copy (pair (j, i)) is written column by column in a
        // pass of its own, so the bin pass leaves the counters to it
        const bool tdump = dump && a.symmetric && i != j;
        {
            const int groups = blockDim.x / wpr;
            const int w = threadIdx.x % wpr, g = threadIdx.x / wpr;
            const bool warp_rows = (wpr & 31) == 0;
            if (g < groups) {
                uint32_t cs0 = 0, cs1 = 0;
                for (int r = g; r < bins; r += groups) {
                    const uint32_t word = words[r * wps + w];
                    uint32_t c0 = 0, c1 = 0;
                    if (word || dump) {
                        if (!tdump) words[r * wps + w] = 0;
                        c0 = word & 0xffffu;
                        c1 = word >> 16;
                        cs0 += c0;
                        cs1 += c1;
                        if (c0) hxy -= __ldg(a.clnc + c0);
                        if (c1) hxy -= __ldg(a.clnc + c1);
                        if (dump)  // bins is even: 8-byte aligned, adjacent lanes adjacent
                            *reinterpret_cast<uint2 *>(a.joint_dump + (((size_t)i * a.m + j) * bins + r) * bins +
                                                       2 * w) = make_uint2(c0, c1);
                    }
                    if (warp_rows) {
                        const uint32_t rs = __reduce_add_sync(0xffffffffu, c0 + c1);
                        if (lane == 0 && rs) atomicAdd(&s_rowsum[r], rs);
                    } else if (c0 + c1) {
                        atomicAdd(&s_rowsum[r], c0 + c1);
                    }
                }
                if (cs0) atomicAdd(&s_colsum[2 * w], cs0);
                if (cs1) atomicAdd(&s_colsum[2 * w + 1], cs1);
            }
        }
        __syncthreads();
        if (tdump) {
            // lanes take consecutive rows r of one counter-word column: two
            // 128-byte stores per warp, and shared reads wps = bins/2 + 3
            // words apart (odd for a multiple of 4 bins: conflict-free)
            uint32_t *tj = a.joint_dump + ((size_t)j * a.m + i) * bins * bins;
            for (int idx = threadIdx.x; idx < wpr * bins; idx += blockDim.x) {
                const int w = idx / bins, r = idx - w * bins;
                const uint32_t word = words[r * wps + w];
                words[r * wps + w] = 0;
                tj[(size_t)(2 * w) * bins + r] = word & 0xffffu;
                tj[(size_t)(2 * w + 1) * bins + r] = word >> 16;
            }
            __syncthreads();  // the corrected bins below overwrite these
        }
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
                const int r = bin / rs, c = bin % rs;
                const uint32_t val = (uint32_t)ev[e].w;
                a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + c] = val;
                if (a.symmetric && i != j) a.joint_dump[(((size_t)j * a.m + i) * bins + c) * bins + r] = val;
            }
        }
        double hx = 0.0, hy = 0.0;
        for (int c = threadIdx.x; c < bins; c += blockDim.x) {
            const unsigned long long cs = s_colsum[c], rs = s_rowsum[c];  // exact: true sums < 2^32
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

// ---------------------------------------------------------------------------
// 32-bit counters for up to WIDE_MAX_BINS bins
//
// A bins^2 histogram of 32-bit counters fits in shared memory up to 224 bins
// (196 KB): each voxel is one plain atomic add, without the packed halves'
// parity, increment and wrap checks.  Same tasks, bucket arithmetic and FP64
// NMI as joint_histogram_mi_kernel.
// ---------------------------------------------------------------------------

constexpr int WIDE_MAX_BINS = ISO_WIDE_MAX_BINS;

template <int FB>
__global__ void __launch_bounds__(HIST_THREADS, 1) joint_histogram_wide_kernel(PairArgs a)
{
    constexpr int FRS = FB ? wide_stride(FB) : 0;
    extern __shared__ uint32_t words[];
    __shared__ int s_task;
    __shared__ double s_red[3][HIST_THREADS / 32];
    __shared__ uint32_t s_colsum[WIDE_MAX_BINS];  // marginals (n < 2^32)
    __shared__ uint32_t s_rowsum[WIDE_MAX_BINS];

    const int bins = a.bins;
    const int nb = bins * bins;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    // with a multiple of 32 bins a warp reads part of one row; with a divisor
    // of the block size as bins each thread reads one column
    const bool warp_rows = (bins & 31) == 0;
    const bool col_own = (blockDim.x % bins) == 0;
    for (int w = threadIdx.x; w < wide_words(bins); w += blockDim.x) words[w] = 0;

    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(a.counter, 1u);
        for (int c = threadIdx.x; c < bins; c += blockDim.x) {
            s_colsum[c] = 0;
            s_rowsum[c] = 0;
        }
        __syncthreads();
        const int t = s_task;
        if (t >= a.num_tasks) break;
        const int2 task = a.tasks[t];
        const int i = task.x, j = task.y;
        const Binner bn = make_binner(a.mma, a.mmb, i, j, bins, wide_stride(bins));
        const float *f1 = a.fa + (size_t)i * a.stride;
        const float *f2 = a.fb + (size_t)j * a.stride;
        const WideCounter cnt{words};
        if (bn.mode == 0) stream_values<0, FB, FRS, false, true>(bn, f1, f2, 0, a.n, cnt);
        else stream_values<1, FB, FRS, false, true>(bn, f1, f2, 0, a.n, cnt);
        __syncthreads();

        // bins: sum(c ln c), marginals, optional dump; clears the counters
        const bool dump = a.joint_dump != nullptr;
        const bool tdump = dump && a.symmetric && i != j;  // transposed copy: a pass of its own
        double hxy = 0.0;
        uint32_t cs = 0;
        for (int idx = threadIdx.x; idx < nb; idx += blockDim.x) {
            const int r = idx / bins, col = idx - r * bins;
            const uint32_t c = words[idx + r];  // padded row r starts at r * (bins + 1)
            if (c) {
                if (!tdump) words[idx + r] = 0;
                hxy -= clnc_of(a.clnc, c);
            }
            if (dump) a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + col] = c;
            if (warp_rows) {
                const uint32_t rs = __reduce_add_sync(0xffffffffu, c);
                if (lane == 0 && rs) atomicAdd(&s_rowsum[r], rs);
            } else if (c) {
                atomicAdd(&s_rowsum[r], c);
            }
            if (col_own) cs += c;
            else if (c) atomicAdd(&s_colsum[col], c);
        }
        if (col_own && cs) atomicAdd(&s_colsum[threadIdx.x % bins], cs);
        __syncthreads();
        if (tdump) {
            // lanes take consecutive rows of one column: coalesced stores, and
            // shared reads bins + 1 words apart
            uint32_t *tj = a.joint_dump + ((size_t)j * a.m + i) * nb;
            for (int idx = threadIdx.x; idx < nb; idx += blockDim.x) {
                const int col = idx / bins, r = idx - col * bins;
                tj[idx] = words[r * (bins + 1) + col];
                words[r * (bins + 1) + col] = 0;
            }
            __syncthreads();
        }
        double hx = 0.0, hy = 0.0;
        for (int c = threadIdx.x; c < bins; c += blockDim.x) {
            const unsigned long long cs64 = s_colsum[c], rs64 = s_rowsum[c];
            if (cs64) hx -= clnc_of(a.clnc, cs64);
            if (rs64) hy -= clnc_of(a.clnc, rs64);
            if (a.colrow_dump) {
                const size_t mm = (size_t)a.m * a.m * bins;
                const size_t bij = ((size_t)i * a.m + j) * bins, bji = ((size_t)j * a.m + i) * bins;
                a.colrow_dump[bij + c] = (uint32_t)cs64;
                a.colrow_dump[mm + bij + c] = (uint32_t)rs64;
                if (a.symmetric && i != j) {
                    a.colrow_dump[bji + c] = (uint32_t)rs64;
                    a.colrow_dump[mm + bji + c] = (uint32_t)cs64;
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

// ---------------------------------------------------------------------------
// Segment-major schedule for long fields
//
// With fields of many megabytes, pairs running concurrently drift apart along
// the voxel axis and their working set outgrows L2, so every pair re-reads its
// fields from DRAM.  Here a task is (voxel segment, pair).  The pairs of a
// chunk (up to ISO_HIST_CHUNK_BYTES of global histograms) run segment by
// segment, in 16 x 16 tiles of pairs within a segment, so the running CTAs
// read the same slice of a few fields.  A task's shared-memory histogram is added
// into the pair's global histogram (16-bit wraps corrected directly there);
// joint_mi_kernel then reduces each global histogram to its NMI.
// ---------------------------------------------------------------------------

struct SegArgs {
    const float *fa, *fb;
    int64_t n, stride;
    int64_t seg_len;     // values per task and field
    const uint32_t *mma, *mmb;
    const int2 *tasks;   // the chunk's pairs
    int num_pairs, num_segs, bins;
    int group;           // pairs whose segments run together (the whole chunk)
    uint32_t *ghist;     // num_pairs x bins*bins
    unsigned int *counter;
    // precomputed row buckets (row_code_kernel) of the fields of fa and fb,
    // or null: then every pair computes both buckets from the values
    const uint32_t *codes_a, *codes_b;
};

// Wrap corrections straight into the pair's global histogram (see count4):
// lo and hi are the global indices of the word's low and high counters.
__device__ __noinline__ void log_wrap_global(uint32_t *gh, int lo, int hi, uint32_t odd, uint32_t old)
{
    if (!odd) {
        atomicAdd(&gh[lo], 65536u);
        atomicAdd(&gh[hi], 0xFFFFFFFFu);  // -1: the carry the high half received
        if ((old >> 16) == 0xffffu) atomicAdd(&gh[hi], 65536u);
    } else {
        atomicAdd(&gh[hi], 65536u);
    }
}

// Wraps corrected straight in the pair's global histogram (segment-major
// kernel).  The global histogram is unpadded, row = bucket of the pair's
// first field: shared counter (r, c) at index r * packed_stride(bins) + c is
// global (r, c), or global (c, r) when the shared histogram is transposed
// (its rows are the pair's second field).
struct GlobalWrap {
    uint32_t *gh;
    int rs;  // packed_stride(bins)
    int bins;
    int transposed;
    __device__ __forceinline__ void operator()(int bin, uint32_t odd, uint32_t old) const
    {
        const int r = bin / rs, c0 = (bin - r * rs) & ~1;
        if (transposed) log_wrap_global(gh, c0 * bins + r, (c0 + 1) * bins + r, odd, old);
        else log_wrap_global(gh, r * bins + c0, r * bins + c0 + 1, odd, old);
    }
};

// ---- precomputed row buckets ----------------------------------------------
// For the segment-major schedule a field's bucket is computed once and reused
// by every pair in which that field has the larger maximum M.  Such a pair's
// interval is [mn, M] with mn between the smallest minimum of all fields
// (m_lo) and the field's own minimum (m_f), and its bucket of value v is
// clamp(trunc(RN(RN(v - mn) / RN(RN(M - mn) / bins)))).  RN is monotone, so
// RN(v - mn) lies in [RN(v - m_f), RN(v - m_lo)], the step in
// [RN(RN(M - m_f)/bins), RN(RN(M - m_lo)/bins)], and the quotient, monotone in
// both, in [RN(d_lo / s_hi), RN(d_hi / s_lo)]: where both ends give the same
// bucket, that is the bucket for every such pair.  The code is that bucket
// times the shared-histogram row stride, or CODE_UNSTABLE (the pair then
// divides, as for any other value near a bucket edge).
constexpr uint32_t CODE_UNSTABLE = 0x80000000u;

__global__ void min_of_mins_kernel(const uint32_t *mma, int ma, const uint32_t *mmb, int mb, uint32_t *out)
{
    // minima are non-negative floats: their bit patterns order like the values
    uint32_t v = 0xffffffffu;
    for (int k = threadIdx.x; k < ma; k += blockDim.x) v = min(v, mma[2 * k]);
    for (int k = threadIdx.x; k < mb; k += blockDim.x) v = min(v, mmb[2 * k]);
    v = __reduce_min_sync(0xffffffffu, v);
    __shared__ uint32_t red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t u = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0xffffffffu;
        u = __reduce_min_sync(0xffffffffu, u);
        if (threadIdx.x == 0) *out = u;
    }
}

__global__ void row_code_kernel(const float *fields, int64_t n, int64_t stride, const uint32_t *minmax,
                                const uint32_t *m_lo_bits, int bins, int rs, uint32_t *codes)
{
    const int f = blockIdx.y;
    const float mf = bits_to_float(minmax[2 * f]), M = bits_to_float(minmax[2 * f + 1]);
    const float mlo = bits_to_float(*m_lo_bits);
    const float s_lo = __fdiv_rn(__fsub_rn(M, mf), (float)bins), s_hi = __fdiv_rn(__fsub_rn(M, mlo), (float)bins);
    const bool usable = s_lo >= 1.17549435e-38f && isfinite(s_hi) && mlo <= mf;
    const float *src = fields + (size_t)f * stride;
    uint32_t *dst = codes + (size_t)f * stride;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const float x = src[v];
        uint32_t code = CODE_UNSTABLE;
        if (usable && x == x) {
            const float q_lo = __fdiv_rn(__fsub_rn(x, mf), s_hi), q_hi = __fdiv_rn(__fsub_rn(x, mlo), s_lo);
            int b_lo = __float2int_rz(q_lo), b_hi = __float2int_rz(q_hi);
            b_lo = b_lo >= bins ? bins - 1 : (b_lo < 0 ? 0 : b_lo);
            b_hi = b_hi >= bins ? bins - 1 : (b_hi < 0 ? 0 : b_hi);
            if (b_lo == b_hi && q_lo >= 0.0f) code = (uint32_t)(b_lo * rs);
        }
        dst[v] = code;
    }
}

// As stream_values, with the first side's buckets read from its codes: the
// second side's buckets come from the bracketed floors, and any voxel whose
// code is CODE_UNSTABLE or whose floors disagree takes the divisions of both
// sides (from the values, reloaded from fcode and fother).
template <int FB, int FRS, bool CSTEP, class Count>
__device__ __forceinline__ void stream_coded(const Binner &bn, const uint32_t *codes, const float *fcode,
                                             const float *fother, int64_t v0, int64_t v1, const Count &count)
{
    const uint4 *pc = reinterpret_cast<const uint4 *>(codes + v0);
    const float4 *p1 = reinterpret_cast<const float4 *>(fcode + v0);
    const float4 *p2 = reinterpret_cast<const float4 *>(fother + v0);
    const int bins = FB ? FB : bn.bins;
    const int rstride = FRS ? FRS : bn.rstride;
    const int n4 = (int)((v1 - v0) >> 2);
    const int step = CSTEP ? HIST_THREADS : (int)blockDim.x;
    const float2 nm = make_float2(-bn.mn, -bn.mn);
    const float2 rl = make_float2(bn.rlo, bn.rlo), nrh = make_float2(-bn.rhi, -bn.rhi);
    const float2 pb = make_float2(FLOOR_BASE, FLOOR_BASE), nb = make_float2(-FLOOR_BASE, -FLOOR_BASE);
    const uint32_t top = (uint32_t)(bins - 1);
    int q = (int)threadIdx.x;
    uint4 ca = make_uint4(0u, 0u, 0u, 0u), cb = ca;
    float4 ya = make_float4(0.f, 0.f, 0.f, 0.f), yb = ya;
    if (q < n4) {
        ca = __ldg(pc + q);
        ya = __ldg(p2 + q);
    }
    auto bin_and_count = [&](const uint4 &c, const float4 &y, int qq) {
        const float2 dy01 = __fadd2_rn(make_float2(y.x, y.y), nm), dy23 = __fadd2_rn(make_float2(y.z, y.w), nm);
        const float2 ly01 = __ffma2_rd(dy01, rl, pb), ly23 = __ffma2_rd(dy23, rl, pb);
        const float2 hy01 = __ffma2_ru(dy01, nrh, nb), hy23 = __ffma2_ru(dy23, nrh, nb);
        const float2 zy01 = __fadd2_rn(ly01, hy01), zy23 = __fadd2_rn(ly23, hy23);
        int b0 = (int)(c.x + min(__float_as_uint(ly01.x) - FLOOR_BASE_BITS, top));
        int b1 = (int)(c.y + min(__float_as_uint(ly01.y) - FLOOR_BASE_BITS, top));
        int b2 = (int)(c.z + min(__float_as_uint(ly23.x) - FLOOR_BASE_BITS, top));
        int b3 = (int)(c.w + min(__float_as_uint(ly23.y) - FLOOR_BASE_BITS, top));
        const bool slow = (((c.x | c.y | c.z | c.w) & CODE_UNSTABLE) |
                           (__float_as_uint(zy01.x) | __float_as_uint(zy01.y) | __float_as_uint(zy23.x) |
                            __float_as_uint(zy23.y))) != 0u;
        if (__builtin_expect(slow, 0)) {
            const int4 e = exact_bins4_at(bn.mn, bn.step, bins, rstride, p1, p2, qq);
            b0 = e.x;
            b1 = e.y;
            b2 = e.z;
            b3 = e.w;
        }
        count.add4(b0, b1, b2, b3);
    };
    while (q < n4) {
        const int qb = q + step;
        if (qb < n4) {
            cb = __ldg(pc + qb);
            yb = __ldg(p2 + qb);
        }
        bin_and_count(ca, ya, q);
        if (qb >= n4) break;
        const int qa = qb + step;
        if (qa < n4) {
            ca = __ldg(pc + qa);
            ya = __ldg(p2 + qa);
        }
        bin_and_count(cb, yb, qb);
        q = qa;
    }
    for (int64_t v = v0 + ((int64_t)n4 << 2) + threadIdx.x; v < v1; v += step)
        count.add1(exact_bucket(bn, fcode[v]) * bn.rstride + exact_bucket(bn, fother[v]));
}

template <int FB, bool CSTEP, bool RELOAD>
__global__ void __launch_bounds__(HIST_THREADS, 1) joint_histogram_seg_kernel(SegArgs a)
{
    constexpr int FRS = FB ? packed_stride(FB) : 0;
    extern __shared__ uint32_t words[];
    __shared__ int s_task;
    const int bins = a.bins;
    const int nwords = packed_words(bins);
    const int wps = packed_row_words(bins), rs = packed_stride(bins);
    for (int w = threadIdx.x; w < nwords; w += blockDim.x) words[w] = 0;
    const int total = a.num_pairs * a.num_segs;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int t = s_task;
        if (t >= total) break;
        // task order: groups of `group` pairs; within a group segment by
        // segment, and within a segment pair by pair
        int seg, p;
        {
            const int per_group = a.group * a.num_segs;
            const int full = a.num_pairs / a.group;
            if (t < full * per_group) {
                const int g = t / per_group, r = t - g * per_group;
                seg = r / a.group;
                p = g * a.group + (r - seg * a.group);
            } else {
                const int r = t - full * per_group, cnt = a.num_pairs - full * a.group;
                seg = r / cnt;
                p = full * a.group + (r - seg * cnt);
            }
        }
        const int2 task = a.tasks[p];
        const int i = task.x, j = task.y;
        const Binner bn = make_binner(a.mma, a.mmb, i, j, bins, rs);
        uint32_t *gh = a.ghist + (size_t)p * bins * bins;
        const int64_t v0 = (int64_t)seg * a.seg_len;
        const int64_t v1 = v0 + a.seg_len < a.n ? v0 + a.seg_len : a.n;
        // the segment as a range of its own (same loop code as one pair per CTA)
        const float *f1 = a.fa + (size_t)i * a.stride + v0;
        const float *f2 = a.fb + (size_t)j * a.stride + v0;
        // with codes, the field with the larger maximum reads its codes and
        // indexes the shared rows; the histogram is transposed when that is the
        // pair's second field
        const bool coded = a.codes_a != nullptr && bn.mode == 0;
        const bool transposed = coded && bits_to_float(a.mmb[2 * j + 1]) > bits_to_float(a.mma[2 * i + 1]);
        const Counter<GlobalWrap> cnt{words, GlobalWrap{gh, rs, bins, transposed ? 1 : 0}};
        if (coded) {
            if (transposed)
                stream_coded<FB, FRS, CSTEP>(bn, a.codes_b + (size_t)j * a.stride + v0, f2, f1, 0, v1 - v0, cnt);
            else
                stream_coded<FB, FRS, CSTEP>(bn, a.codes_a + (size_t)i * a.stride + v0, f1, f2, 0, v1 - v0, cnt);
        } else if (bn.mode == 0) {
            stream_values<0, FB, FRS, CSTEP, RELOAD>(bn, f1, f2, 0, v1 - v0, cnt);
        } else {
            stream_values<1, FB, FRS, CSTEP, RELOAD>(bn, f1, f2, 0, v1 - v0, cnt);
        }
        __syncthreads();
        for (int w = threadIdx.x; w < nwords; w += blockDim.x) {
            const uint32_t val = words[w];
            if (val) {  // the pad words stay 0
                words[w] = 0;
                const int r = w / wps, c = 2 * (w - r * wps);  // the word's low counter (r, c)
                const int glo = transposed ? c * bins + r : r * bins + c;
                const int ghi = transposed ? glo + bins : glo + 1;
                if (val & 0xffffu) atomicAdd(&gh[glo], val & 0xffffu);
                if (val >> 16) atomicAdd(&gh[ghi], val >> 16);
            }
        }
        __syncthreads();
    }
}

struct MiArgs {
    const int2 *tasks;
    const uint32_t *ghist;
    int bins, m, symmetric;
    int64_t n;
    const double *clnc;
    float *ism;
    uint32_t *joint_dump;
    uint32_t *colrow_dump;
};

// One block of MI_THREADS per pair: marginals and sum(c ln c) of the global
// histogram, NMI.  FB: bins as a compile-time constant (0: a.bins).  With a
// multiple of 32 bins a warp reads part of one row and one warp sum replaces
// the row-sum atomics; with a divisor of the block size as bins every thread
// reads a single column and sums it in a register.
constexpr int MI_THREADS = 256;

template <int FB>
__global__ void __launch_bounds__(MI_THREADS) joint_mi_kernel(MiArgs a)
{
    __shared__ uint32_t s_row[ISO_MAX_BINS], s_col[ISO_MAX_BINS];  // n < 2^32
    __shared__ double s_red[3][MI_THREADS / 32];
    const int p = blockIdx.x;
    const int2 task = a.tasks[p];
    const int i = task.x, j = task.y;
    const int bins = FB ? FB : a.bins;
    const int lane = threadIdx.x & 31;
    const bool warp_rows = (bins & 31) == 0;
    const bool col_own = (MI_THREADS % bins) == 0;
    const uint32_t *gh = a.ghist + (size_t)p * bins * bins;
    for (int c = threadIdx.x; c < bins; c += blockDim.x) {
        s_row[c] = 0;
        s_col[c] = 0;
    }
    __syncthreads();
    double hxy = 0.0;
    const bool dump = a.joint_dump != nullptr;
    uint32_t cs_own = 0;
    if constexpr (FB == 256) {
        // 128-bit loads of four bins: a warp reads half a row, and thread t
        // always the columns 4 (t % 64) .. 4 (t % 64) + 3
        static_assert((MI_THREADS * 4) % FB == 0, "one column group per thread");
        const uint4 *gh4 = reinterpret_cast<const uint4 *>(gh);
        uint4 cs4 = make_uint4(0u, 0u, 0u, 0u);
        // the transposed dump (pair (j, i)) goes through a shared tile of
        // T_ROWS rows (dynamic shared memory, present only when dumping), so
        // that each of its rows leaves as whole 128-byte warp stores
        constexpr int T_ROWS = 32, T_STRIDE = FB + 1;
        extern __shared__ uint32_t s_tile[];  // [T_ROWS][T_STRIDE]
        const bool transpose = dump && a.symmetric && i != j;
        uint32_t *dump_ij = dump ? a.joint_dump + ((size_t)i * a.m + j) * FB * FB : nullptr;
        uint32_t *dump_ji = transpose ? a.joint_dump + ((size_t)j * a.m + i) * FB * FB : nullptr;
        for (int q = threadIdx.x; q < FB * FB / 4; q += MI_THREADS) {
            const uint4 c = __ldcs(gh4 + q);
            const int r = q / (FB / 4), col = (q % (FB / 4)) * 4;
            if (dump) {
                reinterpret_cast<uint4 *>(dump_ij)[q] = c;
                if (transpose) {
                    uint32_t *t = s_tile + (r % T_ROWS) * T_STRIDE + col;
                    t[0] = c.x;
                    t[1] = c.y;
                    t[2] = c.z;
                    t[3] = c.w;
                    // every thread runs the same iterations: the block meets
                    // here after each T_ROWS rows
                    if ((q / MI_THREADS + 1) % (T_ROWS * FB / 4 / MI_THREADS) == 0) {
                        __syncthreads();
                        const int r0 = r - r % T_ROWS;
                        const int w = threadIdx.x >> 5;
                        for (int oc = w; oc < FB; oc += MI_THREADS / 32)
                            dump_ji[(size_t)oc * FB + r0 + lane] = s_tile[lane * T_STRIDE + oc];
                        __syncthreads();
                    }
                }
            }
            if (c.x) hxy -= clnc_of(a.clnc, c.x);
            if (c.y) hxy -= clnc_of(a.clnc, c.y);
            if (c.z) hxy -= clnc_of(a.clnc, c.z);
            if (c.w) hxy -= clnc_of(a.clnc, c.w);
            const uint32_t rs = __reduce_add_sync(0xffffffffu, c.x + c.y + c.z + c.w);
            if (lane == 0 && rs) atomicAdd(&s_row[r], rs);
            cs4.x += c.x;
            cs4.y += c.y;
            cs4.z += c.z;
            cs4.w += c.w;
        }
        const int col = (threadIdx.x % (FB / 4)) * 4;
        if (cs4.x) atomicAdd(&s_col[col], cs4.x);
        if (cs4.y) atomicAdd(&s_col[col + 1], cs4.y);
        if (cs4.z) atomicAdd(&s_col[col + 2], cs4.z);
        if (cs4.w) atomicAdd(&s_col[col + 3], cs4.w);
    } else {
    // bins^2 is a multiple of the block size whenever warp_rows holds, so all
    // lanes of a warp run the same iterations for the warp sum
    for (int idx = threadIdx.x; idx < bins * bins; idx += MI_THREADS) {
        const uint32_t c = gh[idx];
        const int r = idx / bins, col = idx - r * bins;
        if (dump) {
            a.joint_dump[(((size_t)i * a.m + j) * bins + r) * bins + col] = c;
            if (a.symmetric && i != j) a.joint_dump[(((size_t)j * a.m + i) * bins + col) * bins + r] = c;
        }
        if (c) hxy -= clnc_of(a.clnc, c);
        if (warp_rows) {
            const uint32_t rs = __reduce_add_sync(0xffffffffu, c);
            if (lane == 0 && rs) atomicAdd(&s_row[r], rs);
        } else if (c) {
            atomicAdd(&s_row[r], c);
        }
        if (col_own) cs_own += c;
        else if (c) atomicAdd(&s_col[col], c);
    }
    if (col_own && cs_own) atomicAdd(&s_col[threadIdx.x % bins], cs_own);
    }
    __syncthreads();
    double hx = 0.0, hy = 0.0;
    for (int c = threadIdx.x; c < bins; c += blockDim.x) {
        const unsigned long long cs = s_col[c], rs = s_row[c];
        if (cs) hx -= clnc_of(a.clnc, cs);
        if (rs) hy -= clnc_of(a.clnc, rs);
        if (a.colrow_dump) {
            const size_t mm = (size_t)a.m * a.m * bins;
            const size_t bij = ((size_t)i * a.m + j) * bins, bji = ((size_t)j * a.m + i) * bins;
            a.colrow_dump[bij + c] = (uint32_t)cs;
            a.colrow_dump[mm + bij + c] = (uint32_t)rs;
            if (a.symmetric && i != j) {
                a.colrow_dump[bji + c] = (uint32_t)rs;
                a.colrow_dump[mm + bji + c] = (uint32_t)cs;
            }
        }
    }
    const int warp = threadIdx.x >> 5;
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
        for (int w = 0; w < MI_THREADS / 32; ++w) {
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
}

// The histogram kernels specialised for the common bin counts (bins and row
// stride as constants in the streaming loop), else the generic instance.
using PairKernel = void (*)(PairArgs);
using SegKernel = void (*)(SegArgs);
// clamp: some value lies above its pair's interval (only the generic
// instances clamp the fast path's buckets).
PairKernel mi_kernel_for(int bins, bool clamp)
{
    return bins == 256 && !clamp ? joint_histogram_mi_kernel<256, false, false>
                                 : joint_histogram_mi_kernel<0, false, false>;
}
PairKernel wide_kernel_for(int bins, bool clamp)
{
    return bins == 128 && !clamp ? joint_histogram_wide_kernel<128> : joint_histogram_wide_kernel<0>;
}
SegKernel seg_kernel_for(int bins, bool clamp)
{
    return bins == 256 && !clamp ? joint_histogram_seg_kernel<256, true, true>
                                 : joint_histogram_seg_kernel<0, true, true>;
}

__global__ void clnc_table_kernel(double *table)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < 65536) table[c] = c < 2 ? 0.0 : (double)c * log((double)c);
}

// Per-field min/max over the first n values: min starts at FLT_MAX and max at
// FLT_MIN as in types/src/DistanceField.cpp:159-200.  Values are >= 0, so
// unsigned comparison of the bit patterns orders them.
// Float order as unsigned keys (negative values below positive ones).
__device__ __forceinline__ uint32_t minmax_key(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ uint32_t minmax_key_to_bits(uint32_t k) { return (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k; }

// Field interval of DistanceField.cpp:159-200: min starts at FLT_MAX, max at
// FLT_MIN, NaN never compares.  Reduced as order keys, then stored as float bits.
__global__ void field_minmax_kernel(const float *fields, int64_t n, int64_t stride, uint32_t *minmax)
{
    const int f = blockIdx.y;
    const float *row = fields + (size_t)f * stride;
    uint32_t lo = 0xff7fffffu, hi = 0x80800000u;  // keys of FLT_MAX and FLT_MIN
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const float x = row[v];
        if (x != x) continue;
        const uint32_t k = minmax_key(x);
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
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
        minmax[2 * f] = 0xff7fffffu;
        minmax[2 * f + 1] = 0x80800000u;
    }
}

__global__ void minmax_finish_kernel(uint32_t *minmax, int m)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < m) {
        minmax[2 * f] = minmax_key_to_bits(minmax[2 * f]);
        minmax[2 * f + 1] = minmax_key_to_bits(minmax[2 * f + 1]);
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
    minmax_finish_kernel<<<(m + 255) / 256, 256, 0, ctx->stream>>>(d_minmax, m);
    ISO_LAUNCHED(ctx);
    return ISO_OK;
}

// Pair tasks ordered in 16-field tiles so concurrently running CTAs share fields
// in L2.  symmetric: i <= j over one set; otherwise all (i, j) of two sets.
// Pair tasks in 16 x 16 tiles.  perm (symmetric runs only, may be null):
// tiles run over perm's positions, and a task (perm[a], perm[b]) has a <= b.
static void build_tasks(int m, bool symmetric, int2 *out, int *count, const int *perm = nullptr)
{
    const int T = 16;
    int c = 0;
    for (int bi = 0; bi < m; bi += T)
        for (int bj = symmetric ? bi : 0; bj < m; bj += T)
            for (int i = bi; i < bi + T && i < m; ++i)
                for (int j = bj; j < bj + T && j < m; ++j)
                    if (!symmetric || j >= i) out[c++] = perm ? make_int2(perm[i], perm[j]) : make_int2(i, j);
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
    std::vector<int> perm;
    if (symmetric && ctx->hist_row_codes && bins > WIDE_MAX_BINS && ctx->hist_segment_values > 0 &&
        n > ctx->hist_segment_values) {
        // precomputed row buckets: order the fields by their maximum, so that
        // every task's first field is the one whose codes it reads and a tile
        // of tasks reads the codes of one 16-field group and the values of
        // another (the same L2 working set as without codes)
        std::vector<uint32_t> mm((size_t)2 * m);
        ISO_CUDA(cudaMemcpyAsync(mm.data(), d_minmax_a, mm.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                 ctx->stream));
        ISO_CUDA(cudaStreamSynchronize(ctx->stream));
        perm.resize(m);
        for (int k = 0; k < m; ++k) perm[k] = k;
        // non-negative maxima: bit order is value order
        std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return mm[2 * x + 1] > mm[2 * y + 1]; });
    }
    build_tasks(m, symmetric, h_tasks.data(), &num_tasks, perm.empty() ? nullptr : perm.data());
    if (ctx->mi_mode == ISO_MI_REF32 && !d_joint_dump) {
        // the reference's FP32 MI walks every ordered pair's histogram: keep them all
        void *p;
        ISO_TRY(iso_buf(ctx, BUF_HIST_DUMP, (size_t)m * m * bins * bins * sizeof(uint32_t), &p));
        d_joint_dump = (uint32_t *)p;
    }
    if (ctx->mi_mode == ISO_MI_REF32 && !d_colrow_dump) {
        // and its marginals (exact integers: their summation order is free)
        void *p;
        ISO_TRY(iso_buf(ctx, BUF_REF32_SUMS, (size_t)2 * m * m * bins * sizeof(uint32_t), &p));
        d_colrow_dump = (uint32_t *)p;
    }
    ISO_TRY(iso_run_similarity_tasks(ctx, d_fields_a, symmetric ? d_fields_a : d_fields_b, m, n, stride, bins,
                                     d_minmax_a, symmetric ? d_minmax_a : d_minmax_b, d_ism, h_tasks.data(), num_tasks,
                                     symmetric, d_joint_dump, d_colrow_dump));
    ctx->joint_m = 0;
    if (ctx->mi_mode == ISO_MI_REF32) {
        ISO_TRY(iso_run_mi_ref32(ctx, d_joint_dump, d_colrow_dump, m, bins, n, d_ism));
        if (d_joint_dump == (uint32_t *)ctx->buf[BUF_HIST_DUMP]) {
            ctx->joint_m = m;
            ctx->joint_bins = bins;
        }
    }
    return ISO_OK;
}

int iso_run_similarity_tasks(iso_ctx *ctx, const float *d_fields_a, const float *d_fields_b, int m, int64_t n,
                             int64_t stride, int bins, const uint32_t *d_minmax_a, const uint32_t *d_minmax_b,
                             float *d_ism, const int2 *h_tasks, int64_t num_tasks_in, bool symmetric,
                             uint32_t *d_joint_dump, uint32_t *d_colrow_dump)
{
    if (num_tasks_in <= 0) return ISO_OK;
    if (num_tasks_in > 0x7fffffff) return iso_fail(ISO_ERR_ARG, "too many pair tasks");
    if (n > (int64_t)0xffffffff) return iso_fail(ISO_ERR_ARG, "fields longer than 2^32 - 1 values");
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

    const size_t smem = (size_t)packed_words(bins) * sizeof(uint32_t);
    const int64_t seg_len = ctx->hist_segment_values;
    if (seg_len > 0 && n > seg_len && bins > WIDE_MAX_BINS) {
        // long fields, packed counters: segment-major schedule, pairs in chunks
        // bounding the global histograms to ISO_HIST_CHUNK_BYTES (and the task
        // count to int range)
        const SegKernel seg_kernel = seg_kernel_for(bins, ctx->hist_clamp_top);
        ISO_CUDA(cudaFuncSetAttribute(seg_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(packed_words(ISO_MAX_BINS) * sizeof(uint32_t))));
        const size_t hist_bytes = (size_t)bins * bins * sizeof(uint32_t);
        const int64_t num_segs64 = (n + seg_len - 1) / seg_len;
        if (num_segs64 > (1 << 24)) return iso_fail(ISO_ERR_ARG, "histogram segments: %lld too many", (long long)num_segs64);
        const int num_segs = (int)num_segs64;
        size_t chunk_sz = std::min<size_t>((size_t)num_tasks, ISO_HIST_CHUNK_BYTES / hist_bytes);
        chunk_sz = std::min<size_t>(chunk_sz, (size_t)(((int64_t)1 << 30) / num_segs64));
        const int chunk = (int)std::max<size_t>(1, chunk_sz);
        // the whole chunk runs segment by segment (256^3, 256 fields: 415 ms
        // for the stage against 424 ms with groups of 128 pairs, 436 ms with
        // 64 and 467 ms with 32)
        const int group = chunk;
        void *d_gh;
        ISO_TRY(iso_buf(ctx, BUF_HIST_DUMP_SEG, (size_t)chunk * hist_bytes, &d_gh));
        // precomputed row buckets of both field sets (one set when the pairs
        // are taken within one), with the smallest minimum of all fields
        const bool one_set = fb == d_fields_a && mmb == d_minmax_a;
        const int nsets = one_set ? 1 : 2;
        uint32_t *codes_a = nullptr, *codes_b = nullptr;
        if (ctx->hist_row_codes) {
            void *d_codes, *d_mlo;
            ISO_TRY(iso_buf(ctx, BUF_ROW_CODES, (size_t)nsets * m * stride * sizeof(uint32_t), &d_codes));
            ISO_TRY(iso_buf(ctx, BUF_MISC, 256, &d_mlo));
            min_of_mins_kernel<<<1, 256, 0, ctx->stream>>>(d_minmax_a, m, one_set ? nullptr : mmb, one_set ? 0 : m,
                                                           (uint32_t *)d_mlo);
            ISO_LAUNCHED(ctx);
            codes_a = (uint32_t *)d_codes;
            codes_b = one_set ? codes_a : codes_a + (size_t)m * stride;
            const int64_t per = (n + 255) / 256;
            const unsigned gx = (unsigned)(per < 512 ? (per < 1 ? 1 : per) : 512);
            row_code_kernel<<<dim3(gx, m), 256, 0, ctx->stream>>>(d_fields_a, n, stride, d_minmax_a,
                                                                  (const uint32_t *)d_mlo, bins, packed_stride(bins),
                                                                  codes_a);
            ISO_LAUNCHED(ctx);
            if (!one_set) {
                row_code_kernel<<<dim3(gx, m), 256, 0, ctx->stream>>>(fb, n, stride, mmb, (const uint32_t *)d_mlo,
                                                                      bins, packed_stride(bins), codes_b);
                ISO_LAUNCHED(ctx);
            }
        }
        int per_sm_seg = 0;
        ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_seg, seg_kernel, HIST_THREADS, smem));
        if (per_sm_seg < 1) per_sm_seg = 1;
        for (int c0 = 0; c0 < num_tasks; c0 += chunk) {
            const int np = std::min(chunk, num_tasks - c0);
            ISO_CUDA(cudaMemsetAsync(d_gh, 0, (size_t)np * hist_bytes, ctx->stream));
            ISO_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), ctx->stream));
            SegArgs sa;
            sa.fa = d_fields_a;
            sa.fb = fb;
            sa.n = n;
            sa.stride = stride;
            sa.seg_len = seg_len;
            sa.mma = d_minmax_a;
            sa.mmb = mmb;
            sa.tasks = (const int2 *)d_tasks + c0;
            sa.num_pairs = np;
            sa.num_segs = num_segs;
            sa.bins = bins;
            sa.group = std::min(group, np);
            sa.ghist = (uint32_t *)d_gh;
            sa.counter = (unsigned int *)d_counter;
            sa.codes_a = codes_a;
            sa.codes_b = codes_b;
            const int64_t seg_tasks = (int64_t)np * num_segs;
            const int grid_seg = (int)std::min<int64_t>((int64_t)ctx->num_sms * per_sm_seg, seg_tasks);
            seg_kernel<<<grid_seg, HIST_THREADS, smem, ctx->stream>>>(sa);
            ISO_LAUNCHED(ctx);
            MiArgs ma;
            ma.tasks = (const int2 *)d_tasks + c0;
            ma.ghist = (const uint32_t *)d_gh;
            ma.bins = bins;
            ma.m = m;
            ma.symmetric = symmetric ? 1 : 0;
            ma.n = n;
            ma.clnc = (const double *)d_clnc;
            ma.ism = d_ism;
            ma.joint_dump = d_joint_dump;
            ma.colrow_dump = d_colrow_dump;
            // the 256-bin kernel's transposed dump tile: 32 rows of 257 words
            const size_t mi_smem = (bins == 256 && d_joint_dump && symmetric) ? (size_t)32 * 257 * sizeof(uint32_t) : 0;
            (bins == 256 ? joint_mi_kernel<256> : joint_mi_kernel<0>)<<<np, MI_THREADS, mi_smem, ctx->stream>>>(ma);
            ISO_LAUNCHED(ctx);
        }
        return ISO_OK;
    }
    if (bins <= WIDE_MAX_BINS) {
        // 32-bit counters: no wrap events
        const size_t wsmem = (size_t)wide_words(bins) * sizeof(uint32_t);
        const PairKernel wide_kernel = wide_kernel_for(bins, ctx->hist_clamp_top);
        ISO_CUDA(cudaFuncSetAttribute(wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(wide_words(WIDE_MAX_BINS) * sizeof(uint32_t))));
        int per_sm_w = 0;
        ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_w, wide_kernel, HIST_THREADS,
                                                               wsmem));
        if (per_sm_w < 1) per_sm_w = 1;
        const int grid_w = std::min(ctx->num_sms * per_sm_w, num_tasks);
        PairArgs w;
        w.fa = d_fields_a;
        w.fb = fb;
        w.n = n;
        w.stride = stride;
        w.mma = d_minmax_a;
        w.mmb = mmb;
        w.tasks = (const int2 *)d_tasks;
        w.num_tasks = num_tasks;
        w.m = m;
        w.bins = bins;
        w.symmetric = symmetric ? 1 : 0;
        w.ism = d_ism;
        w.events = nullptr;
        w.event_cap = 0;
        w.clnc = (const double *)d_clnc;
        w.counter = (unsigned int *)d_counter;
        w.error = (int *)d_counter + 1;
        w.joint_dump = d_joint_dump;
        w.colrow_dump = d_colrow_dump;
        wide_kernel<<<grid_w, HIST_THREADS, wsmem, ctx->stream>>>(w);
        ISO_LAUNCHED(ctx);
        return ISO_OK;
    }
    const PairKernel mi_kernel = mi_kernel_for(bins, ctx->hist_clamp_top);
    ISO_CUDA(cudaFuncSetAttribute(mi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(packed_words(ISO_MAX_BINS) * sizeof(uint32_t))));
    int per_sm = 0;
    ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mi_kernel, HIST_THREADS, smem));
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
    mi_kernel<<<grid, HIST_THREADS, smem, ctx->stream>>>(a);
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
        for (int b : {0, 256})
            ISO_CUDA(cudaFuncSetAttribute(mi_kernel_for(b, false), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(packed_words(ISO_MAX_BINS) * sizeof(uint32_t))));
        int sms = 0, per_sm = 0;
        ISO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        ISO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mi_kernel_for(0, false), HIST_THREADS,
                                                               packed_words(ISO_MAX_BINS) * sizeof(uint32_t)));
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
        minmax_finish_kernel<<<(m + 255) / 256, 256, 0, st>>>(minmax, m);
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
    const size_t smem = (size_t)packed_words(bins) * sizeof(uint32_t);
    mi_kernel_for(bins, false)<<<grid, HIST_THREADS, smem, st>>>(a);  // intervals of its own fields
    ISO_CUDA(cudaGetLastError());
    int err = 0;
    ISO_CUDA(cudaMemcpyAsync(&err, ctrl + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    ISO_CUDA(cudaStreamSynchronize(st));
    if (err) return iso_fail(ISO_ERR_INTERNAL, "iso_similarity_map_noalloc: wrap-event list overflow (code %d)", err);
    return ISO_OK;
}

// ---------------------------------------------------------------------------
// Calibration: the peak rate of the histogram's counter update alone
// ---------------------------------------------------------------------------

namespace {

// Every thread draws pseudo-random bins from a 32-bit LCG and counts them
// with the same packed 16-bit atomic and wrap check as the histogram kernel,
// without bucket arithmetic or global loads.  Wrap corrections are skipped
// (the counts are discarded); the shared words are summed into `sink` so the
// work is not removed.
__global__ void __launch_bounds__(HIST_THREADS, 1) atomic_rate_kernel(int iters, int bins, unsigned int *sink)
{
    extern __shared__ uint32_t words[];
    const int nwords = bins * bins / 2;
    for (int w = threadIdx.x; w < nwords; w += blockDim.x) words[w] = 0;
    __syncthreads();
    uint32_t x = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u + 12345u;
    const uint32_t mask_bins = (uint32_t)(bins * bins - 1);
    uint32_t wraps = 0;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            x = x * 1664525u + 1013904223u;
            const uint32_t bin = (x >> 8) & mask_bins;
            const uint32_t odd = bin & 1u;
            const uint32_t inc = odd * 0xFFFFu + 1u;
            const uint32_t mask = inc * 0xFFFFu;
            const uint32_t old = atomicAdd(&words[bin >> 1], inc);
            wraps += (old & mask) == mask;
        }
    }
    __syncthreads();
    uint32_t acc = wraps;
    for (int w = threadIdx.x; w < nwords; w += blockDim.x) acc += words[w];
    atomicAdd(sink, acc);
}

}  // namespace

extern "C" int iso_probe_counter_rate(iso_ctx *ctx, int bins, double *updates_per_s)
{
    iso_clear_error();
    if (!ctx || !updates_per_s || bins < 2 || bins > ISO_MAX_BINS || (bins & (bins - 1)))
        return iso_fail(ISO_ERR_ARG, "iso_probe_counter_rate: bins must be a power of two in [2, %d]", ISO_MAX_BINS);
    ISO_CUDA(cudaSetDevice(ctx->device));
    void *d_sink;
    ISO_TRY(iso_buf(ctx, BUF_MISC, 256, &d_sink));
    const size_t smem = (size_t)bins * bins / 2 * sizeof(uint32_t);
    ISO_CUDA(cudaFuncSetAttribute(atomic_rate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(ISO_MAX_BINS * ISO_MAX_BINS / 2 * sizeof(uint32_t))));
    const int grid = ctx->num_sms;
    const int iters = 4096;
    cudaEvent_t e0, e1;
    ISO_CUDA(cudaEventCreate(&e0));
    ISO_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        ISO_CUDA(cudaEventRecord(e0, ctx->stream));
        atomic_rate_kernel<<<grid, HIST_THREADS, smem, ctx->stream>>>(iters, bins, (unsigned int *)d_sink);
        ISO_CUDA(cudaEventRecord(e1, ctx->stream));
        ISO_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        ISO_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;  // the first launch warms up
    }
    ctx->launches += 4;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *updates_per_s = (double)grid * HIST_THREADS * iters * 4 / (best * 1e-3);
    return ISO_OK;
}
