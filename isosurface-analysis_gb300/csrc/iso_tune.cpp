// iso_tune.cpp -- the engine's autotuner: picks the launch shapes of the
// distance and histogram stages for one workload by timed trials of the whole
// pipeline, applies them to the context and caches them on disk.
//
// What it replaces: the reference fixes its launch shapes (the one-thread-per-
// pair histogram grid of JointHistogram.cu:362-364, the BVH query launch of
// BVH.cu:667-673, the classify grid of MarchingCube.cpp:599-608); here the
// shapes that decide speed are context settings with identical results for
// every value, so they can be chosen per workload:
//   * ISO_LIMIT_QUERY_RUN           samples each LBVH query lane sweeps along x;
//   * ISO_LIMIT_LBVH_GROUP_POINTS   points per LBVH build-and-query group;
//   * ISO_LIMIT_HIST_SEGMENT_VALUES segment length of the segment-major
//                                   histogram schedule (0: one CTA per pair).
// Each candidate runs the pipeline twice (the faster run counts) and is
// judged by the time of the stage it affects (iso_timing); knobs are tuned one
// after the other, each from the best settings found so far.  The tuned set
// is kept only if the whole pipeline is at least as fast as with the settings
// the context had.  Cache lines: "<key> <segment> <group> <run> <tuned ms>
// <default ms>", the key naming the GPU, the volume shape, the isovalues
// (hash of their bits), bins and the surface, frame, distance and downscale
// options.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "iso_internal.cuh"

namespace {

struct Knobs {
    int64_t seg, group;
    int run;
};

struct Trial {
    float total = 1e30f, surface = 0, distance = 1e30f, histogram = 1e30f;
};

int apply(iso_ctx *ctx, const Knobs &k)
{
    ISO_TRY(iso_ctx_set_limit(ctx, ISO_LIMIT_HIST_SEGMENT_VALUES, k.seg));
    ISO_TRY(iso_ctx_set_limit(ctx, ISO_LIMIT_LBVH_GROUP_POINTS, k.group));
    return iso_ctx_set_limit(ctx, ISO_LIMIT_QUERY_RUN, k.run);
}

std::string make_key(int device, int X, int Y, int Z, const float *iso, int n, const iso_opts *o)
{
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        cudaGetLastError();
        std::memset(&p, 0, sizeof p);
    }
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the isovalues' bits
    for (int i = 0; i < n; ++i) {
        uint32_t b;
        std::memcpy(&b, &iso[i], 4);
        for (int k = 0; k < 4; ++k) {
            h ^= (b >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
    }
    std::string name(p.name);
    for (auto &c : name)
        if (c == ' ') c = '_';
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s/sm%d|%dx%dx%d|n%d|%016llx|b%d|s%d|f%d|d%d|ds%d", name.c_str(),
                  p.multiProcessorCount, X, Y, Z, n, (unsigned long long)h, o->bins, o->surface, o->frame,
                  o->df_method, o->df_downscale);
    return buf;
}

bool lookup(const char *path, const std::string &key, Knobs *k, float *tuned, float *base)
{
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {  // the last line for a key wins
        std::istringstream ss(line);
        std::string kk;
        Knobs t;
        float a, b;
        if (ss >> kk >> t.seg >> t.group >> t.run >> a >> b && kk == key) {
            *k = t;
            *tuned = a;
            *base = b;
            found = true;
        }
    }
    return found;
}

}  // namespace

extern "C" int iso_autotune(iso_ctx *ctx, const float *volume, int X, int Y, int Z, const float *isovalues, int n,
                            const iso_opts *opts, const char *cache_path, iso_tuning *out)
{
    iso_clear_error();
    if (!ctx || !volume || !isovalues || !opts || !out || n <= 0)
        return iso_fail(ISO_ERR_ARG, "iso_autotune: bad argument");
    std::memset(out, 0, sizeof *out);
    const std::string key = make_key(ctx->device, X, Y, Z, isovalues, n, opts);
    Knobs k;
    if (lookup(cache_path, key, &k, &out->tuned_ms, &out->default_ms)) {
        ISO_TRY(apply(ctx, k));
        out->hist_segment_values = k.seg;
        out->lbvh_group_points = k.group;
        out->query_run = k.run;
        out->from_cache = 1;
        return ISO_OK;
    }
    std::vector<float> ism((size_t)n * n);
    std::vector<int32_t> ids(n);
    int trials = 0;
    auto timed = [&](const Knobs &kn, Trial *t) -> int {
        ISO_TRY(apply(ctx, kn));
        *t = Trial();
        for (int r = 0; r < 2; ++r) {
            iso_timing tm;
            int32_t m = 0;
            ISO_TRY(iso_ism(ctx, volume, X, Y, Z, isovalues, n, opts, ism.data(), ids.data(), &m, nullptr, &tm));
            ++trials;
            if (tm.total_ms < t->total) {
                t->total = tm.total_ms;
                t->surface = tm.surface_ms;
            }
            if (tm.distance_ms < t->distance) t->distance = tm.distance_ms;
            if (tm.histogram_ms < t->histogram) t->histogram = tm.histogram_ms;
        }
        return ISO_OK;
    };
    const Knobs base{ctx->hist_segment_values, ctx->lbvh_group_points, ctx->query_run};
    Trial tb;
    ISO_TRY(timed(base, &tb));
    Knobs best = base;
    Trial cur = tb;
    const int64_t F = (int64_t)(X / opts->df_downscale) * (Y / opts->df_downscale) * (Z / opts->df_downscale);
    if (opts->df_method == ISO_DF_LBVH) {
        for (int run : {8, 16, 32, 64}) {
            Knobs c = best;
            c.run = run;
            Trial t;
            ISO_TRY(timed(c, &t));
            if (t.distance < cur.distance) {
                best = c;
                cur = t;
            }
        }
        for (int64_t group : {(int64_t)1 << 25, (int64_t)1 << 26, (int64_t)1 << 27, (int64_t)1 << 28}) {
            if (group == best.group) continue;
            Knobs c = best;
            c.group = group;
            Trial t;
            ISO_TRY(timed(c, &t));
            if (t.distance < cur.distance) {
                best = c;
                cur = t;
            }
        }
    }
    if (opts->bins > ISO_WIDE_MAX_BINS && F > 65536) {
        for (int64_t seg : {(int64_t)0, (int64_t)1 << 20, (int64_t)1 << 21, (int64_t)1 << 22, (int64_t)1 << 23}) {
            if (seg == best.seg || (seg > 0 && seg >= F)) continue;
            Knobs c = best;
            c.seg = seg;
            Trial t;
            ISO_TRY(timed(c, &t));
            if (t.histogram < cur.histogram) {
                best = c;
                cur = t;
            }
        }
    }
    // the chosen set against the settings the context had, on the whole pipeline
    Trial tt;
    ISO_TRY(timed(best, &tt));
    if (tt.total > tb.total) {
        best = base;
        tt = tb;
    }
    ISO_TRY(apply(ctx, best));
    out->hist_segment_values = best.seg;
    out->lbvh_group_points = best.group;
    out->query_run = best.run;
    out->default_ms = tb.total;
    out->tuned_ms = tt.total;
    out->trials = trials;
    if (cache_path) {
        std::ofstream f(cache_path, std::ios::app);
        if (f)
            f << key << " " << best.seg << " " << best.group << " " << best.run << " " << tt.total << " " << tb.total
              << "\n";
    }
    return ISO_OK;
}
