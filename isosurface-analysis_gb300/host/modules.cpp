// modules.cpp -- the reference's module surface (single, script, multi,
// stitch, check) on top of the C ABI.  Inputs are the reference's JSON configs;
// outputs are its files: <var>-<t>/similarityMap-<appendix>/map.dat,
// <var>-<t>/distancefields/distancefield-<k>.df, the meta.json run ledger and
// runtimes.csv.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <functional>
#include <map>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "dao.hpp"
#include "isosim.h"
#include "modules.hpp"

namespace isomod {

using namespace isodao;

static std::string strprintf(const char *fmt, ...)
{
    char buf[4096];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return buf;
}

static bool file_exists(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

static void make_dirs(const std::string &path)
{
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur += path[i];
        if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
    }
    if (!cur.empty()) mkdir(cur.c_str(), 0755);
}

static void check(int rc, const char *what)
{
    if (rc < 0) throw std::runtime_error(std::string(what) + ": " + iso_last_error());
}

static std::vector<float> read_floats(const std::string &path, size_t count)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<float> v(count);
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(count * sizeof(float)));
    if ((size_t)f.gcount() != count * sizeof(float))
        throw std::runtime_error("short read: " + path + " holds fewer than " + std::to_string(count) + " floats");
    return v;
}

static void write_floats(const std::string &path, const float *v, size_t count)
{
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error("cannot write " + path);
    f.write(reinterpret_cast<const char *>(v), (std::streamsize)(count * sizeof(float)));
}

// Single::checkIfAlreadyProcessed (runtime/src/Single.cpp:115-138)
static bool already_processed(const std::string &ledger, const std::string &var, int ts)
{
    if (!file_exists(ledger)) return false;
    RunInformation r = RunInformation::from(load_json(ledger));
    for (auto &v : r.volumes)
        if (v.variable >= 0 && v.variable < (int)r.variables.size() && r.variables[v.variable] == var &&
            v.timestep == ts)
            return true;
    return false;
}

// One volume: Single::run (runtime/src/Single.cpp:143-281) on the engine.
int run_single(iso_ctx *ctx, const SingleConfig &cfg, bool approximation, const RunOptions &opt)
{
    const auto t0 = std::chrono::steady_clock::now();
    const std::string outputFolder = cfg.outputFolder + "/";
    const std::string ledger = outputFolder + cfg.jsonFile;
    if (already_processed(ledger, cfg.variableName, cfg.timestep)) {
        printf("ts %d already processed... skipping\n", cfg.timestep);
        return 0;
    }
    if (cfg.dimensions.size() != 3) throw std::runtime_error("dimensions must have 3 entries");
    const int X = cfg.dimensions[0], Y = cfg.dimensions[1], Z = cfg.dimensions[2];
    const size_t V = (size_t)X * Y * Z;
    const EngineOptions &eng = cfg.engine;
    const bool approx = eng.surface < 0 ? approximation : eng.surface == 1;

    // Isosurface::loadFile: x-fastest .dat -> img order (z fastest)
    std::vector<float> raw = read_floats(cfg.fileName + ".dat", V);
    std::vector<float> img(V);
    check(iso_transpose_xfastest(ctx, raw.data(), X, Y, Z, img.data()), "transpose");
    raw.clear();
    raw.shrink_to_fit();
    float vmin = 0, vmax = 0;
    check(iso_real_range(ctx, img.data(), (int64_t)V, cfg.minValue, cfg.maxValue, &vmin, &vmax), "real range");

    std::vector<float> isovalues = eng.list;
    if (isovalues.empty()) {
        isovalues.resize(eng.isovalues);
        check(iso_isovalues(ctx, img.data(), (int64_t)V, vmin, vmax, eng.isovalues, eng.uniform ? 1 : 0,
                            isovalues.data()),
              "isovalues");
    }
    const int n = (int)isovalues.size();

    iso_opts o;
    o.surface = approx ? ISO_SURFACE_APPROX : ISO_SURFACE_MC;
    o.frame = ISO_FRAME_REF;
    o.df_method = eng.distance == 0 ? ISO_DF_BRUTE : ISO_DF_LBVH;
    o.df_downscale = cfg.dfDownscale;
    o.bins = eng.bins;
    std::vector<float> ism((size_t)n * n);
    std::vector<int32_t> ids(n);
    int32_t m = 0;
    iso_timing timing{};
    // map.dat holds the reference's own FP32 map unless the config asks for FP64
    check(iso_ctx_set_limit(ctx, ISO_LIMIT_MI_MODE, eng.mi ? ISO_MI_REF32 : ISO_MI_FP64), "MI mode");
    check(iso_ism(ctx, img.data(), X, Y, Z, isovalues.data(), n, &o, ism.data(), ids.data(), &m, nullptr, &timing),
          "similarity map");
    ism.resize((size_t)m * m);

    // output folders (Single::createFolder, runtime/src/Single.cpp:399-429)
    const std::string approxstr = approx ? std::string("-approx") + "-scale_1" : "";
    const std::string appendix = std::to_string(n) + "-" + approxstr;
    const std::string varFolder = outputFolder + cfg.variableName + "-" + std::to_string(cfg.timestep);
    const std::string isoSurfaceFolder = varFolder + "/isosurfaces-" + appendix + "/";
    const std::string simMapFolder = varFolder + "/similarityMap-" + appendix + "/";
    const std::string dfFolder = varFolder + "/distancefields/";
    make_dirs(simMapFolder);
    make_dirs(dfFolder);
    write_floats(simMapFolder + "map.dat", ism.data(), ism.size());

    // representatives and their distance fields (printResults, :473-552)
    std::vector<iso_rep> reps((size_t)std::max(eng.representatives, 1));
    const int k = iso_select_representatives(ism.data(), m, ids.data(), isovalues.data(), eng.representatives,
                                             reps.data());
    check(k, "representatives");
    std::vector<int> rep_ids;
    for (int r = 0; r < k; ++r) rep_ids.push_back(reps[r].id);
    std::sort(rep_ids.begin(), rep_ids.end());
    const std::string fname = cfg.fileName.substr(cfg.fileName.find_last_of('/') + 1);
    const size_t F = (size_t)(X / cfg.dfDownscale) * (Y / cfg.dfDownscale) * (Z / cfg.dfDownscale);
    std::vector<float> field(F);
    std::vector<RepresentativesInfo> repInfo;
    for (int r = 0; r < k; ++r) {
        const float cur = isovalues[reps[r].id];
        RepresentativesInfo ri;
        ri.valueId = reps[r].id;
        ri.isovalue = cur;
        ri.repId = r;
        ri.importance = reps[r].priority;
        ri.filename = strprintf("%s%s-%04d-%0.2f-%0.2f.dat", isoSurfaceFolder.c_str(), fname.c_str(), r, cur,
                                reps[r].isovalue);
        ri.mapId = reps[r].map_id;
        repInfo.push_back(ri);
        const int rank = (int)(std::lower_bound(rep_ids.begin(), rep_ids.end(), reps[r].id) - rep_ids.begin());
        check(iso_copy_field(ctx, reps[r].map_id, field.data()), "copy field");
        write_floats(dfFolder + strprintf("distancefield-%d.df", rank), field.data(), F);
    }

    const double runtime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    {
        std::ofstream csv(outputFolder + "runtimes.csv", std::ios::app);
        csv << cfg.variableName << fname << "," << timing.surface_ms << "," << timing.distance_ms << ","
            << timing.histogram_ms << "," << runtime * 1e3 << "\n";
    }
    // saveRunInfo (:603-633)
    RunInformation ri;
    if (file_exists(ledger)) {
        ri = RunInformation::from(load_json(ledger));
    } else {
        ri.dimensions = cfg.dimensions;
        ri.dfDownscale = cfg.dfDownscale;
    }
    ri.addVolumeInformation(cfg.variableName, cfg.timestep, m, repInfo, runtime);
    ri.addSimilarityMap(cfg.variableName, cfg.variableName, cfg.timestep, cfg.timestep, simMapFolder + "map.dat");
    save_json(ri.to_json(), ledger);
    if (opt.verbose)
        printf("%s t=%d: %d isovalues, %d surfaces, %d representatives, %.1f ms on the GPU\n", cfg.variableName.c_str(),
               cfg.timestep, n, m, k, timing.total_ms);
    return 0;
}

int module_single(const std::string &json, const RunOptions &opt)
{
    SingleConfig cfg = SingleConfig::from(load_json(json));
    iso_ctx *ctx = nullptr;
    check(iso_ctx_create(opt.device, &ctx), "context");
    int rc = run_single(ctx, cfg, /*approximation=*/true, opt);  // runtime/main.cpp:236
    iso_ctx_destroy(ctx);
    return rc;
}

// Scripting::run with SINGLE (runtime/src/Scripting.cpp:22-236): entries x
// variables x timesteps, marching cubes.
int module_script(const std::string &json, const RunOptions &opt)
{
    Value root = load_json(json);
    iso_ctx *ctx = nullptr;
    check(iso_ctx_create(opt.device, &ctx), "context");
    for (auto &e : root.at("entries").items()) {
        DataInfo d = DataInfo::from(e);
        for (auto &var : d.variables) {
            for (int ts : d.timesteps) {
                std::string fileName = strprintf(d.fileFormatString.c_str(), d.inputFolder.c_str(),
                                                 var.variableFolder.c_str(), var.name.c_str(), ts);
                if (!file_exists(fileName + ".dat")) {
                    printf("%s.dat\n", fileName.c_str());
                    continue;
                }
                SingleConfig c;
                c.dimensions = d.dimensions;
                c.fileName = fileName;
                c.jsonFile = d.jsonFile;
                c.maxValue = var.maxValue;
                c.minValue = var.minValue;
                c.outputFolder = d.outputFolder;
                c.timestep = ts;
                c.variableName = var.name;
                c.dfDownscale = d.dfDownscale;
                c.engine = d.engine;
                run_single(ctx, c, /*approximation=*/false, opt);
            }
        }
    }
    iso_ctx_destroy(ctx);
    return 0;
}

// MultiVar::run / computeMultiMap (runtime/src/MultiVar.cpp:76-249): 16 x 16
// cross maps between representative distance fields of variable pairs at one
// timestep and of one variable across timesteps.
// Timestep and variable similarity matrices over the cross maps in the
// ledger (no counterpart in the reference, which stops at the cross maps,
// runtime/src/MultiVar.cpp:122-160): entry (a, b) summarises the R x R cross
// map between the representative fields of volumes a and b by its mean and
// its best-match score (iso_block_similarity); the diagonal is 1.  A TSM per
// variable over the configured timesteps, a VSM per timestep over the
// variables; missing maps give null entries.
static void write_aggregate_maps(iso_ctx *ctx, RunInformation &run, const MultiVarConfig &cfg,
                                 const std::string &folder, int R)
{
    std::map<std::tuple<int, int, int, int>, std::string> files;
    for (auto &m : run.similarityMaps) files[{m.var1, m.t1, m.var2, m.t2}] = m.filename;
    auto score = [&](int v1, int t1, int v2, int t2, double &mean, double &best) {
        auto it = files.find({v1, t1, v2, t2});
        bool swapped = false;
        if (it == files.end()) {
            it = files.find({v2, t2, v1, t1});
            swapped = true;
        }
        if (it == files.end() || !file_exists(it->second)) return false;
        std::vector<float> map = read_floats(it->second, (size_t)R * R);
        if (swapped) {
            std::vector<float> tr((size_t)R * R);
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < R; ++j) tr[(size_t)j * R + i] = map[(size_t)i * R + j];
            map.swap(tr);
        }
        const int32_t block[2] = {0, 0};
        float out[2];
        check(iso_block_similarity(ctx, map.data(), R, R, block, 1, out), "block similarity");
        mean = out[0];
        best = out[1];
        return true;
    };
    auto matrix = [&](const std::vector<std::pair<int, int>> &axis) {
        const size_t k = axis.size();
        Value mean = Value::array(), best = Value::array();
        for (size_t a = 0; a < k; ++a) {
            Value rm = Value::array(), rb = Value::array();
            for (size_t b = 0; b < k; ++b) {
                double mv = 1.0, bv = 1.0;
                if (a != b && !score(axis[a].first, axis[a].second, axis[b].first, axis[b].second, mv, bv)) {
                    rm.push(Value());
                    rb.push(Value());
                    continue;
                }
                rm.push(Value(mv));
                rb.push(Value(bv));
            }
            mean.push(rm);
            best.push(rb);
        }
        return std::make_pair(mean, best);
    };
    make_dirs(folder);
    for (size_t v = 0; v < run.variables.size(); ++v) {
        std::vector<std::pair<int, int>> axis;
        Value ts = Value::array();
        for (int t : cfg.timeSteps) {
            axis.push_back({(int)v, t});
            ts.push(Value(t));
        }
        auto mb = matrix(axis);
        Value o = Value::object();
        o.set("kind", Value("TSM"));
        o.set("variable", Value(run.variables[v]));
        o.set("timesteps", ts);
        o.set("mean", mb.first);
        o.set("bestMatch", mb.second);
        const std::string file = folder + "tsm-" + run.variables[v] + ".json";
        save_json(o, file);
        run.setAggregateMap("TSM", (int)v, -1, file);
    }
    for (int t : cfg.timeSteps) {
        std::vector<std::pair<int, int>> axis;
        Value vs = Value::array();
        for (size_t v = 0; v < run.variables.size(); ++v) {
            axis.push_back({(int)v, t});
            vs.push(Value(run.variables[v]));
        }
        auto mb = matrix(axis);
        Value o = Value::object();
        o.set("kind", Value("VSM"));
        o.set("timestep", Value(t));
        o.set("variables", vs);
        o.set("mean", mb.first);
        o.set("bestMatch", mb.second);
        const std::string file = folder + "vsm-" + std::to_string(t) + ".json";
        save_json(o, file);
        run.setAggregateMap("VSM", -1, t, file);
    }
}

int module_multi(const std::string &json, const RunOptions &opt)
{
    MultiVarConfig cfg = MultiVarConfig::from(load_json(json));
    const std::string dataJson = cfg.dataRoot + "/" + cfg.jsonFile;
    RunInformation run = RunInformation::from(load_json(dataJson));
    std::set<std::tuple<std::string, std::string, int, int>> done;
    for (auto &m : run.similarityMaps) done.insert({run.variables[m.var1], run.variables[m.var2], m.t1, m.t2});
    const int X = run.dimensions[0], Y = run.dimensions[1], Z = run.dimensions[2];
    const int ds = cfg.dfDownscale;
    const size_t size = (size_t)(X / ds) * (Y / ds) * (Z / ds);
    const int R = 16;  // MULTI_MAP_DF_NUMBER
    const std::string prefix = cfg.dataRoot + "-multi-tmp/";
    iso_ctx *ctx = nullptr;
    check(iso_ctx_create(opt.device, &ctx), "context");
    // the cross maps hold the reference's own FP32 values (its multi mode of
    // calculate_histogram_h) unless the config asks for FP64
    check(iso_ctx_set_limit(ctx, ISO_LIMIT_MI_MODE, cfg.mi ? ISO_MI_REF32 : ISO_MI_FP64), "MI mode");
    std::vector<float> a((size_t)R * size), b((size_t)R * size), out((size_t)R * R);

    auto load_set = [&](const std::string &var, int t, std::vector<float> &dst) {
        const std::string dir = cfg.dataRoot + "/" + var + "-" + std::to_string(t) + "/distancefields/";
        for (int i = 0; i < R; ++i) {
            const std::string f = dir + "distancefield-" + std::to_string(i) + ".df";
            if (!file_exists(f)) return false;
            std::vector<float> v = read_floats(f, size);
            std::copy(v.begin(), v.end(), dst.begin() + (size_t)i * size);
        }
        return true;
    };
    auto cross = [&](const std::string &v1, const std::string &v2, int t1, int t2, const std::string &folder) {
        if (done.count({v1, v2, t1, t2})) return;
        const auto t0 = std::chrono::steady_clock::now();
        if (!load_set(v1, t1, a) || !load_set(v2, t2, b)) {
            printf("failed\n");
            return;
        }
        check(iso_cross_map(ctx, a.data(), b.data(), R, (int64_t)size, cfg.bins, out.data()), "cross map");
        const std::string file = strprintf("%s/TMP-multiMap-%d-%s-%d-%s-%d.dat", folder.c_str(), R, v1.c_str(), t1,
                                           v2.c_str(), t2);
        write_floats(file, out.data(), out.size());
        run.addSimilarityMap(v1, v2, t1, t2, file);
        done.insert({v1, v2, t1, t2});
        std::ofstream csv(cfg.dataRoot + "-multi-tmp/runtimes-tmp.csv", std::ios::app);
        csv << file << "," << std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() << "\n";
        if (opt.verbose) printf("%s\n", file.c_str());
    };

    const std::vector<std::string> vars = run.variables;
    for (size_t i = 0; i < vars.size(); ++i) {
        for (size_t j = i; j < vars.size(); ++j) {
            for (size_t k = 0; k < cfg.timeSteps.size(); ++k) {
                const int t1 = cfg.timeSteps[k];
                const std::string folder = prefix + vars[i] + "-" + std::to_string(t1);
                make_dirs(folder);
                if (i != j) {
                    cross(vars[i], vars[j], t1, t1, folder);
                } else {
                    for (size_t l = k + 1; l < cfg.timeSteps.size(); ++l) cross(vars[i], vars[j], t1, cfg.timeSteps[l], folder);
                    save_json(run.to_json(), dataJson);
                }
            }
        }
    }
    write_aggregate_maps(ctx, run, cfg, prefix, R);
    save_json(run.to_json(), dataJson);
    iso_ctx_destroy(ctx);
    return 0;
}

// Stitch::run (runtime/src/Stitch.cpp:57-85): append every volume and map of
// the partial ledgers to the first one, written to stitched.json.
int module_stitch(const std::vector<std::string> &files, const RunOptions &)
{
    if (files.size() < 2) {
        printf("Error: at least 2 files needed to stitch\n");
        return 1;
    }
    RunInformation host = RunInformation::from(load_json(files[0]));
    for (size_t f = 1; f < files.size(); ++f) {
        RunInformation part = RunInformation::from(load_json(files[f]));
        for (auto &v : part.volumes)
            host.addVolumeInformation(part.variables[v.variable], v.timestep, v.numIsovalues, v.representatives,
                                      v.runtime);
        for (auto &m : part.similarityMaps)
            host.addSimilarityMap(part.variables[m.var1], part.variables[m.var2], m.t1, m.t2, m.filename);
        for (auto &a : part.aggregateMaps)
            host.setAggregateMap(a.kind, a.variable < 0 ? -1 : host.variable_index(part.variables[a.variable]),
                                 a.timestep, a.filename);
    }
    save_json(host.to_json(), "stitched.json");
    return 0;
}

// Check::run (runtime/src/Check.cpp:13-68): list the cross maps missing for
// timesteps [ts1, ts2).
int module_check(const std::string &json, int ts1, int ts2, const RunOptions &)
{
    RunInformation r = RunInformation::from(load_json(json));
    std::set<std::tuple<int, int, int, int>> have;
    for (auto &m : r.similarityMaps) have.insert({m.var1, m.var2, m.t1, m.t2});
    int missing = 0;
    for (int v1 = 0; v1 < (int)r.variables.size(); ++v1)
        for (int v2 = v1; v2 < (int)r.variables.size(); ++v2)
            for (int t1 = ts1; t1 < ts2; ++t1) {
                if (v1 != v2) {
                    if (!have.count({v1, v2, t1, t1})) {
                        printf("Missing %s %s %d %d\n", r.variables[v1].c_str(), r.variables[v2].c_str(), t1, t1);
                        ++missing;
                    }
                } else {
                    for (int t2 = t1 + 1; t2 < ts2; ++t2)
                        if (!have.count({v1, v2, t1, t2})) {
                            printf("Missing %s %s %d %d\n", r.variables[v1].c_str(), r.variables[v2].c_str(), t1, t2);
                            ++missing;
                        }
                }
            }
    printf("%d missing\n", missing);
    return missing == 0 ? 0 : 2;
}


// ---------------------------------------------------------------------------
// distance: isovalue equalisation (DistanceEqualization,
// runtime/src/DistanceEqualization.cpp, dispatched at runtime/main.cpp:281)
// with the reference's default settings (runtime/hdr/DistanceEqualization.h:
// 20-53): 16 distances between 17 isovalues, no estimation iterations, 180
// refinement iterations that alternate every 5 between moving the odd and the
// even isovalues, each moved isovalue placed where the two neighbouring
// distances become equal on the secant of its bracket.  Distance d_j =
// 1 - ISM[j][j+1] over voxel-approximation surfaces; every iteration is one
// 17-isovalue iso_ism call on the GPU.
//
// Two deliberate differences: the start is the evenly spaced isovalues of
// compute_isovalues' first run (:846-882) or the config's isovalueList -- the
// reference overwrites them with 17 constants tuned to one dataset
// (DistanceEqualization.h:221); and the result is the refined isovalues --
// the reference overwrites its best set with the starting set once the
// refinement returns (:720-723).
// ---------------------------------------------------------------------------
namespace {

constexpr int ND = 16;            // NUM_DISTANCES
constexpr int BIN_MAX_ITR = 180;  // BIN_SEARCH_MAX_ITR
constexpr int BIN_STEP_ITR = 5;   // BIN_SEARCH_STEP_ITR
constexpr int NUDGE_LIMIT = 100000;

struct Bound {  // boundInformation
    float value = 0, left = 0, right = 0;
};

struct Iteration {  // iterationInfo
    float iso[ND + 1];
    float dist[ND];
    Bound upper[ND + 1], lower[ND + 1];
};

struct Moving {  // movingValueAndDistance
    float dRight = 0, isovalue = 0;
};

class Equalizer {
  public:
    Equalizer(iso_ctx *ctx, const std::vector<float> &img, int X, int Y, int Z, float vmin, float vmax, int bins,
              int ds, const std::string &varFolder)
        : ctx_(ctx), img_(img), X_(X), Y_(Y), Z_(Z), vmin_(vmin), vmax_(vmax), bins_(bins), ds_(ds), folder_(varFolder)
    {
        for (int i = 0; i <= ND; ++i) fixed_[i] = false;
        fixed_[0] = fixed_[ND] = true;  // init(), :963-964
    }

    // Points of the voxel approximation at one isovalue.
    int64_t points(float iso)
    {
        int64_t count = 0;
        check(iso_surface_points(ctx_, img_.data(), X_, Y_, Z_, &iso, 1, ISO_SURFACE_APPROX, ISO_FRAME_REF, &count,
                                 nullptr, 0, nullptr),
              "surface count");
        return count;
    }

    // approximation() (:84-131): an empty surface moves its isovalue up in
    // sixteenths of the gap to the next one (past the range maximum it
    // restarts from the previous isovalue); then the ISM of the 17 surfaces
    // and the 16 neighbour distances (computeDistances, :601-617).
    void measure(float *iso)
    {
        // counts of all 17 at once; an isovalue is counted again only if it
        // changed since (the search below moves and swaps them one by one)
        float batch[ND + 1];
        int64_t counts[ND + 1];
        std::copy(iso, iso + ND + 1, batch);
        check(iso_surface_points(ctx_, img_.data(), X_, Y_, Z_, batch, ND + 1, ISO_SURFACE_APPROX, ISO_FRAME_REF,
                                 counts, nullptr, 0, nullptr),
              "surface count");
        for (int d = 0; d <= ND; ++d) {
            int64_t len = iso[d] == batch[d] ? counts[d] : points(iso[d]);
            float cur = iso[d];
            const float val = d < ND ? iso[d + 1] : cur + (vmax_ - vmin_) / ND;
            float incr = (val - cur) / ND;
            for (int tries = 0; len == 0; ++tries) {
                if (tries == NUDGE_LIMIT) throw std::runtime_error("distance: no non-empty surface near an isovalue");
                cur += incr;
                if (cur > vmax_ || cur != cur) {
                    cur = d > 0 ? iso[d - 1] : vmin_;
                    incr = (iso[d] - cur) / 16;
                    cur += incr;
                }
                if (d < ND && cur > iso[d + 1]) {
                    iso[d] = iso[d + 1];
                    iso[d + 1] = cur;
                    cur = iso[d];
                }
                iso[d] = cur;
                len = points(cur);
            }
        }
        iso_opts o;
        o.surface = ISO_SURFACE_APPROX;
        o.frame = ISO_FRAME_REF;
        o.df_method = ISO_DF_LBVH;
        o.df_downscale = ds_;
        o.bins = bins_;
        ism_.assign((size_t)(ND + 1) * (ND + 1), 0.0f);
        std::vector<int32_t> ids(ND + 1);
        int32_t m = 0;
        check(iso_ism(ctx_, img_.data(), X_, Y_, Z_, iso, ND + 1, &o, ism_.data(), ids.data(), &m, nullptr, nullptr),
              "similarity map");
        if (m != ND + 1) throw std::runtime_error("distance: a surface is empty after the isovalue search");
        for (int j = 0; j < ND; ++j) dist_[j] = 1 - ism_[(size_t)j * (ND + 1) + j + 1];
    }

    // fixInversions (:192-215)
    void fix_inversions(float *iso)
    {
        for (int i = 0; i <= ND; ++i)
            for (int j = i + 1; j <= ND; ++j)
                if (iso[i] > iso[j]) {
                    std::swap(iso[i], iso[j]);
                    std::swap(fixed_[i], fixed_[j]);
                }
    }

    // evaluateDistances (:333-557) on the default path: the error statistics,
    // the best set by average error, and the best moving values of the pairs
    // that moved (TAKE_BEST_AT_FIX_SWITCH).
    void evaluate(const float *iso, bool fixEven, const std::string &label)
    {
        float acc = 0;
        for (int j = 0; j < ND; ++j) acc += dist_[j];
        const float avgD = acc / ND;
        float errAcc = 0, errV = 0, maxE = -1;
        for (int k = 0; k < ND; ++k) {
            const float e = std::abs(dist_[k] - avgD);
            errV += e * e;
            errAcc += e;
            if (e > maxE) maxE = e;
        }
        const float avgE = errAcc / ND;
        const float stdDev = std::sqrt(errV / ND);
        if (avgE / avgD < bestAvg_) {
            bestAvg_ = avgE / avgD;
            std::copy(iso, iso + ND + 1, best_);
        }
        if (maxE < bestMax_) bestMax_ = maxE;
        for (int i = fixEven ? 1 : 0; i < ND - 1; i += 2) {
            if (i == 0) continue;
            const float dl = dist_[i - 1], dr = dist_[i];
            if (std::abs(dl - dr) < std::abs(moving_[i - 1].dRight - moving_[i].dRight)) {
                moving_[i - 1] = {dl, iso[i - 1]};
                moving_[i] = {dr, iso[i]};
            }
        }
        std::ofstream d(folder_ + "/distances.csv", std::ios::app), v(folder_ + "/isovalues.csv", std::ios::app);
        d << label << ",";
        v << label << ",";
        for (int j = 0; j < ND; ++j) d << strprintf("%.9g,", dist_[j]);
        for (int j = 0; j <= ND; ++j) v << strprintf("%.9g,", iso[j]);
        d << strprintf("%.9g,%.9g,%.9g,%.9g,%.9g,%.9g\n", avgD, maxE, avgE, stdDev, maxE / avgD, avgE / avgD);
        v << "\n";
    }

    // binaryIsoValueSearch (:1338-1449)
    void move(bool fixedEven, int iterations, float *iso, Iteration &cur)
    {
        const int phase = iterations % BIN_STEP_ITR;
        for (int i = fixedEven ? 1 : 2; i < ND; i += 2) {
            const int j = i - 1, k = i + 1;
            const float dji = dist_[j], dik = dist_[i], sum = dji + dik;
            Bound up, lo;
            if (phase == 0) {
                up = {iso[k], sum, 0.0f};
                lo = {iso[j], 0.0f, sum};
            } else {
                up = infos_[iterations - 1].upper[i];
                lo = infos_[iterations - 1].lower[i];
            }
            if (dji > dik) up = {iso[i], dji, dik};
            if (dji < dik) lo = {iso[i], dji, dik};
            const float incr1 = (lo.left - up.left) / (lo.value - up.value);
            const float fix1 = lo.left - incr1 * lo.value;
            const float incr2 = (lo.right - up.right) / (lo.value - up.value);
            const float fix2 = lo.right - incr2 * lo.value;
            const float nv = (fix2 - fix1) / (incr1 - incr2);
            if (!std::isnan(nv) && !fixed_[i]) iso[i] = nv;
            cur.upper[i] = up;
            cur.lower[i] = lo;
        }
    }

    // run() then binarySearchEqualization (:626-774, :1451-1619).  Calls
    // save(iteration, isovalues) every 10 iterations and at the end.
    template <class Save>
    void run(float *start, const Save &save)
    {
        float iso[ND + 1];
        std::copy(start, start + ND + 1, iso);
        measure(iso);
        evaluate(iso, false, "estimate");
        float cur_iso[ND + 1];
        std::copy(best_, best_ + ND + 1, cur_iso);
        for (int j = 0; j < ND; ++j) moving_[j] = {dist_[j], best_[j]};
        bool fixedEven = true;
        for (int it = 0;; ++it) {
            if (it > 0) std::copy(infos_.back().iso, infos_.back().iso + ND + 1, cur_iso);
            fix_inversions(cur_iso);
            Iteration info;
            move(fixedEven, it, cur_iso, info);
            measure(cur_iso);
            const bool finished = it == BIN_MAX_ITR;
            evaluate(cur_iso, fixedEven, finished ? "final" : std::to_string(it));
            std::copy(cur_iso, cur_iso + ND + 1, info.iso);
            std::copy(dist_, dist_ + ND, info.dist);
            infos_.push_back(info);
            if (it % 10 == 0 || finished) save(it, cur_iso, ism_);
            if (finished) break;
            if ((it + 1) % BIN_STEP_ITR == 0) {
                // at a switch of the moving set the distances restart from the
                // best of the moving pairs (the isovalues restart from the last
                // iteration, as in the reference)
                for (int i = 0; i < ND; ++i) dist_[i] = moving_[i].dRight;
                fixedEven = !fixedEven;
            }
        }
    }

    float best_avg_error() const { return bestAvg_; }
    const float *best() const { return best_; }
    const float *distances() const { return dist_; }

  private:
    iso_ctx *ctx_;
    const std::vector<float> &img_;
    int X_, Y_, Z_;
    float vmin_, vmax_;
    int bins_, ds_;
    std::string folder_;
    float dist_[ND] = {};
    bool fixed_[ND + 1];
    float bestAvg_ = 10e20f, bestMax_ = 10e20f;
    float best_[ND + 1] = {};
    Moving moving_[ND];
    std::vector<Iteration> infos_;
    std::vector<float> ism_;
};

}  // namespace

int module_distance(const std::string &json, const RunOptions &opt)
{
    const auto t0 = std::chrono::steady_clock::now();
    SingleConfig cfg = SingleConfig::from(load_json(json));
    const std::string outputFolder = cfg.outputFolder + "/";
    const std::string ledger = outputFolder + cfg.jsonFile;
    // checkIfAlreadyProcessed (:971-996): any volume of this timestep
    if (file_exists(ledger)) {
        RunInformation r = RunInformation::from(load_json(ledger));
        for (auto &v : r.volumes)
            if (v.timestep == cfg.timestep) {
                printf("timestep %d already processed... skipping\n", cfg.timestep);
                return 0;
            }
    }
    if (cfg.dimensions.size() != 3) throw std::runtime_error("dimensions must have 3 entries");
    const int X = cfg.dimensions[0], Y = cfg.dimensions[1], Z = cfg.dimensions[2];
    const size_t V = (size_t)X * Y * Z;
    iso_ctx *ctx = nullptr;
    check(iso_ctx_create(opt.device, &ctx), "context");
    check(iso_ctx_set_limit(ctx, ISO_LIMIT_MI_MODE, cfg.engine.mi ? ISO_MI_REF32 : ISO_MI_FP64), "MI mode");
    std::vector<float> raw = read_floats(cfg.fileName + ".dat", V);
    std::vector<float> img(V);
    check(iso_transpose_xfastest(ctx, raw.data(), X, Y, Z, img.data()), "transpose");
    float vmin = 0, vmax = 0;
    check(iso_real_range(ctx, img.data(), (int64_t)V, cfg.minValue, cfg.maxValue, &vmin, &vmax), "real range");

    // createFolder (:1003-1043), approximation folders with 17 isovalues
    const std::string varFolder = outputFolder + cfg.variableName + "-" + std::to_string(cfg.timestep);
    const std::string appendix = std::to_string(ND + 1) + "--approx-scale_1";
    const std::string simMapFolder = varFolder + "/similarityMap-" + appendix + "/";
    make_dirs(simMapFolder);
    {
        std::ofstream d(varFolder + "/distances.csv", std::ios::app), v(varFolder + "/isovalues.csv", std::ios::app);
        d << "iterations,";
        v << "iterations,";
        for (int i = 0; i <= ND; ++i) {
            if (i != ND) d << "d" << i << ",";
            v << "iv" << i << ",";
        }
        d << "avgD,maxError,averageError,stdDev,normMaxE,normAvgE\n";
        v << "\n";
    }

    float start[ND + 1];
    if (cfg.engine.list.size() == (size_t)ND + 1) {
        std::copy(cfg.engine.list.begin(), cfg.engine.list.end(), start);
    } else {
        if (!cfg.engine.list.empty()) throw std::runtime_error("distance: isovalueList needs 17 values");
        const float step = (vmax - vmin) / ND;
        for (int i = 0; i <= ND; ++i) start[i] = vmin + step * i;
    }
    // saveIteration / saveRunInfo (:776-793, :1282-1314): one ledger volume
    // per saved iteration, named <variable>-<DAMPENING_FACTOR>
    const std::string name = cfg.variableName + "-" + std::to_string(0.66);
    const std::string mapFile = simMapFolder + "map-" + std::to_string(0.66) + ".dat";
    auto save = [&](int iteration, const float *iso, const std::vector<float> &ism) {
        RunInformation ri;
        if (file_exists(ledger)) {
            ri = RunInformation::from(load_json(ledger));
        } else {
            ri.dimensions = cfg.dimensions;
            ri.dfDownscale = cfg.dfDownscale;
        }
        std::vector<RepresentativesInfo> reps;
        for (int i = 0; i <= ND; ++i) {
            RepresentativesInfo r;
            r.valueId = i;
            r.isovalue = iso[i];
            r.repId = i;
            r.importance = (float)i;
            r.mapId = i;
            r.filename = std::to_string(iteration) + "-surface-" + std::to_string(i) + ".dat";
            reps.push_back(r);
        }
        ri.addVolumeInformation(name, cfg.timestep, ND + 1, reps, (double)iteration);
        ri.addSimilarityMap(name, name, cfg.timestep, cfg.timestep, mapFile);
        save_json(ri.to_json(), ledger);
        write_floats(mapFile, ism.data(), ism.size());
    };
    Equalizer eq(ctx, img, X, Y, Z, vmin, vmax, cfg.engine.bins, cfg.dfDownscale, varFolder);
    eq.run(start, save);
    iso_ctx_destroy(ctx);
    if (opt.verbose)
        printf("%s t=%d: %d refinement iterations, best normalised average error %.4g, %.1f s\n",
               cfg.variableName.c_str(), cfg.timestep, BIN_MAX_ITR, eq.best_avg_error(),
               std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    return 0;
}

}  // namespace isomod
