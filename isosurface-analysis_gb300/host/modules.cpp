// modules.cpp -- the reference's module surface (single, script, multi,
// stitch, check) on top of the C ABI.  Inputs are the reference's JSON configs;
// outputs are its files: <var>-<t>/similarityMap-<appendix>/map.dat,
// <var>-<t>/distancefields/distancefield-<k>.df, the meta.json run ledger and
// runtimes.csv.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <functional>
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

}  // namespace isomod
