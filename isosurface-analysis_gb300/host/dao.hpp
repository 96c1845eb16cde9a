// dao.hpp -- the reference's JSON records with the same field names and
// order (L/json/src/JSONHandler.cpp:17-25, L/DAO/hdr/*.h), read and written
// with isojson.
#pragma once

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "json.hpp"

namespace isodao {

using isojson::Value;

inline std::vector<int> ints(const Value &v)
{
    std::vector<int> out;
    for (auto &x : v.items()) out.push_back(x.integer());
    return out;
}

inline Value ints_json(const std::vector<int> &v)
{
    Value a = Value::array();
    for (int x : v) a.push(Value(x));
    return a;
}

// Optional engine block (not in the reference): overrides of the compile-time
// defaults HIST_SIZE, MAP_SIZE, uniform equalisation, surface and distance
// method, plus an explicit isovalue list.
struct EngineOptions {
    int bins = 128;           // HIST_SIZE (runtime/hdr/globals.h:11)
    int isovalues = 256;      // MAP_SIZE (globals.h:12)
    bool uniform = true;      // histogram equalisation (Single.cpp:294)
    int surface = -1;         // -1: the module's default; 0 marching cubes; 1 approximation
    int distance = 1;         // 0 brute force; 1 LBVH
    int representatives = 16; // MULTI_MAP_DF_NUMBER (globals.h:32)
    int mi = 1;               // "ref32" (1, default): the reference's own FP32 map; "fp64" (0)
    std::vector<float> list;  // explicit isovalues (overrides isovalues/uniform)

    static EngineOptions from(const Value &parent)
    {
        EngineOptions e;
        if (!parent.has("engine")) return e;
        const Value &v = parent.at("engine");
        if (v.has("bins")) e.bins = v.at("bins").integer();
        if (v.has("isovalues")) e.isovalues = v.at("isovalues").integer();
        if (v.has("uniform")) e.uniform = v.at("uniform").boolean();
        if (v.has("surface")) e.surface = v.at("surface").str() == "mc" ? 0 : 1;
        if (v.has("distance")) e.distance = v.at("distance").str() == "brute" ? 0 : 1;
        if (v.has("representatives")) e.representatives = v.at("representatives").integer();
        if (v.has("mi")) {
            const std::string mi = v.at("mi").str();
            if (mi != "ref32" && mi != "fp64") throw std::runtime_error("engine.mi must be \"ref32\" or \"fp64\"");
            e.mi = mi == "ref32" ? 1 : 0;
        }
        if (v.has("isovalueList"))
            for (auto &x : v.at("isovalueList").items()) e.list.push_back((float)x.num());
        return e;
    }
};

struct SingleConfig {  // DAO/hdr/SingleConfig.h
    std::vector<int> dimensions;
    int timestep = 0;
    std::string fileName;
    float minValue = 0, maxValue = 0;
    std::string outputFolder, variableName, jsonFile;
    int dfDownscale = 1;
    EngineOptions engine;

    static SingleConfig from(const Value &v)
    {
        SingleConfig c;
        c.fileName = v.at("fileName").str();
        c.dimensions = ints(v.at("dimensions"));
        c.minValue = (float)v.at("minValue").num();
        c.maxValue = (float)v.at("maxValue").num();
        c.outputFolder = v.at("outputFolder").str();
        c.variableName = v.at("variableName").str();
        c.timestep = v.at("timestep").integer();
        c.dfDownscale = v.at("dfDownscale").integer();
        c.jsonFile = v.at("jsonFile").str();
        c.engine = EngineOptions::from(v);
        return c;
    }
};

struct VariableInfo {  // DAO/hdr/VariableInfo.h
    std::string name;
    float minValue = 0, maxValue = 0;
    std::string variableFolder;
};

struct DataInfo {  // DAO/hdr/DataInfo.h
    std::vector<int> dimensions;
    std::vector<VariableInfo> variables;
    std::vector<int> timesteps;
    int dfDownscale = 1;
    std::string fileFormatString, inputFolder, outputFolder, jsonFile;
    EngineOptions engine;

    static DataInfo from(const Value &v)
    {
        DataInfo d;
        d.dimensions = ints(v.at("dimensions"));
        for (auto &x : v.at("variables").items())
            d.variables.push_back(VariableInfo{x.at("name").str(), (float)x.at("minValue").num(),
                                               (float)x.at("maxValue").num(), x.at("variableFolder").str()});
        d.timesteps = ints(v.at("timesteps"));
        d.dfDownscale = v.at("dfDownscale").integer();
        d.fileFormatString = v.at("fileFormatString").str();
        d.inputFolder = v.at("inputFolder").str();
        d.outputFolder = v.at("outputFolder").str();
        d.jsonFile = v.at("jsonFile").str();
        d.engine = EngineOptions::from(v);
        return d;
    }
};

struct MultiVarConfig {  // DAO/hdr/MultiVarConfig.h
    std::string jsonFile;
    std::vector<int> timeSteps;
    std::string dataRoot;
    int dfDownscale = 1;
    int bins = 128;
    int mi = 1;  // EngineOptions::mi

    static MultiVarConfig from(const Value &v)
    {
        MultiVarConfig c;
        c.jsonFile = v.at("jsonFile").str();
        c.timeSteps = ints(v.at("timeSteps"));
        c.dataRoot = v.at("dataRoot").str();
        c.dfDownscale = v.at("dfDownscale").integer();
        const EngineOptions e = EngineOptions::from(v);
        c.bins = e.bins;
        c.mi = e.mi;
        return c;
    }
};

struct RepresentativesInfo {  // DAO/hdr/RepresentativesInfo.h
    int valueId = 0;
    float isovalue = 0;
    int repId = 0;
    float importance = 0;
    std::string filename;
    int mapId = 0;
};

struct VolumeInformation {  // DAO/hdr/VolumeInformation.h
    int variable = 0, timestep = 0, numIsovalues = 0;
    double runtime = 0;
    std::vector<RepresentativesInfo> representatives;
};

struct SimilarityMapInformation {  // DAO/hdr/SimilarityMapInformation.h
    int var1 = 0, t1 = 0, var2 = 0, t2 = 0;
    std::string filename;
};

// A timestep (TSM) or variable (VSM) similarity matrix built from cross maps.
// No counterpart in the reference's ledger schema: written under the
// additional key "aggregateMaps", and only when there are some, so that
// ledgers without them keep the reference's keys exactly.
struct AggregateMapInformation {
    std::string kind;  // "TSM" (one variable over timesteps) or "VSM" (one timestep over variables)
    int variable = -1; // TSM: variable index; VSM: -1
    int timestep = -1; // VSM: timestep; TSM: -1
    std::string filename;
};

struct RunInformation {  // DAO/hdr/RunInformation.h, src/RunInformation.cpp
    std::vector<int> dimensions;
    std::vector<std::string> variables;
    int dfDownscale = 1;
    std::vector<VolumeInformation> volumes;
    std::vector<SimilarityMapInformation> similarityMaps;
    std::vector<AggregateMapInformation> aggregateMaps;

    int variable_index(const std::string &name)
    {
        for (size_t i = 0; i < variables.size(); ++i)
            if (variables[i] == name) return (int)i;
        variables.push_back(name);
        return (int)variables.size() - 1;
    }
    void addVolumeInformation(const std::string &var, int ts, int n, const std::vector<RepresentativesInfo> &reps,
                              double runtime)
    {
        VolumeInformation v;
        v.variable = variable_index(var);
        v.timestep = ts;
        v.numIsovalues = n;
        v.runtime = runtime;
        v.representatives = reps;
        volumes.push_back(v);
    }
    void addSimilarityMap(const std::string &v1, const std::string &v2, int t1, int t2, const std::string &file)
    {
        SimilarityMapInformation m;
        m.var1 = variable_index(v1);
        m.var2 = variable_index(v2);
        m.t1 = t1;
        m.t2 = t2;
        m.filename = file;
        similarityMaps.push_back(m);
    }

    // Replaces any earlier matrix of the same kind, variable and timestep.
    void setAggregateMap(const std::string &kind, int variable, int timestep, const std::string &file)
    {
        for (auto &a : aggregateMaps)
            if (a.kind == kind && a.variable == variable && a.timestep == timestep) {
                a.filename = file;
                return;
            }
        aggregateMaps.push_back({kind, variable, timestep, file});
    }

    static RunInformation from(const Value &v)
    {
        RunInformation r;
        r.dimensions = ints(v.at("dimensions"));
        for (auto &x : v.at("variables").items()) r.variables.push_back(x.str());
        r.dfDownscale = v.at("dfDownscale").integer();
        for (auto &x : v.at("volumes").items()) {
            VolumeInformation vi;
            vi.variable = x.at("variable").integer();
            vi.timestep = x.at("timestep").integer();
            vi.numIsovalues = x.at("numIsovalues").integer();
            vi.runtime = x.at("runtime").num();
            for (auto &y : x.at("representatives").items()) {
                RepresentativesInfo ri;
                ri.valueId = y.at("valueId").integer();
                ri.isovalue = (float)y.at("isovalue").num();
                ri.repId = y.at("repId").integer();
                ri.importance = (float)y.at("importance").num();
                ri.filename = y.at("filename").str();
                ri.mapId = y.at("mapId").integer();
                vi.representatives.push_back(ri);
            }
            r.volumes.push_back(vi);
        }
        for (auto &x : v.at("similarityMaps").items()) {
            SimilarityMapInformation m;
            m.var1 = x.at("var1").integer();
            m.t1 = x.at("t1").integer();
            m.var2 = x.at("var2").integer();
            m.t2 = x.at("t2").integer();
            m.filename = x.at("filename").str();
            r.similarityMaps.push_back(m);
        }
        if (v.has("aggregateMaps"))
            for (auto &x : v.at("aggregateMaps").items())
                r.aggregateMaps.push_back({x.at("kind").str(), x.at("variable").integer(), x.at("timestep").integer(),
                                           x.at("filename").str()});
        return r;
    }

    Value to_json() const
    {
        Value o = Value::object();
        o.set("dimensions", ints_json(dimensions));
        Value vars = Value::array();
        for (auto &s : variables) vars.push(Value(s));
        o.set("variables", vars);
        o.set("dfDownscale", Value(dfDownscale));
        Value vols = Value::array();
        for (auto &v : volumes) {
            Value x = Value::object();
            x.set("variable", Value(v.variable));
            x.set("timestep", Value(v.timestep));
            x.set("numIsovalues", Value(v.numIsovalues));
            Value reps = Value::array();
            for (auto &r : v.representatives) {
                Value y = Value::object();
                y.set("valueId", Value(r.valueId));
                y.set("isovalue", Value((double)r.isovalue));
                y.set("repId", Value(r.repId));
                y.set("importance", Value((double)r.importance));
                y.set("filename", Value(r.filename));
                y.set("mapId", Value(r.mapId));
                reps.push(y);
            }
            x.set("representatives", reps);
            x.set("runtime", Value(v.runtime));
            vols.push(x);
        }
        o.set("volumes", vols);
        Value maps = Value::array();
        for (auto &m : similarityMaps) {
            Value x = Value::object();
            x.set("var1", Value(m.var1));
            x.set("t1", Value(m.t1));
            x.set("var2", Value(m.var2));
            x.set("t2", Value(m.t2));
            x.set("filename", Value(m.filename));
            maps.push(x);
        }
        o.set("similarityMaps", maps);
        if (!aggregateMaps.empty()) {
            Value agg = Value::array();
            for (auto &a : aggregateMaps) {
                Value x = Value::object();
                x.set("kind", Value(a.kind));
                x.set("variable", Value(a.variable));
                x.set("timestep", Value(a.timestep));
                x.set("filename", Value(a.filename));
                agg.push(x);
            }
            o.set("aggregateMaps", agg);
        }
        return o;
    }
};

inline std::string read_text(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

inline Value load_json(const std::string &path) { return Value::parse(read_text(path)); }

inline void save_json(const Value &v, const std::string &path)
{
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error("cannot write " + path);
    f << v.dump(2) << "\n";
}

}  // namespace isodao
