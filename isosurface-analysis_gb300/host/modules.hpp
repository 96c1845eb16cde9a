// modules.hpp -- the reference's CLI modules on the engine.
#pragma once

#include <string>
#include <vector>

#include "dao.hpp"

struct iso_ctx;

namespace isomod {

struct RunOptions {
    int device = 0;
    bool verbose = true;
};

int run_single(iso_ctx *ctx, const isodao::SingleConfig &cfg, bool approximation, const RunOptions &opt);
int module_single(const std::string &json, const RunOptions &opt);
int module_script(const std::string &json, const RunOptions &opt);
int module_multi(const std::string &json, const RunOptions &opt);
int module_distance(const std::string &json, const RunOptions &opt);
int module_stitch(const std::vector<std::string> &files, const RunOptions &opt);
int module_check(const std::string &json, int ts1, int ts2, const RunOptions &opt);

}  // namespace isomod
