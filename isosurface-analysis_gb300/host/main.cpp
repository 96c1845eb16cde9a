// main.cpp -- `isosim <module> <args>`, the module surface of the reference's
// `isosurfaces <module> <json>` (runtime/main.cpp:51-118).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "modules.hpp"

static void usage()
{
    fprintf(stderr,
            "usage: isosim <module> <args>\n"
            "  single <SingleConfig.json>        one volume (voxel approximation)\n"
            "  script <ScriptingInput.json>      entries x variables x timesteps (marching cubes)\n"
            "  multi  <MultiVarConfig.json>      16x16 cross maps between representative fields,\n"
            "                                    timestep and variable similarity matrices\n"
            "  distance <SingleConfig.json>      equalise 16 distances between 17 isovalues\n"
            "  stitch <host.json> <part.json>... merge run ledgers into stitched.json\n"
            "  check  <meta.json> <ts1> <ts2>    list missing cross maps\n"
            "options (before the module): --device N, --quiet\n");
}

int main(int argc, char **argv)
{
    isomod::RunOptions opt;
    int a = 1;
    while (a < argc && strncmp(argv[a], "--", 2) == 0) {
        if (!strcmp(argv[a], "--device") && a + 1 < argc) opt.device = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--quiet")) opt.verbose = false;
        else { usage(); return 1; }
        ++a;
    }
    if (a >= argc) { usage(); return 1; }
    const std::string module = argv[a++];
    std::vector<std::string> rest(argv + a, argv + argc);
    try {
        if (module == "single" && rest.size() == 1) return isomod::module_single(rest[0], opt);
        if (module == "script" && rest.size() == 1) return isomod::module_script(rest[0], opt);
        if (module == "multi" && rest.size() == 1) return isomod::module_multi(rest[0], opt);
        if (module == "distance" && rest.size() == 1) return isomod::module_distance(rest[0], opt);
        if (module == "stitch") return isomod::module_stitch(rest, opt);
        if (module == "check" && rest.size() == 3)
            return isomod::module_check(rest[0], atoi(rest[1].c_str()), atoi(rest[2].c_str()), opt);
    } catch (const std::exception &e) {
        fprintf(stderr, "isosim %s: %s\n", module.c_str(), e.what());
        return 2;
    }
    usage();
    return 1;
}
