// facetcu_main.cpp — the reference's process seam on the CUDA backend.
//
// `facetcu <mode> [input] [output]` with the argument handling and exit
// codes of the reference's `histream` executable
// (models/histream/src/main.cpp:56-80, base/engine.cpp:162-165): an unknown
// mode prints the usage and exits 2; eFacetRT runs runFacetRTCore
// (facetrtcore.cpp:3116-3161) through facetcu_run_facetrt_core and exits 0 on
// success, 1 on failure.  eFacetEB runs runFacetEBCore's node sequence
// through `python3 -m streamsim_gb300.faceteb` (the same library; exit 0,
// or 1 with `faceteb: <message>`).  The voxel and ray-tracing modes are not
// built on this backend and exit 3, the code the reference uses when engine
// resources cannot be created.
#include <unistd.h>

#include <cstdlib>
#include <filesystem>
#include <iostream>
#include <string>

#include "facetcu.h"

namespace {

// eFacetEB: the node sequence runs in Python over the same library
// (streamsim_gb300/faceteb.py, runFacetEBCore); this executable lives in
// the package folder, whose parent goes on PYTHONPATH.
int exec_faceteb(const char* self, const std::string& input, const std::string& output)
{
    std::error_code ec;
    const std::filesystem::path exe = std::filesystem::canonical("/proc/self/exe", ec);
    const std::filesystem::path root =
        (ec ? std::filesystem::absolute(self) : exe).parent_path().parent_path();
    const char* old = std::getenv("PYTHONPATH");
    const std::string path = root.string() + (old && *old ? ":" + std::string(old) : "");
    setenv("PYTHONPATH", path.c_str(), 1);
    const char* python = std::getenv("FACETCU_PYTHON");
    if (!python || !*python) python = "python3";
    if (output.empty())
        execlp(python, python, "-m", "streamsim_gb300.faceteb", input.c_str(), (char*)nullptr);
    else
        execlp(python, python, "-m", "streamsim_gb300.faceteb", input.c_str(), output.c_str(),
               (char*)nullptr);
    std::cerr << "Failed to create engine resources for eFacetEB: cannot start " << python
              << '\n';
    return 3;
}

}  // namespace

int main(int argc, char** argv)
{
    const std::string mode = argc > 1 ? argv[1] : "eVoxelEB";
    const std::string input = argc > 2 ? argv[2] : "";
    const std::string output = argc > 3 ? argv[3] : "";
    if (mode != "eVoxelEB" && mode != "eFacetEB" && mode != "eFacetRT" && mode != "eVoxelRT" &&
        mode != "eRaytracing") {
        std::cerr << "Usage: facetcu [eVoxelEB|eFacetEB|eFacetRT|eVoxelRT|eRaytracing] "
                     "[project.json] [output.json]\n";
        return 2;
    }
    if (mode == "eFacetEB") return exec_faceteb(argv[0], input, output);
    if (mode != "eFacetRT") {
        std::cerr << "Failed to create engine resources for " << mode
                  << ": only eFacetRT and eFacetEB run on the CUDA backend\n";
        return 3;
    }
    return facetcu_run_facetrt_core(input.c_str(), "", output.c_str()) == 0 ? 0 : 1;
}
