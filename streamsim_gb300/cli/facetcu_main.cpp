// facetcu_main.cpp — the reference's process seam on the CUDA backend.
//
// `facetcu <mode> [input] [output]` with the argument handling and exit
// codes of the reference's `histream` executable
// (models/histream/src/main.cpp:56-80, base/engine.cpp:162-165): an unknown
// mode prints the usage and exits 2; eFacetRT runs runFacetRTCore
// (facetrtcore.cpp:3116-3161) through facetcu_run_facetrt_core and exits 0 on
// success, 1 on failure.  The other reference modes exit 3, the code the
// reference uses when engine resources cannot be created: the voxel and
// ray-tracing engines are not built on this backend, and eFacetEB runs from
// Python (python -m streamsim_gb300.faceteb, the same library).
#include <iostream>
#include <string>

#include "facetcu.h"

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
    if (mode != "eFacetRT") {
        std::cerr << "Failed to create engine resources for " << mode
                  << ": only eFacetRT runs in this executable";
        if (mode == "eFacetEB") std::cerr << " (eFacetEB: python -m streamsim_gb300.faceteb)";
        std::cerr << '\n';
        return 3;
    }
    return facetcu_run_facetrt_core(input.c_str(), "", output.c_str()) == 0 ? 0 : 1;
}
