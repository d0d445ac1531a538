// facetcu_module.hpp — the reference's module seam over this library.
//
// HiStream drives the eFacetRT mode through
//   class Facetrt { setup, upload, create, run, destroy }(std::shared_ptr<FacetrtIO>&)
// (models/histream/src/facetrt/facetrt.h:14-29, facetrtio.h:7-21,
// facetrt.cpp:16-59 with buffer.cpp, descriptor.cpp, pipeline.cpp and
// command.cpp): a chain of readiness flags, then
// runFacetRTCore(inputPath, shaderDirectory, outputPath) == 0.  The same
// class, members and flags here, header only; the buffer, descriptor,
// pipeline and command stages are the same flag transitions (this library
// allocates its device memory when the run starts), and the run goes
// through facetcu_run_facetrt_core.  Every member returns bool as the
// reference's do.
#pragma once

#include <memory>
#include <string>

#include "facetcu.h"

class FacetrtIO {
public:
    std::string inputPath;
    std::string shaderDirectory;  // accepted and unused by the library, as a path
    std::string outputPath;       // empty: facetrt.json next to the input

    facetcu_config setting{};     // facetvk::Config (the run reads the input's own settings)
    bool setupReady{false};
    bool uploadReady{false};
    bool bufferReady{false};
    bool descriptorReady{false};
    bool pipelineReady{false};
    bool commandReady{false};
};

class Facetrt {
public:
    // facetrt.cpp:16-23: an input and a shader directory are required
    bool setup(std::shared_ptr<FacetrtIO>& io)
    {
        if (!io || io->inputPath.empty() || io->shaderDirectory.empty()) return false;
        io->setupReady = true;
        return true;
    }
    bool upload(std::shared_ptr<FacetrtIO>& io)
    {
        if (!io || !io->setupReady) return false;
        io->uploadReady = true;
        return true;
    }
    // facetrt.cpp:34-43: buffer, descriptor, pipeline, command in turn; the
    // pipeline stage needs the shader directory
    bool create(std::shared_ptr<FacetrtIO>& io)
    {
        if (!io || !io->uploadReady) return false;
        io->bufferReady = true;
        io->descriptorReady = true;
        if (io->shaderDirectory.empty()) return false;
        io->pipelineReady = true;
        io->commandReady = true;
        return true;
    }
    // command.cpp:16-24: runFacetRTCore(...) == 0
    bool run(std::shared_ptr<FacetrtIO>& io)
    {
        if (!io || !io->commandReady) return false;
        return facetcu_run_facetrt_core(io->inputPath.c_str(), io->shaderDirectory.c_str(),
                                        io->outputPath.c_str()) == 0;
    }
    // facetrt.cpp:50-59: the stages are released in reverse order
    bool destroy(std::shared_ptr<FacetrtIO>& io)
    {
        if (!io) return true;
        io->commandReady = false;
        io->pipelineReady = false;
        io->descriptorReady = false;
        io->bufferReady = false;
        return true;
    }
};
