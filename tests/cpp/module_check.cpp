// The module seam (include/facetcu_module.hpp): the readiness chain of the
// reference's Facetrt, and, given an input and an output path, one run.
#include <cstdio>
#include <memory>

#include "facetcu_module.hpp"

#define CHECK(c)                                                     \
    do {                                                             \
        if (!(c)) {                                                  \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                                \
        }                                                            \
    } while (0)

int main(int argc, char** argv)
{
    Facetrt model;
    auto io = std::make_shared<FacetrtIO>();
    std::shared_ptr<FacetrtIO> none;
    CHECK(!model.setup(none) && !model.upload(none) && !model.create(none) && !model.run(none));
    CHECK(model.destroy(none));
    CHECK(!model.setup(io));  // no input, no shader directory
    io->inputPath = argc > 1 ? argv[1] : "scene.obj";
    CHECK(!model.setup(io));  // still no shader directory
    CHECK(!model.upload(io) && !model.create(io) && !model.run(io));
    io->shaderDirectory = "shaders";
    CHECK(model.setup(io) && io->setupReady);
    CHECK(!model.create(io) && !io->bufferReady);  // upload first
    CHECK(model.upload(io) && io->uploadReady);
    CHECK(!model.run(io));  // not created
    CHECK(model.create(io));
    CHECK(io->bufferReady && io->descriptorReady && io->pipelineReady && io->commandReady);
    if (argc > 2) {
        io->outputPath = argv[2];
        CHECK(model.run(io));
    }
    CHECK(model.destroy(io));
    CHECK(!io->commandReady && !io->pipelineReady && !io->descriptorReady && !io->bufferReady);
    CHECK(io->setupReady && io->uploadReady);  // destroy keeps them, as the reference's does
    CHECK(!model.run(io));
    // an empty shader directory stops create at the pipeline stage
    auto bare = std::make_shared<FacetrtIO>();
    bare->inputPath = "x.obj";
    bare->shaderDirectory = "s";
    CHECK(model.setup(bare) && model.upload(bare));
    bare->shaderDirectory.clear();
    CHECK(!model.create(bare) && bare->descriptorReady && !bare->pipelineReady);
    std::printf("module seam ok\n");
    return 0;
}
