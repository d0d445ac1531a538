// facetcu.hpp — C++ wrapper over the facetcu C ABI with the interface of the
// reference's facetvk::FacetrtVulkan (models/histream/src/facetrt/facetrt_vulkan.h:70-104).
//
// Same member names, argument order, defaults, return types and exception
// classes, so a caller written against FacetrtVulkan (runGpu in
// facetrtcore.cpp:1621-1780, runFacetEBCore :3345-3392) compiles against
// facetcu::FacetrtCuda after swapping the type.  Header-only; link with
// libfacetcu.so.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "facetcu.h"

namespace facetcu {

// facetvk POD types, same layout (facetrt_vulkan.h:15-62).
struct Vertex {
    float position[3]{};
    float normal[3]{};
};
struct Direction {
    float x{};
    float y{};
    float z{1.0f};
};
struct SurfaceOptics {
    float reflectance{};
    float transmittance{};
    float emission{};
    float directIrradiance{};
};
struct Config {
    uint32_t rasterWidth{512};
    uint32_t rasterHeight{512};
    uint32_t maxFragmentsPerPixel{32};
    uint32_t edgeHashCapacity{0};
    bool enableValidation{false};
    uint32_t gpuIndex{0};
    uint32_t periodicNeighborCount{0};
    float periodicSizeX{1.0f};
    float periodicSizeZ{1.0f};
};
struct GraphDiagnostics {
    uint32_t facetCount{};
    uint32_t surfaceCount{};
    uint32_t directedEdgeCount{};
    uint32_t fragmentOverflow{};
    uint32_t hashOverflow{};
    float maxClosureError{};
};
struct SolveResult {
    std::vector<float> radiosity;
    uint32_t iterations{};
    float maxDelta{};
};

static_assert(sizeof(Vertex) == sizeof(facetcu_vertex), "Vertex layout");
static_assert(sizeof(Direction) == sizeof(facetcu_direction), "Direction layout");
static_assert(sizeof(SurfaceOptics) == sizeof(facetcu_surface_optics), "SurfaceOptics layout");
static_assert(sizeof(Config) == sizeof(facetcu_config), "Config layout");
static_assert(sizeof(GraphDiagnostics) == sizeof(facetcu_graph_diagnostics), "GraphDiagnostics layout");

// Thrown for FACETCU_CUDA_ERROR / NO_DEVICE / OUT_OF_MEMORY /
// DEVICE_CAPACITY / NOT_CONVERGED (the Vulkan backend throws runtime_error
// for its device failures, facetrt_vulkan.cpp:89-96).
struct DeviceError : std::runtime_error {
    int code;
    DeviceError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void throw_status(int status, const char* message)
{
    const std::string m = message ? message : "";
    switch (status) {
    case FACETCU_OK: return;
    case FACETCU_INVALID_ARGUMENT: throw std::invalid_argument(m);
    case FACETCU_LOGIC_ERROR: throw std::logic_error(m);
    case FACETCU_RUNTIME_ERROR: throw std::runtime_error(m);
    case FACETCU_OVERFLOW_ERROR: throw std::overflow_error(m);
    default: throw DeviceError(status, m);
    }
}

class FacetrtCuda {
public:
    FacetrtCuda()
    {
        if (facetcu_create(&m_ctx) != FACETCU_OK) throw std::bad_alloc();
    }
    ~FacetrtCuda() { facetcu_release(m_ctx); }
    FacetrtCuda(const FacetrtCuda&) = delete;
    FacetrtCuda& operator=(const FacetrtCuda&) = delete;

    // The shader directory of the Vulkan backend has no meaning here.
    void initialize(const Config& config, const std::string& /*shaderDirectory*/ = {})
    {
        check(facetcu_initialize(m_ctx, reinterpret_cast<const facetcu_config*>(&config)));
        m_initialized = true;
    }
    void setGeometry(const std::vector<Vertex>& vertices)
    {
        check(facetcu_set_geometry(m_ctx, reinterpret_cast<const facetcu_vertex*>(vertices.data()),
                                   vertices.size()));
        m_facets = uint32_t(vertices.size() / 3U);
    }
    GraphDiagnostics buildVisibilityGraph(const std::vector<Direction>& directions)
    {
        GraphDiagnostics d{};
        check(facetcu_build_visibility_graph(
            m_ctx, reinterpret_cast<const facetcu_direction*>(directions.data()),
            uint32_t(directions.size()), reinterpret_cast<facetcu_graph_diagnostics*>(&d)));
        return d;
    }
    SolveResult solve(const std::vector<SurfaceOptics>& optics, float skyRadiosity,
                      uint32_t iterations = 64, float relaxation = 1.0f)
    {
        SolveResult r;
        r.radiosity.resize(optics.size());
        check(facetcu_solve(m_ctx, reinterpret_cast<const facetcu_surface_optics*>(optics.data()),
                            optics.size(), skyRadiosity, iterations, relaxation,
                            r.radiosity.data(), &r.iterations, &r.maxDelta));
        return r;
    }
    SolveResult solveAccelerated(const std::vector<SurfaceOptics>& optics, float skyRadiosity,
                                 const std::vector<float>* initialRadiosity = nullptr,
                                 uint32_t maximumIterations = 64, uint32_t batchIterations = 8,
                                 float tolerance = 1.0e-4f, float relaxation = 1.0f)
    {
        if (initialRadiosity && initialRadiosity->size() != optics.size())
            throw std::invalid_argument(
                "Initial radiosity must contain one finite non-negative value per surface");
        SolveResult r;
        r.radiosity.resize(optics.size());
        check(facetcu_solve_accelerated(
            m_ctx, reinterpret_cast<const facetcu_surface_optics*>(optics.data()), optics.size(),
            skyRadiosity, initialRadiosity ? initialRadiosity->data() : nullptr,
            maximumIterations, batchIterations, tolerance, relaxation, r.radiosity.data(),
            &r.iterations, &r.maxDelta));
        return r;
    }
    std::vector<float> incidentIrradiance(const SolveResult& solution,
                                          const std::vector<SurfaceOptics>& optics,
                                          float skyRadiosity) const
    {
        if (solution.radiosity.size() != optics.size())
            throw std::invalid_argument(
                "Incident irradiance requires a completed solve and visibility graph");
        std::vector<float> out(optics.size());
        check(facetcu_incident_irradiance(
            m_ctx, solution.radiosity.data(),
            reinterpret_cast<const facetcu_surface_optics*>(optics.data()), optics.size(),
            skyRadiosity, out.data()));
        return out;
    }
    std::vector<float> computeSunlitFraction(const Direction& sunDirection)
    {
        std::vector<float> out(size_t(m_facets) * 2U);
        check(facetcu_compute_sunlit_fraction(
            m_ctx, reinterpret_cast<const facetcu_direction*>(&sunDirection), out.data()));
        return out;
    }
    void destroy()
    {
        facetcu_destroy(m_ctx);
        m_initialized = false;
        m_facets = 0;
    }

    [[nodiscard]] bool initialized() const noexcept { return m_initialized; }
    [[nodiscard]] uint32_t facetCount() const noexcept { return m_facets; }
    [[nodiscard]] uint32_t surfaceCount() const noexcept { return m_facets * 2U; }
    [[nodiscard]] facetcu_context* handle() const noexcept { return m_ctx; }

private:
    void check(int status) const { throw_status(status, facetcu_last_error(m_ctx)); }

    facetcu_context* m_ctx{nullptr};
    bool m_initialized{false};
    uint32_t m_facets{0};
};

}  // namespace facetcu
