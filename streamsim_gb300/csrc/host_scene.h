// host_scene.h — host-side scene assembly and the eFacetRT run's output,
// shared by the OBJ loader (scene.cpp) and the XML project loader
// (project.cpp).  Triangles are appended as the reference's appendTriangle
// does (facetrtcore.cpp:287-306): the unit normal of (b - a) x (c - a) on all
// three vertices, degenerate triangles dropped.
#pragma once

#include <array>
#include <chrono>
#include <cstdint>
#include <filesystem>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/facetcu.h"

namespace facetcu {
namespace host {

using V3 = std::array<float, 3>;
using Clock = std::chrono::steady_clock;

struct HostScene {
    std::vector<facetcu_vertex> vertices;
    std::vector<uint32_t> material;
    uint32_t leaf = 0;
    V3 lo{}, hi{};
    uint32_t facets() const { return uint32_t(vertices.size() / 3); }
};

V3 sub(const V3& a, const V3& b);
V3 scaled(const V3& v, float s);
float dot3(const V3& a, const V3& b);
V3 cross3(const V3& a, const V3& b);
V3 unit(const V3& v);
bool push_triangle(HostScene& sc, const V3& a, const V3& b, const V3& c, uint32_t material);
// 0-based position index of an OBJ face token (negative = relative)
int obj_position(const std::string& token, size_t count);

struct RunOutput {
    std::string backend = "CUDA GPU";
    std::string quantity = "hemispherical radiosity";
    std::string units = "W m-2";
    facetcu_graph_diagnostics graph{};
    std::vector<float> radiosity, sunlit, enhancement, wavelengths, band_radiosity;
    uint32_t iterations = 0;
    float max_delta = 0.0f;
    double total_ms = 0, visibility_ms = 0, sunlight_ms = 0, solve_ms = 0;
};

double ms_between(Clock::time_point a, Clock::time_point b);
void progress(int value, const std::string& stage);
// writeWebResult (facetrtcore.cpp:1782-1840)
void write_web_result(const std::string& file, const HostScene& sc, const RunOutput& r);

// A context that throws the library's message on failure.
struct Context {
    facetcu_context* ctx = nullptr;
    Context();
    ~Context();
    void check(int status) const;
};

}  // namespace host

namespace dem {
// DemHeightField (facetrtcore.cpp:2618-2650): band 1 as float32, nodata and
// non-finite cells replaced by the minimum of the valid ones.
struct HeightField {
    int width = 0, height = 0;
    float minimum = 0.0f;
    std::vector<float> values;
    bool valid() const
    {
        return width >= 2 && height >= 2 && values.size() == size_t(width) * size_t(height);
    }
    float above_minimum(float north_x, float east_z, float scene_width, float scene_depth) const;
};
// readDemHeightField's file step (facetrtcore.cpp:2660-2696) over ESRI ASCII
// grids and baseline GeoTIFF; throws the reference's messages.
HeightField read_height_field(const std::filesystem::path& path);
// Up to max_bands raster bands as bytes (GDAL's RasterIO into GDT_Byte);
// failures throw open_error / read_error followed by the path.
struct ByteBands {
    int width = 0, height = 0, count = 0;
    std::vector<uint8_t> values[3];
};
ByteBands read_byte_bands(const std::filesystem::path& path, int max_bands,
                          const std::string& open_error, const std::string& read_error);
}  // namespace dem

namespace project {
// The XML view of a project.json (facetInputView, facetrtcore.cpp:1888-2036).
std::string xml_view(const std::string& path);
// The eFacetRT run of an XML project (runFacetRTCore with loadProjectScene
// and facetRTParametersFromInput, facetrtcore.cpp:3116-3161); writes
// result_file.  Throws on failure.
void run_facetrt(const std::string& input, const std::string& result_file);
}  // namespace project

}  // namespace facetcu
