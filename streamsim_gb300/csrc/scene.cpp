// scene.cpp — host side of the eFacetRT process seam on the CUDA backend.
//
// The reference's OBJ path through runFacetRTCore
// (models/histream/src/facetrt/facetrtcore.cpp:3116-3161):
//   loadTreeWithSoil (:361-473)   OBJ positions and faces, Y shifted to start
//                                 at 0, a 48 x 48 soil grid under the object
//                                 unless an `o STREAMSIM_TERRAIN` block exists
//   runGpu (:1621-1780)           40-direction graph, sun raster, makeOptics
//                                 (:500-522), a 64-sweep solve, a diffuse
//                                 solve and lightEnhancement (:1561-1583)
//   writeWebResult (:1782-1840)   facetrt.json, 9 significant digits
// with the context calls of this library in place of FacetrtVulkan.  The
// float arithmetic (normals, bounds, soil grid, direct irradiance) is written
// in the reference's operation order and compiled without contraction, so
// scenes and optics are bit-identical to the reference's.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "facetcu.h"
#include "host_scene.h"

namespace {

thread_local std::string g_host_error;

}  // namespace

// The message facetcu_host_last_error() reports for host-only entry points.
void facetcu_set_host_error(const std::string& message) { g_host_error = message; }

namespace facetcu {
namespace host {

V3 sub(const V3& a, const V3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
V3 scaled(const V3& v, float s) { return {v[0] * s, v[1] * s, v[2] * s}; }
float dot3(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
V3 cross3(const V3& a, const V3& b)
{
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
V3 unit(const V3& v)
{
    const float length = std::sqrt(dot3(v, v));
    if (!(length > 1.0e-8f)) throw std::runtime_error("Zero-length direction or degenerate triangle");
    return scaled(v, 1.0f / length);
}

bool push_triangle(HostScene& sc, const V3& a, const V3& b, const V3& c, uint32_t material)
{
    const V3 n = cross3(sub(b, a), sub(c, a));
    if (dot3(n, n) <= 1.0e-16f) return false;
    const V3 u = unit(n);
    for (const V3* p : {&a, &b, &c}) {
        facetcu_vertex v{};
        std::memcpy(v.position, p->data(), 12);
        std::memcpy(v.normal, u.data(), 12);
        sc.vertices.push_back(v);
    }
    sc.material.push_back(material);
    return true;
}

int obj_position(const std::string& token, size_t count)
{
    const std::string digits = token.substr(0, token.find('/'));
    if (digits.empty()) throw std::runtime_error("OBJ face has no position index");
    const int raw = std::stoi(digits);
    const long index = raw > 0 ? long(raw) - 1 : long(count) + raw;
    if (index < 0 || size_t(index) >= count)
        throw std::runtime_error("OBJ position index is out of range");
    return int(index);
}

// ---- the run --------------------------------------------------------------
double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

void progress(int value, const std::string& stage)
{
    std::cout << "PROGRESS\t" << value << '\t' << stage << std::endl;
}

Context::Context()
{
    if (facetcu_create(&ctx) != FACETCU_OK) throw std::bad_alloc();
}
Context::~Context() { facetcu_release(ctx); }
void Context::check(int status) const
{
    if (status != FACETCU_OK) throw std::runtime_error(facetcu_last_error(ctx));
}

void write_web_result(const std::string& file, const HostScene& sc, const RunOutput& r)
{
    std::ofstream out(file, std::ios::binary);
    if (!out) throw std::runtime_error("Cannot write web result: " + file);
    out << std::setprecision(9) << "{\n"
        << "  \"backend\": \"" << r.backend << "\",\n"
        << "  \"quantity\": \"" << r.quantity << "\",\n"
        << "  \"units\": \"" << r.units << "\",\n"
        << "  \"facetCount\": " << sc.facets() << ",\n"
        << "  \"leafFacetCount\": " << sc.leaf << ",\n"
        << "  \"vertexPositions\": [";
    for (size_t i = 0; i < sc.vertices.size(); ++i) {
        const float* p = sc.vertices[i].position;
        out << (i ? "," : "") << p[0] << ',' << p[1] << ',' << p[2];
    }
    out << "],\n"
        << "  \"graph\": {\"directedEdges\":" << r.graph.directed_edge_count
        << ",\"closureError\":" << r.graph.max_closure_error
        << ",\"fragmentOverflow\":" << r.graph.fragment_overflow
        << ",\"hashOverflow\":" << r.graph.hash_overflow << "},\n"
        << "  \"timing\": {\"totalMs\":" << r.total_ms << ",\"visibilityMs\":" << r.visibility_ms
        << ",\"sunlightMs\":" << r.sunlight_ms << ",\"solveMs\":" << r.solve_ms << "},\n"
        << "  \"iterations\": " << r.iterations << ",\n"
        << "  \"maxDelta\": " << r.max_delta << ",\n";
    auto array = [&out](const char* name, const std::vector<float>& v, bool comma) {
        out << "  \"" << name << "\": [";
        for (size_t i = 0; i < v.size(); ++i) out << (i ? "," : "") << v[i];
        out << ']' << (comma ? "," : "") << '\n';
    };
    array("wavelengths", r.wavelengths, true);
    array("sunlit", r.sunlit, true);
    array("radiosity", r.radiosity, true);
    array("lightEnhancement", r.enhancement, !r.band_radiosity.empty());
    if (!r.band_radiosity.empty()) array("bandRadiosity", r.band_radiosity, false);
    out << "}\n";
    if (!out) throw std::runtime_error("Cannot write web result: " + file);
}

}  // namespace host
}  // namespace facetcu

namespace {

using namespace facetcu::host;

constexpr uint32_t kSoilGrid = 48;        // facetrtcore.cpp:83
constexpr float kBeam = 700.0f;           // facetrtcore.cpp:84
constexpr float kSky = 100.0f;            // facetrtcore.cpp:85
constexpr uint32_t kSweeps = 64;          // facetrtcore.cpp:82
constexpr uint32_t kRaster = 1024;        // facetrtcore.cpp:74
constexpr uint32_t kLayers = 64;          // facetrtcore.cpp:75

HostScene load_tree_with_soil(const std::string& path)
{
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Cannot open tree OBJ: " + path);
    std::vector<V3> points;
    std::vector<std::array<int, 3>> faces;
    const size_t none = std::numeric_limits<size_t>::max();
    size_t terrain_start = none;
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream fields(line);
        std::string kind;
        fields >> kind;
        if (kind == "v") {
            V3 p{};
            if (!(fields >> p[0] >> p[1] >> p[2])) throw std::runtime_error("Invalid OBJ vertex");
            points.push_back(p);
        } else if (kind == "f") {
            std::vector<int> poly;
            std::string token;
            while (fields >> token) poly.push_back(obj_position(token, points.size()));
            for (size_t i = 1; i + 1 < poly.size(); ++i) faces.push_back({poly[0], poly[i], poly[i + 1]});
        } else if (kind == "o") {
            std::string name;
            fields >> name;
            if (name == "STREAMSIM_TERRAIN" && terrain_start == none) terrain_start = faces.size();
        }
    }
    if (points.empty() || faces.empty()) throw std::runtime_error("Tree OBJ contains no usable geometry");

    const float big = std::numeric_limits<float>::max();
    V3 lo{big, big, big}, hi{-big, -big, -big};
    for (const V3& p : points)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    for (V3& p : points) p[1] -= lo[1];

    const bool terrain = terrain_start != none && terrain_start < faces.size();
    HostScene sc;
    sc.vertices.reserve((faces.size() + (terrain ? 0 : 2 * kSoilGrid * kSoilGrid)) * 3);
    uint32_t objects = 0;
    for (size_t i = 0; i < faces.size(); ++i) {
        const bool ground = terrain && i >= terrain_start;
        if (push_triangle(sc, points[faces[i][0]], points[faces[i][1]], points[faces[i][2]],
                          ground ? 1u : 0u) &&
            !ground)
            ++objects;
    }
    sc.leaf = terrain ? objects : sc.facets();

    float x0 = lo[0], x1 = hi[0], z0 = lo[2], z1 = hi[2];
    if (!terrain) {
        const float margin = 0.5f * std::max(hi[0] - lo[0], hi[2] - lo[2]);
        x0 -= margin;
        x1 += margin;
        z0 -= margin;
        z1 += margin;
        const float n = float(kSoilGrid), y = -0.01f;
        for (uint32_t r = 0; r < kSoilGrid; ++r) {
            const float za = z0 + (z1 - z0) * float(r) / n;
            const float zb = z0 + (z1 - z0) * float(r + 1) / n;
            for (uint32_t c = 0; c < kSoilGrid; ++c) {
                const float xa = x0 + (x1 - x0) * float(c) / n;
                const float xb = x0 + (x1 - x0) * float(c + 1) / n;
                push_triangle(sc, {xa, y, za}, {xb, y, zb}, {xb, y, za}, 1u);
                push_triangle(sc, {xa, y, za}, {xa, y, zb}, {xb, y, zb}, 1u);
            }
        }
    }
    sc.lo = {x0, terrain ? 0.0f : -0.01f, z0};
    sc.hi = {x1, hi[1] - lo[1], z1};
    return sc;
}

void make_optics(const facetcu_vertex* v, uint32_t facets, uint32_t leaf, const float* sunlit,
                 const facetcu_direction& sun_dir, facetcu_surface_optics* out)
{
    const V3 sun{sun_dir.x, sun_dir.y, sun_dir.z};
    for (uint32_t f = 0; f < facets; ++f) {
        const bool object = f < leaf;
        const V3 n{v[3 * f].normal[0], v[3 * f].normal[1], v[3 * f].normal[2]};
        for (uint32_t k = 0; k < 2; ++k) {
            const uint32_t s = 2 * f + k;
            const V3 side = scaled(n, k == 0 ? 1.0f : -1.0f);
            out[s].reflectance = object ? 0.10f : 0.20f;
            out[s].transmittance = object ? 0.05f : 0.0f;
            out[s].emission = 0.0f;
            out[s].direct_irradiance = sunlit[s] * std::max(0.0f, dot3(side, sun)) * kBeam;
        }
    }
}

RunOutput run_gpu(const HostScene& sc)
{
    RunOutput r;
    const auto t_begin = Clock::now();
    progress(3, "Creating CUDA context and device buffers");
    Context c;
    facetcu_config cfg{};
    cfg.raster_width = kRaster;
    cfg.raster_height = kRaster;
    cfg.max_fragments_per_pixel = kLayers;
    cfg.periodic_size_x = 1.0f;
    cfg.periodic_size_z = 1.0f;
    c.check(facetcu_initialize(c.ctx, &cfg));
    c.check(facetcu_set_geometry(c.ctx, sc.vertices.data(), sc.vertices.size()));

    progress(10, "GPU visibility graph: 40 directions at " + std::to_string(kRaster) + " x " +
                     std::to_string(kRaster));
    const auto t_vis = Clock::now();
    std::vector<facetcu_direction> dirs(40);
    facetcu_hemisphere_directions(40, dirs.data());
    c.check(facetcu_build_visibility_graph(c.ctx, dirs.data(), 40, &r.graph));
    const auto t_vis_end = Clock::now();
    r.visibility_ms = ms_between(t_vis, t_vis_end);

    progress(72, "GPU sunlight visibility raster");
    const uint32_t S = sc.facets() * 2;
    const facetcu_direction sun = facetcu_sun_direction(30.0f, 135.0f);
    r.sunlit.resize(S);
    c.check(facetcu_compute_sunlit_fraction(c.ctx, &sun, r.sunlit.data()));
    const auto t_sun_end = Clock::now();
    r.sunlight_ms = ms_between(t_vis_end, t_sun_end);

    progress(82, "GPU Jacobi radiosity: 64 iterations");
    std::vector<facetcu_surface_optics> optics(S);
    make_optics(sc.vertices.data(), sc.facets(), sc.leaf, r.sunlit.data(), sun, optics.data());
    r.radiosity.resize(S);
    c.check(facetcu_solve(c.ctx, optics.data(), S, kSky, kSweeps, 1.0f, r.radiosity.data(),
                          &r.iterations, &r.max_delta));
    progress(98, "GPU diffuse baseline and direct-light enhancement");
    for (auto& o : optics) o.direct_irradiance = 0.0f;
    std::vector<float> diffuse(S);
    uint32_t it = 0;
    float md = 0.0f;
    c.check(facetcu_solve(c.ctx, optics.data(), S, kSky, kSweeps, 1.0f, diffuse.data(), &it, &md));
    r.enhancement.resize(S);
    for (uint32_t s = 0; s < S; ++s) r.enhancement[s] = std::max(0.0f, r.radiosity[s] - diffuse[s]);
    const auto t_end = Clock::now();
    r.solve_ms = ms_between(t_sun_end, t_end);
    r.total_ms = ms_between(t_begin, t_end);
    progress(100, "CUDA GPU complete");
    return r;
}

bool has_obj_extension(const std::filesystem::path& p)
{
    return p.extension() == ".obj" || p.extension() == ".OBJ";
}

}  // namespace

extern "C" {

const char* facetcu_host_last_error(void) { return g_host_error.c_str(); }

int facetcu_load_tree_with_soil(const char* path, facetcu_vertex* vertices,
                                uint32_t* material_indices, uint32_t capacity_facets,
                                facetcu_scene_info* info)
{
    g_host_error.clear();
    if (!path || !info) {
        g_host_error = "path and info are required";
        return FACETCU_INVALID_ARGUMENT;
    }
    try {
        const HostScene sc = load_tree_with_soil(path);
        info->facet_count = sc.facets();
        info->leaf_facet_count = sc.leaf;
        std::memcpy(info->minimum, sc.lo.data(), 12);
        std::memcpy(info->maximum, sc.hi.data(), 12);
        if (vertices || material_indices) {
            if (capacity_facets < sc.facets()) {
                g_host_error = "capacity_facets is smaller than the scene";
                return FACETCU_INVALID_ARGUMENT;
            }
            if (vertices) std::memcpy(vertices, sc.vertices.data(), sc.vertices.size() * 24);
            if (material_indices)
                std::memcpy(material_indices, sc.material.data(), sc.material.size() * 4);
        }
        return FACETCU_OK;
    } catch (const std::exception& e) {
        g_host_error = e.what();
        return FACETCU_RUNTIME_ERROR;
    }
}

int facetcu_make_optics(const facetcu_vertex* vertices, uint32_t facet_count,
                        uint32_t leaf_facet_count, const float* sunlit,
                        const facetcu_direction* sun, facetcu_surface_optics* optics)
{
    g_host_error.clear();
    if (!vertices || !sunlit || !sun || !optics) {
        g_host_error = "vertices, sunlit, sun and optics are required";
        return FACETCU_INVALID_ARGUMENT;
    }
    make_optics(vertices, facet_count, leaf_facet_count, sunlit, *sun, optics);
    return FACETCU_OK;
}

float facetcu_planck_radiance(float wavelength, float temperature)
{
    // Planck's law in W m-2 sr-1 um-1: c1 = 2 h c^2, c2 = h c / k (um K),
    // wavelength in nm above 50 (else um), in double like the reference
    // (facetrtcore.cpp:524-536).
    const double c1 = 1.1910439340652e8, c2 = 14388.291040407;
    const double um = wavelength > 50.0f ? double(wavelength) / 1000.0 : double(wavelength);
    const double x = c2 / (std::max(1.0, double(temperature)) * std::max(1.0e-6, um));
    return float(c1 / (std::pow(um, 5.0) * std::expm1(x)));
}

int facetcu_run_facetrt_core(const char* input_path, const char* shader_directory,
                             const char* output_file)
{
    (void)shader_directory;  // the Vulkan backend's SPIR-V directory; nothing to load here
    try {
        const std::string input = input_path ? input_path : "";
        if (input.empty()) throw std::invalid_argument("FacetRT requires project.json");
        const std::filesystem::path in(input);
        std::string result_file = output_file ? output_file : "";
        if (result_file.empty()) result_file = (in.parent_path() / "facetrt.json").lexically_normal().string();
        if (!has_obj_extension(in)) {
            // an XML project (the reference's Input.xml): loadProjectScene
            facetcu::project::run_facetrt(input, result_file);
            std::cout << "RESULT\t" << result_file << std::endl;
            return 0;
        }
        const HostScene sc = load_tree_with_soil(input);
        const char* env = std::getenv("HISTREAM_FACET_BACKEND");
        if (env && std::string(env) == "cpu")
            std::cerr << "facetrt: the retained CPU raster backend is not part of this build; "
                         "running the CUDA backend\n";
        const RunOutput r = run_gpu(sc);
        const std::filesystem::path parent = std::filesystem::path(result_file).parent_path();
        if (!parent.empty()) std::filesystem::create_directories(parent);
        write_web_result(result_file, sc, r);
        std::cout << "RESULT\t" << result_file << std::endl;
        return 0;
    } catch (const std::exception& e) {
        std::cerr << "facetrt: " << e.what() << '\n';
        return 1;
    }
}

}  // extern "C"
