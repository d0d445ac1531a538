// api.cpp — the extern "C" entry points of include/facetcu.h.
//
// Each entry point mirrors a member of facetvk::FacetrtVulkan
// (models/histream/src/facetrt/facetrt_vulkan.{h,cpp}): same preconditions,
// same validation rules and messages, same outputs; exceptions become status
// codes (see facetcu.h).  Host arithmetic that must round as the reference's
// CPU rasterizer does (the orthographic frame) is compiled with
// -ffp-contract=off.
#include <algorithm>
#include <array>
#include <chrono>
#include <fstream>
#include <map>
#include <sstream>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "internal.h"

using namespace facetcu;

struct facetcu_context {
    std::string last_error;
    bool initialized = false;
    facetcu_config config{};
    int device = -1;
    cudaStream_t stream = nullptr;

    uint32_t facets = 0;
    std::vector<facetcu_vertex> vertices_host;
    DeviceBuffer vertices;
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    bool bounds_override = false;
    float omin[3] = {0, 0, 0}, omax[3] = {0, 0, 0};

    DeviceGraph graph;
    bool graph_ready = false;

    RasterBuffers raster;
    DeviceBuffer pairs, pair_count, denom_tmp;
    Workspace ws;

    DeviceBuffer optics, rad_a, rad_b, residual, host_io, scratch;
    DeviceBuffer sun_total, sun_visible;
    BatchState batch;
    DeviceBuffer batch_inputs;

    Lbvh bvh;
    bool bvh_ready = false;
    mlp::Net net;
    mlp::Scratch mlp_scratch;
    mlp::TensorScratch mlp_tensor;
    DeviceBuffer mlp_io, warm_b1, warm_x, warm_y, warm_x0;
    DeviceBuffer samples_uv, samples_dir, fraction;
    spectral::Tables spec;
    DeviceBuffer spec_io;
    DeviceBuffer eb_io, eb_tab;  // FacetEB node fields and per-material tables
    DeviceBuffer img_io;         // sensor image scratch and outputs
    // autotuned settings by problem key: the panel width and the pipelined
    // int8 step's CTAs per SM (0: as many as fit)
    struct Tuned {
        uint32_t panel_width = 0, step_ctas = 0;
    };
    std::map<std::string, Tuned> tuned;
    std::string gpu_name;                   // for the autotuner's key
};

namespace {

int fail(facetcu_context* ctx, int code, const std::string& msg)
{
    if (ctx) ctx->last_error = msg;
    return code;
}

template <typename F>
int guarded(facetcu_context* ctx, F&& body)
{
    if (!ctx) return FACETCU_INVALID_ARGUMENT;
    try {
        ctx->last_error.clear();
        return body();
    } catch (const Error& e) {
        return fail(ctx, e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(ctx, FACETCU_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(ctx, FACETCU_RUNTIME_ERROR, e.what());
    }
}

void require_initialized(facetcu_context* ctx, const char* what)
{
    if (!ctx->initialized)
        throw Error(FACETCU_LOGIC_ERROR, std::string("initialize() must be called before ") + what);
    FCU_CHECK(cudaSetDevice(ctx->device));
}

void require_graph(facetcu_context* ctx, const char* what)
{
    require_initialized(ctx, what);
    if (!ctx->graph_ready)
        throw Error(FACETCU_LOGIC_ERROR,
                    std::string("buildVisibilityGraph() must be called before ") + what);
}

// ---- host frame arithmetic (facetrtcore.cpp:262-269, :1222-1255) ----------
using V3 = std::array<float, 3>;
float dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
V3 cross(const V3& a, const V3& b)
{
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
V3 normalized(const V3& v, const char* what)
{
    const float length = std::sqrt(dot(v, v));
    if (!(length > 1.0e-8f)) throw Error(FACETCU_INVALID_ARGUMENT, what);
    const float inv = 1.0f / length;
    return {v[0] * inv, v[1] * inv, v[2] * inv};
}
const int kTileOffsets[20][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {-1, 1}, {1, -1},
                                 {1, 1},  {-2, 0}, {2, 0}, {0, -2}, {0, 2}, {-2, -1}, {-2, 1},
                                 {2, -1}, {2, 1},  {-1, -2}, {1, -2}, {-1, 2}, {1, 2}};

PeriodicTiles make_tiles(const facetcu_context* ctx)
{
    PeriodicTiles p;
    p.count = std::min(ctx->config.periodic_neighbor_count, 20u);
    for (uint32_t t = 1; t <= p.count; ++t) {
        p.dx[t] = float(kTileOffsets[t - 1][0]) * ctx->config.periodic_size_x;
        p.dz[t] = float(kTileOffsets[t - 1][1]) * ctx->config.periodic_size_z;
    }
    return p;
}

RasterFrame make_frame(const facetcu_context* ctx)
{
    RasterFrame f{};
    const float* mn = ctx->bounds_override ? ctx->omin : ctx->bmin;
    const float* mx = ctx->bounds_override ? ctx->omax : ctx->bmax;
    V3 emin{mn[0], mn[1], mn[2]}, emax{mx[0], mx[1], mx[2]};
    const uint32_t neighbours = std::min(ctx->config.periodic_neighbor_count, 20u);
    f.tiles = neighbours + 1u;
    f.tile_dx[0] = 0.0f;
    f.tile_dz[0] = 0.0f;
    for (uint32_t t = 1; t <= neighbours; ++t) {
        const int* o = kTileOffsets[t - 1];
        const float ox = float(o[0]) * ctx->config.periodic_size_x;
        const float oz = float(o[1]) * ctx->config.periodic_size_z;
        f.tile_dx[t] = ox;
        f.tile_dz[t] = oz;
        emin[0] = std::min(emin[0], mn[0] + ox);
        emax[0] = std::max(emax[0], mx[0] + ox);
        emin[2] = std::min(emin[2], mn[2] + oz);
        emax[2] = std::max(emax[2], mx[2] + oz);
    }
    const V3 diag{emax[0] - emin[0], emax[1] - emin[1], emax[2] - emin[2]};
    f.center[0] = (emin[0] + emax[0]) * 0.5f;
    f.center[1] = (emin[1] + emax[1]) * 0.5f;
    f.center[2] = (emin[2] + emax[2]) * 0.5f;
    f.radius = std::max(0.5f * std::sqrt(dot(diag, diag)) * 1.001f, 1.0e-4f);
    f.width = ctx->config.raster_width;
    f.height = ctx->config.raster_height;
    f.facets = ctx->facets;
    return f;
}

RasterView make_view(const facetcu_direction& d)
{
    const V3 view = normalized({d.x, d.y, d.z}, "A visibility direction has zero length");
    const V3 ref = std::abs(view[2]) < 0.9f ? V3{0.0f, 0.0f, 1.0f} : V3{0.0f, 1.0f, 0.0f};
    const V3 right = normalized(cross(ref, view), "A visibility direction has zero length");
    const V3 up = cross(view, right);
    RasterView v{};
    for (int i = 0; i < 3; ++i) {
        v.right[i] = right[i];
        v.up[i] = up[i];
        v.view[i] = view[i];
    }
    return v;
}

int side_bits_for(uint32_t surfaces)
{
    int b = 1;
    while ((1ull << b) < surfaces) ++b;
    return b;
}

uint32_t chain_cap(const facetcu_context* ctx) { return ctx->config.max_fragments_per_pixel; }

// facetrt_vulkan.cpp:1160-1175
void validate_optics(const facetcu_surface_optics* optics, size_t n)
{
    if (!optics) throw Error(FACETCU_INVALID_ARGUMENT, "Optics array must contain exactly two sides per facet");
    for (size_t i = 0; i < n; ++i) {
        const facetcu_surface_optics& v = optics[i];
        if (!std::isfinite(v.reflectance) || !std::isfinite(v.transmittance) ||
            !std::isfinite(v.emission) || !std::isfinite(v.direct_irradiance) ||
            v.reflectance < 0.0f || v.transmittance < 0.0f || v.emission < 0.0f ||
            v.direct_irradiance < 0.0f || v.reflectance + v.transmittance > 1.0001f) {
            throw Error(FACETCU_INVALID_ARGUMENT,
                        "Optical values must be finite, non-negative, and reflectance+transmittance<=1");
        }
    }
}

void validate_count(uint64_t count, uint32_t surfaces)
{
    if (count != surfaces)
        throw Error(FACETCU_INVALID_ARGUMENT, "Optics array must contain exactly two sides per facet");
}

void validate_sky(float sky)
{
    if (!std::isfinite(sky) || sky < 0.0f)
        throw Error(FACETCU_INVALID_ARGUMENT, "skyRadiosity must be finite and non-negative");
}

void validate_relax(float r)
{
    if (!(r > 0.0f && r <= 1.0f))
        throw Error(FACETCU_INVALID_ARGUMENT, "GPU Jacobi relaxation must be in (0,1]");
}

void upload(DeviceBuffer& buf, const void* src, size_t bytes, cudaStream_t s)
{
    buf.reserve(bytes);
    if (bytes) FCU_CHECK(cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, s));
}

// The plain Jacobi loop shared by solve and solveAccelerated.  Runs `count`
// sweeps starting from buffer `ping`; each sweep's max|dB| lands in
// residual[sweep_index].  Returns the new ping.
uint32_t run_sweeps(facetcu_context* ctx, float sky, float relax, uint32_t count, uint32_t ping,
                    uint32_t first_slot)
{
    float* a = ctx->rad_a.as<float>();
    float* b = ctx->rad_b.as<float>();
    uint32_t* res = ctx->residual.as<uint32_t>();
    for (uint32_t i = 0; i < count; ++i) {
        const float* in = ping == 0 ? a : b;
        float* out = ping == 0 ? b : a;
        jacobi_plain_sweep(ctx->graph, ctx->optics.as<facetcu_surface_optics>(), sky, relax, in,
                           out, res + first_slot + i, ctx->stream);
        ping ^= 1u;
    }
    return ping;
}

}  // namespace

extern "C" {

// facetrtcore.cpp:475-489
void facetcu_hemisphere_directions(uint32_t count, facetcu_direction* out)
{
    if (!out) return;
    const float golden = 2.39996322972865332f;
    for (uint32_t i = 0; i < count; ++i) {
        const float y = (static_cast<float>(i) + 0.5f) / static_cast<float>(count);
        const float radius = std::sqrt(std::max(0.0f, 1.0f - y * y));
        const float azimuth = golden * static_cast<float>(i);
        out[i] = {radius * std::cos(azimuth), y, radius * std::sin(azimuth)};
    }
}

// facetrtcore.cpp:491-498
facetcu_direction facetcu_sun_direction(float zenith_degrees, float azimuth_degrees)
{
    const float pi = 3.14159265358979323846f;
    const float zenith = zenith_degrees * pi / 180.0f;
    const float azimuth = azimuth_degrees * pi / 180.0f;
    return {std::sin(zenith) * std::cos(azimuth), std::cos(zenith),
            std::sin(zenith) * std::sin(azimuth)};
}

int facetcu_create(facetcu_context** out)
{
    if (!out) return FACETCU_INVALID_ARGUMENT;
    try {
        *out = new facetcu_context();
    } catch (...) {
        return FACETCU_OUT_OF_MEMORY;
    }
    return FACETCU_OK;
}

void facetcu_release(facetcu_context* ctx)
{
    if (!ctx) return;
    facetcu_destroy(ctx);
    delete ctx;
}

const char* facetcu_last_error(const facetcu_context* ctx)
{
    return ctx ? ctx->last_error.c_str() : "null context";
}

int facetcu_device_count(int* count)
{
    if (!count) return FACETCU_INVALID_ARGUMENT;
    int n = 0;
    const cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *count = 0;
        return FACETCU_OK;
    }
    *count = n;
    return FACETCU_OK;
}

// FacetrtVulkan::initialize (facetrt_vulkan.cpp:98-110)
int facetcu_initialize(facetcu_context* ctx, const facetcu_config* config)
{
    return guarded(ctx, [&] {
        facetcu_destroy(ctx);
        if (!config) throw Error(FACETCU_INVALID_ARGUMENT, "config is null");
        if (config->raster_width == 0 || config->raster_height == 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "Raster dimensions must be positive");
        if (config->max_fragments_per_pixel == 0 || config->max_fragments_per_pixel > 1024)
            throw Error(FACETCU_INVALID_ARGUMENT, "maxFragmentsPerPixel must be in [1, 1024]");
        if (uint64_t(config->raster_width) * config->raster_height > (1ull << 26))
            throw Error(FACETCU_INVALID_ARGUMENT, "Raster exceeds 8192 x 8192 pixels");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
            cudaGetLastError();
            throw Error(FACETCU_NO_DEVICE, "No CUDA device is available for FacetRT");
        }
        if (int(config->gpu_index) >= n)
            throw Error(FACETCU_INVALID_ARGUMENT, "gpuIndex exceeds the number of CUDA devices");
        ctx->device = int(config->gpu_index);
        FCU_CHECK(cudaSetDevice(ctx->device));
        FCU_CHECK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->config = *config;
        ctx->initialized = true;
        return FACETCU_OK;
    });
}

// FacetrtVulkan::destroy (facetrt_vulkan.cpp:1486-1516)
int facetcu_destroy(facetcu_context* ctx)
{
    if (!ctx) return FACETCU_INVALID_ARGUMENT;
    if (!ctx->initialized) return FACETCU_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->vertices.release();
    ctx->graph.row_offsets.release();
    ctx->graph.edges.release();
    ctx->graph.denominators.release();
    ctx->graph.sky.release();
    ctx->graph.packed.release();
    ctx->graph.packed_valid = false;
    for (DeviceBuffer* b : {&ctx->graph.order, &ctx->graph.rank, &ctx->graph.p_rows,
                            &ctx->graph.p_packed, &ctx->graph.p_denom, &ctx->graph.p_sky})
        b->release();
    ctx->graph.perm_valid = false;
    ctx->graph.scene_facets.clear();
    ctx->graph.p_scene.release();
    ctx->graph_ready = false;
    for (DeviceBuffer* b : {&ctx->raster.counts, &ctx->raster.offsets, &ctx->raster.records,
                            &ctx->raster.big_list, &ctx->raster.deep_list, &ctx->raster.stats,
                            &ctx->pairs, &ctx->pair_count, &ctx->denom_tmp, &ctx->ws.a, &ctx->ws.b,
                            &ctx->ws.c, &ctx->ws.d, &ctx->ws.e, &ctx->optics, &ctx->rad_a,
                            &ctx->rad_b, &ctx->residual, &ctx->host_io, &ctx->scratch,
                            &ctx->sun_total, &ctx->sun_visible, &ctx->batch.x0, &ctx->batch.x1,
                            &ctx->batch.half, &ctx->batch.colstats, &ctx->batch.q,
                            &ctx->batch.corr, &ctx->batch.i8, &ctx->batch_inputs, &ctx->spec_io,
                            &ctx->spec.dev, &ctx->eb_io, &ctx->eb_tab, &ctx->img_io})
        b->release();
    release_graphs(ctx->batch);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = nullptr;
    ctx->facets = 0;
    for (DeviceBuffer* b : {&ctx->bvh.nodes, &ctx->bvh.tri, &ctx->bvh.parent, &ctx->bvh.flags,
                            &ctx->samples_uv, &ctx->samples_dir, &ctx->fraction, &ctx->mlp_io,
                            &ctx->warm_b1, &ctx->warm_x, &ctx->warm_y, &ctx->warm_x0,
                            &ctx->net.params, &ctx->net.bf16, &ctx->net.adam_m, &ctx->net.adam_v,
                            &ctx->net.grad})
        b->release();
    for (DeviceBuffer* b : {&ctx->mlp_scratch.z1, &ctx->mlp_scratch.a1, &ctx->mlp_scratch.z2,
                            &ctx->mlp_scratch.a2, &ctx->mlp_scratch.y, &ctx->mlp_scratch.dy,
                            &ctx->mlp_scratch.da, &ctx->mlp_scratch.dz, &ctx->mlp_scratch.part,
                            &ctx->mlp_scratch.lossp, &ctx->mlp_scratch.idx, &ctx->mlp_scratch.xb,
                            &ctx->mlp_scratch.tb, &ctx->mlp_tensor.xb, &ctx->mlp_tensor.a1,
                            &ctx->mlp_tensor.a2, &ctx->mlp_tensor.w1p, &ctx->mlp_tensor.error})
        b->release();
    ctx->net.ready = false;
    ctx->bvh_ready = false;
    ctx->vertices_host.clear();
    ctx->bounds_override = false;
    ctx->initialized = false;
    return FACETCU_OK;
}

int facetcu_get_stream(facetcu_context* ctx, void** stream)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "getStream()");
        if (!stream) throw Error(FACETCU_INVALID_ARGUMENT, "stream is null");
        *stream = ctx->stream;
        return FACETCU_OK;
    });
}

// FacetrtVulkan::setGeometry + validateGeometry (facetrt_vulkan.cpp:425-471)
int facetcu_set_geometry(facetcu_context* ctx, const facetcu_vertex* vertices,
                         uint64_t vertex_count)
{
    return guarded(ctx, [&] {
        if (!ctx->initialized)
            throw Error(FACETCU_LOGIC_ERROR, "initialize() must be called before setGeometry()");
        FCU_CHECK(cudaSetDevice(ctx->device));
        if (!vertices || vertex_count == 0 || vertex_count % 3 != 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "Geometry must be a non-empty triangle list");
        if (vertex_count / 3 > (1ull << 30))
            throw Error(FACETCU_OVERFLOW_ERROR, "Geometry exceeds 2^30 facets");
        for (uint64_t i = 0; i < vertex_count; ++i) {
            const facetcu_vertex& v = vertices[i];
            for (float c : v.position)
                if (!std::isfinite(c))
                    throw Error(FACETCU_INVALID_ARGUMENT, "Geometry contains a non-finite position");
            const float len = std::sqrt(v.normal[0] * v.normal[0] + v.normal[1] * v.normal[1] +
                                        v.normal[2] * v.normal[2]);
            if (!(len > 0.99f && len < 1.01f))
                throw Error(FACETCU_INVALID_ARGUMENT, "Facet normals must be normalized");
        }
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        ctx->graph_ready = false;
        ctx->graph.packed_valid = false;
        ctx->graph.perm_valid = false;
        ctx->graph.scene_facets.clear();
        ctx->bvh_ready = false;
        ctx->facets = uint32_t(vertex_count / 3);
        ctx->vertices_host.assign(vertices, vertices + vertex_count);
        for (int a = 0; a < 3; ++a) {
            ctx->bmin[a] = std::numeric_limits<float>::max();
            ctx->bmax[a] = std::numeric_limits<float>::lowest();
        }
        for (uint64_t i = 0; i < vertex_count; ++i)
            for (int a = 0; a < 3; ++a) {
                ctx->bmin[a] = std::min(ctx->bmin[a], vertices[i].position[a]);
                ctx->bmax[a] = std::max(ctx->bmax[a], vertices[i].position[a]);
            }
        upload(ctx->vertices, vertices, vertex_count * sizeof(facetcu_vertex), ctx->stream);
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        return FACETCU_OK;
    });
}

int facetcu_set_raster_bounds(facetcu_context* ctx, const float minimum[3], const float maximum[3])
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "setRasterBounds()");
        if (!minimum || !maximum) {
            ctx->bounds_override = false;
            return FACETCU_OK;
        }
        for (int a = 0; a < 3; ++a) {
            if (!std::isfinite(minimum[a]) || !std::isfinite(maximum[a]) || maximum[a] < minimum[a])
                throw Error(FACETCU_INVALID_ARGUMENT, "Raster bounds must be finite and ordered");
            ctx->omin[a] = minimum[a];
            ctx->omax[a] = maximum[a];
        }
        ctx->bounds_override = true;
        return FACETCU_OK;
    });
}

// FacetrtVulkan::buildVisibilityGraph (facetrt_vulkan.cpp:866-1062)
int facetcu_build_visibility_graph(facetcu_context* ctx, const facetcu_direction* directions,
                                   uint32_t direction_count,
                                   facetcu_graph_diagnostics* diagnostics)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "buildVisibilityGraph()");
        if (ctx->facets == 0)
            throw Error(FACETCU_LOGIC_ERROR, "setGeometry() must be called before buildVisibilityGraph()");
        if (!directions || direction_count == 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "At least one visibility direction is required");
        ctx->graph_ready = false;
        const uint32_t S = ctx->facets * 2u;
        const int side_bits = side_bits_for(S);
        std::vector<RasterView> views(direction_count);
        for (uint32_t d = 0; d < direction_count; ++d) views[d] = make_view(directions[d]);
        const RasterFrame frame = make_frame(ctx);
        if (uint64_t(frame.tiles) * ctx->facets >= (1ull << 31))
            throw Error(FACETCU_OVERFLOW_ERROR, "facets x periodic tiles exceeds 2^31");
        cudaStream_t s = ctx->stream;
        DeviceGraph& g = ctx->graph;
        g.surfaces = S;
        uint32_t* denom = static_cast<uint32_t*>(g.denominators.reserve(size_t(S) * 4));
        uint32_t* sky = static_cast<uint32_t*>(g.sky.reserve(size_t(S) * 4));
        FCU_CHECK(cudaMemsetAsync(denom, 0, size_t(S) * 4, s));
        FCU_CHECK(cudaMemsetAsync(sky, 0, size_t(S) * 4, s));
        unsigned long long* pair_count =
            static_cast<unsigned long long*>(ctx->pair_count.reserve(16));
        FCU_CHECK(cudaMemsetAsync(pair_count, 0, 8, s));
        // directions per chunk: keep the per-pixel count/offset arrays near 1 GiB
        const uint64_t pixels = uint64_t(frame.width) * frame.height;
        uint32_t chunk = uint32_t(std::max<uint64_t>(1, (1ull << 30) / (8 * pixels)));
        chunk = std::min<uint32_t>(std::min<uint32_t>(chunk, 64u), direction_count);
        uint64_t overflow = 0, pairs_used = 0, pairs_cap = ctx->pairs.bytes / 8;
        uint32_t capacity_error = 0, max_chain = 0;
        for (uint32_t d0 = 0; d0 < direction_count; d0 += chunk) {
            const uint32_t n = std::min(chunk, direction_count - d0);
            RasterStats st{};
            raster_fragments(ctx->vertices.as<facetcu_vertex>(), frame, views.data() + d0, n,
                             ctx->raster, ctx->ws, st, s);
            // pairs of this chunk are at most the fragments of it
            const uint64_t need = pairs_used + st.fragments + 1;
            if (need > pairs_cap) {
                DeviceBuffer grown;
                grown.reserve(std::max<uint64_t>(need, pairs_cap * 2) * 8);
                if (pairs_used)
                    FCU_CHECK(cudaMemcpyAsync(grown.ptr, ctx->pairs.ptr, pairs_used * 8,
                                              cudaMemcpyDeviceToDevice, s));
                FCU_CHECK(cudaStreamSynchronize(s));
                std::swap(ctx->pairs.ptr, grown.ptr);
                std::swap(ctx->pairs.bytes, grown.bytes);
                pairs_cap = ctx->pairs.bytes / 8;
            }
            raster_resolve_graph(frame, n, chain_cap(ctx), ctx->raster, denom, sky,
                                 ctx->pairs.as<uint64_t>(), pair_count, side_bits, st, s);
            unsigned long long used = 0;
            FCU_CHECK(cudaMemcpyAsync(&used, pair_count, 8, cudaMemcpyDeviceToHost, s));
            FCU_CHECK(cudaStreamSynchronize(s));
            pairs_used = used;
            overflow += st.overflow;
            capacity_error += st.capacity_error;
            max_chain = std::max(max_chain, st.max_chain);
        }
        facetcu_graph_diagnostics diag{};
        diag.facet_count = ctx->facets;
        diag.surface_count = S;
        diag.fragment_overflow = uint32_t(std::min<uint64_t>(overflow, 0xffffffffu));
        diag.hash_overflow = 0;
        if (diagnostics) *diagnostics = diag;
        if (overflow)
            throw Error(FACETCU_RUNTIME_ERROR,
                        "Visibility A-buffer overflow; increase Config::maxFragmentsPerPixel");
        if (capacity_error)
            throw Error(FACETCU_DEVICE_CAPACITY, "a pixel chain exceeded the 1024-fragment device capacity");
        graph_from_pairs(ctx->pairs.as<uint64_t>(), pairs_used, side_bits, g, ctx->ws, s);
        float closure = 0.0f;
        uint32_t sampled = 0;
        graph_closure(g, &closure, &sampled, ctx->ws, s);
        diag.directed_edge_count = uint32_t(g.nnz);
        diag.max_closure_error = closure;
        if (diagnostics) *diagnostics = diag;
        if (sampled == 0)
            throw Error(FACETCU_RUNTIME_ERROR,
                        "Visibility raster has no surface samples; radiation results are invalid");
        graph_pack(g, ctx->ws, s);
        FCU_CHECK(cudaStreamSynchronize(s));
        ctx->graph_ready = true;
        return FACETCU_OK;
    });
}

// FacetrtVulkan::computeSunlitFraction (facetrt_vulkan.cpp:1064-1158)
int facetcu_compute_sunlit_fraction(facetcu_context* ctx, const facetcu_direction* sun,
                                    float* fraction)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "computeSunlitFraction()");
        if (ctx->facets == 0)
            throw Error(FACETCU_LOGIC_ERROR, "setGeometry() must be called before computeSunlitFraction()");
        if (!sun || !fraction) throw Error(FACETCU_INVALID_ARGUMENT, "sun direction and output are required");
        const uint32_t S = ctx->facets * 2u;
        const RasterView view = make_view(*sun);
        const RasterFrame frame = make_frame(ctx);
        cudaStream_t s = ctx->stream;
        RasterStats st{};
        raster_fragments(ctx->vertices.as<facetcu_vertex>(), frame, &view, 1, ctx->raster, ctx->ws,
                         st, s);
        uint32_t* total = static_cast<uint32_t*>(ctx->sun_total.reserve(size_t(S) * 4));
        uint32_t* visible = static_cast<uint32_t*>(ctx->sun_visible.reserve(size_t(S) * 4));
        FCU_CHECK(cudaMemsetAsync(total, 0, size_t(S) * 4, s));
        FCU_CHECK(cudaMemsetAsync(visible, 0, size_t(S) * 4, s));
        raster_resolve_sunlit(frame, chain_cap(ctx), ctx->raster, total, visible, st, s);
        if (st.overflow)
            throw Error(FACETCU_RUNTIME_ERROR,
                        "Direct-light A-buffer overflow; increase Config::maxFragmentsPerPixel");
        std::vector<uint32_t> t(S), v(S);
        FCU_CHECK(cudaMemcpyAsync(t.data(), total, size_t(S) * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaMemcpyAsync(v.data(), visible, size_t(S) * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        for (uint32_t i = 0; i < S; ++i)
            fraction[i] = t[i] ? float(v[i]) / float(t[i]) : 0.0f;
        return FACETCU_OK;
    });
}

namespace {
void ensure_bvh(facetcu_context* ctx)
{
    if (ctx->bvh_ready) return;
    for (int a = 0; a < 3; ++a) {
        ctx->bvh.scene_min[a] = ctx->bmin[a];
        ctx->bvh.scene_max[a] = ctx->bmax[a];
    }
    const uint32_t periodic = std::min(ctx->config.periodic_neighbor_count, 20u);
    ctx->bvh.hit_margin = hit_margin(ctx->bmin, ctx->bmax, periodic, ctx->config.periodic_size_x,
                                     ctx->config.periodic_size_z);
    lbvh_build(ctx->vertices.as<facetcu_vertex>(), ctx->facets, ctx->bvh, ctx->ws, ctx->stream);
    ctx->bvh_ready = true;
}
}  // namespace

}  // extern "C"

namespace {

// The rays of each sample set in the order of their directions: a Morton
// curve over the direction's tangent-plane components (dx, dy), 8 bits each.
// A warp traces 32 consecutive rays at a time, so neighbouring directions
// keep its BVH traversal coherent.  A side's row depends only on the set of
// its rays (hits are sorted and counted), so the graph is unchanged.
void order_samples(const float* uv, const float* dir, uint32_t sets, uint32_t rays,
                   std::vector<float>& uv_out, std::vector<float>& dir_out)
{
    const size_t n = size_t(sets) * rays;
    uv_out.resize(n * 2);
    dir_out.resize(n * 3);
    std::vector<uint32_t> key(rays), idx(rays);
    auto q8 = [](float v) {
        const float c = std::isfinite(v) ? std::min(1.0f, std::max(-1.0f, v)) : 0.0f;
        return uint32_t((c + 1.0f) * 127.5f);
    };
    for (uint32_t set = 0; set < sets; ++set) {
        const size_t b = size_t(set) * rays;
        for (uint32_t j = 0; j < rays; ++j) {
            const uint32_t x = q8(dir[3 * (b + j)]), y = q8(dir[3 * (b + j) + 1]);
            uint32_t k = 0;
            for (int bit = 0; bit < 8; ++bit)
                k |= ((x >> bit) & 1u) << (2 * bit) | ((y >> bit) & 1u) << (2 * bit + 1);
            key[j] = k;
            idx[j] = j;
        }
        std::stable_sort(idx.begin(), idx.end(),
                         [&](uint32_t a, uint32_t c) { return key[a] < key[c]; });
        for (uint32_t j = 0; j < rays; ++j) {
            const size_t from = b + idx[j], to = b + j;
            uv_out[2 * to] = uv[2 * from];
            uv_out[2 * to + 1] = uv[2 * from + 1];
            for (int c = 0; c < 3; ++c) dir_out[3 * to + c] = dir[3 * from + c];
        }
    }
}

}  // namespace

extern "C" {

int facetcu_build_hemisphere_graph(facetcu_context* ctx, const facetcu_hemisphere_config* config,
                                   const float* sample_uv, const float* sample_dir,
                                   facetcu_graph_diagnostics* diagnostics, uint64_t* dropped)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "buildHemisphereGraph()");
        if (ctx->facets == 0)
            throw Error(FACETCU_LOGIC_ERROR, "setGeometry() must be called before buildHemisphereGraph()");
        if (!config || !sample_uv || !sample_dir)
            throw Error(FACETCU_INVALID_ARGUMENT, "hemisphere config and sample tables are required");
        if (config->rays_per_side == 0 || config->rays_per_side > 1023)
            throw Error(FACETCU_INVALID_ARGUMENT, "rays_per_side must be in [1, 1023]");
        if (config->top_k == 0 || config->sample_sets == 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "top_k and sample_sets must be positive");
        const uint32_t S = ctx->facets * 2u;
        if (S > (1u << 22))
            throw Error(FACETCU_OVERFLOW_ERROR, "hemisphere graphs support at most 2^22 sides");
        cudaStream_t s = ctx->stream;
        ctx->graph_ready = false;
        const size_t n = size_t(config->sample_sets) * config->rays_per_side;
        std::vector<float> uv_sorted, dir_sorted;
        order_samples(sample_uv, sample_dir, config->sample_sets, config->rays_per_side,
                      uv_sorted, dir_sorted);
        upload(ctx->samples_uv, uv_sorted.data(), n * 8, s);
        upload(ctx->samples_dir, dir_sorted.data(), n * 12, s);
        FCU_CHECK(cudaStreamSynchronize(s));  // the host tables go out of scope
        ensure_bvh(ctx);
        DeviceGraph& g = ctx->graph;
        unsigned long long drop = 0;
        hemisphere_graph(ctx->vertices.as<facetcu_vertex>(), ctx->facets, ctx->bvh,
                         ctx->samples_uv.as<float>(), ctx->samples_dir.as<float>(),
                         config->rays_per_side, config->sample_sets, config->top_k,
                         make_tiles(ctx), g, &drop, ctx->ws, s);
        float closure = 0.0f;
        uint32_t sampled = 0;
        graph_closure(g, &closure, &sampled, ctx->ws, s);
        graph_pack(g, ctx->ws, s);
        FCU_CHECK(cudaStreamSynchronize(s));
        facetcu_graph_diagnostics diag{};
        diag.facet_count = ctx->facets;
        diag.surface_count = S;
        diag.directed_edge_count = uint32_t(g.nnz);
        diag.max_closure_error = closure;
        if (diagnostics) *diagnostics = diag;
        if (dropped) *dropped = drop;
        ctx->graph_ready = true;
        return FACETCU_OK;
    });
}

int facetcu_hemisphere_sunlit(facetcu_context* ctx, const facetcu_direction* sun, uint32_t samples,
                              uint32_t sample_sets, const float* sample_uv, float* fraction)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "hemisphereSunlit()");
        if (ctx->facets == 0)
            throw Error(FACETCU_LOGIC_ERROR, "setGeometry() must be called before hemisphereSunlit()");
        if (!sun || !sample_uv || !fraction || samples == 0 || sample_sets == 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "sun, samples and output are required");
        if (!std::isfinite(sun->x) || !std::isfinite(sun->y) || !std::isfinite(sun->z) ||
            !(sun->x * sun->x + sun->y * sun->y + sun->z * sun->z > 0.0f))
            throw Error(FACETCU_INVALID_ARGUMENT, "sun direction must be finite and non-zero");
        cudaStream_t s = ctx->stream;
        const uint32_t S = ctx->facets * 2u;
        upload(ctx->samples_uv, sample_uv, size_t(sample_sets) * samples * 8, s);
        ensure_bvh(ctx);
        float* d = static_cast<float*>(ctx->fraction.reserve(size_t(S) * 4));
        hemisphere_sunlit(ctx->vertices.as<facetcu_vertex>(), ctx->facets, ctx->bvh,
                          ctx->samples_uv.as<float>(), samples, sample_sets,
                          make_float3(sun->x, sun->y, sun->z), make_tiles(ctx), d, s);
        FCU_CHECK(cudaMemcpyAsync(fraction, d, size_t(S) * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return FACETCU_OK;
    });
}

int facetcu_graph_size(facetcu_context* ctx, uint32_t* surface_count, uint64_t* edges)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "graphSize()");
        if (surface_count) *surface_count = ctx->graph.surfaces;
        if (edges) *edges = ctx->graph.nnz;
        return FACETCU_OK;
    });
}

int facetcu_get_graph(facetcu_context* ctx, uint32_t* row_offsets, facetcu_csr_edge* edges,
                      uint32_t* denominators, uint32_t* sky_counts)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "getGraph()");
        const DeviceGraph& g = ctx->graph;
        cudaStream_t s = ctx->stream;
        if (row_offsets)
            FCU_CHECK(cudaMemcpyAsync(row_offsets, g.row_offsets.ptr, (size_t(g.surfaces) + 1) * 4,
                                      cudaMemcpyDeviceToHost, s));
        if (edges && g.nnz)
            FCU_CHECK(cudaMemcpyAsync(edges, g.edges.ptr, g.nnz * 8, cudaMemcpyDeviceToHost, s));
        if (denominators)
            FCU_CHECK(cudaMemcpyAsync(denominators, g.denominators.ptr, size_t(g.surfaces) * 4,
                                      cudaMemcpyDeviceToHost, s));
        if (sky_counts)
            FCU_CHECK(cudaMemcpyAsync(sky_counts, g.sky.ptr, size_t(g.surfaces) * 4,
                                      cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return FACETCU_OK;
    });
}

int facetcu_set_graph(facetcu_context* ctx, uint32_t surface_count, const uint32_t* row_offsets,
                      const facetcu_csr_edge* edges, const uint32_t* denominators,
                      const uint32_t* sky_counts)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "setGraph()");
        if (ctx->facets == 0)
            throw Error(FACETCU_LOGIC_ERROR, "setGeometry() must be called before setGraph()");
        if (surface_count != ctx->facets * 2u || !row_offsets || !denominators || !sky_counts)
            throw Error(FACETCU_INVALID_ARGUMENT, "graph must have two rows per facet");
        if (row_offsets[0] != 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "row offsets must start at 0");
        for (uint32_t i = 0; i < surface_count; ++i)
            if (row_offsets[i + 1] < row_offsets[i])
                throw Error(FACETCU_INVALID_ARGUMENT, "row offsets must be non-decreasing");
        const uint64_t nnz = row_offsets[surface_count];
        if (nnz && !edges) throw Error(FACETCU_INVALID_ARGUMENT, "edges are required");
        for (uint64_t e = 0; e < nnz; ++e)
            if (edges[e].neighbor >= surface_count)
                throw Error(FACETCU_INVALID_ARGUMENT, "graph contains an invalid surface index");
        DeviceGraph& g = ctx->graph;
        cudaStream_t s = ctx->stream;
        g.surfaces = surface_count;
        g.nnz = nnz;
        upload(g.row_offsets, row_offsets, (size_t(surface_count) + 1) * 4, s);
        upload(g.edges, edges, nnz * 8 + 8, s);
        upload(g.denominators, denominators, size_t(surface_count) * 4, s);
        upload(g.sky, sky_counts, size_t(surface_count) * 4, s);
        g.packed_valid = false;
        g.perm_valid = false;
        g.scene_facets.clear();
        float closure;
        uint32_t sampled;
        graph_closure(g, &closure, &sampled, ctx->ws, s);
        graph_pack(g, ctx->ws, s);
        FCU_CHECK(cudaStreamSynchronize(s));
        ctx->graph_ready = true;
        return FACETCU_OK;
    });
}

// FacetrtVulkan::solve (facetrt_vulkan.cpp:1177-1247)
int facetcu_solve(facetcu_context* ctx, const facetcu_surface_optics* optics,
                  uint64_t optics_count, float sky, uint32_t iterations, float relaxation,
                  float* radiosity, uint32_t* iterations_done, float* max_delta)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "solve()");
        const uint32_t S = ctx->graph.surfaces;
        validate_count(optics_count, S);
        validate_optics(optics, S);
        validate_sky(sky);
        validate_relax(relaxation);
        cudaStream_t s = ctx->stream;
        upload(ctx->optics, optics, size_t(S) * 16, s);
        ctx->rad_a.reserve(size_t(S) * 4);
        ctx->rad_b.reserve(size_t(S) * 4);
        ctx->residual.reserve((size_t(iterations) + 1) * 4);
        FCU_CHECK(cudaMemsetAsync(ctx->rad_a.ptr, 0, size_t(S) * 4, s));
        FCU_CHECK(cudaMemsetAsync(ctx->rad_b.ptr, 0, size_t(S) * 4, s));
        FCU_CHECK(cudaMemsetAsync(ctx->residual.ptr, 0, (size_t(iterations) + 1) * 4, s));
        const uint32_t ping = run_sweeps(ctx, sky, relaxation, iterations, 0, 0);
        const float* final_buf = ping == 0 ? ctx->rad_a.as<float>() : ctx->rad_b.as<float>();
        uint32_t bits = 0;
        if (radiosity)
            FCU_CHECK(cudaMemcpyAsync(radiosity, final_buf, size_t(S) * 4, cudaMemcpyDeviceToHost, s));
        if (iterations)
            FCU_CHECK(cudaMemcpyAsync(&bits, ctx->residual.as<uint32_t>() + iterations - 1, 4,
                                      cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        if (iterations_done) *iterations_done = iterations;
        if (max_delta) std::memcpy(max_delta, &bits, 4);
        return FACETCU_OK;
    });
}

// FacetrtVulkan::solveAccelerated (facetrt_vulkan.cpp:1249-1358)
int facetcu_solve_accelerated(facetcu_context* ctx, const facetcu_surface_optics* optics,
                              uint64_t optics_count, float sky, const float* initial,
                              uint32_t maximum_iterations, uint32_t batch_iterations,
                              float tolerance, float relaxation, float* radiosity,
                              uint32_t* iterations_done, float* max_delta)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "solveAccelerated()");
        const uint32_t S = ctx->graph.surfaces;
        validate_count(optics_count, S);
        validate_optics(optics, S);
        validate_sky(sky);
        validate_relax(relaxation);
        if (maximum_iterations == 0 || batch_iterations == 0 || !std::isfinite(tolerance) ||
            tolerance < 0.0f)
            throw Error(FACETCU_INVALID_ARGUMENT,
                        "Accelerated solve iterations must be positive and tolerance non-negative");
        if (initial) {
            for (uint32_t i = 0; i < S; ++i)
                if (!std::isfinite(initial[i]) || initial[i] < 0.0f)
                    throw Error(FACETCU_INVALID_ARGUMENT,
                                "Initial radiosity must contain one finite non-negative value per surface");
        }
        cudaStream_t s = ctx->stream;
        upload(ctx->optics, optics, size_t(S) * 16, s);
        ctx->rad_a.reserve(size_t(S) * 4);
        ctx->rad_b.reserve(size_t(S) * 4);
        ctx->residual.reserve((size_t(maximum_iterations) + 1) * 4);
        FCU_CHECK(cudaMemsetAsync(ctx->residual.ptr, 0, (size_t(maximum_iterations) + 1) * 4, s));
        if (initial) {
            FCU_CHECK(cudaMemcpyAsync(ctx->rad_a.ptr, initial, size_t(S) * 4, cudaMemcpyHostToDevice, s));
            FCU_CHECK(cudaMemcpyAsync(ctx->rad_b.ptr, initial, size_t(S) * 4, cudaMemcpyHostToDevice, s));
        } else {
            FCU_CHECK(cudaMemsetAsync(ctx->rad_a.ptr, 0, size_t(S) * 4, s));
            FCU_CHECK(cudaMemsetAsync(ctx->rad_b.ptr, 0, size_t(S) * 4, s));
        }
        uint32_t done = 0, ping = 0;
        float md = 0.0f;
        while (done < maximum_iterations) {
            const uint32_t count = std::min(batch_iterations, maximum_iterations - done);
            ping = run_sweeps(ctx, sky, relaxation, count, ping, done);
            done += count;
            uint32_t bits = 0;
            FCU_CHECK(cudaMemcpyAsync(&bits, ctx->residual.as<uint32_t>() + done - 1, 4,
                                      cudaMemcpyDeviceToHost, s));
            FCU_CHECK(cudaStreamSynchronize(s));
            std::memcpy(&md, &bits, 4);
            if (md <= tolerance) break;
        }
        const float* final_buf = ping == 0 ? ctx->rad_a.as<float>() : ctx->rad_b.as<float>();
        if (radiosity)
            FCU_CHECK(cudaMemcpyAsync(radiosity, final_buf, size_t(S) * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        if (iterations_done) *iterations_done = done;
        if (max_delta) *max_delta = md;
        return FACETCU_OK;
    });
}

// FacetrtVulkan::incidentIrradiance (facetrt_vulkan.cpp:1360-1399)
int facetcu_incident_irradiance(facetcu_context* ctx, const float* radiosity,
                                const facetcu_surface_optics* optics, uint64_t count, float sky,
                                float* irradiance)
{
    return guarded(ctx, [&] {
        if (!ctx->initialized || !ctx->graph_ready || !radiosity || !optics || !irradiance ||
            count != uint64_t(ctx->graph.surfaces))
            throw Error(FACETCU_INVALID_ARGUMENT,
                        "Incident irradiance requires a completed solve and visibility graph");
        FCU_CHECK(cudaSetDevice(ctx->device));
        if (!std::isfinite(sky) || sky < 0.0f)
            throw Error(FACETCU_INVALID_ARGUMENT, "Sky radiosity must be finite and non-negative");
        const uint32_t S = ctx->graph.surfaces;
        cudaStream_t s = ctx->stream;
        upload(ctx->optics, optics, size_t(S) * 16, s);
        float* rad = static_cast<float*>(ctx->scratch.reserve(size_t(S) * 8));
        FCU_CHECK(cudaMemcpyAsync(rad, radiosity, size_t(S) * 4, cudaMemcpyHostToDevice, s));
        incident_irradiance(ctx->graph, ctx->optics.as<facetcu_surface_optics>(), sky, rad, rad + S, s);
        FCU_CHECK(cudaMemcpyAsync(irradiance, rad + S, size_t(S) * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return FACETCU_OK;
    });
}

}  // extern "C"

namespace {

void validate_batch(const facetcu_batch_config* cfg)
{
    if (!cfg) throw Error(FACETCU_INVALID_ARGUMENT, "batch config is null");
    if (cfg->band_count == 0 || cfg->sun_count == 0)
        throw Error(FACETCU_INVALID_ARGUMENT, "band_count and sun_count must be positive");
    if (cfg->precision > 2u) throw Error(FACETCU_INVALID_ARGUMENT, "unknown precision");
    if (cfg->warm_start > FACETCU_WARM_MLP) throw Error(FACETCU_INVALID_ARGUMENT, "unknown warm start");
    if (cfg->warm_start == FACETCU_WARM_MLP && cfg->band_count != uint32_t(mlp::kOutputs))
        throw Error(FACETCU_INVALID_ARGUMENT, "the MLP warm start needs 64 bands");
    if (!std::isfinite(cfg->tolerance) || cfg->tolerance < 0.0f)
        throw Error(FACETCU_INVALID_ARGUMENT, "tolerance must be finite and non-negative");
    if (uint64_t(cfg->band_count) * cfg->sun_count > (1ull << 31))
        throw Error(FACETCU_OVERFLOW_ERROR, "band_count x sun_count exceeds 2^31");
}

// The reference's optics checks (facetrt_vulkan.cpp solve), run on the
// device over every band and side.
void check_batch_inputs(facetcu_context* ctx, const float* rho, const float* tau,
                        const float* emis, size_t n, const float* sky, const float* beam,
                        uint32_t bands)
{
    const uint32_t bad = validate_inputs(rho, tau, emis, n, sky, beam, bands, ctx->scratch,
                                         ctx->stream);
    if (bad & 1u)
        throw Error(FACETCU_INVALID_ARGUMENT,
                    "Optical values must be finite, non-negative, and reflectance+transmittance<=1");
    if (bad & 2u) throw Error(FACETCU_INVALID_ARGUMENT, "skyRadiosity must be finite and non-negative");
    if (bad & 4u)
        throw Error(FACETCU_INVALID_ARGUMENT, "beam irradiance must be finite and non-negative");
}

// The autotuner's key: GPU, graph size, columns, precision.
std::string tune_key(facetcu_context* ctx, const facetcu_batch_config* cfg)
{
    if (ctx->gpu_name.empty()) {
        cudaDeviceProp prop{};
        FCU_CHECK(cudaGetDeviceProperties(&prop, ctx->device));
        ctx->gpu_name = prop.name;
    }
    std::ostringstream k;
    k << ctx->gpu_name << "|S=" << ctx->graph.surfaces << "|nnz=" << ctx->graph.nnz
      << "|R=" << uint64_t(cfg->band_count) * cfg->sun_count << "|precision=" << cfg->precision;
    return k.str();
}

int run_batched(facetcu_context* ctx, const facetcu_batch_config* cfg_in, const float* rho,
                const float* tau, const float* emis, const float* sky, const float* beam,
                const float* dgeo, const float* initial, float* out, facetcu_batch_result* result,
                uint32_t step_ctas = 0)
{
    facetcu_batch_config tuned_cfg = *cfg_in;
    if (tuned_cfg.panel_width == 0 && !ctx->tuned.empty()) {
        const auto it = ctx->tuned.find(tune_key(ctx, cfg_in));
        if (it != ctx->tuned.end()) {
            tuned_cfg.panel_width = it->second.panel_width;
            step_ctas = it->second.step_ctas;
        }
    }
    const facetcu_batch_config* cfg = &tuned_cfg;
    BatchProblem p{};
    p.step_ctas_per_sm = step_ctas;
    p.vertices = ctx->vertices.as<facetcu_vertex>();
    for (int a = 0; a < 3; ++a) {
        p.lo[a] = ctx->bmin[a];
        p.hi[a] = ctx->bmax[a];
    }
    p.S = ctx->graph.surfaces;
    p.bands = cfg->band_count;
    p.suns = cfg->sun_count;
    p.rho = rho;
    p.tau = tau;
    p.emis = emis;
    p.sky = sky;
    p.beam = beam;
    p.dgeo = dgeo;
    cudaEvent_t e0, e1;
    FCU_CHECK(cudaEventCreate(&e0));
    FCU_CHECK(cudaEventCreate(&e1));
    FCU_CHECK(cudaEventRecord(e0, ctx->stream));
    int rc;
    if (cfg->warm_start == FACETCU_WARM_MLP) {
        // first-order sweep, features, network, B1 + prediction as the start
        const uint32_t S = p.S, R = p.bands * p.suns;
        float* b1 = static_cast<float*>(ctx->warm_b1.reserve(size_t(R) * S * 4));
        float* x = static_cast<float*>(ctx->warm_x.reserve(size_t(p.suns) * S * mlp::kInputs * 4));
        float* y = static_cast<float*>(ctx->warm_y.reserve(size_t(p.suns) * S * mlp::kOutputs * 4));
        float* x0 = static_cast<float*>(ctx->warm_x0.reserve(size_t(R) * S * 4));
        facetcu_batch_config first = *cfg;
        first.precision = FACETCU_PRECISION_FP32;
        first.warm_start = FACETCU_WARM_NONE;
        first.maximum_iterations = 1;
        first.flags = 0;
        facetcu_batch_result r1{};
        batched_solve(ctx->graph, p, first, nullptr, b1, ctx->batch, ctx->ws, ctx->stream, &r1);
        mlp::features(b1, S, p.bands, p.suns, p.rho, p.tau, p.sky, p.beam,
                      ctx->graph.denominators.as<uint32_t>(), ctx->graph.sky.as<uint32_t>(),
                      ctx->vertices.as<facetcu_vertex>(), x, ctx->stream);
        mlp::infer_tensor(ctx->net, x, size_t(p.suns) * S, ctx->mlp_tensor, y, ctx->stream);
        if (mlp::tensor_error(ctx->mlp_tensor, ctx->stream))
            throw Error(FACETCU_DEVICE_TIMEOUT, "tensor-core MLP kernel timed out");
        mlp::warm_combine(b1, y, S, p.bands, p.suns, p.sky, p.beam, x0, ctx->stream);
        facetcu_batch_config rest = *cfg;
        rest.warm_start = FACETCU_WARM_GIVEN;
        rc = batched_solve(ctx->graph, p, rest, x0, out, ctx->batch, ctx->ws, ctx->stream, result);
        if (result) {
            result->iterations += 1;
            result->sweeps += 1;
            // features + combine, and per inference chunk 3 GEMMs + the bias add
            const size_t chunks = (size_t(p.suns) * S + mlp::kInferChunk - 1) / mlp::kInferChunk;
            result->kernel_launches += r1.kernel_launches + 2 + 4 * uint32_t(chunks);
        }
    } else {
        rc = batched_solve(ctx->graph, p, *cfg, initial, out, ctx->batch, ctx->ws, ctx->stream,
                           result);
    }
    FCU_CHECK(cudaEventRecord(e1, ctx->stream));
    FCU_CHECK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (result) result->seconds = double(ms) * 1e-3;
    if (rc == FACETCU_NOT_CONVERGED) {
        ctx->last_error = "batched solve reached maximum_iterations before the tolerance";
    }
    return rc;
}

}  // namespace

extern "C" {

int facetcu_solve_batched_device(facetcu_context* ctx, const facetcu_batch_config* cfg,
                                 const float* reflectance, const float* transmittance,
                                 const float* emission, const float* sky, const float* beam,
                                 const float* direct_geometry, const float* initial,
                                 float* radiosity, facetcu_batch_result* result)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "solveBatched()");
        validate_batch(cfg);
        if (!reflectance || !transmittance || !sky || !beam || !radiosity)
            throw Error(FACETCU_INVALID_ARGUMENT, "reflectance, transmittance, sky, beam and output are required");
        if (cfg->warm_start == FACETCU_WARM_GIVEN && !initial)
            throw Error(FACETCU_INVALID_ARGUMENT, "warm_start = GIVEN needs an initial radiosity");
        if (cfg->warm_start == FACETCU_WARM_MLP && !ctx->net.ready)
            throw Error(FACETCU_LOGIC_ERROR, "the MLP warm start needs trained parameters");
        check_batch_inputs(ctx, reflectance, transmittance, emission,
                           size_t(cfg->band_count) * ctx->graph.surfaces, sky, beam,
                           cfg->band_count);
        return run_batched(ctx, cfg, reflectance, transmittance, emission, sky, beam,
                           direct_geometry, initial, radiosity, result);
    });
}

int facetcu_solve_batched(facetcu_context* ctx, const facetcu_batch_config* cfg,
                          const float* reflectance, const float* transmittance,
                          const float* emission, const float* sky, const float* beam,
                          const float* direct_geometry, const float* initial, float* radiosity,
                          facetcu_batch_result* result)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "solveBatched()");
        validate_batch(cfg);
        if (!reflectance || !transmittance || !sky || !beam || !radiosity)
            throw Error(FACETCU_INVALID_ARGUMENT, "reflectance, transmittance, sky, beam and output are required");
        if (cfg->warm_start == FACETCU_WARM_GIVEN && !initial)
            throw Error(FACETCU_INVALID_ARGUMENT, "warm_start = GIVEN needs an initial radiosity");
        if (cfg->warm_start == FACETCU_WARM_MLP && !ctx->net.ready)
            throw Error(FACETCU_LOGIC_ERROR, "the MLP warm start needs trained parameters");
        const size_t S = ctx->graph.surfaces, B = cfg->band_count, K = cfg->sun_count;
        const size_t R = B * K;
        // one device block for all inputs: rho, tau, emis, dgeo, sky, beam, initial, out
        const size_t n_bs = B * S, n_ks = direct_geometry ? K * S : 0, n_rs = R * S;
        const size_t init_n = cfg->warm_start == FACETCU_WARM_GIVEN ? n_rs : 0;
        const size_t total = 3 * n_bs + n_ks + 2 * B + init_n + n_rs + 64;
        float* base = static_cast<float*>(ctx->batch_inputs.reserve(total * 4));
        float* d_rho = base;
        float* d_tau = d_rho + n_bs;
        float* d_emis = d_tau + n_bs;
        float* d_dgeo = d_emis + n_bs;
        float* d_sky = d_dgeo + n_ks;
        float* d_beam = d_sky + B;
        float* d_init = d_beam + B;
        float* d_out = d_init + init_n;
        cudaStream_t s = ctx->stream;
        FCU_CHECK(cudaMemcpyAsync(d_rho, reflectance, n_bs * 4, cudaMemcpyHostToDevice, s));
        FCU_CHECK(cudaMemcpyAsync(d_tau, transmittance, n_bs * 4, cudaMemcpyHostToDevice, s));
        if (emission) FCU_CHECK(cudaMemcpyAsync(d_emis, emission, n_bs * 4, cudaMemcpyHostToDevice, s));
        if (n_ks) FCU_CHECK(cudaMemcpyAsync(d_dgeo, direct_geometry, n_ks * 4, cudaMemcpyHostToDevice, s));
        FCU_CHECK(cudaMemcpyAsync(d_sky, sky, B * 4, cudaMemcpyHostToDevice, s));
        FCU_CHECK(cudaMemcpyAsync(d_beam, beam, B * 4, cudaMemcpyHostToDevice, s));
        if (init_n) FCU_CHECK(cudaMemcpyAsync(d_init, initial, init_n * 4, cudaMemcpyHostToDevice, s));
        check_batch_inputs(ctx, d_rho, d_tau, emission ? d_emis : nullptr, n_bs, d_sky, d_beam,
                           uint32_t(B));
        const int rc = run_batched(ctx, cfg, d_rho, d_tau, emission ? d_emis : nullptr, d_sky, d_beam,
                                   n_ks ? d_dgeo : nullptr, init_n ? d_init : nullptr, d_out, result);
        FCU_CHECK(cudaMemcpyAsync(radiosity, d_out, n_rs * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return rc;
    });
}

}  // extern "C"

extern "C" {

int facetcu_mlp_parameter_count(uint32_t* count)
{
    if (!count) return FACETCU_INVALID_ARGUMENT;
    *count = uint32_t(mlp::kParameterCount);
    return FACETCU_OK;
}

int facetcu_mlp_reset(facetcu_context* ctx, uint32_t seed)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpReset()");
        mlp::init_params(ctx->net, seed, ctx->stream);
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        return FACETCU_OK;
    });
}

int facetcu_mlp_get_parameters(facetcu_context* ctx, float* parameters)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpGetParameters()");
        if (!ctx->net.ready) throw Error(FACETCU_LOGIC_ERROR, "the MLP has no parameters yet");
        if (!parameters) throw Error(FACETCU_INVALID_ARGUMENT, "parameters is null");
        FCU_CHECK(cudaMemcpyAsync(parameters, ctx->net.params.ptr, mlp::kParameterCount * 4,
                                  cudaMemcpyDeviceToHost, ctx->stream));
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        return FACETCU_OK;
    });
}

int facetcu_mlp_set_parameters(facetcu_context* ctx, const float* parameters)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpSetParameters()");
        if (!parameters) throw Error(FACETCU_INVALID_ARGUMENT, "parameters is null");
        for (int i = 0; i < mlp::kParameterCount; ++i)
            if (!std::isfinite(parameters[i]))
                throw Error(FACETCU_INVALID_ARGUMENT, "MLP parameters must be finite");
        mlp::set_params(ctx->net, parameters, ctx->stream);
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        return FACETCU_OK;
    });
}

int facetcu_mlp_forward(facetcu_context* ctx, const float* x, uint32_t n, float* y)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpForward()");
        if (!ctx->net.ready) throw Error(FACETCU_LOGIC_ERROR, "the MLP has no parameters yet");
        if (!x || !y || n == 0) throw Error(FACETCU_INVALID_ARGUMENT, "x, y and n are required");
        cudaStream_t s = ctx->stream;
        float* dx = static_cast<float*>(
            ctx->mlp_io.reserve(size_t(n) * (mlp::kInputs + mlp::kOutputs) * 4));
        float* dy = dx + size_t(n) * mlp::kInputs;
        FCU_CHECK(cudaMemcpyAsync(dx, x, size_t(n) * mlp::kInputs * 4, cudaMemcpyHostToDevice, s));
        mlp::infer(ctx->net, dx, n, ctx->mlp_scratch, dy, s);
        FCU_CHECK(cudaMemcpyAsync(y, dy, size_t(n) * mlp::kOutputs * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return FACETCU_OK;
    });
}

int facetcu_mlp_forward_tensor(facetcu_context* ctx, const float* x, uint32_t n, float* y)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpForwardTensor()");
        if (!ctx->net.ready) throw Error(FACETCU_LOGIC_ERROR, "the MLP has no parameters yet");
        if (!x || !y || n == 0) throw Error(FACETCU_INVALID_ARGUMENT, "x, y and n are required");
        cudaStream_t s = ctx->stream;
        float* dx = static_cast<float*>(
            ctx->mlp_io.reserve(size_t(n) * (mlp::kInputs + mlp::kOutputs) * 4));
        float* dy = dx + size_t(n) * mlp::kInputs;
        FCU_CHECK(cudaMemcpyAsync(dx, x, size_t(n) * mlp::kInputs * 4, cudaMemcpyHostToDevice, s));
        mlp::infer_tensor(ctx->net, dx, n, ctx->mlp_tensor, dy, s);
        if (mlp::tensor_error(ctx->mlp_tensor, s))
            throw Error(FACETCU_DEVICE_TIMEOUT, "tensor-core MLP kernel timed out");
        FCU_CHECK(cudaMemcpyAsync(y, dy, size_t(n) * mlp::kOutputs * 4, cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return FACETCU_OK;
    });
}

int facetcu_mlp_loss_and_gradient(facetcu_context* ctx, const float* x, const float* target,
                                  uint32_t n, float* loss, float* gradient)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpLossAndGradient()");
        if (!ctx->net.ready) throw Error(FACETCU_LOGIC_ERROR, "the MLP has no parameters yet");
        if (!x || !target || n == 0) throw Error(FACETCU_INVALID_ARGUMENT, "x, target and n are required");
        if (n > mlp::kMaxRows) throw Error(FACETCU_OVERFLOW_ERROR, "at most 2^21 rows per gradient");
        cudaStream_t s = ctx->stream;
        float* dx = static_cast<float*>(
            ctx->mlp_io.reserve(size_t(n) * (mlp::kInputs + mlp::kOutputs) * 4));
        float* dt = dx + size_t(n) * mlp::kInputs;
        FCU_CHECK(cudaMemcpyAsync(dx, x, size_t(n) * mlp::kInputs * 4, cudaMemcpyHostToDevice, s));
        FCU_CHECK(cudaMemcpyAsync(dt, target, size_t(n) * mlp::kOutputs * 4, cudaMemcpyHostToDevice, s));
        const double l = mlp::loss_and_grad(ctx->net, dx, dt, int(n), ctx->mlp_scratch, s, true);
        if (loss) *loss = float(l);
        if (gradient)
            FCU_CHECK(cudaMemcpyAsync(gradient, ctx->net.grad.ptr, mlp::kParameterCount * 4,
                                      cudaMemcpyDeviceToHost, s));
        FCU_CHECK(cudaStreamSynchronize(s));
        return FACETCU_OK;
    });
}

int facetcu_mlp_train_device(facetcu_context* ctx, const float* x, const float* target, uint64_t n,
                             const facetcu_mlp_train_config* config, float* final_loss)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "mlpTrain()");
        if (!x || !target || n == 0 || !config || config->batch == 0 || config->steps == 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "samples and a training config are required");
        if (n >= (1ull << 32)) throw Error(FACETCU_OVERFLOW_ERROR, "at most 2^32 training samples");
        if (config->batch > mlp::kMaxRows)
            throw Error(FACETCU_OVERFLOW_ERROR, "at most 2^21 samples per training batch");
        if (!std::isfinite(config->learning_rate) || config->learning_rate <= 0.0f)
            throw Error(FACETCU_INVALID_ARGUMENT, "learning_rate must be positive");
        if (!ctx->net.ready) mlp::init_params(ctx->net, config->seed, ctx->stream);
        const double l = mlp::train(ctx->net, x, target, n, config->steps, config->batch,
                                    config->learning_rate, config->seed, ctx->mlp_scratch,
                                    ctx->stream);
        if (final_loss) *final_loss = float(l);
        return FACETCU_OK;
    });
}

int facetcu_mlp_samples_device(facetcu_context* ctx, const facetcu_batch_config* cfg,
                               const float* reflectance, const float* transmittance,
                               const float* emission, const float* sky, const float* beam,
                               const float* direct_geometry, const float* converged,
                               float* features, float* targets)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "mlpSamples()");
        validate_batch(cfg);
        if (cfg->band_count != uint32_t(mlp::kOutputs))
            throw Error(FACETCU_INVALID_ARGUMENT, "MLP samples need 64 bands");
        if (!reflectance || !transmittance || !sky || !beam || !converged || !features || !targets)
            throw Error(FACETCU_INVALID_ARGUMENT, "inputs and outputs are required");
        BatchProblem p{};
        p.vertices = ctx->vertices.as<facetcu_vertex>();
        for (int a = 0; a < 3; ++a) {
            p.lo[a] = ctx->bmin[a];
            p.hi[a] = ctx->bmax[a];
        }
        p.S = ctx->graph.surfaces;
        p.bands = cfg->band_count;
        p.suns = cfg->sun_count;
        p.rho = reflectance;
        p.tau = transmittance;
        p.emis = emission;
        p.sky = sky;
        p.beam = beam;
        p.dgeo = direct_geometry;
        const uint32_t S = p.S, R = p.bands * p.suns;
        float* b1 = static_cast<float*>(ctx->warm_b1.reserve(size_t(R) * S * 4));
        facetcu_batch_config first = *cfg;
        first.precision = FACETCU_PRECISION_FP32;
        first.warm_start = FACETCU_WARM_NONE;
        first.maximum_iterations = 1;
        first.flags = 0;
        facetcu_batch_result r1{};
        batched_solve(ctx->graph, p, first, nullptr, b1, ctx->batch, ctx->ws, ctx->stream, &r1);
        mlp::features(b1, S, p.bands, p.suns, p.rho, p.tau, p.sky, p.beam,
                      ctx->graph.denominators.as<uint32_t>(), ctx->graph.sky.as<uint32_t>(),
                      ctx->vertices.as<facetcu_vertex>(), features, ctx->stream);
        mlp::targets(converged, b1, S, p.bands, p.suns, p.sky, p.beam, targets, ctx->stream);
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        return FACETCU_OK;
    });
}


// ---- spectral optics and the band loop ---------------------------------------
}  // extern "C"

namespace {

void validate_surface(const facetcu_surface_parameters& m)
{
    if ((m.reflectance_count && !m.reflectance) || (m.transmittance_count && !m.transmittance))
        throw Error(FACETCU_INVALID_ARGUMENT, "a surface's band values are missing");
}

void validate_spectral(const facetcu_context* ctx, const facetcu_spectral_parameters* p,
                       const float* sunlit, const facetcu_direction* sun)
{
    if (!p || !sunlit || !sun)
        throw Error(FACETCU_INVALID_ARGUMENT, "parameters, sunlit and sun are required");
    if (!p->wavelengths || p->band_count == 0)
        throw Error(FACETCU_INVALID_ARGUMENT, "at least one wavelength is required");
    for (uint32_t b = 0; b < p->band_count; ++b)
        if (!std::isfinite(p->wavelengths[b]) || p->wavelengths[b] <= 0.0f)
            throw Error(FACETCU_INVALID_ARGUMENT, "wavelengths must be finite and positive");
    if (p->material_count && !p->materials)
        throw Error(FACETCU_INVALID_ARGUMENT, "material_count > 0 needs materials");
    validate_surface(p->object);
    validate_surface(p->ground);
    for (uint32_t m = 0; m < p->material_count; ++m) validate_surface(p->materials[m]);
    if (p->leaf_facet_count > ctx->facets)
        throw Error(FACETCU_INVALID_ARGUMENT, "leaf_facet_count exceeds the facet count");
    if (!std::isfinite(sun->x) || !std::isfinite(sun->y) || !std::isfinite(sun->z))
        throw Error(FACETCU_INVALID_ARGUMENT, "sun direction must be finite");
}

struct SpectralIO {
    uint32_t* material = nullptr;
    float *texture = nullptr, *sunlit = nullptr, *dgeo = nullptr, *rho = nullptr,
          *tau = nullptr, *emis = nullptr, *out = nullptr, *sky = nullptr, *beam = nullptr;
    facetcu_surface_optics* aos = nullptr;
};

// Device inputs for `bands` bands: tables, materials, texture, sunlit, dgeo.
SpectralIO spectral_inputs(facetcu_context* ctx, const facetcu_spectral_parameters& p,
                           const float* sunlit, const facetcu_direction& sun, uint32_t bands)
{
    cudaStream_t st = ctx->stream;
    const size_t F = ctx->facets, S = 2 * F, nb = p.band_count;
    ctx->spec.build(p, st);
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t bytes = al(F * 4) * 2 + al(S * 4) * 2 + al(size_t(bands) * S * 4) * 4 +
                         al(nb * 4) * 2 + al(S * 16);
    char* c = static_cast<char*>(ctx->spec_io.reserve(bytes));
    SpectralIO io;
    auto take = [&](size_t b) {
        char* r = c;
        c += al(b);
        return r;
    };
    io.material = p.material_indices ? reinterpret_cast<uint32_t*>(take(F * 4)) : nullptr;
    io.texture = p.texture_factors ? reinterpret_cast<float*>(take(F * 4)) : nullptr;
    io.sunlit = reinterpret_cast<float*>(take(S * 4));
    io.dgeo = reinterpret_cast<float*>(take(S * 4));
    io.rho = reinterpret_cast<float*>(take(size_t(bands) * S * 4));
    io.tau = reinterpret_cast<float*>(take(size_t(bands) * S * 4));
    io.emis = reinterpret_cast<float*>(take(size_t(bands) * S * 4));
    io.out = reinterpret_cast<float*>(take(size_t(bands) * S * 4));
    io.sky = reinterpret_cast<float*>(take(nb * 4));
    io.beam = reinterpret_cast<float*>(take(nb * 4));
    io.aos = reinterpret_cast<facetcu_surface_optics*>(take(S * 16));
    if (io.material)
        FCU_CHECK(cudaMemcpyAsync(io.material, p.material_indices, F * 4, cudaMemcpyHostToDevice, st));
    if (io.texture)
        FCU_CHECK(cudaMemcpyAsync(io.texture, p.texture_factors, F * 4, cudaMemcpyHostToDevice, st));
    FCU_CHECK(cudaMemcpyAsync(io.sunlit, sunlit, S * 4, cudaMemcpyHostToDevice, st));
    FCU_CHECK(cudaMemcpyAsync(io.sky, ctx->spec.sky.data(), nb * 4, cudaMemcpyHostToDevice, st));
    FCU_CHECK(cudaMemcpyAsync(io.beam, ctx->spec.beam.data(), nb * 4, cudaMemcpyHostToDevice, st));
    spectral::direct_geometry(uint32_t(F), ctx->vertices.as<facetcu_vertex>(), sun, io.sunlit,
                              io.dgeo, st);
    return io;
}

void nested(facetcu_context* ctx, int rc)
{
    if (rc != FACETCU_OK) throw Error(rc, ctx->last_error);
}

}  // namespace

extern "C" {

int facetcu_spectral_optics(facetcu_context* ctx, const facetcu_spectral_parameters* parameters,
                            const float* sunlit, const facetcu_direction* sun, uint32_t band,
                            facetcu_surface_optics* optics)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "spectralOptics()");
        if (!ctx->facets) throw Error(FACETCU_LOGIC_ERROR, "spectralOptics() needs geometry");
        validate_spectral(ctx, parameters, sunlit, sun);
        if (!optics) throw Error(FACETCU_INVALID_ARGUMENT, "optics is required");
        if (band >= parameters->band_count) throw Error(FACETCU_INVALID_ARGUMENT, "band out of range");
        const facetcu_spectral_parameters& p = *parameters;
        const size_t S = 2 * size_t(ctx->facets);
        SpectralIO io = spectral_inputs(ctx, p, sunlit, *sun, 1);
        spectral::optics(ctx->spec, p, ctx->facets, ctx->vertices.as<facetcu_vertex>(), io.material,
                         io.texture, *sun, io.sunlit, band, 1, io.rho, io.tau, io.emis, ctx->stream);
        spectral::pack(S, io.rho, io.tau, io.emis, io.dgeo, ctx->spec.beam[band], io.aos, ctx->stream);
        FCU_CHECK(cudaMemcpyAsync(optics, io.aos, S * 16, cudaMemcpyDeviceToHost, ctx->stream));
        FCU_CHECK(cudaStreamSynchronize(ctx->stream));
        return FACETCU_OK;
    });
}

int facetcu_solve_bands(facetcu_context* ctx, const facetcu_spectral_parameters* parameters,
                        const float* sunlit, const facetcu_direction* sun, float* band_radiosity,
                        float* light_enhancement, facetcu_band_result* result)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "solveBands()");
        validate_spectral(ctx, parameters, sunlit, sun);
        if (!band_radiosity || !light_enhancement)
            throw Error(FACETCU_INVALID_ARGUMENT, "band_radiosity and light_enhancement are required");
        const auto t0 = std::chrono::steady_clock::now();
        const facetcu_spectral_parameters& p = *parameters;
        const uint32_t nb = p.band_count;
        const size_t S = ctx->graph.surfaces;
        if (S != 2 * size_t(ctx->facets))
            throw Error(FACETCU_LOGIC_ERROR, "the graph does not belong to the current geometry");
        cudaStream_t st = ctx->stream;
        SpectralIO io = spectral_inputs(ctx, p, sunlit, *sun, nb);
        spectral::optics(ctx->spec, p, ctx->facets, ctx->vertices.as<facetcu_vertex>(), io.material,
                         io.texture, *sun, io.sunlit, 0, nb, io.rho, io.tau, io.emis, st);
        const bool accel = p.accelerated_solver != 0;
        // band 0 through the reference-semantics solver (it carries the
        // SolveResult of facetrt.json and the direct-light enhancement)
        std::vector<facetcu_surface_optics> o0(S);
        spectral::pack(S, io.rho, io.tau, io.emis, io.dgeo, ctx->spec.beam[0], io.aos, st);
        FCU_CHECK(cudaMemcpyAsync(o0.data(), io.aos, S * 16, cudaMemcpyDeviceToHost, st));
        FCU_CHECK(cudaStreamSynchronize(st));
        auto solve_one = [&](const std::vector<facetcu_surface_optics>& o, float* out,
                             uint32_t* it, float* md) {
            if (accel)
                nested(ctx, facetcu_solve_accelerated(ctx, o.data(), S, ctx->spec.sky[0], nullptr,
                                                      64, 8, 1.0e-4f, 1.0f, out, it, md));
            else
                nested(ctx, facetcu_solve(ctx, o.data(), S, ctx->spec.sky[0], 64, 1.0f, out, it, md));
        };
        facetcu_band_result r{};
        solve_one(o0, band_radiosity, &r.iterations, &r.max_delta);
        if (nb > 1) {
            facetcu_batch_config cfg{};
            cfg.band_count = nb - 1;
            cfg.sun_count = 1;
            cfg.precision = FACETCU_PRECISION_FP32;
            cfg.warm_start = FACETCU_WARM_NONE;
            cfg.maximum_iterations = accel ? 2000u : 64u;
            cfg.tolerance = accel ? 1.0e-6f : 0.0f;
            facetcu_batch_result br{};
            const int rc = facetcu_solve_batched_device(ctx, &cfg, io.rho + S, io.tau + S,
                                                        io.emis + S, io.sky + 1, io.beam + 1,
                                                        io.dgeo, nullptr, io.out + S, &br);
            if (rc != FACETCU_NOT_CONVERGED || accel) nested(ctx, rc);
            r.batched_sweeps = br.sweeps;
        }
        FCU_CHECK(cudaMemcpyAsync(io.out, band_radiosity, S * 4, cudaMemcpyHostToDevice, st));
        const float cosz = std::max(0.0f, sun->y);
        const float ref = 700.0f * cosz + 100.0f * 0.5f;
        if (ref > 1.0e-8f)
            spectral::apparent(io.out, S, nb, ctx->spec.optical_dev, ref, st);
        FCU_CHECK(cudaMemcpyAsync(band_radiosity, io.out, size_t(nb) * S * 4,
                                  cudaMemcpyDeviceToHost, st));
        FCU_CHECK(cudaStreamSynchronize(st));
        for (uint32_t b = 0; b < nb; ++b) r.thermal_bands += ctx->spec.optical[b] ? 0u : 1u;
        std::fill(light_enhancement, light_enhancement + S, 0.0f);
        if (ctx->spec.optical[0]) {
            for (auto& o : o0) o.direct_irradiance = 0.0f;
            std::vector<float> diffuse(S);
            uint32_t it = 0;
            float md = 0.0f;
            solve_one(o0, diffuse.data(), &it, &md);
            for (size_t s = 0; s < S; ++s) {
                float d = diffuse[s];
                if (ref > 1.0e-8f) d = std::clamp(d / ref, 0.0f, 1.0f);
                light_enhancement[s] = std::max(0.0f, band_radiosity[s] - d);
            }
        }
        r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (result) *result = r;
        return FACETCU_OK;
    });
}

// ---- scene batches -------------------------------------------------------
int facetcu_scene_batch(facetcu_context* ctx, facetcu_context* const* scenes,
                        uint32_t scene_count, uint32_t* side_offsets,
                        facetcu_graph_diagnostics* diagnostics)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "sceneBatch()");
        if (!scenes || scene_count == 0)
            throw Error(FACETCU_INVALID_ARGUMENT, "at least one scene is required");
        uint64_t facets = 0, nnz = 0;
        float extent = 0.0f;
        uint32_t max_count = 0;
        for (uint32_t i = 0; i < scene_count; ++i) {
            const facetcu_context* sc = scenes[i];
            if (!sc || sc == ctx || !sc->graph_ready)
                throw Error(FACETCU_LOGIC_ERROR,
                            "every scene of a batch needs its own context with a built graph");
            if (sc->device != ctx->device)
                throw Error(FACETCU_INVALID_ARGUMENT, "the scenes of a batch must share a GPU");
            facets += sc->facets;
            nnz += sc->graph.nnz;
            max_count = std::max(max_count, sc->graph.max_count);
            for (int a = 0; a < 3; ++a) extent = std::max(extent, sc->bmax[a] - sc->bmin[a]);
        }
        if (2 * facets > 0xffffffffull || nnz > 0xffffffffull)
            throw Error(FACETCU_OVERFLOW_ERROR, "the batch exceeds 2^32 sides or edges");
        // Scene i sits in its own cell of an n x n x n grid (cell = 1.25 x the
        // largest scene extent): positions matter here only for the solver's
        // Morton renumbering, which then keeps every scene contiguous.
        uint32_t n = 1;
        while (uint64_t(n) * n * n < scene_count) ++n;
        const float cell = 1.25f * std::max(extent, 1.0f);
        std::vector<facetcu_vertex> all;
        all.reserve(size_t(facets) * 3);
        for (uint32_t i = 0; i < scene_count; ++i) {
            const facetcu_context* sc = scenes[i];
            const float off[3] = {float(i % n) * cell - sc->bmin[0],
                                  float((i / n) % n) * cell - sc->bmin[1],
                                  float(i / (n * n)) * cell - sc->bmin[2]};
            for (facetcu_vertex v : sc->vertices_host) {
                for (int a = 0; a < 3; ++a) v.position[a] += off[a];
                all.push_back(v);
            }
        }
        nested(ctx, facetcu_set_geometry(ctx, all.data(), all.size()));
        DeviceGraph& g = ctx->graph;
        cudaStream_t s = ctx->stream;
        const uint32_t S = uint32_t(2 * facets);
        g.surfaces = S;
        g.nnz = nnz;
        g.row_offsets.reserve((size_t(S) + 1) * 4);
        g.edges.reserve(nnz * 8 + 8);
        g.denominators.reserve(size_t(S) * 4);
        g.sky.reserve(size_t(S) * 4);
        uint32_t side = 0;
        uint64_t edge = 0;
        for (uint32_t i = 0; i < scene_count; ++i) {
            const facetcu_context* sc = scenes[i];
            FCU_CHECK(cudaStreamSynchronize(sc->stream));
            if (side_offsets) side_offsets[i] = side;
            graph_append(g, sc->graph, side, edge, s);
            side += sc->graph.surfaces;
            edge += sc->graph.nnz;
        }
        if (side_offsets) side_offsets[scene_count] = side;
        const uint32_t last = uint32_t(nnz);
        FCU_CHECK(cudaMemcpyAsync(g.row_offsets.as<uint32_t>() + S, &last, 4,
                                  cudaMemcpyHostToDevice, s));
        g.max_count = max_count;
        g.packed_valid = false;
        g.perm_valid = false;
        // the scenes' facet ranges: converged scenes leave the int8 steps
        g.scene_facets.assign(1, 0u);
        for (uint32_t i = 0, f = 0; i < scene_count; ++i) {
            f += scenes[i]->graph.surfaces / 2u;
            g.scene_facets.push_back(f);
        }
        float closure = 0.0f;
        uint32_t sampled = 0;
        graph_closure(g, &closure, &sampled, ctx->ws, s);
        graph_pack(g, ctx->ws, s);
        FCU_CHECK(cudaStreamSynchronize(s));
        ctx->graph_ready = true;
        if (diagnostics) {
            *diagnostics = {};
            diagnostics->facet_count = uint32_t(facets);
            diagnostics->surface_count = S;
            diagnostics->directed_edge_count = uint32_t(nnz);
            diagnostics->max_closure_error = closure;
        }
        return FACETCU_OK;
    });
}

// ---- autotuning ------------------------------------------------------------
}  // extern "C"

namespace {

// JSON-lines cache: {"key": "...", "panel_width": N} per line.
// One JSON object per line: key, panel width and (optional, 0 when absent)
// the pipelined step's CTAs per SM.
void read_tune_cache(const char* path, std::map<std::string, facetcu_context::Tuned>& out)
{
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) {
        const size_t k0 = line.find("\"key\": \"");
        const size_t p0 = line.find("\"panel_width\": ");
        if (k0 == std::string::npos || p0 == std::string::npos) continue;
        const size_t ks = k0 + 8, ke = line.find('"', ks);
        if (ke == std::string::npos) continue;
        facetcu_context::Tuned t;
        t.panel_width = uint32_t(std::strtoul(line.c_str() + p0 + 15, nullptr, 10));
        const size_t c0 = line.find("\"step_ctas_per_sm\": ");
        if (c0 != std::string::npos)
            t.step_ctas = uint32_t(std::strtoul(line.c_str() + c0 + 20, nullptr, 10));
        out[line.substr(ks, ke - ks)] = t;
    }
}

void write_tune_cache(const char* path, const std::map<std::string, facetcu_context::Tuned>& m)
{
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream out(tmp);
        if (!out) throw Error(FACETCU_RUNTIME_ERROR, std::string("cannot write ") + tmp);
        for (const auto& kv : m)
            out << "{\"key\": \"" << kv.first << "\", \"panel_width\": " << kv.second.panel_width
                << ", \"step_ctas_per_sm\": " << kv.second.step_ctas << "}\n";
    }
    if (std::rename(tmp.c_str(), path) != 0)
        throw Error(FACETCU_RUNTIME_ERROR, std::string("cannot replace ") + path);
}

}  // namespace

extern "C" {

int facetcu_autotune_batched(facetcu_context* ctx, const facetcu_batch_config* config,
                             const float* reflectance, const float* transmittance,
                             const float* emission, const float* sky, const float* beam,
                             const float* direct_geometry, float* radiosity,
                             const char* cache_path, uint32_t* panel_width)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "autotuneBatched()");
        validate_batch(config);
        if (!reflectance || !transmittance || !sky || !beam || !radiosity || !panel_width)
            throw Error(FACETCU_INVALID_ARGUMENT,
                        "reflectance, transmittance, sky, beam, output and panel_width are required");
        const std::string key = tune_key(ctx, config);
        if (cache_path) read_tune_cache(cache_path, ctx->tuned);
        auto hit = ctx->tuned.find(key);
        if (hit != ctx->tuned.end()) {
            *panel_width = hit->second.panel_width;
            return FACETCU_OK;
        }
        check_batch_inputs(ctx, reflectance, transmittance, emission,
                           size_t(config->band_count) * ctx->graph.surfaces, sky, beam,
                           config->band_count);
        const uint64_t R = uint64_t(config->band_count) * config->sun_count;
        const uint32_t cap = config->precision == FACETCU_PRECISION_FP64 ? 32u : 128u;
        // panel width x (for the widths whose int8 step is the pipelined
        // kernel, MIXED at 64 and 128 columns) its CTAs per SM
        facetcu_context::Tuned best;
        double best_t = 0.0;
        for (uint32_t P = 32; P <= cap; P *= 2) {
            if (P > R && P != 32) break;  // wider than the columns: only padding
            const bool pipelined =
                config->precision == FACETCU_PRECISION_MIXED && (P == 64 || P == 128);
            for (uint32_t ctas : {0u, 2u, 1u}) {
                if (ctas && !pipelined) break;
                facetcu_batch_config c = *config;
                c.panel_width = P;
                c.warm_start = FACETCU_WARM_NONE;
                c.maximum_iterations = 6;  // a few sweeps of every panel
                c.tolerance = 0.0f;
                c.flags = 0;
                facetcu_batch_result r{};
                run_batched(ctx, &c, reflectance, transmittance, emission, sky, beam,
                            direct_geometry, nullptr, radiosity, &r, ctas);  // warms the graph copies
                run_batched(ctx, &c, reflectance, transmittance, emission, sky, beam,
                            direct_geometry, nullptr, radiosity, &r, ctas);
                if (best.panel_width == 0 || r.seconds < best_t) {
                    best.panel_width = P;
                    best.step_ctas = ctas;
                    best_t = r.seconds;
                }
            }
        }
        ctx->tuned[key] = best;
        if (cache_path) write_tune_cache(cache_path, ctx->tuned);
        *panel_width = best.panel_width;
        return FACETCU_OK;
    });
}

}  // extern "C"

// ---- FacetEB node -----------------------------------------------------------
namespace {

const float kGroundReflectance[1] = {0.20f};
const float kGroundTransmittance[1] = {0.0f};

// surfaceForFacet's fixed fallbacks (facetrtcore.cpp:607-620).
facetcu_energy_surface fallback_surface(bool ground)
{
    facetcu_energy_surface m;
    facetcu_energy_surface_defaults(&m);
    if (ground) {
        m.optics.reflectance = kGroundReflectance;
        m.optics.transmittance = kGroundTransmittance;
        m.optics.tir_reflectance = 0.05f;
        m.optics.sunlit_temperature = 305.0f;
        m.optics.shaded_temperature = 295.0f;
    }
    return m;
}

float value_at(const float* v, uint32_t n, uint32_t i, float fallback)
{
    if (!v || n == 0) return fallback;
    return v[i < n ? i : n - 1];
}

void validate_energy(const facetcu_context* ctx, const facetcu_energy_parameters* p,
                     const facetcu_meteo* meteo, const facetcu_direction* sun, const float* sunlit,
                     const facetcu_shortwave_window* windows, uint32_t window_count,
                     const float* band_direct, const float* band_diffuse,
                     const facetcu_energy_fields* fields)
{
    if (!p || !meteo || !sun || !sunlit || !fields || !fields->temperature)
        throw Error(FACETCU_INVALID_ARGUMENT,
                    "parameters, meteo, sun, sunlit and fields.temperature are required");
    if (window_count && !windows) throw Error(FACETCU_INVALID_ARGUMENT, "windows are required");
    if (p->band_count && (!p->wavelengths || !band_direct || !band_diffuse))
        throw Error(FACETCU_INVALID_ARGUMENT,
                    "sensor bands need wavelengths, band_direct and band_diffuse");
    if (p->band_count && !fields->band_output)
        throw Error(FACETCU_INVALID_ARGUMENT, "sensor bands need fields.band_output");
    for (uint32_t b = 0; b < p->band_count; ++b)
        if (!std::isfinite(p->wavelengths[b]) || p->wavelengths[b] <= 0.0f)
            throw Error(FACETCU_INVALID_ARGUMENT, "wavelengths must be finite and positive");
    if (p->material_count && !p->materials)
        throw Error(FACETCU_INVALID_ARGUMENT, "material_count > 0 needs materials");
    for (uint32_t m = 0; m < p->material_count; ++m) {
        validate_surface(p->materials[m].optics);
        if ((p->materials[m].energy_reflectance_count && !p->materials[m].energy_reflectance) ||
            (p->materials[m].energy_transmittance_count && !p->materials[m].energy_transmittance))
            throw Error(FACETCU_INVALID_ARGUMENT, "a surface's energy band values are missing");
    }
    if (p->leaf_facet_count > ctx->facets)
        throw Error(FACETCU_INVALID_ARGUMENT, "leaf_facet_count exceeds the facet count");
    if (p->coupling_iterations < 1 || p->coupling_iterations > 100)
        throw Error(FACETCU_INVALID_ARGUMENT, "coupling_iterations must be in [1, 100]");
    if (!(p->temperature_relaxation > 0.0f && p->temperature_relaxation <= 1.0f))
        throw Error(FACETCU_INVALID_ARGUMENT, "temperature_relaxation must be in (0, 1]");
    if (!(p->time_step >= 1.0f) || !std::isfinite(p->time_step))
        throw Error(FACETCU_INVALID_ARGUMENT, "time_step must be finite and >= 1");
    if (!(p->temperature_tolerance >= 0.0f) || !(p->solver_tolerance >= 0.0f))
        throw Error(FACETCU_INVALID_ARGUMENT, "tolerances must be non-negative");
    if (p->solver_iterations < 1)
        throw Error(FACETCU_INVALID_ARGUMENT, "solver_iterations must be at least 1");
    if (p->precision != FACETCU_PRECISION_FP32 && p->precision != FACETCU_PRECISION_MIXED)
        throw Error(FACETCU_INVALID_ARGUMENT, "precision must be FP32 or MIXED");
    if (p->precision == FACETCU_PRECISION_MIXED && p->solver_tolerance <= 0.0f)
        throw Error(FACETCU_INVALID_ARGUMENT, "MIXED precision needs a solver_tolerance");
    if (!std::isfinite(sun->x) || !std::isfinite(sun->y) || !std::isfinite(sun->z))
        throw Error(FACETCU_INVALID_ARGUMENT, "sun direction must be finite");
    for (uint32_t w = 0; w < window_count; ++w)
        if (!std::isfinite(windows[w].direct_normal) || !std::isfinite(windows[w].diffuse) ||
            windows[w].direct_normal < 0.0f || windows[w].diffuse < 0.0f)
            throw Error(FACETCU_INVALID_ARGUMENT, "window irradiances must be finite and >= 0");
}

}  // namespace

extern "C" {

int facetcu_faceteb_node(facetcu_context* ctx, const facetcu_energy_parameters* parameters,
                         const facetcu_meteo* meteo, const facetcu_direction* sun,
                         const float* sunlit, const facetcu_shortwave_window* windows,
                         uint32_t window_count, const float* band_direct,
                         const float* band_diffuse, facetcu_energy_fields* fields,
                         facetcu_energy_result* result)
{
    return guarded(ctx, [&] {
        require_graph(ctx, "facetebNode()");
        validate_energy(ctx, parameters, meteo, sun, sunlit, windows, window_count, band_direct,
                        band_diffuse, fields);
        const auto t0 = std::chrono::steady_clock::now();
        const facetcu_energy_parameters& p = *parameters;
        const uint32_t F = ctx->facets, M = p.material_count, W = window_count, nb = p.band_count;
        const size_t S = ctx->graph.surfaces;
        if (S != 2 * size_t(F))
            throw Error(FACETCU_LOGIC_ERROR, "the graph does not belong to the current geometry");
        cudaStream_t st = ctx->stream;
        const facetcu_vertex* V = ctx->vertices.as<facetcu_vertex>();

        // per-slot tables: materials, then the object and ground fallbacks
        const facetcu_energy_surface object_fb = fallback_surface(false);
        const facetcu_energy_surface ground_fb = fallback_surface(true);
        auto surface = [&](uint32_t slot) -> const facetcu_energy_surface& {
            return slot < M ? p.materials[slot] : (slot == M ? object_fb : ground_fb);
        };
        std::vector<energy::Material> mats(M + 2);
        std::vector<float2> sw_table(size_t(M + 2) * 2 * W);
        std::vector<facetcu_surface_parameters> optics(M);
        for (uint32_t slot = 0; slot < M + 2; ++slot) {
            const facetcu_energy_surface& m = surface(slot);
            if (slot < M) optics[slot] = m.optics;
            energy::Material& d = mats[slot];
            d.tir_r = m.optics.tir_reflectance;
            d.tir_t = m.optics.tir_transmittance;
            d.surface_resistance = m.surface_resistance;
            d.heat_capacity = m.heat_capacity_per_area;
            d.soil_moisture = m.soil_moisture;
            d.storage_coefficient = energy::storage_coefficient(m, p.time_step);
            d.pv_eta25 = m.pv_eta25;
            d.pv_gamma = m.pv_gamma;
            d.pv_bifaciality = m.pv_bifaciality;
            d.convective_scale = m.convective_scale;
            d.soil_method = m.soil_temperature_method;
            d.photovoltaic = m.photovoltaic ? 1u : 0u;
            d.vegetation = m.vegetation ? 1u : 0u;
            for (uint32_t obj = 0; obj < 2; ++obj) {
                // the broadband value when no per-sample energy spectrum is given
                const float r_fb = obj ? 0.10f : 0.20f, t_fb = obj ? 0.05f : 0.0f;
                const float r_mean =
                    m.energy_reflectance_count
                        ? 0.0f
                        : energy::shortwave_weighted_value(m.optics.reflectance,
                                                           m.optics.reflectance_count, r_fb);
                const float t_mean =
                    m.energy_transmittance_count
                        ? 0.0f
                        : energy::shortwave_weighted_value(m.optics.transmittance,
                                                           m.optics.transmittance_count, t_fb);
                for (uint32_t w = 0; w < W; ++w) {
                    const uint32_t band = windows[w].energy_band;
                    sw_table[(size_t(slot) * 2 + obj) * W + w] = make_float2(
                        m.energy_reflectance_count
                            ? value_at(m.energy_reflectance, m.energy_reflectance_count, band, r_fb)
                            : r_mean,
                        m.energy_transmittance_count
                            ? value_at(m.energy_transmittance, m.energy_transmittance_count, band,
                                       t_fb)
                            : t_mean);
                }
            }
        }
        // band values of the sensor bands (bandValue of the same surfaces)
        facetcu_spectral_parameters sp{};
        const float one_band = 550.0f;
        sp.wavelengths = nb ? p.wavelengths : &one_band;
        sp.band_count = nb ? nb : 1;
        sp.object = object_fb.optics;
        sp.ground = ground_fb.optics;
        sp.materials = M ? optics.data() : nullptr;
        sp.material_count = M;
        sp.leaf_facet_count = p.leaf_facet_count;
        sp.background_angular_strength = p.background_angular_strength;
        sp.sky_temperature = p.sky_temperature;
        if (nb) ctx->spec.build(sp, st);

        // the node's air (runFacetEBCore :3556-3571)
        const float sky_longwave = meteo->longwave > 0.0f
                                       ? meteo->longwave
                                       : 5.670374419e-8f * std::pow(p.sky_temperature, 4.0f);
        energy::Air air{};
        air.air = std::clamp(meteo->air_temperature + 273.15f, 220.0f, 340.0f);
        air.conductance = 5.8f + 4.1f * std::sqrt(std::max(0.1f, meteo->wind_speed));
        air.pressure = std::max(100.0f, meteo->pressure);
        air.density = air.pressure * 100.0f / (287.05f * air.air);
        air.resistance = air.density * 1005.0f / std::max(0.1f, air.conductance);
        air.vapor = meteo->vapor_pressure;
        air.time_step = p.time_step;
        air.relaxation = p.temperature_relaxation;
        air.vegetation_method = p.vegetation_temperature_method == 1 ? 1 : 0;
        std::vector<float> small(2 * size_t(W) + 3 * size_t(nb) + 2);
        for (uint32_t w = 0; w < W; ++w) {
            small[w] = windows[w].direct_normal;
            small[W + w] = windows[w].diffuse;
        }
        const float cosz = std::max(0.0f, sun->y);
        for (uint32_t b = 0; b < nb; ++b) {
            const bool opt = ctx->spec.optical[b] != 0;
            small[2 * W + b] = opt ? band_diffuse[b] * 0.5f
                                   : facetcu_planck_radiance(p.wavelengths[b], p.sky_temperature);
            small[2 * W + nb + b] = opt ? band_direct[b] : 0.0f;
            small[2 * W + 2 * nb + b] = opt ? band_direct[b] * cosz + band_diffuse[b] * 0.5f : 0.0f;
        }
        small[2 * W + 3 * nb] = sky_longwave;
        small[2 * W + 3 * nb + 1] = 0.0f;

        // device layout
        auto al = [](size_t b) { return (b + 255) / 256 * 256; };
        const size_t tab_bytes = al(mats.size() * sizeof(energy::Material)) +
                                 al(sw_table.size() * 8 + 8) + al(small.size() * 4) +
                                 al(size_t(nb) * 4 + 4) + al(F * 4) * 2 + al(64);
        char* tb = static_cast<char*>(ctx->eb_tab.reserve(tab_bytes));
        auto take_t = [&](size_t b) {
            char* r = tb;
            tb += al(b);
            return r;
        };
        auto* d_mats = reinterpret_cast<energy::Material*>(take_t(mats.size() * sizeof(energy::Material)));
        auto* d_sw_table = reinterpret_cast<float2*>(take_t(sw_table.size() * 8 + 8));
        float* d_small = reinterpret_cast<float*>(take_t(small.size() * 4));
        float* d_wl = reinterpret_cast<float*>(take_t(size_t(nb) * 4 + 4));
        uint32_t* d_material = p.material_indices ? reinterpret_cast<uint32_t*>(take_t(F * 4)) : nullptr;
        float* d_texture = p.texture_factors ? reinterpret_cast<float*>(take_t(F * 4)) : nullptr;
        uint32_t* d_stats = reinterpret_cast<uint32_t*>(take_t(64));
        const float* d_dni = d_small;
        const float* d_diff = d_small + W;
        const float* d_bsky = d_small + 2 * W;
        const float* d_bbeam = d_small + 2 * W + nb;
        const float* d_bref = d_small + 2 * W + 2 * nb;
        const float* d_lwsky = d_small + 2 * W + 3 * nb;
        const float* d_zero = d_lwsky + 1;

        const size_t per_side = 26;  // single-column fields (below)
        const size_t io_bytes = al(S * 4) * per_side + al(size_t(W) * S * 4) * 6 +
                                al(size_t(nb) * S * 4) * 4;
        char* c = static_cast<char*>(ctx->eb_io.reserve(io_bytes));
        auto take = [&](size_t n) {
            float* r = reinterpret_cast<float*>(c);
            c += al(n * 4);
            return r;
        };
        float* d_sunlit = take(S);
        float* d_dgeo = take(2 * S);  // [direct geometry][zeros]: the window solve's two suns
        float* d_T = take(S);
        float* d_Tprev = take(S);
        float* d_abs = take(S);
        float* d_inc = take(S);
        float* d_swb = take(S);
        float* d_db = take(S);
        float* d_lrho = take(S);
        float* d_ltau = take(S);
        float* d_lemis = take(S);
        float* d_lB[2] = {take(S), take(S)};
        float* d_lH = take(S);
        energy::Fluxes fx{};
        fx.net = take(S);
        fx.sensible = take(S);
        fx.latent = take(S);
        fx.latent_slope = take(S);
        fx.storage = take(S);
        fx.storage_slope = take(S);
        fx.pv = take(S);
        fx.pv_slope = take(S);
        float* d_swrho = take(size_t(W) * S);
        float* d_swtau = take(size_t(W) * S);
        float* d_swB = take(2 * size_t(W) * S);
        float* d_swH = take(size_t(W) * S);
        float* d_swBT = take(size_t(W) * S);
        float* d_brho = take(size_t(nb) * S);
        float* d_btau = take(size_t(nb) * S);
        float* d_bemis = take(size_t(nb) * S);
        float* d_bout = take(size_t(nb) * S);

        FCU_CHECK(cudaMemcpyAsync(d_mats, mats.data(), mats.size() * sizeof(energy::Material),
                                  cudaMemcpyHostToDevice, st));
        if (!sw_table.empty())
            FCU_CHECK(cudaMemcpyAsync(d_sw_table, sw_table.data(), sw_table.size() * 8,
                                      cudaMemcpyHostToDevice, st));
        FCU_CHECK(cudaMemcpyAsync(d_small, small.data(), small.size() * 4, cudaMemcpyHostToDevice, st));
        if (nb) FCU_CHECK(cudaMemcpyAsync(d_wl, p.wavelengths, size_t(nb) * 4, cudaMemcpyHostToDevice, st));
        if (d_material)
            FCU_CHECK(cudaMemcpyAsync(d_material, p.material_indices, size_t(F) * 4,
                                      cudaMemcpyHostToDevice, st));
        if (d_texture)
            FCU_CHECK(cudaMemcpyAsync(d_texture, p.texture_factors, size_t(F) * 4,
                                      cudaMemcpyHostToDevice, st));
        FCU_CHECK(cudaMemcpyAsync(d_sunlit, sunlit, S * 4, cudaMemcpyHostToDevice, st));
        FCU_CHECK(cudaMemcpyAsync(d_T, fields->temperature, S * 4, cudaMemcpyHostToDevice, st));
        FCU_CHECK(cudaMemcpyAsync(d_Tprev, d_T, S * 4, cudaMemcpyDeviceToDevice, st));
        FCU_CHECK(cudaMemsetAsync(d_dgeo + S, 0, S * 4, st));
        energy::direct_geometry(F, V, *sun, d_sunlit, d_dgeo, st);

        facetcu_energy_result r{};
        r.kernel_launches = 1;
        const bool accel = p.solver_tolerance > 0.0f;
        auto solve = [&](uint32_t bands, uint32_t suns, uint32_t precision, const float* rho,
                         const float* tau, const float* emis, const float* sky, const float* beam,
                         const float* dgeo, const float* init, float* out) {
            facetcu_batch_config cfg{};
            cfg.band_count = bands;
            cfg.sun_count = suns;
            cfg.precision = precision;
            cfg.warm_start = init ? FACETCU_WARM_GIVEN : FACETCU_WARM_NONE;
            cfg.maximum_iterations = p.solver_iterations;
            cfg.tolerance = p.solver_tolerance;
            facetcu_batch_result br{};
            const int rc = run_batched(ctx, &cfg, rho, tau, emis, sky, beam, dgeo, init, out, &br);
            if (rc != FACETCU_OK && rc != FACETCU_NOT_CONVERGED) nested(ctx, rc);
            r.kernel_launches += br.kernel_launches;
            return br.iterations;
        };

        // shortwave windows: each with and without its direct beam, one solve
        if (W) {
            energy::shortwave_optics(F, W, V, d_material, M, d_texture, p.leaf_facet_count,
                                     d_sw_table, p.background_angular_strength, *sun, d_swrho,
                                     d_swtau, st);
            r.shortwave_sweeps = solve(W, 2, p.precision, d_swrho, d_swtau, nullptr, d_diff, d_dni,
                                       d_dgeo, nullptr, d_swB);
            energy::window_incident(ctx->graph, W, d_swB, d_diff, d_dni, d_dgeo, d_swBT, d_swH,
                                    st);
            energy::shortwave_sum(uint32_t(S), W, d_swrho, d_swtau, d_swH, d_swB, d_abs, d_inc,
                                  d_swb, d_db, st);
            r.kernel_launches += 4;
        } else {
            for (float* z : {d_abs, d_inc, d_swb, d_db}) FCU_CHECK(cudaMemsetAsync(z, 0, S * 4, st));
        }

        // coupling rounds
        uint32_t stats[4] = {0, 0, 0, 0};
        auto read_stats = [&] {
            FCU_CHECK(cudaMemcpyAsync(stats, d_stats, sizeof(stats), cudaMemcpyDeviceToHost, st));
            FCU_CHECK(cudaStreamSynchronize(st));
            if (stats[3]) throw Error(FACETCU_RUNTIME_ERROR, "FacetEB energy residual is not finite");
        };
        auto as_float = [](uint32_t u) {
            float f;
            std::memcpy(&f, &u, 4);
            return f;
        };
        int cur = -1;  // d_lB[cur] holds the latest longwave radiosity
        auto longwave = [&] {
            energy::longwave_optics(F, V, d_material, M, p.leaf_facet_count, d_mats,
                                    p.background_angular_strength, d_T, d_lrho, d_ltau, d_lemis, st);
            const int next = cur < 0 ? 0 : cur ^ 1;
            r.longwave_sweeps += solve(1, 1, p.precision, d_lrho, d_ltau, d_lemis, d_lwsky, d_zero,
                                       nullptr, (accel && cur >= 0) ? d_lB[cur] : nullptr,
                                       d_lB[next]);
            cur = next;
            energy::window_incident(ctx->graph, 1, d_lB[cur], d_lwsky, nullptr, nullptr, nullptr,
                                    d_lH, st);
            r.kernel_launches += 3;  // optics, incident and the balance after it
        };
        float max_dt = 0.0f;
        for (uint32_t round = 0; round < p.coupling_iterations; ++round) {
            longwave();
            energy::balance(F, p.leaf_facet_count, d_material, M, d_mats, air, d_lrho, d_ltau,
                            d_lemis, d_lH, d_abs, d_inc, d_T, d_Tprev, fx, d_stats, true, st);
            read_stats();
            max_dt = as_float(stats[0]);
            r.coupling_iterations = round + 1;
            if (max_dt <= p.temperature_tolerance && as_float(stats[2]) <= p.temperature_tolerance)
                break;
        }
        longwave();
        energy::balance(F, p.leaf_facet_count, d_material, M, d_mats, air, d_lrho, d_ltau, d_lemis,
                        d_lH, d_abs, d_inc, d_T, d_Tprev, fx, d_stats, false, st);
        read_stats();
        r.max_temperature_delta = max_dt;
        r.max_energy_residual = as_float(stats[1]);
        r.max_energy_residual_equivalent = as_float(stats[2]);
        r.converged = (max_dt <= p.temperature_tolerance &&
                       r.max_energy_residual_equivalent <= p.temperature_tolerance)
                          ? 1u
                          : 0u;

        // sensor bands of the solved state
        if (nb) {
            energy::state_optics(F, nb, V, d_material, M, d_texture, p.leaf_facet_count,
                                 ctx->spec.table, d_mats, ctx->spec.optical_dev, d_wl,
                                 p.background_angular_strength, *sun, d_T, d_brho, d_btau, d_bemis,
                                 st);
            r.band_sweeps = solve(nb, 1, p.precision, d_brho, d_btau, d_bemis, d_bsky, d_bbeam,
                                  d_dgeo, nullptr, d_bout);
            energy::state_output(d_bout, S, nb, ctx->spec.optical_dev, d_bref, st);
            r.kernel_launches += 2;
        }
        r.solves = 2 * W + r.coupling_iterations + 1 + nb;

        auto get = [&](float* host, const float* dev, size_t n) {
            if (host) FCU_CHECK(cudaMemcpyAsync(host, dev, n * 4, cudaMemcpyDeviceToHost, st));
        };
        get(fields->temperature, d_T, S);
        get(fields->shortwave_radiosity, d_swb, S);
        get(fields->diffuse_radiosity, d_db, S);
        get(fields->longwave_radiosity, d_lB[cur], S);
        get(fields->absorbed_shortwave, d_abs, S);
        get(fields->incident_shortwave, d_inc, S);
        get(fields->net_radiation, fx.net, S);
        get(fields->sensible_heat, fx.sensible, S);
        get(fields->latent_heat, fx.latent, S);
        get(fields->storage_heat, fx.storage, S);
        get(fields->photovoltaic_power, fx.pv, S);
        get(fields->band_output, d_bout, size_t(nb) * S);
        std::vector<float> sw, lw;
        if (fields->radiosity) {
            sw.resize(S);
            lw.resize(S);
            get(sw.data(), d_swb, S);
            get(lw.data(), d_lB[cur], S);
        }
        FCU_CHECK(cudaStreamSynchronize(st));
        if (fields->radiosity)
            for (size_t s = 0; s < S; ++s) fields->radiosity[s] = lw[s] + sw[s];
        r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (result) *result = r;
        return FACETCU_OK;
    });
}

}  // extern "C"

// ---- sensor images ----------------------------------------------------------
extern "C" {

int facetcu_render_sensor_image(facetcu_context* ctx, const facetcu_sensor* sensor,
                                const float* values, uint32_t band_count,
                                const float* wavelengths, float* image, int32_t* side_index,
                                facetcu_image_info* info)
{
    return guarded(ctx, [&] {
        require_initialized(ctx, "renderSensorImage()");
        if (!ctx->facets) throw Error(FACETCU_LOGIC_ERROR, "renderSensorImage() needs geometry");
        if (!sensor) throw Error(FACETCU_INVALID_ARGUMENT, "sensor is required");
        if (band_count && (!values || !wavelengths || !image))
            throw Error(FACETCU_INVALID_ARGUMENT, "values, wavelengths and image are required");
        if (!band_count && !side_index)
            throw Error(FACETCU_INVALID_ARGUMENT, "nothing to render: no bands and no side_index");
        double nz = 0.0, na = 0.0;
        const image::Camera cam = image::camera(*sensor, &nz, &na);
        const size_t n = size_t(cam.width) * cam.height;
        if (n > (size_t(1) << 28) || size_t(band_count) * n > (size_t(1) << 31))
            throw Error(FACETCU_INVALID_ARGUMENT, "image too large");
        for (uint32_t b = 0; b < band_count; ++b)
            if (!std::isfinite(wavelengths[b]))
                throw Error(FACETCU_INVALID_ARGUMENT, "wavelengths must be finite");
        const uint32_t F = ctx->facets;
        const size_t S = 2 * size_t(F);
        cudaStream_t st = ctx->stream;
        auto al = [](size_t b) { return (b + 255) / 256 * 256; };
        const size_t bytes = al(size_t(F) * 3 * image::kProjBytes) + al(size_t(F) * 4) +
                             al(n * 8) + al(n * 4) * 2 + al(size_t(band_count) * S * 4) +
                             al(size_t(band_count) * 4) + al(size_t(band_count) * n * 4) + al(8);
        char* c = static_cast<char*>(ctx->img_io.reserve(bytes));
        auto take = [&](size_t b) {
            char* r = c;
            c += al(b);
            return r;
        };
        image::Scratch w{};
        w.proj = take(size_t(F) * 3 * image::kProjBytes);
        w.side = reinterpret_cast<int32_t*>(take(size_t(F) * 4));
        w.zbuf = reinterpret_cast<unsigned long long*>(take(n * 8));
        w.index = reinterpret_cast<int32_t*>(take(n * 4));
        int32_t* d_sides = reinterpret_cast<int32_t*>(take(n * 4));
        float* d_values = reinterpret_cast<float*>(take(size_t(band_count) * S * 4));
        float* d_wl = reinterpret_cast<float*>(take(size_t(band_count) * 4));
        float* d_image = reinterpret_cast<float*>(take(size_t(band_count) * n * 4));
        uint32_t* d_counts = reinterpret_cast<uint32_t*>(take(8));
        if (band_count) {
            FCU_CHECK(cudaMemcpyAsync(d_values, values, size_t(band_count) * S * 4,
                                      cudaMemcpyHostToDevice, st));
            FCU_CHECK(cudaMemcpyAsync(d_wl, wavelengths, size_t(band_count) * 4,
                                      cudaMemcpyHostToDevice, st));
        }
        const double sky_t = std::max(120.0, sensor->sky_temperature != 0.0 &&
                                                     std::isfinite(sensor->sky_temperature)
                                                 ? sensor->sky_temperature
                                                 : 250.0);
        image::render(cam, F, ctx->vertices.as<facetcu_vertex>(), d_values, band_count, S, d_wl,
                      sensor->temperature_output != 0, sky_t, w, d_image, d_sides, d_counts, st);
        uint32_t counts[2] = {0, 0};
        if (band_count)
            FCU_CHECK(cudaMemcpyAsync(image, d_image, size_t(band_count) * n * 4,
                                      cudaMemcpyDeviceToHost, st));
        if (side_index)
            FCU_CHECK(cudaMemcpyAsync(side_index, d_sides, n * 4, cudaMemcpyDeviceToHost, st));
        FCU_CHECK(cudaMemcpyAsync(counts, d_counts, 8, cudaMemcpyDeviceToHost, st));
        FCU_CHECK(cudaStreamSynchronize(st));
        if (info) {
            info->observed_pixels = counts[0];
            info->output_pixels = counts[1];
            info->naming_zenith = nz;
            info->naming_azimuth = na;
        }
        return FACETCU_OK;
    });
}

}  // extern "C"
