// internal.h — shared declarations of the facetcu library (not installed).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/facetcu.h"

namespace facetcu {

// Error carrying one of the FACETCU_* status codes.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        throw Error(FACETCU_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    }
    throw Error(FACETCU_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}
#define FCU_CHECK(x) ::facetcu::cuda_check((x), #x)
#define FCU_LAUNCH(what) ::facetcu::cuda_check(cudaGetLastError(), what)

// Owning device buffer that only grows.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { release(); }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    void* reserve(size_t n)
    {
        if (n <= bytes && ptr) return ptr;
        release();
        if (n == 0) n = 16;
        cuda_check(cudaMalloc(&ptr, n), "cudaMalloc");
        bytes = n;
        return ptr;
    }
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

// Per-direction orthographic frame of the CPU rasterizer
// (facetrtcore.cpp:1244-1282): right/up/view basis, centre and radius.
struct RasterView {
    float right[3];
    float up[3];
    float view[3];
};

struct RasterFrame {
    float center[3];
    float radius;
    uint32_t width, height;
    uint32_t facets;
    uint32_t tiles;        // 1 + periodic neighbours (<= 21)
    float tile_dx[21];
    float tile_dz[21];
};

// Scratch used by the device sort and scan.
struct Workspace {
    DeviceBuffer a, b, c, d, e;
};

// ---- device utilities (sort.cu) ----------------------------------------
// Exclusive scan of n uint32 values; out may alias in.  Returns nothing;
// *total_dev (optional) receives the 64-bit sum on the device.
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n,
                        unsigned long long* total_dev, Workspace& ws, cudaStream_t s);
// LSD radix sort of 64-bit keys on bits [0, key_bits), with optional 32-bit
// values; stable.  Result ends in keys/values (the buffers are swapped with
// the alternates as needed).
void radix_sort_u64(uint64_t*& keys, uint64_t*& keys_alt, uint32_t*& values,
                    uint32_t*& values_alt, size_t n, int key_bits, Workspace& ws,
                    cudaStream_t s);

// ---- raster visibility (raster.cu) --------------------------------------
struct RasterBuffers {
    DeviceBuffer counts;    // dirs * pixels
    DeviceBuffer offsets;   // dirs * pixels + 1
    DeviceBuffer records;   // fragments (u64: depth bits << 32 | key)
    DeviceBuffer big_list;  // large-triangle work items
    DeviceBuffer deep_list; // pixels with more than the fast-path chain
    DeviceBuffer stats;     // small counters
};

struct RasterStats {
    unsigned long long fragments;
    unsigned long long overflow;   // sum over pixels of max(0, count - cap)
    unsigned long long pairs;
    unsigned int big;
    unsigned int deep;
    unsigned int capacity_error;
    unsigned int max_chain;
};

// Rasterise `dir_count` directions (views[0..dir_count)) into exact-size
// per-pixel fragment lists.  Leaves counts/offsets/records filled.
void raster_fragments(const facetcu_vertex* d_vertices, const RasterFrame& frame,
                      const RasterView* views, uint32_t dir_count, RasterBuffers& rb,
                      Workspace& ws, RasterStats& stats, cudaStream_t s);
// Resolve the lists of a chunk into denominators, sky counts and pair keys
// (lo << side_bits | hi), appended at pairs[pair_count..].
// chain_cap = the reference's maxFragmentsPerPixel: longer chains count as
// fragment overflow (UINT32_MAX = no limit).
void raster_resolve_graph(const RasterFrame& frame, uint32_t dir_count, uint32_t chain_cap,
                          RasterBuffers& rb, uint32_t* d_denominators, uint32_t* d_sky,
                          uint64_t* d_pairs, unsigned long long* d_pair_count, int side_bits,
                          RasterStats& stats, cudaStream_t s);
// Resolve one direction's lists into sunlit total/visible counts.
void raster_resolve_sunlit(const RasterFrame& frame, uint32_t chain_cap, RasterBuffers& rb,
                           uint32_t* d_total, uint32_t* d_visible, RasterStats& stats,
                           cudaStream_t s);

// ---- graph assembly (graph.cu) ------------------------------------------
struct DeviceGraph {
    uint32_t surfaces = 0;
    uint64_t nnz = 0;
    DeviceBuffer row_offsets;   // S + 1 (u32)
    DeviceBuffer edges;         // nnz * {neighbor, count}
    DeviceBuffer denominators;  // S
    DeviceBuffer sky;           // S
    DeviceBuffer packed;        // nnz u32: neighbor | count << nb_bits (batched solver)
    bool packed_valid = false;
    uint32_t nb_bits = 22;  // neighbour field width of the packed words
    uint32_t max_count = 0;
    // Morton-ordered copy used by the batched solver: facets renumbered along
    // a Morton curve of their centroids, rows and neighbour ids remapped.
    bool perm_valid = false;
    DeviceBuffer order;         // new facet -> old facet
    DeviceBuffer rank;          // old facet -> new facet
    DeviceBuffer p_rows, p_packed, p_denom, p_sky;
    size_t p_nnz = 0;           // edges of the copy (counts above 255 split)
    // Scene batches: the first facet of every scene and the total (empty for
    // one scene); with the Morton copy, the scene of each renumbered facet.
    std::vector<uint32_t> scene_facets;
    DeviceBuffer p_scene;       // F u16, built with the Morton copy for 2..65535 scenes
};
// Sort undirected pair keys, count runs, emit the symmetric CSR.
void graph_from_pairs(uint64_t* d_pairs, size_t pair_count, int side_bits, DeviceGraph& g,
                      Workspace& ws, cudaStream_t s);
// max |(sky + sum counts) / denom - 1| over sides with denom > 0, and the
// number of sides with denom > 0.
void graph_append(DeviceGraph& dst, const DeviceGraph& src, uint32_t side_offset,
                  uint64_t edge_offset, cudaStream_t s);
void graph_closure(const DeviceGraph& g, float* closure, uint32_t* sampled, Workspace& ws,
                   cudaStream_t s);
// Build the 4-byte packed edge array (neighbor in 22 bits, count in 10 bits)
// when the graph fits it.
bool graph_pack(DeviceGraph& g, Workspace& ws, cudaStream_t s);

// ---- solves (solve.cu) ---------------------------------------------------
void jacobi_plain_sweep(const DeviceGraph& g, const facetcu_surface_optics* d_optics,
                        float sky, float relaxation, const float* d_in, float* d_out,
                        uint32_t* d_max_delta_bits, cudaStream_t s);
// The same sweep on raw device pointers (used by facetcu_solve_noalloc).
void jacobi_plain_sweep_raw(uint32_t surfaces, const uint32_t* rows, const facetcu_csr_edge* edges,
                            const uint32_t* denom, const uint32_t* skyc,
                            const facetcu_surface_optics* d_optics, float sky, float relaxation,
                            const float* d_in, float* d_out, uint32_t* d_max_delta_bits,
                            cudaStream_t s);
void incident_irradiance(const DeviceGraph& g, const facetcu_surface_optics* d_optics,
                         float sky, const float* d_radiosity, float* d_out, cudaStream_t s);

// ---- batched solver (batched.cu) ---------------------------------------
struct BatchProblem {
    const facetcu_vertex* vertices;  // for the Morton order of the solver graph
    float lo[3], hi[3];              // scene bounds
    uint32_t S;            // sides
    uint32_t bands, suns;  // R = bands * suns
    const float* rho;      // bands * S
    const float* tau;      // bands * S
    const float* emis;     // bands * S or null
    const float* sky;      // bands
    const float* beam;     // bands
    const float* dgeo;     // suns * S or null
    uint32_t step_ctas_per_sm = 0;  // pipelined int8 step: CTAs per SM (0: as many as fit)
};
struct BatchState {
    DeviceBuffer x0, x1;        // panels, side-major [S][P]
    DeviceBuffer half;          // BF16 copy for mixed precision
    DeviceBuffer colstats;      // per-column max|dB|, max|B| bits
    DeviceBuffer q;             // source term per panel
    DeviceBuffer corr;          // residual / correction panel
    DeviceBuffer i8;            // int8 step panels (two)
    DeviceBuffer scene_state;   // scene batches: [scenes][kMaxP] step records + [scenes] done
    cudaGraphExec_t step_graph = nullptr;  // the int8 phase's loop graph
    bool no_loop_graph = false;            // conditional graph nodes unavailable
    alignas(8) unsigned char step_graph_key[384] = {};
};
void release_graphs(BatchState& st);
// Device-side checks of the batched solve's inputs; returns the error bits
// (1 optics, 2 sky, 4 beam).
uint32_t validate_inputs(const float* rho, const float* tau, const float* emis, size_t n,
                         const float* sky, const float* beam, uint32_t bands, DeviceBuffer& scratch,
                         cudaStream_t s);
int batched_solve(const DeviceGraph& g, const BatchProblem& p, const facetcu_batch_config& cfg,
                  const float* d_initial, float* d_out, BatchState& st, Workspace& ws,
                  cudaStream_t s, facetcu_batch_result* result);

// ---- hemisphere ray casting (lbvh.cu, hemi.cu) ----------------------------
struct Lbvh {
    uint32_t leaves = 0;
    DeviceBuffer nodes;      // internal nodes: 2 children (u32, leaf bit 31) + aabb
    DeviceBuffer tri;        // per sorted leaf: a, e1, e2 (9 floats) + facet id
    DeviceBuffer parent;     // build scratch
    DeviceBuffer flags;      // build scratch
    float scene_min[3], scene_max[3];
    // A hit counts only when o + t d lies in the facet's box widened by
    // hit_margin (set before lbvh_build); leaf boxes are widened by twice it.
    float hit_margin = 0.0f;
};
// The hemisphere caster's hit margin from the vertex bounds and the periodic
// copies traced: 1e-5 of (reach + extent) + 1e-7, where reach is the largest
// coordinate magnitude (plus two periods with copies) and extent the largest
// side of the bounds.
float hit_margin(const float lo[3], const float hi[3], uint32_t periodic_count, float size_x,
                 float size_z);
void lbvh_build(const facetcu_vertex* d_vertices, uint32_t facets, Lbvh& bvh, Workspace& ws,
                cudaStream_t s);
// Facet ids sorted by the 30-bit Morton code of their centroids in [lo, hi].
void morton_order(const facetcu_vertex* d_vertices, uint32_t facets, const float lo[3],
                  const float hi[3], uint32_t* d_order, Workspace& ws, cudaStream_t s);
// Periodic tile offsets (tile 0 = the scene itself), as in RasterFrame.
struct PeriodicTiles {
    uint32_t count = 0;  // neighbour tiles (<= 20)
    float dx[21] = {}, dz[21] = {};
};
void hemisphere_graph(const facetcu_vertex* d_vertices, uint32_t facets, const Lbvh& bvh,
                      const float* d_uv, const float* d_dir, uint32_t rays, uint32_t sets,
                      uint32_t top_k, const PeriodicTiles& periodic, DeviceGraph& g,
                      unsigned long long* dropped, Workspace& ws, cudaStream_t s);
void hemisphere_sunlit(const facetcu_vertex* d_vertices, uint32_t facets, const Lbvh& bvh,
                       const float* d_uv, uint32_t samples, uint32_t sets, float3 sun,
                       const PeriodicTiles& periodic, float* d_fraction, cudaStream_t s);

// ---- warm-start MLP (mlp.cu) -----------------------------------------------
namespace mlp {
constexpr int kInputs = 12, kOutputs = 64;
constexpr int kParameterCount = 128 * 12 + 128 + 128 * 128 + 128 + 64 * 128 + 64;
// Layer sizes and offsets in the parameter vector (W1[128x12], b1, W2, b2,
// W3[64x128], b3; row-major W[out][in]).
constexpr int kIn = 12, kH = 128, kOut = 64;
constexpr int kW1 = kH * kIn, kB1 = kH, kW2 = kH * kH, kB2 = kH, kW3 = kOut * kH, kB3 = kOut;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kW1, kOffW2 = kOffB1 + kB1, kOffB2 = kOffW2 + kW2,
              kOffW3 = kOffB2 + kB2, kOffB3 = kOffW3 + kW3, kParams = kOffB3 + kB3;
static_assert(kParams == kParameterCount, "parameter layout");

struct Net {
    DeviceBuffer params, bf16, adam_m, adam_v, grad;
    bool ready = false;
    uint32_t steps_done = 0;
};
struct Scratch {
    DeviceBuffer z1, a1, z2, a2, y, dy, da, dz, part, lossp, idx, xb, tb;
};
// Buffers of the tensor-core inference (mlp_tc.cu).
struct TensorScratch {
    DeviceBuffer xb, a1, a2, w1p, error;
};
// Inference of n rows on the tensor cores (tcgen05, BF16 activations, FP32
// accumulation): X[n][12] FP32 -> Y[n][64] FP32.  Asynchronous on s; a
// wait that ran out inside a kernel is reported by tensor_error.
void infer_tensor(Net& net, const float* X, size_t n, TensorScratch& ts, float* Y, cudaStream_t s);
// Nonzero when a tensor-core kernel since the last infer_tensor timed out
// (synchronises s).
uint32_t tensor_error(TensorScratch& ts, cudaStream_t s);
void init_params(Net& net, uint32_t seed, cudaStream_t s);
void set_params(Net& net, const float* host, cudaStream_t s);
// Rows per forward pass: kMaxRows keeps the GEMM grid (64 rows per CTA in
// y) under 65,535 CTAs; inference is chunked at kInferChunk rows.
constexpr size_t kMaxRows = size_t(1) << 21;
constexpr size_t kInferChunk = size_t(1) << 19;
void forward_full(Net& net, const float* X, int n, Scratch& sc, float* Y, cudaStream_t s);
void infer(Net& net, const float* X, size_t n, Scratch& sc, float* Y, cudaStream_t s);
double loss_and_grad(Net& net, const float* X, const float* T, int n, Scratch& sc, cudaStream_t s,
                     bool want_loss);
void adam_step(Net& net, float lr, cudaStream_t s);
double train(Net& net, const float* X, const float* T, uint64_t n, uint32_t steps, uint32_t batch,
             float lr, uint32_t seed, Scratch& sc, cudaStream_t s);
void features(const float* B1, uint32_t S, uint32_t bands, uint32_t suns, const float* rho,
              const float* tau, const float* sky, const float* beam, const uint32_t* denom,
              const uint32_t* skyc, const facetcu_vertex* V, float* X, cudaStream_t s);
void warm_combine(const float* B1, const float* Y, uint32_t S, uint32_t bands, uint32_t suns,
                  const float* sky, const float* beam, float* x0, cudaStream_t s);
void targets(const float* B, const float* B1, uint32_t S, uint32_t bands, uint32_t suns,
             const float* sky, const float* beam, float* T, cudaStream_t s);
}  // namespace mlp

// ---- FacetEB node kernels (energy.cu) --------------------------------------
namespace energy {
// Per material slot (materials, then the object and ground fallbacks).
struct Material {
    float tir_r, tir_t;
    float surface_resistance, heat_capacity, soil_moisture;
    float storage_coefficient;  // soilStorageCoefficient(surface, dTime)
    float pv_eta25, pv_gamma, pv_bifaciality, convective_scale;
    int32_t soil_method;
    uint32_t photovoltaic, vegetation;
};
// Per-node air scalars (runFacetEBCore :3560-3571).
struct Air {
    float air;          // K, clamp(T_air + 273.15, 220, 340)
    float conductance;  // 5.8 + 4.1 sqrt(max(0.1, wind))
    float pressure;     // max(100, p) hPa
    float density;      // p 100 / (287.05 T)
    float resistance;   // density 1005 / max(0.1, conductance)
    float vapor;        // hPa
    float time_step;
    float relaxation;
    int32_t vegetation_method;
};
struct Fluxes {
    float *net, *sensible, *latent, *latent_slope, *storage, *storage_slope, *pv, *pv_slope;
};
void shortwave_optics(uint32_t F, uint32_t W, const facetcu_vertex* V, const uint32_t* material,
                      uint32_t M, const float* texture, uint32_t leaf, const float2* table,
                      float strength, facetcu_direction sun, float* rho, float* tau,
                      cudaStream_t s);
void direct_geometry(uint32_t F, const facetcu_vertex* V, facetcu_direction sun,
                     const float* sunlit, float* dgeo, cudaStream_t s);
// BT: scratch of S * W floats (unused for one column without a direct term).
void window_incident(const DeviceGraph& g, uint32_t W, const float* B, const float* sky,
                     const float* dni, const float* dgeo, float* BT, float* H, cudaStream_t s);
void shortwave_sum(uint32_t S, uint32_t W, const float* rho, const float* tau, const float* H,
                   const float* B, float* absorbed, float* incident, float* radiosity,
                   float* diffuse, cudaStream_t s);
void longwave_optics(uint32_t F, const facetcu_vertex* V, const uint32_t* material, uint32_t M,
                     uint32_t leaf, const Material* mats, float strength, const float* T,
                     float* rho, float* tau, float* emis, cudaStream_t s);
void balance(uint32_t F, uint32_t leaf, const uint32_t* material, uint32_t M,
             const Material* mats, const Air& a, const float* lw_rho, const float* lw_tau,
             const float* lw_emis, const float* lw_in, const float* absorbed,
             const float* incident, float* T, const float* T_prev, const Fluxes& out,
             uint32_t* stats, bool update, cudaStream_t s);
void state_optics(uint32_t F, uint32_t nb, const facetcu_vertex* V, const uint32_t* material,
                  uint32_t M, const float* texture, uint32_t leaf, const float4* table,
                  const Material* mats, const uint8_t* optical, const float* wavelengths,
                  float strength, facetcu_direction sun, const float* T, float* rho, float* tau,
                  float* emis, cudaStream_t s);
void state_output(float* B, size_t S, uint32_t nb, const uint8_t* optical, const float* reference,
                  cudaStream_t s);
// Host arithmetic of the reference (faceteb.cpp).
float shortwave_weighted_value(const float* values, uint32_t n, float fallback);
float storage_coefficient(const facetcu_energy_surface& m, float time_step);
}  // namespace energy

// ---- sensor images (image.cu) ----------------------------------------------
namespace image {
struct Camera {
    double right[3], up[3], out[3], forward[3], cam_pos[3];
    double tan_half, min_x, max_y, range_x, range_y;
    double orth_min_z, orth_max_x, orth_east, orth_north, scene_w, scene_d;
    uint32_t width, height;
    int32_t perspective;
};
struct Scratch {
    void* proj;               // 3F projected vertices
    int32_t* side;            // F observed sides
    unsigned long long* zbuf; // W*H depth keys
    int32_t* index;           // W*H facet indices, then observed sides
};
constexpr size_t kProjBytes = 32;  // one projected vertex
Camera camera(const facetcu_sensor& s, double* naming_zenith, double* naming_azimuth);
void render(const Camera& c, uint32_t F, const facetcu_vertex* V, const float* values,
            uint32_t nb, size_t S, const float* wavelengths, bool as_temperature, double sky_t,
            Scratch& w, float* image, int32_t* sides, uint32_t* counts, cudaStream_t s);
}  // namespace image

// ---- spectral optics (spectral.cu) ----------------------------------------
namespace spectral {
bool optical_wavelength(float wavelength);
// Per-material, per-band scalars and per-band flags for one parameter set.
struct Tables {
    DeviceBuffer dev;
    float4* table = nullptr;   // [(slot*2 + object)*bands + b] = {rho, tau, Planck sun, shade}
    float2* tir = nullptr;     // [slot] = {tir rho, tir tau}
    uint8_t* thermal = nullptr;      // [b] wavelength > 2500 (makeSpectralOptics' test)
    uint8_t* optical_dev = nullptr;  // [b] isOpticalWavelength
    std::vector<float> sky, beam;    // per band
    std::vector<uint8_t> optical;
    void build(const facetcu_spectral_parameters& p, cudaStream_t s);
};
void optics(const Tables& t, const facetcu_spectral_parameters& p, uint32_t F,
            const facetcu_vertex* V, const uint32_t* material, const float* texture,
            facetcu_direction sun, const float* sunlit, uint32_t b0, uint32_t bcount, float* rho,
            float* tau, float* emis, cudaStream_t s);
void direct_geometry(uint32_t F, const facetcu_vertex* V, facetcu_direction sun,
                     const float* sunlit, float* dgeo, cudaStream_t s);
void pack(size_t S, const float* rho, const float* tau, const float* emis, const float* dgeo,
          float beam, facetcu_surface_optics* out, cudaStream_t s);
void apparent(float* B, size_t S, uint32_t bands, const uint8_t* optical, float ref,
              cudaStream_t s);
}  // namespace spectral

}  // namespace facetcu
