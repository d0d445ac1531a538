/*
 * facetcu.h — C ABI of the GB300 FacetRT facet-radiosity library.
 *
 * This is the library seam that replaces StreamSim HiStream's Vulkan backend
 * class facetvk::FacetrtVulkan (models/histream/src/facetrt/facetrt_vulkan.h:70-104).
 * Plain C types, plain pointers and sizes; every function returns an int
 * status (FACETCU_OK = 0) and keeps a message for facetcu_last_error().
 * One context = one GPU, one CUDA stream, one thread at a time (the
 * reference object is single-threaded and non-reentrant, facetrt_vulkan.cpp:292-301).
 * Every call is synchronous unless its name ends in _device or _async.
 *
 * Side convention (facetrt_vulkan.h:28-29): side 2f is the geometric-normal
 * side of facet f, side 2f+1 the opposite side.
 */
#ifndef FACETCU_H
#define FACETCU_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FACETCU_ABI_VERSION 1

/* Status codes.  The first four map to the exception classes the reference
 * throws (facetrt_vulkan.cpp), so a C++ wrapper can re-throw them. */
enum {
    FACETCU_OK = 0,
    FACETCU_INVALID_ARGUMENT = 1, /* std::invalid_argument */
    FACETCU_LOGIC_ERROR = 2,      /* std::logic_error: call-order violation */
    FACETCU_RUNTIME_ERROR = 3,    /* std::runtime_error: overflow, no samples */
    FACETCU_OVERFLOW_ERROR = 4,   /* std::overflow_error: capacity exceeded */
    FACETCU_CUDA_ERROR = 5,       /* CUDA runtime failure */
    FACETCU_NO_DEVICE = 6,        /* no usable GPU */
    FACETCU_OUT_OF_MEMORY = 7,    /* device allocation failed */
    FACETCU_DEVICE_CAPACITY = 8,  /* a device-side capacity flag was raised */
    FACETCU_NOT_CONVERGED = 9,    /* iteration budget spent; result still written */
    FACETCU_DEVICE_TIMEOUT = 10   /* a bounded wait inside a kernel ran out (the context
                                     stays usable; the result is not written) */
};

typedef struct facetcu_context facetcu_context;

/* facetvk::Vertex (facetrt_vulkan.h:15-18): 24 bytes. */
typedef struct { float position[3]; float normal[3]; } facetcu_vertex;
/* facetvk::Direction (facetrt_vulkan.h:22-26): towards the camera / sun. */
typedef struct { float x, y, z; } facetcu_direction;
/* facetvk::SurfaceOptics (facetrt_vulkan.h:30-35): 16 bytes per side. */
typedef struct {
    float reflectance, transmittance, emission, direct_irradiance;
} facetcu_surface_optics;
/* facetvk::Config (facetrt_vulkan.h:37-47), same field order and layout.
 * max_fragments_per_pixel is the reference's A-buffer depth: a pixel chain
 * longer than it is reported as fragment overflow and fails the build, as
 * in the reference; the device lists themselves have no fixed depth.
 * edge_hash_capacity is accepted and ignored (the graph is built by sorting,
 * not hashing, so hash overflow cannot occur). */
typedef struct {
    uint32_t raster_width;
    uint32_t raster_height;
    uint32_t max_fragments_per_pixel;
    uint32_t edge_hash_capacity;
    bool enable_validation;
    uint32_t gpu_index;
    uint32_t periodic_neighbor_count;
    float periodic_size_x;
    float periodic_size_z;
} facetcu_config;
/* facetvk::GraphDiagnostics (facetrt_vulkan.h:49-56). */
typedef struct {
    uint32_t facet_count;
    uint32_t surface_count;
    uint32_t directed_edge_count;
    uint32_t fragment_overflow;
    uint32_t hash_overflow;
    float max_closure_error;
} facetcu_graph_diagnostics;
/* FacetrtVulkan::CsrEdge (facetrt_vulkan.h:114-117). */
typedef struct { uint32_t neighbor, count; } facetcu_csr_edge;

/* ---- host helpers (no GPU needed) -------------------------------------- */
/* makeHemisphereDirections (facetrtcore.cpp:475-489): `count` golden-spiral
 * directions of the upper hemisphere (Y up), computed with the C library's
 * float cos/sin like the reference. */
void facetcu_hemisphere_directions(uint32_t count, facetcu_direction *out);
/* sunDirection (facetrtcore.cpp:491-498): +X north, +Z east, Y up. */
facetcu_direction facetcu_sun_direction(float zenith_degrees, float azimuth_degrees);

/* ---- lifetime -------------------------------------------------------- */
int facetcu_create(facetcu_context **out);
void facetcu_release(facetcu_context *ctx);
const char *facetcu_last_error(const facetcu_context *ctx);
int facetcu_device_count(int *count);

/* FacetrtVulkan::initialize (facetrt_vulkan.h:80, facetrt_vulkan.cpp:98). */
int facetcu_initialize(facetcu_context *ctx, const facetcu_config *config);
/* FacetrtVulkan::destroy (facetrt_vulkan.h:102): frees device resources;
 * the context may be initialized again. */
int facetcu_destroy(facetcu_context *ctx);
/* The CUDA stream all of the context's work runs on (cudaStream_t). */
int facetcu_get_stream(facetcu_context *ctx, void **stream);

/* ---- geometry and visibility ----------------------------------------- */
/* FacetrtVulkan::setGeometry (facetrt_vulkan.cpp:445-471): non-indexed
 * triangle list, 3 consecutive vertices per facet with the same unit normal.
 * The orthographic raster frame uses the vertex bounds, as the Vulkan
 * backend does (facetrt_vulkan.cpp:455-464). */
int facetcu_set_geometry(facetcu_context *ctx, const facetcu_vertex *vertices,
                         uint64_t vertex_count);
/* Use explicit scene bounds for the raster frame instead of the vertex
 * bounds — what the reference's CPU backend does (Scene::minimum/maximum in
 * CpuRasterizer, facetrtcore.cpp:1222-1242). */
int facetcu_set_raster_bounds(facetcu_context *ctx, const float minimum[3],
                              const float maximum[3]);
/* FacetrtVulkan::buildVisibilityGraph (facetrt_vulkan.cpp:866-1062), with
 * the raster and pixel-chain rules of buildCpuGraph (facetrtcore.cpp:1348-1436):
 * integer counts equal to the reference CPU backend's. */
int facetcu_build_visibility_graph(facetcu_context *ctx,
                                   const facetcu_direction *directions,
                                   uint32_t direction_count,
                                   facetcu_graph_diagnostics *diagnostics);
/* FacetrtVulkan::computeSunlitFraction (facetrt_vulkan.cpp:1064-1158) with
 * the rules of computeCpuSunlit (facetrtcore.cpp:1438-1474). fraction: 2F. */
int facetcu_compute_sunlit_fraction(facetcu_context *ctx,
                                    const facetcu_direction *sun_direction,
                                    float *fraction);

/* Hemisphere ray-cast view factors (no reference counterpart): for every
 * side, rays_per_side cosine-distributed rays from points on the facet,
 * nearest hit by an LBVH; the top_k most-hit sides are kept per row and the
 * row is renormalised over kept + sky rays (denominator = kept + sky).
 * sample_uv: sets * rays_per_side * 2 barycentric (u, v); sample_dir:
 * sets * rays_per_side * 3 local directions (z along the side normal);
 * side s uses set s % sets. dropped (optional) = rays hitting sides cut by
 * top_k, summed over all rows.  Limits: rays_per_side <= 1023, 2F <= 2^22.
 * The LBVH is built on first use after setGeometry and kept. */
typedef struct {
    uint32_t rays_per_side;
    uint32_t top_k;
    uint32_t sample_sets;
    uint32_t reserved;
} facetcu_hemisphere_config;
int facetcu_build_hemisphere_graph(facetcu_context *ctx,
                                   const facetcu_hemisphere_config *config,
                                   const float *sample_uv, const float *sample_dir,
                                   facetcu_graph_diagnostics *diagnostics,
                                   uint64_t *dropped);
/* Sun visibility by shadow rays from `samples` points per side (set s % sets
 * of sample_uv, which holds sets * samples * 2 floats); sides facing away
 * from the sun get 0. fraction: 2F. */
int facetcu_hemisphere_sunlit(facetcu_context *ctx, const facetcu_direction *sun_direction,
                              uint32_t samples, uint32_t sample_sets,
                              const float *sample_uv, float *fraction);

/* Graph access (count form: F_sn = count_sn / denom_s, sky_s / denom_s). */
int facetcu_graph_size(facetcu_context *ctx, uint32_t *surface_count,
                       uint64_t *directed_edge_count);
/* Rows are sorted by neighbour.  Any pointer may be NULL. */
int facetcu_get_graph(facetcu_context *ctx, uint32_t *row_offsets,
                      facetcu_csr_edge *edges, uint32_t *denominators,
                      uint32_t *sky_counts);
/* Load a graph built elsewhere (e.g. by the reference); needs set_geometry. */
int facetcu_set_graph(facetcu_context *ctx, uint32_t surface_count,
                      const uint32_t *row_offsets, const facetcu_csr_edge *edges,
                      const uint32_t *denominators, const uint32_t *sky_counts);

/* ---- solves (reference semantics) ------------------------------------ */
/* FacetrtVulkan::solve (facetrt_vulkan.cpp:1177-1247): `iterations` Jacobi
 * sweeps from B = 0 with the two-sided update of radiosity.comp:49-106;
 * FP32 gather in CSR order.  optics_count must be 2F (the reference checks
 * optics.size(), facetrt_vulkan.cpp:1162); radiosity receives 2F floats;
 * initial (solve_accelerated) holds 2F floats when given. */
int facetcu_solve(facetcu_context *ctx, const facetcu_surface_optics *optics,
                  uint64_t optics_count, float sky_radiosity, uint32_t iterations,
                  float relaxation, float *radiosity, uint32_t *iterations_done,
                  float *max_delta);
/* FacetrtVulkan::solveAccelerated (facetrt_vulkan.cpp:1249-1358): optional
 * warm start, batches of batch_iterations sweeps, stop when the absolute
 * max|dB| of the last sweep <= tolerance. initial may be NULL. */
int facetcu_solve_accelerated(facetcu_context *ctx, const facetcu_surface_optics *optics,
                              uint64_t optics_count, float sky_radiosity, const float *initial,
                              uint32_t maximum_iterations, uint32_t batch_iterations,
                              float tolerance, float relaxation, float *radiosity,
                              uint32_t *iterations_done, float *max_delta);
/* FacetrtVulkan::incidentIrradiance (facetrt_vulkan.cpp:1360-1399):
 * H_s = max(0, diffuse_s + D_s) from a solution, FP64 gather.  radiosity,
 * optics and irradiance hold `count` = 2F elements. */
int facetcu_incident_irradiance(facetcu_context *ctx, const float *radiosity,
                                const facetcu_surface_optics *optics, uint64_t count,
                                float sky_radiosity, float *irradiance);

/* ---- batched solves (no reference counterpart) ------------------------ */
/* Many right-hand sides against the one graph: R = band_count * sun_count
 * columns, column r = sun * band_count + band.  Per band b and side s:
 * reflectance[b*S+s], transmittance[b*S+s], emission[b*S+s] (NULL = 0),
 * sky[b] and beam[b]; per sun k: direct_geometry[k*S+s] (the sunlit
 * fraction times max(0, n_s . sun_k); NULL = no direct light).  The source
 * for column (k,b) is D = beam[b] * direct_geometry[k*S+s].
 * Iterates the reference's two-sided Jacobi sweep (relaxation 1) until, for
 * every column, max_s |B_new - B| <= tolerance * max_s |B_new|, or
 * maximum_iterations.  radiosity: R * S floats, column-major by RHS
 * (radiosity[r*S + s]). */
enum {
    FACETCU_PRECISION_FP32 = 0,     /* FP32 gather */
    FACETCU_PRECISION_MIXED = 1,    /* FP32 state and residual; int8 steps (BF16 defects below 32 columns) */
    FACETCU_PRECISION_FP64 = 2      /* FP64 state and gather (reference truth) */
};
enum {
    FACETCU_WARM_NONE = 0,          /* start from B = 0 */
    FACETCU_WARM_GIVEN = 1,         /* start from `initial` (R * S floats) */
    FACETCU_WARM_MLP = 2            /* start from the context's trained MLP (64 bands) */
};
typedef struct {
    uint32_t band_count;
    uint32_t sun_count;
    uint32_t precision;         /* FACETCU_PRECISION_* */
    uint32_t warm_start;        /* FACETCU_WARM_* */
    uint32_t maximum_iterations;
    float tolerance;            /* stop when every side's relative change
                                   |dB_s| / max(|B_s|, 1e-6 max|B|) <= tolerance */
    uint32_t panel_width;       /* RHS columns per resident panel (power of two, <= 128;
                                   <= 32 in FP64); 0 = the widest that fits */
    uint32_t flags;             /* FACETCU_BATCH_TIME_SWEEPS: time every sweep kernel;
                                   FACETCU_BATCH_LEGACY_STEP: run the 64-column int8
                                   steps on the register-gather kernel instead of the
                                   asynchronous-copy pipeline (same results; for
                                   comparisons) */
} facetcu_batch_config;
#define FACETCU_BATCH_TIME_SWEEPS 1u
#define FACETCU_BATCH_LEGACY_STEP 2u
typedef struct {
    uint32_t iterations;        /* sweeps of the slowest panel */
    uint32_t residual_corrections;
    uint32_t converged;         /* 1 if every column met the tolerance */
    float max_relative_change;  /* worst column at exit */
    double seconds;             /* device time of the solve (CUDA events) */
    uint32_t kernel_launches;   /* kernels the solve launched */
    uint32_t sweeps;            /* sweep kernels run, summed over panels */
    double sweep_seconds;       /* summed time of the dominant sweep kernel (TIME_SWEEPS) */
    double sweep_bytes;         /* algorithmic HBM bytes of those sweeps */
    uint32_t timed_sweeps;      /* number of sweeps in sweep_seconds */
    uint32_t graph_launches;    /* replays of the captured step batch (CUDA graph); their
                                   kernels are counted in kernel_launches */
} facetcu_batch_result;
int facetcu_solve_batched(facetcu_context *ctx, const facetcu_batch_config *config,
                          const float *reflectance, const float *transmittance,
                          const float *emission, const float *sky, const float *beam,
                          const float *direct_geometry, const float *initial,
                          float *radiosity, facetcu_batch_result *result);
/* Same with every array already in device memory (pointers from
 * cudaMalloc or a framework allocator); runs on the context stream and
 * returns after the solve has finished. */
int facetcu_solve_batched_device(facetcu_context *ctx, const facetcu_batch_config *config,
                                 const float *reflectance, const float *transmittance,
                                 const float *emission, const float *sky, const float *beam,
                                 const float *direct_geometry, const float *initial,
                                 float *radiosity, facetcu_batch_result *result);

/* Autotuning of the batched solve: times the candidate panel widths (32, 64
 * and 128 columns, those not wider than the columns; 32 in FP64) and, for
 * the widths whose MIXED int8 step runs on the pipelined kernel (64 and
 * 128), that kernel's CTAs per SM (as many as fit, 2 or 1) on short solves
 * (6 sweeps of every panel) of the given inputs (device pointers, as
 * facetcu_solve_batched_device; `radiosity` is scratch here) and keeps the
 * fastest for this GPU, graph size, column count and precision: later
 * batched solves with panel_width = 0 use it (the results do not depend on
 * the choice, only the time).  *panel_width receives the width.  cache_path
 * (may be NULL) names a JSON-lines file the choices are read from first and
 * written back to; a cached choice returns without timing.  No counterpart
 * in the reference. */
int facetcu_autotune_batched(facetcu_context *ctx, const facetcu_batch_config *config,
                             const float *reflectance, const float *transmittance,
                             const float *emission, const float *sky, const float *beam,
                             const float *direct_geometry, float *radiosity,
                             const char *cache_path, uint32_t *panel_width);

/* ---- learned warm start (no counterpart in the reference) --------------- */
/* MLP 12 -> 128 -> 128 -> 64 with GELU, BF16 weights (FP32 master copy,
 * FP32 accumulation), trained by the library's own forward, backward and
 * Adam kernels.  Per sun and side its 12 inputs are the first-order
 * radiosity (one sweep from B = 0) of bands 0, 9, ..., 63 divided by
 * sky_b + beam_b, the reflectance and transmittance of band 32, the
 * sky-view fraction sky_s / denom_s and the y (up) component of the side
 * normal; its 64 outputs predict (B_b - B1_b) / (sky_b + beam_b), the
 * multiple-scattering part of every band.  FACETCU_WARM_MLP starts the
 * batched solve from B1 + prediction; the iteration then runs to the same
 * tolerance as without it, so the network only changes the sweep count.
 * Parameters: 26,432 floats, W1[128x12], b1[128], W2[128x128], b2[128],
 * W3[64x128], b3[64] (row-major, [out][in]). */
typedef struct {
    uint32_t steps;
    uint32_t batch;
    float learning_rate;
    uint32_t seed;
} facetcu_mlp_train_config;
int facetcu_mlp_parameter_count(uint32_t *count);
int facetcu_mlp_reset(facetcu_context *ctx, uint32_t seed);
int facetcu_mlp_get_parameters(facetcu_context *ctx, float *parameters);
int facetcu_mlp_set_parameters(facetcu_context *ctx, const float *parameters);
/* Forward pass of n samples (host arrays): x[n * 12] -> y[n * 64]. */
int facetcu_mlp_forward(facetcu_context *ctx, const float *x, uint32_t n, float *y);
/* The same forward pass on the tensor cores (no reference counterpart; the
 * inference the learned warm start runs): each layer is 128-row tiles of
 * tcgen05.mma (BF16 operands staged by TMA, FP32 accumulation in tensor
 * memory) with the bias and GELU applied when the accumulator is read back;
 * hidden activations are BF16, so outputs differ from facetcu_mlp_forward by
 * a BF16 rounding per layer (about 1e-2 of the output scale).
 * FACETCU_DEVICE_TIMEOUT if a kernel's bounded wait ran out. */
int facetcu_mlp_forward_tensor(facetcu_context *ctx, const float *x, uint32_t n, float *y);
/* Mean-squared loss over n x 64 outputs and its FP32 gradient with respect
 * to the parameters (same order), for x[n * 12] and target[n * 64];
 * n <= 2^21 (FACETCU_OVERFLOW_ERROR above). */
int facetcu_mlp_loss_and_gradient(facetcu_context *ctx, const float *x, const float *target,
                                  uint32_t n, float *loss, float *gradient);
/* Adam training on n device-resident samples (x[n * 12], target[n * 64]):
 * `steps` minibatches of `batch` rows (<= 2^21) drawn with replacement
 * (counter-based hash of seed, step, row). */
int facetcu_mlp_train_device(facetcu_context *ctx, const float *x, const float *target,
                             uint64_t n, const facetcu_mlp_train_config *config,
                             float *final_loss);
/* Training samples of the current graph and a 64-band batch problem (device
 * pointers as in facetcu_solve_batched_device, converged radiosity
 * [R][S]): features[(k * S + s) * 12], targets[(k * S + s) * 64]. */
int facetcu_mlp_samples_device(facetcu_context *ctx, const facetcu_batch_config *config,
                               const float *reflectance, const float *transmittance,
                               const float *emission, const float *sky, const float *beam,
                               const float *direct_geometry, const float *converged,
                               float *features, float *targets);

/* ---- allocation-free solve (no counterpart in the reference) ------------- */
/* facetcu_solve without any device allocation, for callers that cannot
 * allocate GPU memory themselves or through us: host frameworks and plugin
 * hosts that own the whole device-memory budget and hand it out from their
 * own pool, and latency-critical loops that must not pay the implicit device
 * synchronisation of cudaMalloc/cudaFree.  The caller passes the graph,
 * optics and output in memory the current device can read and write;
 * the sweep's working memory (one radiosity buffer and the per-sweep max|dB|
 * slots) is a fixed array compiled into the library, about 4.2 MB per GPU
 * that loads it, kept until the process exits.
 *   row_offsets[surface_count + 1], edges[row_offsets[surface_count]],
 *   denominators[surface_count], sky_counts[surface_count], optics and
 *   radiosity[surface_count]: device-accessible; surface_count even,
 *   <= FACETCU_NOALLOC_MAX_SURFACES (else FACETCU_OVERFLOW_ERROR);
 *   1 <= iterations <= FACETCU_NOALLOC_MAX_ITERATIONS.
 * Semantics are those of facetcu_solve (B starts at 0, `iterations`
 * sweeps); the result is written to `radiosity`.  Work is queued on
 * `stream` (a cudaStream_t; NULL = the default stream) of the current
 * device; when max_delta is non-NULL the call waits for the stream and
 * stores the last sweep's max|dB| (max_delta must then be NULL while
 * `stream` is being captured into a graph: FACETCU_INVALID_ARGUMENT),
 * otherwise it returns once the work is queued.  Every call looks up the
 * array's device address (cudaGetSymbolAddress) in the current device's
 * context, so a context reset between calls is harmless.  All calls share
 * the one array: calls whose work overlaps on a GPU (other threads or
 * streams) race and must be serialised by the caller.  Inputs are not read
 * back for validation. */
#define FACETCU_NOALLOC_MAX_SURFACES 1048576u
#define FACETCU_NOALLOC_MAX_ITERATIONS 4096u
int facetcu_solve_noalloc(const uint32_t *row_offsets, const facetcu_csr_edge *edges,
                          const uint32_t *denominators, const uint32_t *sky_counts,
                          uint32_t surface_count, const facetcu_surface_optics *optics,
                          float sky_radiosity, uint32_t iterations, float relaxation,
                          float *radiosity, float *max_delta, void *stream);

/* ---- scene batches ------------------------------------------------------ */
/* Makes ctx's geometry and graph the disjoint union of `scene_count` other
 * contexts, each with a built graph (raster or hemisphere), so that one
 * batched solve (one launch per sweep) covers scenes of uneven size:
 * scene i's sides are [side_offsets[i], side_offsets[i+1]) of the union and
 * its graph block is copied with its neighbour indices offset (no
 * cross-scene edges).  Scene i's vertices are translated into their own cell
 * of a grid (only the solver's Morton renumbering sees positions).  Per-side
 * arrays for the union are the scenes' arrays concatenated in that order.
 * side_offsets holds scene_count + 1 entries; diagnostics may be NULL.  No
 * counterpart in the reference (it solves one scene per run). */
int facetcu_scene_batch(facetcu_context *ctx, facetcu_context *const *scenes,
                        uint32_t scene_count, uint32_t *side_offsets,
                        facetcu_graph_diagnostics *diagnostics);

/* ---- scene files, optics and the eFacetRT process flow ------------------ */
/* Scene facts loadTreeWithSoil returns (Scene, facetrtcore.cpp:148-166). */
typedef struct {
    uint32_t facet_count;
    uint32_t leaf_facet_count; /* facets [0, leaf) are the object, the rest ground */
    float minimum[3];
    float maximum[3];
} facetcu_scene_info;
/* loadTreeWithSoil (facetrtcore.cpp:361-473): OBJ positions and faces (fan
 * triangulated, degenerate triangles dropped), Y shifted so the lowest
 * vertex is at 0, and a 48 x 48 soil grid at y = -0.01 reaching half the
 * object's extent beyond it, unless an `o STREAMSIM_TERRAIN` block marks the
 * ground.  Host only, no GPU.  Call with vertices = material_indices = NULL
 * for `info`, then with arrays for capacity_facets >= info.facet_count facets
 * (3 vertices, one material index per facet: 0 object, 1 ground).  Errors
 * (FACETCU_RUNTIME_ERROR with the reference's message) are read with
 * facetcu_host_last_error(). */
int facetcu_load_tree_with_soil(const char *path, facetcu_vertex *vertices,
                                uint32_t *material_indices, uint32_t capacity_facets,
                                facetcu_scene_info *info);
/* makeOptics (facetrtcore.cpp:500-522): rho 0.10 / 0.20, tau 0.05 / 0 for
 * object / ground sides, D = sunlit * max(0, n_side . sun) * 700.  Host only. */
int facetcu_make_optics(const facetcu_vertex *vertices, uint32_t facet_count,
                        uint32_t leaf_facet_count, const float *sunlit,
                        const facetcu_direction *sun, facetcu_surface_optics *optics);
/* planckRadiance (facetrtcore.cpp:524-536): W m-2 sr-1 um-1; wavelength in
 * nm when above 50, else in um; evaluated in double. */
float facetcu_planck_radiance(float wavelength, float temperature);
/* The message of the last failing host-only call on this thread. */
const char *facetcu_host_last_error(void);
/* runFacetRTCore (facetrtcore.h:5-7, facetrtcore.cpp:3116-3161) for an OBJ
 * scene: loadTreeWithSoil, the runGpu sequence (:1621-1780) on this library
 * (40-direction graph at 1024 x 1024, sun raster at 30/135 deg, makeOptics,
 * 64-sweep solve, diffuse solve, lightEnhancement) and writeWebResult
 * (:1782-1840).  Prints `PROGRESS\t<int>\t<text>` lines and
 * `RESULT\t<path>` to stdout; on failure `facetrt: <message>` to stderr and
 * returns 1 (0 on success).  output_file NULL or "" writes facetrt.json next
 * to the input.  shader_directory is accepted and unused.  An XML project
 * (Input.xml) runs loadProjectScene's scene and the spectral band loop of
 * runGpu (facetcu_project_load, facetcu_solve_bands); a project.json
 * through its XML view. */
int facetcu_run_facetrt_core(const char *input_path, const char *shader_directory,
                             const char *output_file);

/* ---- spectral optics and the band loop ----------------------------------- */
/* SurfaceParameters (facetrtcore.cpp:106-138): the fields the optics read. */
typedef struct {
    const float *reflectance;   /* per band; the last value repeats (bandValue :538-544) */
    uint32_t reflectance_count; /* 0: 0.10 for object facets, 0.20 for ground */
    const float *transmittance;
    uint32_t transmittance_count; /* 0: 0.05 object, 0 ground */
    float tir_reflectance;
    float tir_transmittance;
    float sunlit_temperature; /* K */
    float shaded_temperature; /* K */
} facetcu_surface_parameters;
/* FacetRTParameters (facetrtcore.cpp:140-146) and the Scene fields
 * makeSpectralOptics reads (:148-166). */
typedef struct {
    const float *wavelengths; /* nm; a band is optical when <= 2500 nm (values <= 2.5 are um) */
    uint32_t band_count;
    facetcu_surface_parameters object; /* for object facets without a material */
    facetcu_surface_parameters ground; /* for ground facets without a material */
    const facetcu_surface_parameters *materials; /* Scene::materials */
    uint32_t material_count;
    const uint32_t *material_indices; /* per facet, or NULL */
    const float *texture_factors;     /* per facet reflectance factor, or NULL (1) */
    uint32_t leaf_facet_count;
    float background_angular_strength; /* Hapke blend of ground sides, [0, 1] */
    float sky_temperature;             /* K, sky radiance of thermal bands */
    uint32_t accelerated_solver;       /* FacetRTParameters::acceleratedSolver */
} facetcu_spectral_parameters;
/* makeSpectralOptics (facetrtcore.cpp:1057-1126) for one band on the
 * context's geometry; sunlit[2F] and optics[2F] are host arrays. */
int facetcu_spectral_optics(facetcu_context *ctx, const facetcu_spectral_parameters *parameters,
                            const float *sunlit, const facetcu_direction *sun, uint32_t band,
                            facetcu_surface_optics *optics);
typedef struct {
    uint32_t iterations;    /* band 0's SolveResult::iterations */
    float max_delta;        /* band 0's SolveResult::maxDelta */
    uint32_t thermal_bands; /* bands that are not optical */
    uint32_t batched_sweeps; /* sweeps of the batched solve of bands 1.. */
    double seconds;
} facetcu_band_result;
/* The spectral band loop of runGpu (facetrtcore.cpp:1677-1773) on the
 * context's graph: optics of every band on the device, band 0 through the
 * reference-semantics solver (64 sweeps, or solveAccelerated's rule when
 * accelerated_solver), bands 1.. in one batched FP32 solve (64 sweeps; to a
 * max relative change of 1e-6 when accelerated_solver, with no band-to-band
 * warm start), optical bands converted to apparent reflectance
 * clamp(B / (700 max(0, sun.y) + 50), 0, 1), and lightEnhancement from a
 * direct-free solve of band 0 when it is optical (else zeros).
 * band_radiosity[band_count][2F] and light_enhancement[2F] are host arrays. */
int facetcu_solve_bands(facetcu_context *ctx, const facetcu_spectral_parameters *parameters,
                        const float *sunlit, const facetcu_direction *sun, float *band_radiosity,
                        float *light_enhancement, facetcu_band_result *result);

/* ---- FacetEB: the coupled radiation / energy-balance node ---------------- */
/* The shortwave spectrum of a FacetEB run (ShortwaveSpectrum and
 * loadShortwaveSpectrum, facetrtcore.cpp:2458-2541): direct and diffuse
 * samples per 1 nm from 400 nm, per micrometre.  Fewer than 2 samples (or
 * a non-positive integral) select the reference's flat fallback of 2001
 * samples, 0.5 * direct_fraction and 0.5 * (1 - direct_fraction); otherwise
 * both are scaled so that their summed trapezoid integral is one. */
typedef struct {
    const float *direct;
    const float *diffuse;
    uint32_t sample_count;   /* min of the two lengths */
    float direct_fraction;   /* directScatteringRatio, clamped to [0, 1] */
    uint32_t window_width;   /* spectralAccelerationWidth, samples per window (1..1000) */
} facetcu_shortwave_spectrum;
/* One spectral-acceleration window (runFacetEBCore :3499-3536): solved with
 * the optics of sample `energy_band` (the window centre). */
typedef struct {
    float direct_normal; /* W m^-2 of the window's direct beam, normal to the sun */
    float diffuse;       /* W m^-2 of the window's sky radiosity */
    uint32_t energy_band;
} facetcu_shortwave_window;
/* The windows of one node (total_shortwave W m^-2 on the horizontal,
 * cos_zenith = max(0, sun.y)), skipping windows with no energy as the
 * reference does, and for each of band_count wavelengths the spectral
 * direct and diffuse irradiance total_shortwave * spectrum(lambda) * 0.001
 * (band_direct / band_diffuse may be NULL).  Host only; *window_count is
 * set even when capacity is too small (then FACETCU_OVERFLOW_ERROR). */
int facetcu_shortwave_windows(const facetcu_shortwave_spectrum *spectrum, float total_shortwave,
                              float cos_zenith, const float *wavelengths, uint32_t band_count,
                              facetcu_shortwave_window *windows, uint32_t capacity,
                              uint32_t *window_count, float *band_direct, float *band_diffuse);

/* The energy-balance fields of SurfaceParameters (facetrtcore.cpp:113-138);
 * facetcu_energy_surface_defaults() fills the reference's defaults. */
typedef struct {
    facetcu_surface_parameters optics;     /* band values, TIR reflectance/transmittance */
    const float *energy_reflectance;       /* per shortwave sample; empty: the Planck(5778 K)- */
    uint32_t energy_reflectance_count;     /*   weighted mean of optics.reflectance */
    const float *energy_transmittance;
    uint32_t energy_transmittance_count;
    float surface_resistance;      /* s m^-1 */
    float specific_heat;           /* J kg^-1 K^-1 */
    float density;                 /* kg m^-3 */
    float thermal_conductivity;    /* W m^-1 K^-1 */
    float soil_moisture;           /* below 0.03: dry soil, no latent heat */
    float heat_capacity_per_area;  /* J m^-2 K^-1 of object facets */
    int32_t soil_temperature_method; /* 0: storage = 0.35 Rn; 1: force-restore; 2: 1.5 x force-restore */
    uint32_t photovoltaic;
    uint32_t vegetation;
    float pv_eta25, pv_gamma, pv_bifaciality;
    float convective_scale;
} facetcu_energy_surface;
void facetcu_energy_surface_defaults(facetcu_energy_surface *surface);

/* runFacetEBCore's settings (facetrtcore.cpp:3196-3233) and scene fields.
 * Facets without a material take the reference's fixed fallbacks
 * (surfaceForFacet :607-620): SurfaceParameters{} for objects, reflectance
 * 0.20 / transmittance 0 / TIR 0.05 for the ground. */
typedef struct {
    const facetcu_energy_surface *materials; /* Scene::materials */
    uint32_t material_count;
    const uint32_t *material_indices; /* per facet, or NULL */
    const float *texture_factors;     /* per facet reflectance factor, or NULL (1) */
    uint32_t leaf_facet_count;
    float background_angular_strength;
    const float *wavelengths;         /* sensor bands of the node output, may be 0 */
    uint32_t band_count;
    float sky_temperature;            /* K, clamped by the caller to [150, 350] */
    float time_step;                  /* dTime, s (>= 1) */
    uint32_t coupling_iterations;     /* 1..100 */
    float temperature_tolerance;      /* K */
    float temperature_relaxation;     /* 0.05..1 */
    int32_t vegetation_temperature_method; /* 0 Ball-Berry, 1 Farquhar */
    uint32_t solver_iterations;       /* Jacobi sweeps per solve: 64 = kIterations */
    float solver_tolerance;           /* 0: every solve runs solver_iterations sweeps from
                                         zero, as the reference; > 0: stop on the per-side
                                         rule and start each longwave solve from the last */
    uint32_t precision;               /* FACETCU_PRECISION_FP32 or _MIXED (needs solver_tolerance > 0) */
} facetcu_energy_parameters;
/* One meteorological row (MeteoStep :3172-3181). */
typedef struct {
    float air_temperature;   /* deg C */
    float vapor_pressure;    /* hPa */
    float pressure;          /* hPa */
    float wind_speed;        /* m s^-1 */
    float shortwave;         /* W m^-2 */
    float longwave;          /* W m^-2; <= 0: sigma T_sky^4 */
} facetcu_meteo;
/* Per-side fields of a node (host arrays of 2F floats; NULL = not wanted,
 * except temperature). */
typedef struct {
    float *temperature;        /* in: the state at the node start; out: the solved state */
    float *radiosity;          /* shortwave + final longwave (combineRadiativeSolutions) */
    float *shortwave_radiosity;
    float *diffuse_radiosity;  /* shortwave without direct light */
    float *longwave_radiosity;
    float *absorbed_shortwave;
    float *incident_shortwave;
    float *net_radiation;
    float *sensible_heat;
    float *latent_heat;
    float *storage_heat;
    float *photovoltaic_power;
    float *band_output;        /* [band_count][2F]: apparent reflectance (optical), radiance */
} facetcu_energy_fields;
typedef struct {
    uint32_t coupling_iterations;
    uint32_t converged;
    float max_temperature_delta;           /* K */
    float max_energy_residual;             /* W m^-2 */
    float max_energy_residual_equivalent;  /* K */
    uint32_t shortwave_sweeps;             /* of the window solve */
    uint32_t longwave_sweeps;              /* summed over the coupling solves */
    uint32_t band_sweeps;
    uint32_t solves;                       /* radiosity solves the reference would run */
    uint32_t kernel_launches;              /* kernels the node launched */
    double seconds;
} facetcu_energy_result;
/* One FacetEB time node (runFacetEBCore :3462-3908) on the context's graph:
 * every shortwave window solved with and without its direct beam as one
 * batched solve, incident and absorbed shortwave accumulated in window order,
 * then up to coupling_iterations rounds of longwave optics from the
 * temperatures, a longwave solve, incident longwave, the per-facet energy
 * fluxes (net radiation, sensible, latent, storage, PV), the residual and
 * the relaxed Newton temperature update, all on the device; a final
 * longwave solve and flux evaluation; and the sensor bands (spectral optics
 * of the solved state, one batched solve, apparent reflectance).  sunlit is
 * the node's sun raster (2F floats), sun its direction.  Returns
 * FACETCU_RUNTIME_ERROR "FacetEB energy residual is not finite" as the
 * reference throws. */
int facetcu_faceteb_node(facetcu_context *ctx, const facetcu_energy_parameters *parameters,
                         const facetcu_meteo *meteo, const facetcu_direction *sun,
                         const float *sunlit, const facetcu_shortwave_window *windows,
                         uint32_t window_count, const float *band_direct,
                         const float *band_diffuse, facetcu_energy_fields *fields,
                         facetcu_energy_result *result);

/* The sun of a FacetEB node.  The reference calls NREL's SPA (the vendored
 * thirdparty/spa.h, SPA_ZA) from updateSolarPosition
 * (facetrtcore.cpp:3290-3327); here the sun's coordinates follow Meeus's
 * published formulas (about 0.01 deg from SPA) with SPA's input ranges,
 * error codes and refraction.  facetcu_solar_input holds spa_data's inputs
 * (spa.h: local time, hours east of UTC, degrees east/north, metres,
 * millibars, degrees Celsius, delta_t in seconds).  zenith and azimuth
 * (eastward from north) in degrees; *spa_error = SPA's error code (0, or
 * 1-16 with FACETCU_INVALID_ARGUMENT). */
typedef struct {
    int32_t year, month, day, hour, minute, second;
    double delta_t, timezone, longitude, latitude, elevation, pressure, temperature;
    double atmos_refract;
} facetcu_solar_input;
int facetcu_solar_position(const facetcu_solar_input *input, double *zenith, double *azimuth,
                           int32_t *spa_error);
/* updateSolarPosition on one meteorology row: day of year and local time
 * from julian_time (2019, UTC+8, whole minutes), the site's latitude and
 * longitude, the row's pressure (at least 100 mbar) and air temperature.
 * FACETCU_RUNTIME_ERROR "FacetEB solar-position calculation failed" as the
 * reference throws. */
int facetcu_faceteb_sun(float julian_time, float latitude, float longitude, float pressure,
                        float air_temperature, float *zenith, float *azimuth);

/* ---- sensor images (server.mjs:1127-1600, writeRadiosityTiffForAngle) ---- */
/* The sensor of a project: image size, parallel or perspective projection,
 * view angles, field of view, scene extent and sensor position.  Values
 * that the reference reads as "not a number" take its defaults: pass NaN
 * (position) or 0 (fov: 60, scene_x/scene_y: 1, sky_temperature: 250). */
typedef struct {
    uint32_t width, height;     /* sensor.x, sensor.y */
    uint32_t perspective;       /* projection perspective / central / center */
    double view_zenith;         /* vza, degrees */
    double view_azimuth;        /* vaa, degrees clockwise from +X (north) toward +Z (east) */
    double fov;                 /* vertical field of view (perspective), clamped to [0.1, 120] */
    double scene_x, scene_y;    /* scene extent along x (north) and z (east), m */
    double position[3];         /* positionX, positionY, height (m); any NaN: centre at 3000 m */
    double sky_temperature;     /* K (max 120) for the thermal sky of perspective views */
    uint32_t temperature_output; /* the values are temperatures (a FacetEB temperature image) */
} facetcu_sensor;
typedef struct {
    uint32_t observed_pixels;   /* pixels of the observed (oblique) raster that see a facet */
    uint32_t output_pixels;     /* pixels of the output image that see a facet */
    double naming_zenith;       /* the view angles the output file is named by */
    double naming_azimuth;
} facetcu_image_info;
/* Renders band_count images of per-side values (values[band][2F], host)
 * seen by the sensor, on the context's geometry: the observed side of each
 * facet, a z-buffered raster of side indices (barycentric test at pixel
 * centres in double precision, the nearest depth wins and the first facet
 * among equal depths), for a parallel sensor the nadir remap of that oblique
 * raster onto the scene's ground grid, and for a perspective sensor the
 * analytic sky where a pixel's ray looks up (wavelengths[band] in nm or um;
 * the atmosphere table of the reference is not applied).  image[band][H][W]
 * (float, NaN where nothing is seen) and side_index[H][W] (int32, -1; may be
 * NULL) are host arrays. */
int facetcu_render_sensor_image(facetcu_context *ctx, const facetcu_sensor *sensor,
                                const float *values, uint32_t band_count,
                                const float *wavelengths, float *image, int32_t *side_index,
                                facetcu_image_info *info);

/* ---- XML projects (scene and material ingestion) ------------------------ */
/* A HiStream XML project (the reference's Input.xml) read as
 * loadProjectScene and facetRTParametersFromInput do
 * (facetrtcore.cpp:2038-3025): objects from OBJ files (groups bound to
 * materials by mesh name) or cubes, placed from position files (x y z
 * [scale [rotation]]) and clipped to the scene domain, then a flat ground
 * grid, raised by the project's DEM (facetcu_dem_height_field) under the
 * ground and every placement; materials from custom, file, PROSPECT and BSM
 * spectra (the models' optipar.txt beside the sun spectrum), thermal blocks,
 * soil sets and surface-energy blocks, physical reflectance textures (ESRI
 * ASCII grids, baseline GeoTIFF and PNG).  A project.json is read through
 * its XML view (facetcu_project_xml_view).  Host only; errors through
 * facetcu_host_last_error(). */
typedef struct facetcu_project facetcu_project;
typedef struct {
    uint32_t facet_count;
    uint32_t leaf_facet_count;      /* object facets come first, the ground last */
    uint32_t material_count;        /* Scene::materials (the ground's is the last) */
    uint32_t band_count;
    float sun_zenith, sun_azimuth;  /* degrees */
    uint32_t periodic_neighbor_count;
    float periodic_size_x, periodic_size_z;
    uint32_t raster_size, raster_layers;
    float background_angular_strength;
    float minimum[3], maximum[3];
    float sky_temperature;
    uint32_t accelerated_solver;
} facetcu_project_info;
int facetcu_project_load(const char *path, facetcu_project **project);
void facetcu_project_release(facetcu_project *project);
int facetcu_project_get_info(const facetcu_project *project, facetcu_project_info *info);
/* vertices[3F], material_indices[F], texture_factors[F] (any may be NULL) */
int facetcu_project_get_geometry(const facetcu_project *project, facetcu_vertex *vertices,
                                 uint32_t *material_indices, float *texture_factors);
/* material index < material_count, or material_count for the parameters'
 * object surface and material_count + 1 for the ground; the pointers stay
 * valid while the project lives.  output_component: 0 unknown, 1 soil,
 * 2 vegetation, 3 building, 4 PV, 5 water. */
int facetcu_project_get_material(const facetcu_project *project, uint32_t index,
                                 facetcu_energy_surface *surface, uint32_t *output_component);
/* The XML view of a project.json (facetInputView, facetrtcore.cpp:1888-2036,
 * over projectjson.cpp's accessors): the form facetcu_project_load reads a
 * project.json in.  Files are resolved against the project's folder, the
 * runtime "defined" folder (sun spectra, optipar.txt) is ./defined.
 * *length = the view's length; buffer (capacity bytes, NUL-terminated) may
 * be NULL to ask for the length. */
int facetcu_project_xml_view(const char *path, char *buffer, uint64_t capacity,
                             uint64_t *length);
/* A DEM height field as readDemHeightField makes it (facetrtcore.cpp:
 * 2618-2697, which reads band 1 with GDAL): values[height][width] in
 * metres, rows from north to south, nodata and non-finite cells set to
 * *minimum, the minimum of the valid cells.  Reads ESRI ASCII grids and
 * baseline GeoTIFF (classic or BigTIFF, strips or tiles, no compression,
 * LZW, deflate or PackBits, predictors 1-3, integer or IEEE samples, the
 * GDAL_NODATA tag).  values may be NULL to ask for the size; capacity is
 * its length in floats.  FACETCU_RUNTIME_ERROR with the reference's
 * messages ("Cannot open DEM: ", "Cannot read DEM elevations: ", "DEM must
 * contain at least 2 x 2 cells: ", "DEM contains no valid elevations: "). */
int facetcu_dem_height_field(const char *path, int32_t *width, int32_t *height, float *minimum,
                             float *values, uint64_t capacity);
/* The project's FacetRTParameters and scene fields as spectral parameters
 * for facetcu_spectral_optics / facetcu_solve_bands. */
int facetcu_project_spectral_parameters(const facetcu_project *project,
                                        facetcu_spectral_parameters *parameters);

#ifdef __cplusplus
}
#endif
#endif /* FACETCU_H */
