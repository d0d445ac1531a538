/*
 * facet_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the FacetRT facet-radiosity path of StreamSim's HiStream
 * engine (models/histream/src/facetrt/facetrtcore.cpp).  It is the checker
 * for the CUDA library: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg may call it.  Nothing in the product links it.
 *
 * Floating-point expressions are written in the same order as the reference
 * and the file is compiled with -ffp-contract=off, so that every float
 * result (projected vertices, edge functions, depths) is the IEEE-rounded
 * value the reference's own CPU backend computes on x86-64.
 *
 * Parity pin: the raster graph, sunlit fraction and Jacobi solve are checked
 * against (1) the reference's CPU functions compiled in place by
 * oracle/build_ref.py and (2) the radiosity/sunlit vectors the reference
 * shipped in validation/<scene>/output/radiosity_gpu.json (tests/golden/).
 */
#ifndef FACET_ORACLE_H
#define FACET_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float position[3]; float normal[3]; } orc_vertex;
typedef struct { float x, y, z; } orc_direction;
typedef struct { float reflectance, transmittance, emission, direct; } orc_optics;

/* Count-form visibility graph over oriented sides (side 2f = geometric
 * normal side, 2f+1 = opposite side).  Rows are sorted by neighbour. */
typedef struct {
    uint32_t surface_count;
    uint64_t nnz;
    uint32_t *row_offsets;   /* surface_count + 1 */
    uint32_t *neighbors;     /* nnz */
    uint32_t *counts;        /* nnz */
    uint32_t *denominators;  /* surface_count */
    uint32_t *sky_counts;    /* surface_count */
    uint32_t fragment_overflow;
    uint32_t max_depth;      /* deepest fragment chain seen */
    float max_closure_error;
} orc_graph;

/* Raster configuration shared by the graph and sunlit passes. */
typedef struct {
    uint32_t raster_size;
    uint32_t layers;
    uint32_t periodic_count;
    float periodic_size_x;
    float periodic_size_z;
    float bounds_min[3];
    float bounds_max[3];
} orc_raster_config;

/* facetrtcore.cpp:475-489 */
void orc_hemisphere_directions(uint32_t count, orc_direction *out);
/* facetrtcore.cpp:491-498 */
orc_direction orc_sun_direction(float zenith_deg, float azimuth_deg);
/* facetrtcore.cpp:168-188 */
uint32_t orc_adaptive_layers(uint32_t facet_count, uint32_t periodic_count,
                             uint32_t raster_size, uint32_t base_layers);

/* facetrtcore.cpp:1348-1436 (buildCpuGraph).  Returns 0, or 1 when the
 * A-buffer overflowed (the reference throws "CPU A-buffer overflow"; the
 * graph is still filled so the diagnostic can be compared). */
int orc_build_graph(const orc_vertex *vertices, uint32_t facet_count,
                    const orc_raster_config *cfg,
                    const orc_direction *directions, uint32_t direction_count,
                    orc_graph *out);
void orc_free_graph(orc_graph *g);

/* facetrtcore.cpp:1438-1474 (computeCpuSunlit).  Returns 0 or 1 (overflow). */
int orc_sunlit(const orc_vertex *vertices, uint32_t facet_count,
               const orc_raster_config *cfg, orc_direction sun, float *fraction);

/* facetrtcore.cpp:1476-1529 (solveCpu): FP32 state, FP64 gather. */
float orc_solve(const orc_graph *g, const orc_optics *optics, float sky,
                uint32_t iterations, float relaxation, float *radiosity);
/* Same Jacobi sweep but with every quantity in double; used as the FP64
 * truth.  Iterates until max|dB| <= tol*max|B| or max_iterations. */
uint32_t orc_solve_f64(const orc_graph *g, const orc_optics *optics, double sky,
                       uint32_t max_iterations, double tol, double *radiosity);
/* facetrtcore.cpp:1531-1559 (incidentIrradianceCpu). */
void orc_incident(const orc_graph *g, const float *radiosity,
                  const orc_optics *optics, float sky, float *irradiance);
/* Energy closure of a converged count-form solution (weights = denom):
 * returns (lhs, rhs) of
 *   sum w D + sum sky L + sum w e = sum w (1 - rho - tau_opp) H + sum sky B. */
void orc_energy_closure(const orc_graph *g, const orc_optics *optics, double sky,
                        const double *radiosity, double *lhs, double *rhs);

/* facetrtcore.cpp:362-473 (loadTreeWithSoil).  Caller frees *vertices and
 * *materials with orc_free.  Returns 0 or a negative error code. */
int orc_load_tree_with_soil(const char *path, orc_vertex **vertices,
                            uint32_t **materials, uint32_t *facet_count,
                            uint32_t *leaf_facet_count,
                            float bounds_min[3], float bounds_max[3]);
/* facetrtcore.cpp:500-522 (makeOptics) with the constants exposed. */
void orc_make_optics(const orc_vertex *vertices, uint32_t facet_count,
                     uint32_t leaf_facet_count, const float *sunlit,
                     orc_direction sun, float beam, float leaf_rho,
                     float leaf_tau, float ground_rho, float ground_tau,
                     orc_optics *optics);

/* Hemisphere ray-cast view factors (the CUDA library's second visibility
 * mode; the reference has no counterpart).  Same sample tables, same
 * arithmetic and same tie rules as the device kernel, by brute force over
 * all facets.  Output rows are the top_k largest counts (ties: lower side
 * index first), denominators = kept + sky, sorted by neighbour. */
int orc_hemisphere_graph(const orc_vertex *vertices, uint32_t facet_count,
                         const float *sample_uv, const float *sample_dir,
                         uint32_t rays_per_side, uint32_t sets, uint32_t top_k,
                         orc_graph *out, uint64_t *dropped);
int orc_hemisphere_sunlit(const orc_vertex *vertices, uint32_t facet_count,
                          const float *sample_uv, uint32_t samples, uint32_t sets,
                          orc_direction sun, float *fraction);
/* The same with the scene's periodic copies (the raster mode's tiles,
 * facetrtcore.cpp:226-237): nearest hit over the scene and up to 20 copies
 * offset by (tx * size_x, tz * size_z); the origin facet is skipped in the
 * scene's own tile only. */
int orc_hemisphere_graph_periodic(const orc_vertex *vertices, uint32_t facet_count,
                                  const float *sample_uv, const float *sample_dir,
                                  uint32_t rays_per_side, uint32_t sets, uint32_t top_k,
                                  uint32_t periodic_count, float size_x, float size_z,
                                  orc_graph *out, uint64_t *dropped);
int orc_hemisphere_sunlit_periodic(const orc_vertex *vertices, uint32_t facet_count,
                                   const float *sample_uv, uint32_t samples, uint32_t sets,
                                   orc_direction sun, uint32_t periodic_count, float size_x,
                                   float size_z, float *fraction);

/* The same two results with a BVH over the facets and `threads` host
 * threads (0: every online core), for scenes where the brute force is too
 * slow.  Identical output: the BVH only skips facets whose widened box the
 * ray misses.  Return 0, or -1 when memory ran out. */
int orc_hemisphere_graph_bvh(const orc_vertex *vertices, uint32_t facet_count,
                             const float *sample_uv, const float *sample_dir,
                             uint32_t rays_per_side, uint32_t sets, uint32_t top_k,
                             uint32_t periodic_count, float size_x, float size_z,
                             uint32_t threads, orc_graph *out, uint64_t *dropped);
int orc_hemisphere_sunlit_bvh(const orc_vertex *vertices, uint32_t facet_count,
                              const float *sample_uv, uint32_t samples, uint32_t sets,
                              orc_direction sun, uint32_t periodic_count, float size_x,
                              float size_z, uint32_t threads, float *fraction);

/* Per-ray hits of the listed sides (side seen or 0xFFFFFFFF, distance or
 * -1), by brute force (use_bvh = 0) or the BVH (use_bvh = 1): the
 * diagnostic behind a graph difference. */
int orc_hemisphere_rays(const orc_vertex *vertices, uint32_t facet_count,
                        const float *sample_uv, const float *sample_dir, uint32_t rays_per_side,
                        uint32_t sets, const uint32_t *sides, uint32_t side_count, int use_bvh,
                        uint32_t *hit_side, float *hit_t);

void orc_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
