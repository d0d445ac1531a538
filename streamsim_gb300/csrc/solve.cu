// solve.cu — the reference's single-RHS Jacobi sweep and incident irradiance.
//
// k_jacobi_plain is the "plain FP32 GPU solver": the sweep of the
// reference's radiosity.comp:49-106 (FacetrtVulkan::solve), one thread per
// facet updating both sides, FP32 gather over the count-form CSR in row
// order, mix() relaxation, max|dB| as an atomicMax over float bits.  It is
// kept literal on purpose: it is the baseline the batched solver is
// measured against, and the solver behind facetcu_solve/_accelerated.
#include "internal.h"

namespace facetcu {
namespace {

__device__ __forceinline__ float incoming(uint32_t s, const uint32_t* rows,
                                          const facetcu_csr_edge* edges, const uint32_t* denom,
                                          const uint32_t* skyc, float sky, const float* B)
{
    const uint32_t d = denom[s];
    if (d == 0u) return sky;
    float v = float(skyc[s]) * sky;
    for (uint32_t e = rows[s]; e < rows[s + 1]; ++e) {
        const facetcu_csr_edge ed = edges[e];
        v += float(ed.count) * B[ed.neighbor];
    }
    return v / float(d);
}

__global__ void __launch_bounds__(64) k_jacobi_plain(
    uint32_t facets, const uint32_t* rows, const facetcu_csr_edge* edges, const uint32_t* denom,
    const uint32_t* skyc, const facetcu_surface_optics* optics, float sky, float relax,
    const float* Bin, float* Bout, uint32_t* max_delta_bits)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= facets) return;
    const uint32_t s0 = 2u * f, s1 = s0 + 1u;
    const facetcu_surface_optics o0 = optics[s0], o1 = optics[s1];
    const float h0 = incoming(s0, rows, edges, denom, skyc, sky, Bin) + o0.direct_irradiance;
    const float h1 = incoming(s1, rows, edges, denom, skyc, sky, Bin) + o1.direct_irradiance;
    const float t0 = o0.emission + o0.reflectance * h0 + o0.transmittance * h1;
    const float t1 = o1.emission + o1.reflectance * h1 + o1.transmittance * h0;
    const float old0 = Bin[s0], old1 = Bin[s1];
    // GLSL mix(x, y, a) = x * (1 - a) + y * a
    const float n0 = old0 * (1.0f - relax) + t0 * relax;
    const float n1 = old1 * (1.0f - relax) + t1 * relax;
    Bout[s0] = n0;
    Bout[s1] = n1;
    const float delta = fmaxf(fabsf(n0 - old0), fabsf(n1 - old1));
    atomicMax(max_delta_bits, __float_as_uint(delta));
}

// FacetrtVulkan::incidentIrradiance / incidentIrradianceCpu
// (facetrt_vulkan.cpp:1360-1399, facetrtcore.cpp:1531-1559): FP64 gather.
__global__ void __launch_bounds__(128) k_incident(
    uint32_t surfaces, const uint32_t* rows, const facetcu_csr_edge* edges, const uint32_t* denom,
    const uint32_t* skyc, const facetcu_surface_optics* optics, float sky, const float* B,
    float* out)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= surfaces) return;
    double diffuse = sky;
    const uint32_t d = denom[s];
    if (d != 0u) {
        diffuse = double(skyc[s]) * double(sky);
        for (uint32_t e = rows[s]; e < rows[s + 1]; ++e) {
            const facetcu_csr_edge ed = edges[e];
            diffuse += double(ed.count) * double(B[ed.neighbor]);
        }
        diffuse /= double(d);
    }
    out[s] = fmaxf(0.0f, float(diffuse) + optics[s].direct_irradiance);
}

}  // namespace

void jacobi_plain_sweep(const DeviceGraph& g, const facetcu_surface_optics* d_optics, float sky,
                        float relaxation, const float* d_in, float* d_out,
                        uint32_t* d_max_delta_bits, cudaStream_t s)
{
    const uint32_t facets = g.surfaces / 2u;
    if (!facets) return;
    k_jacobi_plain<<<(facets + 63) / 64, 64, 0, s>>>(
        facets, g.row_offsets.as<uint32_t>(), g.edges.as<facetcu_csr_edge>(),
        g.denominators.as<uint32_t>(), g.sky.as<uint32_t>(), d_optics, sky, relaxation, d_in,
        d_out, d_max_delta_bits);
    FCU_LAUNCH("k_jacobi_plain");
}

void jacobi_plain_sweep_raw(uint32_t surfaces, const uint32_t* rows, const facetcu_csr_edge* edges,
                            const uint32_t* denom, const uint32_t* skyc,
                            const facetcu_surface_optics* d_optics, float sky, float relaxation,
                            const float* d_in, float* d_out, uint32_t* d_max_delta_bits,
                            cudaStream_t s)
{
    const uint32_t facets = surfaces / 2u;
    if (!facets) return;
    k_jacobi_plain<<<(facets + 63) / 64, 64, 0, s>>>(facets, rows, edges, denom, skyc, d_optics,
                                                      sky, relaxation, d_in, d_out,
                                                      d_max_delta_bits);
    FCU_LAUNCH("k_jacobi_plain");
}

void incident_irradiance(const DeviceGraph& g, const facetcu_surface_optics* d_optics, float sky,
                         const float* d_radiosity, float* d_out, cudaStream_t s)
{
    if (!g.surfaces) return;
    k_incident<<<(g.surfaces + 127) / 128, 128, 0, s>>>(
        g.surfaces, g.row_offsets.as<uint32_t>(), g.edges.as<facetcu_csr_edge>(),
        g.denominators.as<uint32_t>(), g.sky.as<uint32_t>(), d_optics, sky, d_radiosity, d_out);
    FCU_LAUNCH("k_incident");
}

}  // namespace facetcu
