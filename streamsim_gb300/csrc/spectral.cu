// spectral.cu — makeSpectralOptics for every band at once, and the pieces of
// the runGpu band loop that run on the device.
//
// makeSpectralOptics (models/histream/src/facetrt/facetrtcore.cpp:1057-1126)
// evaluates, per band and side, the material's band value (bandValue,
// :538-544) times the facet's texture factor, the ground's Hapke angular
// reflectance (backgroundHapkeReflectance :565-587, facetHapkeKernel
// :552-563, facetHapkeH :546-550) or infrared emissivity
// (infraredHapkeEmissivity :589-605), and for thermal bands the emission
// eps * Planck of the sunlit/shaded temperature mix (:1112-1118).  Here one
// thread handles one (band, side) and writes the batched solver's band-major
// inputs rho[b][s], tau[b][s], emis[b][s]; the direct term stays factored as
// dgeo[s] = sunlit_s max(0, n_s . sun) times a per-band beam (700 for optical
// bands, 0 for thermal ones), the product the reference forms.
//
// Per-material, per-band scalars (band values with their object/ground
// fallbacks, Planck radiances in double) are tabulated on the host, so the
// kernel reads a small table and does the per-side float arithmetic in the
// reference's operation order.  This file is compiled with -fmad=false: the
// clamps, mixes and products round exactly as the reference's host code.
// The Hapke terms call CUDA's sqrtf/tanf/acosf/powf, whose results may
// differ from the C library's in the last place; with the reference's default
// angular strength 0 they cancel exactly and the optics are bit-identical.
#include <cmath>
#include <vector>

#include "internal.h"
#include "optics_math.cuh"

namespace facetcu {
namespace spectral {
namespace {

using namespace optics_math;

__global__ void k_spectral_optics(uint32_t F, uint32_t nb, uint32_t b0, uint32_t bcount,
                                  const facetcu_vertex* __restrict__ V,
                                  const uint32_t* __restrict__ material, uint32_t M,
                                  const float* __restrict__ texture, uint32_t leaf,
                                  const float4* __restrict__ table, const float2* __restrict__ tir,
                                  const uint8_t* __restrict__ thermal, float strength, F3 sun,
                                  const float* __restrict__ sunlit, float* __restrict__ rho,
                                  float* __restrict__ tau, float* __restrict__ emis)
{
    const size_t S = size_t(F) * 2;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= S * bcount) return;
    const uint32_t b = b0 + uint32_t(i / S);
    const uint32_t s = uint32_t(i % S), f = s >> 1;
    const bool object = f < leaf;
    const uint32_t mi = material ? material[f] : 0xffffffffu;
    const uint32_t slot = mi < M ? mi : (object ? M : M + 1);
    const float4 tb = table[(size_t(slot) * 2 + (object ? 1 : 0)) * nb + b];
    const float2 tt = tir[slot];
    const bool th = thermal[b] != 0;
    const float tex = (texture && !th) ? texture[f] : 1.0f;
    float r = sclamp((th ? tt.x : tb.x) * tex, 0.0f, 1.0f);
    const float t = sclamp(th ? tt.y : tb.y, 0.0f, 1.0f - r);
    const facetcu_vertex& v = V[3 * size_t(f)];
    const F3 side = mulf(F3{v.normal[0], v.normal[1], v.normal[2]}, (s & 1u) ? -1.0f : 1.0f);
    float eps = smax(0.0f, 1.0f - r - t);
    if (!object && th) {
        eps = ground_emissivity(eps, fabsf(side.y), strength);
        r = sclamp(1.0f - t - eps, 0.0f, 1.0f);
    } else if (!object) {
        r = ground_reflectance(r, sun, side, side, strength);
    }
    const size_t o = size_t(b - b0) * S + s;
    rho[o] = r;
    tau[o] = smin(t, 1.0f - r);
    float e = 0.0f;
    if (th) {
        const float lit = sclamp(sunlit[s], 0.0f, 1.0f);
        const float black = lit * tb.z + (1.0f - lit) * tb.w;
        e = eps * black;
    }
    emis[o] = e;
}

// dgeo[s] = sunlit_s * max(0, n_s . sun)
__global__ void k_direct_geometry(uint32_t F, const facetcu_vertex* __restrict__ V, F3 sun,
                                  const float* __restrict__ sunlit, float* __restrict__ dgeo)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 2 * F) return;
    const facetcu_vertex& v = V[3 * size_t(s >> 1)];
    const F3 side = mulf(F3{v.normal[0], v.normal[1], v.normal[2]}, (s & 1u) ? -1.0f : 1.0f);
    dgeo[s] = sunlit[s] * smax(0.0f, dotf(side, sun));
}

// One band's optics as the reference's array of structs.
__global__ void k_pack(size_t S, const float* rho, const float* tau, const float* emis,
                       const float* dgeo, float beam, facetcu_surface_optics* out)
{
    const size_t s = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= S) return;
    out[s] = {rho[s], tau[s], emis[s], dgeo[s] * beam};
}

// Apparent reflectance of optical bands: clamp(B / reference, 0, 1).
__global__ void k_apparent(float* B, size_t S, uint32_t bands, const uint8_t* optical, float ref)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= S * bands) return;
    if (!optical[i / S]) return;
    B[i] = sclamp(B[i] / ref, 0.0f, 1.0f);
}

inline unsigned blocks(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

float band_value(const float* v, uint32_t n, uint32_t band, float fallback)
{
    if (!v || n == 0) return fallback;
    return v[band < n ? band : n - 1];
}

}  // namespace

bool optical_wavelength(float wavelength)
{
    const float nm = wavelength <= 2.5f ? wavelength * 1000.0f : wavelength;
    return nm <= 2500.0f;
}

void Tables::build(const facetcu_spectral_parameters& p, cudaStream_t s)
{
    const uint32_t nb = p.band_count, M = p.material_count;
    std::vector<float4> tab(size_t(M + 2) * 2 * nb);
    std::vector<float2> tr(M + 2);
    std::vector<uint8_t> th(nb), opt(nb);
    auto surface = [&](uint32_t slot) -> const facetcu_surface_parameters& {
        return slot < M ? p.materials[slot] : (slot == M ? p.object : p.ground);
    };
    for (uint32_t slot = 0; slot < M + 2; ++slot) {
        const facetcu_surface_parameters& m = surface(slot);
        tr[slot] = make_float2(m.tir_reflectance, m.tir_transmittance);
        for (uint32_t obj = 0; obj < 2; ++obj)
            for (uint32_t b = 0; b < nb; ++b) {
                const float wl = p.wavelengths[b];
                tab[(size_t(slot) * 2 + obj) * nb + b] = make_float4(
                    band_value(m.reflectance, m.reflectance_count, b, obj ? 0.10f : 0.20f),
                    band_value(m.transmittance, m.transmittance_count, b, obj ? 0.05f : 0.0f),
                    facetcu_planck_radiance(wl, m.sunlit_temperature),
                    facetcu_planck_radiance(wl, m.shaded_temperature));
            }
    }
    sky.resize(nb);
    beam.resize(nb);
    for (uint32_t b = 0; b < nb; ++b) {
        const float wl = p.wavelengths[b];
        th[b] = wl > 2500.0f ? 1 : 0;  // makeSpectralOptics' own thermal test (:1063)
        opt[b] = optical_wavelength(wl) ? 1 : 0;
        sky[b] = opt[b] ? 100.0f * 0.5f : facetcu_planck_radiance(wl, p.sky_temperature);
        beam[b] = th[b] ? 0.0f : 700.0f;
    }
    optical.assign(opt.begin(), opt.end());
    const size_t bytes = tab.size() * 16 + tr.size() * 8 + 2 * size_t(nb) + 64;
    char* base = static_cast<char*>(dev.reserve(bytes));
    table = reinterpret_cast<float4*>(base);
    tir = reinterpret_cast<float2*>(base + tab.size() * 16);
    thermal = reinterpret_cast<uint8_t*>(base + tab.size() * 16 + tr.size() * 8);
    optical_dev = thermal + nb;
    FCU_CHECK(cudaMemcpyAsync(table, tab.data(), tab.size() * 16, cudaMemcpyHostToDevice, s));
    FCU_CHECK(cudaMemcpyAsync(tir, tr.data(), tr.size() * 8, cudaMemcpyHostToDevice, s));
    FCU_CHECK(cudaMemcpyAsync(thermal, th.data(), nb, cudaMemcpyHostToDevice, s));
    FCU_CHECK(cudaMemcpyAsync(optical_dev, opt.data(), nb, cudaMemcpyHostToDevice, s));
    FCU_CHECK(cudaStreamSynchronize(s));  // the host vectors go out of scope
}

void optics(const Tables& t, const facetcu_spectral_parameters& p, uint32_t F,
            const facetcu_vertex* V, const uint32_t* material, const float* texture,
            facetcu_direction sun, const float* sunlit, uint32_t b0, uint32_t bcount, float* rho,
            float* tau, float* emis, cudaStream_t s)
{
    const size_t n = size_t(F) * 2 * bcount;
    if (!n) return;
    k_spectral_optics<<<blocks(n, 256), 256, 0, s>>>(
        F, p.band_count, b0, bcount, V, material, p.material_count, texture, p.leaf_facet_count,
        t.table, t.tir, t.thermal, p.background_angular_strength, F3{sun.x, sun.y, sun.z}, sunlit,
        rho, tau, emis);
    FCU_LAUNCH("k_spectral_optics");
}

void direct_geometry(uint32_t F, const facetcu_vertex* V, facetcu_direction sun,
                     const float* sunlit, float* dgeo, cudaStream_t s)
{
    if (!F) return;
    k_direct_geometry<<<blocks(size_t(F) * 2, 256), 256, 0, s>>>(F, V, F3{sun.x, sun.y, sun.z},
                                                                 sunlit, dgeo);
    FCU_LAUNCH("k_direct_geometry");
}

void pack(size_t S, const float* rho, const float* tau, const float* emis, const float* dgeo,
          float beam, facetcu_surface_optics* out, cudaStream_t s)
{
    if (!S) return;
    k_pack<<<blocks(S, 256), 256, 0, s>>>(S, rho, tau, emis, dgeo, beam, out);
    FCU_LAUNCH("k_pack");
}

void apparent(float* B, size_t S, uint32_t bands, const uint8_t* optical, float ref,
              cudaStream_t s)
{
    if (!S || !bands) return;
    k_apparent<<<blocks(S * bands, 256), 256, 0, s>>>(B, S, bands, optical, ref);
    FCU_LAUNCH("k_apparent");
}

}  // namespace spectral
}  // namespace facetcu
