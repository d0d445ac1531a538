// energy.cu — the device side of one FacetEB time node.
//
// runFacetEBCore (models/histream/src/facetrt/facetrtcore.cpp:3462-3908)
// loops, per node, over shortwave windows (solve with and without the direct
// beam, incident irradiance, absorbed = absorptance x incident), then over
// coupling rounds (longwave optics from the temperatures, a longwave solve,
// incident longwave, the per-facet energy fluxes, the residual and a relaxed
// Newton temperature update) and finally over sensor bands.  The reference
// does each of these on the host, side by side, between GPU solves.  Here
// every per-side step is a kernel on device-resident arrays, so a node moves
// no per-side data across PCIe until its fields are read back:
//
//   k_shortwave_optics   all windows' optics at once (makeEnergyShortwaveOptics
//                        :952-1003), window-major planes for the batched solver
//   k_direct_geometry    clamp(sunlit) max(0, n . sun), times a beam per column
//   k_window_incident    H[w][s] for every window column (incidentIrradianceCpu
//                        :1531-1559: an FP64 gather there, a compensated FP32 one
//                        here), a warp per side over a side-major copy of the
//                        windows (k_transpose)
//   k_incident_one       the same for the single longwave column
//   k_shortwave_sum      the window accumulation in window order (:3536-3552)
//   k_longwave_optics    makeEnergyLongwaveOptics (:1005-1036)
//   k_balance            evaluateEnergyFluxes + measureEnergyResidual + the
//                        temperature update (:3590-3826), one thread per facet
//   k_state_optics       makeStateSpectralOptics (:1135-1200) for all bands
//   k_state_output       the sensor bands' apparent reflectance (:3893-3906)
//
// This file is compiled with -fmad=false and keeps the reference's operation
// order, so sums and products round as its host code does; the powers and
// exponentials go through double precision (pow(T, 3), pow(T, 4), 10^x and
// exp are correctly rounded to float in all but rare halfway cases, as the C
// library's are).
#include <cmath>

#include "internal.h"
#include "optics_math.cuh"

namespace facetcu {
namespace energy {
namespace {

using namespace optics_math;

constexpr float kSigma = 5.670374419e-8f;  // kStefanBoltzmann (:86)

__device__ __forceinline__ uint32_t slot_of(const uint32_t* material, uint32_t M, uint32_t f,
                                            bool object)
{
    const uint32_t mi = material ? material[f] : 0xffffffffu;
    return mi < M ? mi : (object ? M : M + 1);
}

__device__ __forceinline__ F3 side_normal(const facetcu_vertex* V, uint32_t s)
{
    const facetcu_vertex& v = V[3 * size_t(s >> 1)];
    return mulf(F3{v.normal[0], v.normal[1], v.normal[2]}, (s & 1u) ? -1.0f : 1.0f);
}

__device__ __forceinline__ float pow3(float x)
{
    const double d = double(x);
    return float(d * d * d);
}

__device__ __forceinline__ float pow4(float x)
{
    const double d2 = double(x) * double(x);
    return float(d2 * d2);
}

__device__ __forceinline__ float square(float x) { return float(double(x) * double(x)); }

// saturationVaporPressure (:853-857), hPa
__device__ float saturation(float temperature)
{
    const float celsius = sclamp(temperature - 273.15f, -80.0f, 80.0f);
    return 6.107f * float(exp10(double(7.5f * celsius / (237.3f + celsius))));
}

// saturationVaporPressureSlope (:859-865)
__device__ float saturation_slope(float temperature)
{
    const float celsius = sclamp(temperature - 273.15f, -80.0f, 80.0f);
    const float sat = saturation(temperature);
    return sat * 2.3026f * 7.5f * 237.3f / square(237.3f + celsius);
}

// latentHeatFlux (:868-883)
__device__ float latent_flux(float temperature, const Air& a, float surface_resistance)
{
    const float celsius = temperature - 273.15f;
    const float heat = (2.501f - 0.002361f * celsius) * 1.0e6f;
    const float deficit =
        0.622f * smax(0.0f, saturation(temperature) - a.vapor) / smax(100.0f, a.pressure);
    return a.density * heat * deficit / smax(1.0f, a.resistance + surface_resistance);
}

// latentHeatFluxDerivative (:885-906)
__device__ float latent_slope(float temperature, const Air& a, float surface_resistance)
{
    const float celsius = temperature - 273.15f;
    const float sat = saturation(temperature);
    const float slope = saturation_slope(temperature);
    const float heat = (2.501f - 0.002361f * celsius) * 1.0e6f;
    const float deficit = 0.622f * smax(0.0f, sat - a.vapor) / smax(100.0f, a.pressure);
    const float derivative = a.density / smax(1.0f, a.resistance + surface_resistance) *
                             (-2361.0f * deficit + heat * 0.622f * slope / smax(100.0f, a.pressure));
    return smax(0.0f, derivative);
}

// planckRadiance (:524-536) in double, as the reference.
__device__ float planck(float wavelength, float temperature)
{
    const double c1 = 1.1910439340652e8;
    const double c2 = 14388.291040407;
    const double um = wavelength > 50.0f ? double(wavelength) / 1000.0 : double(wavelength);
    const double exponent = c2 / (fmax(1.0, double(temperature)) * fmax(1.0e-6, um));
    return float(c1 / (pow(um, 5.0) * expm1(exponent)));
}

__device__ __forceinline__ void atomic_max_pos(uint32_t* p, float v)
{
    atomicMax(p, __float_as_uint(v));  // v >= 0: the bit patterns order as the values
}

__global__ void k_shortwave_optics(uint32_t F, uint32_t W, const facetcu_vertex* __restrict__ V,
                                   const uint32_t* __restrict__ material, uint32_t M,
                                   const float* __restrict__ texture, uint32_t leaf,
                                   const float2* __restrict__ table, float strength, F3 sun,
                                   float* __restrict__ rho, float* __restrict__ tau)
{
    const size_t S = size_t(F) * 2;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= S * W) return;
    const uint32_t w = uint32_t(i / S), s = uint32_t(i % S), f = s >> 1;
    const bool object = f < leaf;
    const uint32_t slot = slot_of(material, M, f, object);
    const float2 tb = table[(size_t(slot) * 2 + (object ? 1 : 0)) * W + w];
    const float tex = texture ? texture[f] : 1.0f;
    const float r = sclamp(tb.x * tex, 0.0f, 1.0f);
    const float t = sclamp(tb.y, 0.0f, 1.0f - r);
    const F3 side = side_normal(V, s);
    const float sr = object ? r : ground_reflectance(r, sun, side, side, strength);
    rho[i] = sr;
    tau[i] = smin(t, 1.0f - sr);
}

// dgeo[s] = clamp(sunlit_s, 0, 1) max(0, n_s . sun): a side's direct
// irradiance is dgeo times the beam, the product the reference forms.
__global__ void k_direct_geometry(uint32_t F, const facetcu_vertex* __restrict__ V, F3 sun,
                                  const float* __restrict__ sunlit, float* __restrict__ dgeo)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 2 * F) return;
    dgeo[s] = sclamp(sunlit[s], 0.0f, 1.0f) * smax(0.0f, dotf(side_normal(V, s), sun));
}

// Side-major copy of the first W columns of a column-major [R][S] block.
__global__ void k_transpose(uint32_t S, uint32_t W, const float* __restrict__ B,
                            float* __restrict__ BT)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(S) * W) return;
    const uint32_t s = uint32_t(i / W), w = uint32_t(i % W);
    BT[i] = B[size_t(w) * S + s];
}

// Compensated FP32 sum of count x B terms: each product split exactly into
// p + e (TwoProduct with an explicit fmaf) and each addition into s + err
// (Neumaier's TwoSum); the errors accumulate in c.  sum + c then carries
// about twice the float precision, as close to the reference's FP64 sum as
// its conversion back to float can tell, at FP32 throughput (GB300's FP64
// rate is a small fraction of it).
struct Csum {
    float s, c;
};
__device__ __forceinline__ void csum_add(Csum& a, float t, float e)
{
    const float s = a.s + t;
    const float err = fabsf(a.s) >= fabsf(t) ? (a.s - s) + t : (t - s) + a.s;
    a.s = s;
    a.c += err + e;
}
__device__ __forceinline__ void csum_term(Csum& a, uint32_t count, float v)
{
    const float n = float(count);  // exact below 2^24
    const float p = n * v;
    csum_add(a, p, fmaf(n, v, -p));
}
__device__ __forceinline__ double csum_value(const Csum& a) { return double(a.s) + double(a.c); }

// H[w][s] = max(0, diffuse + D): one warp per side, lane w of each 32-wide
// window group sums its window's gather in the reference's edge order (each
// edge is one broadcast load, its W values one contiguous row of BT).
__global__ void k_window_incident(uint32_t S, uint32_t W, const uint32_t* __restrict__ rows,
                                  const facetcu_csr_edge* __restrict__ edges,
                                  const uint32_t* __restrict__ denom,
                                  const uint32_t* __restrict__ skyc, const float* __restrict__ BT,
                                  const float* __restrict__ sky, const float* __restrict__ dni,
                                  const float* __restrict__ dgeo, float* __restrict__ H)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (warp >= S) return;
    const uint32_t s = warp;
    const uint32_t d = denom[s], start = rows[s], end = rows[s + 1];
    const float g = dgeo ? dgeo[s] : 0.0f;
    for (uint32_t w0 = 0; w0 < W; w0 += 32) {
        const uint32_t w = w0 + lane;
        const bool on = w < W;
        const float L = on ? sky[w] : 0.0f;
        double diffuse = L;
        if (d != 0u) {
            Csum acc{0.0f, 0.0f};
            uint32_t e = start;
            for (; e + 4 <= end; e += 4) {
                facetcu_csr_edge ed[4];
                float v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) ed[k] = edges[e + k];
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = on ? BT[size_t(ed[k].neighbor) * W + w] : 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) csum_term(acc, ed[k].count, v[k]);
            }
            for (; e < end; ++e) {
                const facetcu_csr_edge ed = edges[e];
                csum_term(acc, ed.count, on ? BT[size_t(ed.neighbor) * W + w] : 0.0f);
            }
            diffuse = (double(skyc[s]) * double(L) + csum_value(acc)) / double(d);
        }
        if (on) {
            const float D = dgeo ? g * dni[w] : 0.0f;
            H[size_t(w) * S + s] = smax(0.0f, float(diffuse) + D);
        }
    }
}

// One column, no direct term: a warp per side, lanes over the edges, the
// lanes' compensated partial sums combined by shuffles.
__global__ void k_incident_one(uint32_t S, const uint32_t* __restrict__ rows,
                               const facetcu_csr_edge* __restrict__ edges,
                               const uint32_t* __restrict__ denom,
                               const uint32_t* __restrict__ skyc, const float* __restrict__ B,
                               const float* __restrict__ sky, float* __restrict__ H)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31u;
    if (warp >= S) return;
    const uint32_t s = warp;
    const uint32_t d = denom[s];
    const float L = sky[0];
    Csum acc{0.0f, 0.0f};
    if (d != 0u) {
        const uint32_t end = rows[s + 1];
        for (uint32_t e = rows[s] + lane; e < end; e += 32) {
            const facetcu_csr_edge ed = edges[e];
            csum_term(acc, ed.count, B[ed.neighbor]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float os = __shfl_xor_sync(0xffffffffu, acc.s, o);
        const float oc = __shfl_xor_sync(0xffffffffu, acc.c, o);
        csum_add(acc, os, oc);
    }
    if (lane == 0) {
        double diffuse = L;
        if (d != 0u) diffuse = (double(skyc[s]) * double(L) + csum_value(acc)) / double(d);
        H[s] = smax(0.0f, float(diffuse));
    }
}

// Window accumulation in window order; columns [0, W) of B are the direct
// solutions, [W, 2W) the direct-free ones.
__global__ void k_shortwave_sum(uint32_t S, uint32_t W, const float* __restrict__ rho,
                                const float* __restrict__ tau, const float* __restrict__ H,
                                const float* __restrict__ B, float* __restrict__ absorbed,
                                float* __restrict__ incident, float* __restrict__ radiosity,
                                float* __restrict__ diffuse)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    float a = 0.0f, in = 0.0f, b = 0.0f, bd = 0.0f;
    for (uint32_t w = 0; w < W; ++w) {
        const size_t o = size_t(w) * S + s;
        const float absorptance = sclamp(1.0f - rho[o] - tau[o], 0.0f, 1.0f);
        in += H[o];
        a += absorptance * H[o];
        b += B[o];
        bd += B[size_t(W) * S + o];
    }
    absorbed[s] = a;
    incident[s] = in;
    radiosity[s] = b;
    diffuse[s] = bd;
}

__global__ void k_longwave_optics(uint32_t F, const facetcu_vertex* __restrict__ V,
                                  const uint32_t* __restrict__ material, uint32_t M, uint32_t leaf,
                                  const Material* __restrict__ mats, float strength,
                                  const float* __restrict__ T, float* __restrict__ rho,
                                  float* __restrict__ tau, float* __restrict__ emis)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= 2 * F) return;
    const uint32_t f = s >> 1;
    const bool ground = f >= leaf;
    const Material& m = mats[slot_of(material, M, f, !ground)];
    const float r = sclamp(m.tir_r, 0.0f, 1.0f);
    const float t = sclamp(m.tir_t, 0.0f, 1.0f - r);
    const float eps = smax(0.0f, 1.0f - r - t);
    const F3 side = side_normal(V, s);
    const float se = ground ? ground_emissivity(eps, fabsf(side.y), strength) : eps;
    rho[s] = sclamp(1.0f - t - se, 0.0f, 1.0f);
    tau[s] = t;
    emis[s] = se * kSigma * pow4(sclamp(T[s], 1.0f, 1000.0f));
}

// evaluateEnergyFluxes, measureEnergyResidual and (update != 0) the
// temperature update of one coupling round, one thread per facet.
// stats: [0] max |dT| bits, [1] max |residual| bits, [2] max residual
// equivalent bits, [3] non-finite residual seen.
__global__ void k_balance(uint32_t F, uint32_t leaf, const uint32_t* __restrict__ material,
                          uint32_t M, const Material* __restrict__ mats, Air a,
                          const float* __restrict__ lw_rho, const float* __restrict__ lw_tau,
                          const float* __restrict__ lw_emis, const float* __restrict__ lw_in,
                          const float* __restrict__ absorbed, const float* __restrict__ incident,
                          float* __restrict__ T, const float* __restrict__ T_prev, Fluxes out,
                          uint32_t* __restrict__ stats, int update)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const bool object = f < leaf;
    const Material& m = mats[slot_of(material, M, f, object)];
    const uint32_t s0 = 2 * f;
    float eps[2], rn[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const uint32_t s = s0 + k;
        eps[k] = sclamp(1.0f - lw_rho[s] - lw_tau[s], 0.0f, 1.0f);
        rn[k] = absorbed[s] + eps[k] * lw_in[s] - lw_emis[s];
    }
    float max_res = 0.0f, max_eq = 0.0f, max_dt = 0.0f;
    bool bad = false;
    if (object) {
        const float t0 = T[s0];
        const float net = rn[0] + rn[1];
        const float sens = 2.0f * a.conductance * m.convective_scale * (t0 - a.air);
        float leaf_resistance = m.surface_resistance;
        if (a.vegetation_method == 1) {
            const float par = smax(0.0f, absorbed[s0] + absorbed[s0 + 1]);
            const float opening = 0.25f + 0.75f * par / (par + 180.0f);
            const float celsius = t0 - 273.15f;
            const float response = float(exp(-double(square((celsius - 25.0f) / 18.0f))));
            leaf_resistance = sclamp(m.surface_resistance / smax(0.08f, opening * response), 40.0f,
                                     100000.0f);
        }
        const float veg = m.vegetation ? 2.0f : 0.0f;
        const float lat = veg * latent_flux(t0, a, leaf_resistance);
        const float lat_slope = veg * latent_slope(t0, a, leaf_resistance);
        const float stor_slope = smax(0.0f, m.heat_capacity) / a.time_step;
        const float stor = stor_slope * (t0 - T_prev[s0]);
        const float effective = incident[s0] + m.pv_bifaciality * incident[s0 + 1];
        const float eta = m.pv_eta25 * (1.0f + m.pv_gamma * (t0 - 298.15f));
        const float available = absorbed[s0] + absorbed[s0 + 1];
        const float raw = eta * effective;
        const float pv = m.photovoltaic ? sclamp(raw, 0.0f, available) : 0.0f;
        const float pv_slope = (m.photovoltaic && raw > 0.0f && raw < available)
                                   ? m.pv_eta25 * m.pv_gamma * effective
                                   : 0.0f;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t s = s0 + k;
            out.net[s] = net;
            out.sensible[s] = sens;
            out.latent[s] = lat;
            out.latent_slope[s] = lat_slope;
            out.storage[s] = stor;
            out.storage_slope[s] = stor_slope;
            out.pv[s] = pv;
            out.pv_slope[s] = pv_slope;
        }
        // the object's energy equation is checked and solved on side 0
        const float p3 = pow3(t0);
        const float residual = net - sens - lat - stor - pv;
        const float response = 8.0f * eps[0] * kSigma * p3 +
                               a.conductance * (2.0f * m.convective_scale) + lat_slope +
                               stor_slope + pv_slope;
        bad = !isfinite(residual) || !isfinite(response);
        max_res = fabsf(residual);
        max_eq = fabsf(residual) / smax(1.0f, response);
        if (update) {
            const float derivative = 8.0f * eps[0] * kSigma * p3 +
                                     2.0f * a.conductance * m.convective_scale + lat_slope +
                                     stor_slope + pv_slope;
            const float candidate =
                sclamp(t0 + residual / smax(1.0f, derivative), 220.0f, 360.0f);
            const float updated = t0 + a.relaxation * (candidate - t0);
            max_dt = fabsf(updated - t0);
            T[s0] = updated;
            T[s0 + 1] = updated;
        }
    } else {
        const bool dry = m.soil_moisture < 0.03f;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const uint32_t s = s0 + k;
            const float ts = T[s];
            const float sens = a.conductance * (ts - a.air);
            const float lat = dry ? 0.0f : latent_flux(ts, a, m.surface_resistance);
            const float lat_slope = dry ? 0.0f : latent_slope(ts, a, m.surface_resistance);
            float stor, stor_slope;
            if (m.soil_method == 0) {
                stor_slope = 0.0f;
                stor = 0.35f * rn[k];
            } else {
                stor_slope = m.storage_coefficient * (m.soil_method == 2 ? 1.5f : 1.0f);
                stor = stor_slope * (ts - T_prev[s]);
            }
            out.net[s] = rn[k];
            out.sensible[s] = sens;
            out.latent[s] = lat;
            out.latent_slope[s] = lat_slope;
            out.storage[s] = stor;
            out.storage_slope[s] = stor_slope;
            out.pv[s] = 0.0f;
            out.pv_slope[s] = 0.0f;
            const float p3 = pow3(ts);
            const float residual = rn[k] - sens - lat - stor;
            const float response = 4.0f * eps[k] * kSigma * p3 + a.conductance + lat_slope +
                                   stor_slope;
            bad = bad || !isfinite(residual) || !isfinite(response);
            max_res = smax(max_res, fabsf(residual));
            max_eq = smax(max_eq, fabsf(residual) / smax(1.0f, response));
            if (update) {
                const float candidate =
                    sclamp(ts + residual / smax(1.0f, response), 220.0f, 360.0f);
                const float updated = ts + a.relaxation * (candidate - ts);
                max_dt = smax(max_dt, fabsf(updated - ts));
                T[s] = updated;
            }
        }
    }
    if (bad) {
        atomicExch(stats + 3, 1u);
        return;
    }
    atomic_max_pos(stats + 0, max_dt);
    atomic_max_pos(stats + 1, max_res);
    atomic_max_pos(stats + 2, max_eq);
}

__global__ void k_state_optics(uint32_t F, uint32_t nb, const facetcu_vertex* __restrict__ V,
                               const uint32_t* __restrict__ material, uint32_t M,
                               const float* __restrict__ texture, uint32_t leaf,
                               const float4* __restrict__ table, const Material* __restrict__ mats,
                               const uint8_t* __restrict__ optical,
                               const float* __restrict__ wavelengths, float strength, F3 sun,
                               const float* __restrict__ T, float* __restrict__ rho,
                               float* __restrict__ tau, float* __restrict__ emis)
{
    const size_t S = size_t(F) * 2;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= S * nb) return;
    const uint32_t b = uint32_t(i / S), s = uint32_t(i % S), f = s >> 1;
    const bool object = f < leaf;
    const uint32_t slot = slot_of(material, M, f, object);
    const float4 tb = table[(size_t(slot) * 2 + (object ? 1 : 0)) * nb + b];
    const Material& m = mats[slot];
    const bool opt = optical[b] != 0;
    const float tex = (opt && texture) ? texture[f] : 1.0f;
    float r = sclamp((opt ? tb.x : m.tir_r) * tex, 0.0f, 1.0f);
    const float t = sclamp(opt ? tb.y : m.tir_t, 0.0f, 1.0f - r);
    const F3 side = side_normal(V, s);
    float eps = smax(0.0f, 1.0f - r - t);
    if (!object && opt) {
        r = ground_reflectance(r, sun, side, side, strength);
    } else if (!object) {
        eps = ground_emissivity(eps, fabsf(side.y), strength);
        r = sclamp(1.0f - t - eps, 0.0f, 1.0f);
    }
    rho[i] = r;
    tau[i] = smin(t, 1.0f - r);
    emis[i] = opt ? 0.0f : eps * planck(wavelengths[b], sclamp(T[s], 1.0f, 2000.0f));
}

// Optical bands: clamp(B / reference, 0, 1) where the reference irradiance
// is above 1e-8, else 0; thermal bands keep their radiance.
__global__ void k_state_output(float* B, size_t S, uint32_t nb, const uint8_t* optical,
                               const float* reference)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= S * nb) return;
    const uint32_t b = uint32_t(i / S);
    if (!optical[b]) return;
    const float ref = reference[b];
    B[i] = ref > 1.0e-8f ? sclamp(B[i] / ref, 0.0f, 1.0f) : 0.0f;
}

inline unsigned blocks(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

}  // namespace

void shortwave_optics(uint32_t F, uint32_t W, const facetcu_vertex* V, const uint32_t* material,
                      uint32_t M, const float* texture, uint32_t leaf, const float2* table,
                      float strength, facetcu_direction sun, float* rho, float* tau,
                      cudaStream_t s)
{
    const size_t n = size_t(F) * 2 * W;
    if (!n) return;
    k_shortwave_optics<<<blocks(n, 256), 256, 0, s>>>(F, W, V, material, M, texture, leaf, table,
                                                      strength, F3{sun.x, sun.y, sun.z}, rho, tau);
    FCU_LAUNCH("k_shortwave_optics");
}

void direct_geometry(uint32_t F, const facetcu_vertex* V, facetcu_direction sun,
                     const float* sunlit, float* dgeo, cudaStream_t s)
{
    if (!F) return;
    k_direct_geometry<<<blocks(size_t(F) * 2, 256), 256, 0, s>>>(F, V, F3{sun.x, sun.y, sun.z},
                                                                 sunlit, dgeo);
    FCU_LAUNCH("k_direct_geometry");
}

void window_incident(const DeviceGraph& g, uint32_t W, const float* B, const float* sky,
                     const float* dni, const float* dgeo, float* BT, float* H, cudaStream_t s)
{
    const size_t S = g.surfaces;
    if (!S || !W) return;
    const uint32_t* rows = g.row_offsets.as<uint32_t>();
    const facetcu_csr_edge* edges = g.edges.as<facetcu_csr_edge>();
    const uint32_t* den = g.denominators.as<uint32_t>();
    const uint32_t* skyc = g.sky.as<uint32_t>();
    if (W == 1 && !dgeo) {
        k_incident_one<<<blocks(S * 32, 256), 256, 0, s>>>(uint32_t(S), rows, edges, den, skyc, B,
                                                            sky, H);
        FCU_LAUNCH("k_incident_one");
        return;
    }
    k_transpose<<<blocks(S * W, 256), 256, 0, s>>>(uint32_t(S), W, B, BT);
    FCU_LAUNCH("k_transpose");
    k_window_incident<<<blocks(S * 32, 256), 256, 0, s>>>(uint32_t(S), W, rows, edges, den, skyc,
                                                          BT, sky, dni, dgeo, H);
    FCU_LAUNCH("k_window_incident");
}

void shortwave_sum(uint32_t S, uint32_t W, const float* rho, const float* tau, const float* H,
                   const float* B, float* absorbed, float* incident, float* radiosity,
                   float* diffuse, cudaStream_t s)
{
    if (!S) return;
    k_shortwave_sum<<<blocks(S, 256), 256, 0, s>>>(S, W, rho, tau, H, B, absorbed, incident,
                                                   radiosity, diffuse);
    FCU_LAUNCH("k_shortwave_sum");
}

void longwave_optics(uint32_t F, const facetcu_vertex* V, const uint32_t* material, uint32_t M,
                     uint32_t leaf, const Material* mats, float strength, const float* T,
                     float* rho, float* tau, float* emis, cudaStream_t s)
{
    if (!F) return;
    k_longwave_optics<<<blocks(size_t(F) * 2, 256), 256, 0, s>>>(F, V, material, M, leaf, mats,
                                                                 strength, T, rho, tau, emis);
    FCU_LAUNCH("k_longwave_optics");
}

void balance(uint32_t F, uint32_t leaf, const uint32_t* material, uint32_t M,
             const Material* mats, const Air& a, const float* lw_rho, const float* lw_tau,
             const float* lw_emis, const float* lw_in, const float* absorbed,
             const float* incident, float* T, const float* T_prev, const Fluxes& out,
             uint32_t* stats, bool update, cudaStream_t s)
{
    FCU_CHECK(cudaMemsetAsync(stats, 0, 4 * sizeof(uint32_t), s));
    if (!F) return;
    k_balance<<<blocks(F, 128), 128, 0, s>>>(F, leaf, material, M, mats, a, lw_rho, lw_tau,
                                             lw_emis, lw_in, absorbed, incident, T, T_prev, out,
                                             stats, update ? 1 : 0);
    FCU_LAUNCH("k_balance");
}

void state_optics(uint32_t F, uint32_t nb, const facetcu_vertex* V, const uint32_t* material,
                  uint32_t M, const float* texture, uint32_t leaf, const float4* table,
                  const Material* mats, const uint8_t* optical, const float* wavelengths,
                  float strength, facetcu_direction sun, const float* T, float* rho, float* tau,
                  float* emis, cudaStream_t s)
{
    const size_t n = size_t(F) * 2 * nb;
    if (!n) return;
    k_state_optics<<<blocks(n, 256), 256, 0, s>>>(F, nb, V, material, M, texture, leaf, table,
                                                  mats, optical, wavelengths, strength,
                                                  F3{sun.x, sun.y, sun.z}, T, rho, tau, emis);
    FCU_LAUNCH("k_state_optics");
}

void state_output(float* B, size_t S, uint32_t nb, const uint8_t* optical, const float* reference,
                  cudaStream_t s)
{
    if (!S || !nb) return;
    k_state_output<<<blocks(S * nb, 256), 256, 0, s>>>(B, S, nb, optical, reference);
    FCU_LAUNCH("k_state_output");
}

}  // namespace energy
}  // namespace facetcu
