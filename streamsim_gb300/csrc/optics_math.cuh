// optics_math.cuh — the per-side optics arithmetic shared by spectral.cu and
// energy.cu (both compiled with -fmad=false so every product and sum rounds
// as the reference's host code does).
//
// Ground sides take the reference's Hapke angular reflectance
// (backgroundHapkeReflectance, models/histream/src/facetrt/facetrtcore.cpp
// :565-587, with facetHapkeKernel :552-563 and facetHapkeH :546-550) and its
// infrared emissivity (infraredHapkeEmissivity :589-605).
#pragma once
#include <cstdint>

namespace facetcu {
namespace optics_math {

__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float sclamp(float v, float lo, float hi)
{
    return (v < lo) ? lo : ((hi < v) ? hi : v);
}

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ float dotf(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 mulf(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ F3 unitf(F3 a) { return mulf(a, 1.0f / sqrtf(dotf(a, a))); }

constexpr float kPi = 3.14159265358979323846f;

// Chandrasekhar H function in the two-stream form the reference uses.
__device__ inline float hapke_h(float mu, float w)
{
    const float gamma = sqrtf(smax(1.0f - w, 1.0e-6f));
    return (1.0f + 2.0f * mu) / (1.0f + 2.0f * mu * gamma);
}

// Bidirectional kernel with a shadow-hiding opposition surge (amplitude 1,
// width 0.1) and the multiple-scattering H(mu0) H(mu) - 1 term.
__device__ inline float hapke_kernel(float mu0, float mu, float phase, float w)
{
    const float surge = 1.0f / (1.0f + tanf(0.5f * phase) / 0.1f);
    const float multiple = hapke_h(mu0, w) * hapke_h(mu, w) - 1.0f;
    return w / (4.0f * kPi) * mu0 / smax(mu0 + mu, 1.0e-5f) * (1.0f + surge + multiple);
}

__device__ inline float ground_reflectance(float rho, F3 in, F3 out, F3 normal, float strength)
{
    const F3 n = unitf(normal);
    in = unitf(in);
    out = unitf(out);
    if (dotf(in, n) < 0.0f) in = mulf(in, -1.0f);
    if (dotf(out, n) < 0.0f) out = mulf(out, -1.0f);
    const float mu0 = smax(dotf(n, in), 1.0e-4f);
    const float mu = smax(dotf(n, out), 1.0e-4f);
    const float phase = acosf(sclamp(dotf(in, out), -1.0f, 1.0f));
    const float base = sclamp(rho, 0.0f, 0.999f);
    const float w = sclamp(4.0f * base / powf(1.0f + base, 2.0f), 1.0e-5f, 0.999f);
    const float directional = hapke_kernel(mu0, mu, phase, w);
    const float h1 = hapke_h(1.0f, w);
    const float reference = w / (8.0f * kPi) * h1 * h1;
    const float hapke = sclamp(base * directional / smax(reference, 1.0e-6f), 0.0f, 1.0f);
    return base + (hapke - base) * sclamp(strength, 0.0f, 1.0f);
}

__device__ inline float ground_emissivity(float eps, float cosine, float strength)
{
    const float base = sclamp(eps, 0.0f, 1.0f);
    const float w = sclamp(1.0f - base * base, 1.0e-5f, 0.999f);
    const float root = sqrtf(1.0f - w);
    auto directional = [root](float mu) {
        return root * (1.0f + 2.0f * mu / 1.5f) / (1.0f + 2.0f * mu / 1.5f * root);
    };
    const float hapke = sclamp(
        base * directional(sclamp(cosine, 1.0e-4f, 1.0f)) / smax(directional(1.0f), 1.0e-6f),
        0.0f, 1.0f);
    return base + (hapke - base) * sclamp(strength, 0.0f, 1.0f);
}

}  // namespace optics_math
}  // namespace facetcu
