// faceteb.cpp — host arithmetic of a FacetEB node: the shortwave spectrum and
// its spectral-acceleration windows, Planck-weighted broadband values,
// soil storage coefficients and the reference's SurfaceParameters defaults.
//
// Each function restates the reference's host code with the same operation
// order and types (this file is compiled with -ffp-contract=off), so the
// windows and per-material scalars are bit-identical to the reference's:
//   loadShortwaveSpectrum / ShortwaveSpectrum   facetrtcore.cpp:2458-2541
//   the window loop of runFacetEBCore           facetrtcore.cpp:3485-3536
//   shortwaveWeightedBandValue                  facetrtcore.cpp:915-950
//   soilStorageCoefficient                      facetrtcore.cpp:908-914
//   SurfaceParameters defaults                  facetrtcore.cpp:113-138
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "internal.h"

void facetcu_set_host_error(const std::string& message);

namespace facetcu {
namespace energy {

namespace {
constexpr float kPi = 3.14159265358979323846f;
constexpr uint32_t kSpectrumSamples = 2001;  // 400..2400 nm at 1 nm

struct Spectrum {
    std::vector<float> direct, diffuse;

    static float sample(const std::vector<float>& v, float wavelength)
    {
        if (v.empty()) return 0.0f;
        const float nm = wavelength <= 2.5f ? wavelength * 1000.0f : wavelength;
        const long i = std::clamp(long(std::lround(nm - 400.0f)), 0L, long(v.size()) - 1);
        return v[size_t(i)];
    }
    size_t count() const { return std::min(direct.size(), diffuse.size()); }
    // trapezoid over samples [first, last], per micrometre -> per 1 nm step
    static float integrate(const std::vector<float>& v, size_t first, size_t last)
    {
        if (v.size() < 2 || first >= v.size() - 1) return 0.0f;
        last = std::min(last, v.size() - 1);
        double integral = 0.0;
        for (size_t s = first; s < last; ++s) integral += 0.5 * double(v[s] + v[s + 1]);
        return float(integral * 0.001);
    }
};

Spectrum normalized(const facetcu_shortwave_spectrum& in)
{
    Spectrum sp;
    const float fraction = in.direct_fraction;
    auto flat = [&] {
        sp.direct.assign(kSpectrumSamples, 0.5f * fraction);
        sp.diffuse.assign(kSpectrumSamples, 0.5f * (1.0f - fraction));
    };
    // a spectrum file's values: non-finite -> 0, negative -> 0, at most 2001
    auto read = [](const float* v, uint32_t n) {
        std::vector<float> out;
        if (!v) return out;
        n = std::min(n, kSpectrumSamples);
        out.reserve(n);
        for (uint32_t i = 0; i < n; ++i) out.push_back(std::isfinite(v[i]) ? std::max(0.0f, v[i]) : 0.0f);
        return out;
    };
    sp.direct = read(in.direct, in.sample_count);
    sp.diffuse = read(in.diffuse, in.sample_count);
    const size_t count = sp.count();
    if (count < 2) {
        flat();
        return sp;
    }
    sp.direct.resize(count);
    sp.diffuse.resize(count);
    double integral = 0.0;
    for (size_t i = 0; i + 1 < count; ++i)
        integral += 0.5 * (sp.direct[i] + sp.direct[i + 1] + sp.diffuse[i] + sp.diffuse[i + 1]);
    integral *= 0.001;
    if (!(integral > 0.0) || !std::isfinite(integral)) {
        flat();
        return sp;
    }
    const float inverse = float(1.0 / integral);
    for (float& v : sp.direct) v *= inverse;
    for (float& v : sp.diffuse) v *= inverse;
    return sp;
}

const float kObjectReflectance[1] = {0.10f};
const float kObjectTransmittance[1] = {0.05f};
}  // namespace

float shortwave_weighted_value(const float* v, uint32_t n, float fallback)
{
    if (!v || n == 0) return fallback;
    if (n == 1) return std::isfinite(v[0]) ? v[0] : fallback;
    if (n == 2) {
        // visible and NIR/SWIR broad bands
        const float visible = std::isfinite(v[0]) ? v[0] : fallback;
        const float infrared = std::isfinite(v[1]) ? v[1] : visible;
        return 0.43f * visible + 0.57f * infrared;
    }
    double weighted = 0.0, weights = 0.0;
    for (uint32_t b = 0; b < n; ++b) {
        if (!std::isfinite(v[b])) continue;
        const float wavelength = 400.0f + 2000.0f * float(b) / float(n - 1);
        const double w = std::max(0.0f, facetcu_planck_radiance(wavelength, 5778.0f));
        weighted += w * double(v[b]);
        weights += w;
    }
    return weights > 0.0 ? float(weighted / weights) : fallback;
}

float storage_coefficient(const facetcu_energy_surface& m, float time_step)
{
    const float inertia =
        std::sqrt(std::max(0.0f, m.specific_heat * m.density * m.thermal_conductivity));
    return 2.0f * inertia / std::sqrt(kPi * std::max(1.0f, time_step));
}

}  // namespace energy
}  // namespace facetcu

extern "C" {

void facetcu_energy_surface_defaults(facetcu_energy_surface* s)
{
    if (!s) return;
    *s = facetcu_energy_surface{};
    s->optics.reflectance = facetcu::energy::kObjectReflectance;
    s->optics.reflectance_count = 1;
    s->optics.transmittance = facetcu::energy::kObjectTransmittance;
    s->optics.transmittance_count = 1;
    s->optics.tir_reflectance = 0.03f;
    s->optics.tir_transmittance = 0.0f;
    s->optics.sunlit_temperature = 300.0f;
    s->optics.shaded_temperature = 296.0f;
    s->surface_resistance = 120.0f;
    s->specific_heat = 1180.0f;
    s->density = 1800.0f;
    s->thermal_conductivity = 1.55f;
    s->soil_moisture = 0.25f;
    s->heat_capacity_per_area = 60000.0f;
    s->soil_temperature_method = 1;
    s->photovoltaic = 0;
    s->vegetation = 1;
    s->pv_eta25 = 0.22f;
    s->pv_gamma = -0.0035f;
    s->pv_bifaciality = 0.0f;
    s->convective_scale = 1.0f;
}

int facetcu_shortwave_windows(const facetcu_shortwave_spectrum* spectrum, float total_shortwave,
                              float cos_zenith, const float* wavelengths, uint32_t band_count,
                              facetcu_shortwave_window* windows, uint32_t capacity,
                              uint32_t* window_count, float* band_direct, float* band_diffuse)
{
    using facetcu::energy::Spectrum;
    facetcu_set_host_error("");
    if (!spectrum || !window_count || (capacity && !windows) || (band_count && !wavelengths)) {
        facetcu_set_host_error("spectrum, window_count, windows and wavelengths are required");
        return FACETCU_INVALID_ARGUMENT;
    }
    if (spectrum->window_width == 0) {
        facetcu_set_host_error("window_width must be at least 1");
        return FACETCU_INVALID_ARGUMENT;
    }
    const Spectrum sp = facetcu::energy::normalized(*spectrum);
    const float total = std::max(0.0f, total_shortwave);
    const float cosz = std::max(0.0f, cos_zenith);
    const size_t count = sp.count();
    const float direct_integral = count >= 2 ? Spectrum::integrate(sp.direct, 0, count - 1) : 0.0f;
    const float normal_scale = cosz > 1.0e-4f && direct_integral > 1.0e-8f
                                   ? std::min(1400.0f, total * direct_integral / cosz) / direct_integral
                                   : 0.0f;
    uint32_t n = 0;
    if (total > 0.0f && count >= 2) {
        const size_t width = spectrum->window_width;
        for (size_t first = 0; first + 1 < count; first += width) {
            const size_t last = std::min(first + width, count - 1);
            const size_t centre = (first + last) / 2;
            const float df = Spectrum::integrate(sp.direct, first, last);
            const float ff = Spectrum::integrate(sp.diffuse, first, last);
            if (df + ff <= 1.0e-10f) continue;
            if (n < capacity)
                windows[n] = {normal_scale * df, total * ff, uint32_t(centre)};
            ++n;
        }
    }
    *window_count = n;
    for (uint32_t b = 0; b < band_count; ++b) {
        const bool optical = facetcu::spectral::optical_wavelength(wavelengths[b]);
        if (band_direct)
            band_direct[b] = optical ? total * Spectrum::sample(sp.direct, wavelengths[b]) * 0.001f : 0.0f;
        if (band_diffuse)
            band_diffuse[b] = optical ? total * Spectrum::sample(sp.diffuse, wavelengths[b]) * 0.001f : 0.0f;
    }
    if (n > capacity) {
        facetcu_set_host_error("window capacity is smaller than the window count");
        return FACETCU_OVERFLOW_ERROR;
    }
    return FACETCU_OK;
}

}  // extern "C"
