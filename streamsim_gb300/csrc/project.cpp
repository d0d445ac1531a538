// project.cpp — scene and material ingestion of a HiStream XML project
// (the reference's Input.xml) and the eFacetRT run on it.
//
// Restates, with the same operation order and types (host code compiled
// with -ffp-contract=off), the reference's
//   XML helpers            facetrtcore.cpp:2052-2220 (firstXmlTag, xmlFloat,
//                          numberList, nameList, xmlAttribute, namedXmlBlock)
//   loadOpticalCoefficients :2223-2252 (optipar.txt beside the sun spectrum)
//   loadSurfaceParameters   :2254-2358, loadSoilParameters :2360-2383
//   facetRTParametersFromInput :2385-2426, xmlObjectBlocks :2428-2449
//   readObjGeometry         :2559-2608 (groups per triangle, y shifted to 0)
//   readPlacements, transformPosition, appendGeometry, cubeGeometry,
//   appendProjectGround     :2699-2878 (clipped to the scene domain
//                          :307-357)
//   loadProjectScene        :2880-3025
// and the spectral models they call (Compo::resolveSpectrals with the
// PROSPECT-style fluspect and the BSM soil model, compo.cpp:15-90, 152-341,
// 436-479; Utils::expint, utils.cpp:459-471).  In the reference's
// translation unit the unqualified float math calls (sin, exp, log, sqrt,
// pow) resolve to the C library's double functions; here they are written as
// std::fn(double(x)) with the same float/double promotions.
//
// DEM height fields and physical reflectance textures are read by dem.cpp
// (ESRI ASCII grids and baseline GeoTIFF, the formats GDAL would open for the
// reference); the texture steps (loadReflectanceVarianceTexture,
// sampledReflectanceVariance, finalizeReflectanceTextureFactors,
// facetrtcore.cpp:623-846) are restated here.  A project.json is read
// through its XML view (project_json.cpp), as the reference's readTextFile
// does.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <iterator>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/facetcu.h"
#include "host_scene.h"

void facetcu_set_host_error(const std::string& message);

namespace facetcu {
namespace project {

using host::V3;

constexpr int kSamples = 2001;  // 400..2400 nm at 1 nm (N1)
constexpr float kPi = 3.14159265358979323846f;

// ReflectanceVarianceTexture (facetrtcore.cpp:88-111): luminance deviations
// in [-1, 1], sampled bilinearly with wrap-around.
struct Texture {
    int width = 0, height = 0;
    std::vector<float> values;
    float sample(float u, float v) const
    {
        if (width <= 0 || height <= 0 || values.empty()) return 0.0f;
        const float x = (u - std::floor(u)) * float(width);
        const float y = (v - std::floor(v)) * float(height);
        const int x0 = int(std::floor(x)) % width, y0 = int(std::floor(y)) % height;
        const int x1 = (x0 + 1) % width, y1 = (y0 + 1) % height;
        const float tx = x - std::floor(x), ty = y - std::floor(y);
        const auto at = [this](int c, int r) { return values[size_t(r) * size_t(width) + size_t(c)]; };
        const float top = at(x0, y0) * (1.0f - tx) + at(x1, y0) * tx;
        const float bottom = at(x0, y1) * (1.0f - tx) + at(x1, y1) * tx;
        return top * (1.0f - ty) + bottom * ty;
    }
};

// SurfaceParameters with the reference's defaults (facetrtcore.cpp:113-138).
struct Surface {
    std::vector<float> r{0.10f}, t{0.05f}, er, et;
    float tir_r = 0.03f, tir_t = 0.0f, t_sun = 300.0f, t_shade = 296.0f;
    float rs = 120.0f, c = 1180.0f, density = 1800.0f, k = 1.55f, moisture = 0.25f;
    float hcap = 60000.0f;
    int soil_method = 1;
    bool pv = false, vegetation = true;
    float eta25 = 0.22f, gamma = -0.0035f, bif = 0.0f, conv = 1.0f;
    uint8_t component = 0;
    float tex_strength = 0.0f, tex_repeat = 1.0f;
    std::shared_ptr<const Texture> texture;
};

// srgbToLinear (facetrtcore.cpp:623-629).
float srgb_to_linear(float value)
{
    value = std::clamp(value, 0.0f, 1.0f);
    return value <= 0.04045f ? value / 12.92f : std::pow((value + 0.055f) / 1.055f, 2.4f);
}

// loadReflectanceVarianceTexture (facetrtcore.cpp:631-702): up to three
// bands as bytes, linear luminance, its mean removed and the deviations
// scaled to [-1, 1].  The raster is read by dem.cpp (ESRI ASCII grids and
// baseline GeoTIFF, the formats GDAL would open here).
std::shared_ptr<const Texture> load_texture(const std::filesystem::path& path)
{
    const std::string key = std::filesystem::absolute(path).lexically_normal().string();
    const dem::ByteBands b = dem::read_byte_bands(key, 3,
                                                  "Cannot open reflectance variance texture: ",
                                                  "Cannot read reflectance variance texture: ");
    if (b.width < 2 || b.height < 2)
        throw std::runtime_error(
            "Reflectance variance texture must contain at least 2 x 2 pixels: " + key);
    auto t = std::make_shared<Texture>();
    t->width = b.width;
    t->height = b.height;
    const size_t n = size_t(b.width) * size_t(b.height);
    t->values.resize(n);
    double mean = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const float red = srgb_to_linear(b.values[0][i] / 255.0f);
        const float green = b.count > 1 ? srgb_to_linear(b.values[1][i] / 255.0f) : red;
        const float blue = b.count > 2 ? srgb_to_linear(b.values[2][i] / 255.0f) : red;
        const float luminance = 0.2126f * red + 0.7152f * green + 0.0722f * blue;
        t->values[i] = luminance;
        mean += luminance;
    }
    mean /= double(n);
    float max_abs = 0.0f;
    for (float& v : t->values) {
        v -= float(mean);
        max_abs = std::max(max_abs, std::abs(v));
    }
    if (!(max_abs > 1.0e-6f))
        throw std::runtime_error("Reflectance variance texture is effectively constant: " + key);
    for (float& v : t->values) v /= max_abs;
    return t;
}

struct Parameters {  // FacetRTParameters (:140-146)
    std::vector<float> wavelengths{550.0f};
    Surface object;
    Surface ground;
    float sky_temperature = 250.0f;
    bool accelerated = false;
    Parameters()
    {
        ground.r = {0.20f};
        ground.t = {0.0f};
        ground.tir_r = 0.05f;
        ground.tir_t = 0.0f;
        ground.t_sun = 305.0f;
        ground.t_shade = 295.0f;
    }
};

struct Project {
    host::HostScene scene;
    std::vector<Surface> materials;
    std::vector<float> texture;
    float sun_zenith = 30.0f, sun_azimuth = 135.0f, strength = 0.0f;
    uint32_t periodic = 0, raster = 1024, layers = 64;
    float periodic_x = 1.0f, periodic_z = 1.0f;
    Parameters params;
    // C views (pointers into the vectors above)
    std::vector<facetcu_surface_parameters> optics_view;
    facetcu_surface_parameters object_view{}, ground_view{};
};

namespace {

// ---- XML -------------------------------------------------------------------
std::string decode(std::string value)
{
    const std::pair<const char*, const char*> entities[] = {
        {"&amp;", "&"}, {"&lt;", "<"}, {"&gt;", ">"}, {"&quot;", "\""}, {"&apos;", "'"}};
    for (const auto& e : entities) {
        size_t at = 0;
        while ((at = value.find(e.first, at)) != std::string::npos) {
            value.replace(at, std::strlen(e.first), e.second);
            at += std::strlen(e.second);
        }
    }
    return value;
}

std::string first_tag(const std::string& xml, const char* tag)
{
    const std::string open = "<" + std::string(tag), close = "</" + std::string(tag) + ">";
    const size_t begin = xml.find(open);
    if (begin == std::string::npos) return {};
    const size_t content = xml.find('>', begin + open.size());
    if (content == std::string::npos) return {};
    const size_t end = xml.find(close, content + 1);
    if (end == std::string::npos) return {};
    return decode(xml.substr(content + 1, end - content - 1));
}

std::string trim(std::string v)
{
    auto space = [](unsigned char ch) { return std::isspace(ch) != 0; };
    v.erase(v.begin(), std::find_if(v.begin(), v.end(), [&](char ch) { return !space(ch); }));
    v.erase(std::find_if(v.rbegin(), v.rend(), [&](char ch) { return !space(ch); }).base(),
            v.end());
    return v;
}

float xml_float(const std::string& xml, const char* tag, float fallback)
{
    const std::string v = trim(first_tag(xml, tag));
    if (v.empty()) return fallback;
    try {
        const float x = std::stof(v);
        return std::isfinite(x) ? x : fallback;
    } catch (...) {
        return fallback;
    }
}

std::vector<float> number_list(const std::string& text)
{
    std::string t = text;
    std::replace(t.begin(), t.end(), ';', ',');
    std::istringstream in(t);
    std::vector<float> out;
    std::string token;
    while (std::getline(in, token, ',')) {
        std::istringstream words(token);
        float v = 0.0f;
        while (words >> v)
            if (std::isfinite(v)) out.push_back(v);
    }
    return out;
}

std::string first_list_name(const std::string& text)
{
    return trim(text.substr(0, text.find_first_of(",;")));
}

std::vector<std::string> name_list(const std::string& text)
{
    std::string t = text;
    std::replace(t.begin(), t.end(), ';', ',');
    std::istringstream in(t);
    std::vector<std::string> out;
    std::string v;
    while (std::getline(in, v, ',')) {
        v = trim(v);
        if (!v.empty()) out.push_back(v);
    }
    return out;
}

bool iequal(const std::string& a, const std::string& b)
{
    return a.size() == b.size() &&
           std::equal(a.begin(), a.end(), b.begin(), [](unsigned char x, unsigned char y) {
               return std::tolower(x) == std::tolower(y);
           });
}

std::string attribute(const std::string& opening, const char* name)
{
    const std::string prefix = std::string(name) + '=';
    size_t at = opening.find(prefix);
    while (at != std::string::npos) {
        if (at == 0 || std::isspace(static_cast<unsigned char>(opening[at - 1]))) {
            size_t start = at + prefix.size();
            if (start < opening.size() && (opening[start] == '"' || opening[start] == '\'')) {
                const char quote = opening[start++];
                const size_t end = opening.find(quote, start);
                if (end != std::string::npos) return decode(opening.substr(start, end - start));
            }
        }
        at = opening.find(prefix, at + prefix.size());
    }
    return {};
}

// The first <element ...>...</element> block whose name attribute is `name`
// (any block when name is empty).
std::string named_block(const std::string& xml, const char* element, const std::string& name)
{
    const std::string open = "<" + std::string(element), close = "</" + std::string(element) + ">";
    size_t at = 0;
    while ((at = xml.find(open, at)) != std::string::npos) {
        const size_t suffix = at + open.size();
        if (suffix < xml.size() &&
            !(xml[suffix] == '>' || std::isspace(static_cast<unsigned char>(xml[suffix])))) {
            at = suffix;
            continue;
        }
        const size_t opening_end = xml.find('>', suffix);
        if (opening_end == std::string::npos) return {};
        const std::string opening = xml.substr(at, opening_end - at + 1);
        const size_t end = xml.find(close, opening_end + 1);
        if (end == std::string::npos) return {};
        if (name.empty() || attribute(opening, "name") == name)
            return xml.substr(at, end + close.size() - at);
        at = end + close.size();
    }
    return {};
}

std::vector<std::string> object_blocks(const std::string& xml)
{
    std::vector<std::string> out;
    const std::string open = "<object", close = "</object>";
    size_t at = 0;
    while ((at = xml.find(open, at)) != std::string::npos) {
        const size_t suffix = at + open.size();
        if (suffix >= xml.size() ||
            !(xml[suffix] == '>' || std::isspace(static_cast<unsigned char>(xml[suffix])))) {
            at = suffix;
            continue;
        }
        const size_t end = xml.find(close, suffix);
        if (end == std::string::npos) break;
        out.push_back(xml.substr(at, end + close.size() - at));
        at = end + close.size();
    }
    return out;
}

std::filesystem::path resolve(const std::filesystem::path& input, const std::string& value)
{
    const std::filesystem::path p(trim(value));
    return p.is_absolute() ? p : (input.parent_path() / p).lexically_normal();
}

std::string read_text(const std::string& path)
{
    std::string ext = std::filesystem::path(path).extension().string();
    std::transform(ext.begin(), ext.end(), ext.begin(),
                   [](unsigned char ch) { return char(std::tolower(ch)); });
    if (ext == ".json") return xml_view(path);
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("Cannot open HiStream input: " + path);
    return {std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>()};
}

// ---- spectral models -------------------------------------------------------
struct Coefficients {  // the optipar.txt columns the models read
    std::vector<float> wl, nr, kab, kdm, ks, kw, phi1, phi2, gsv1, gsv2, gsv3, nw;
};

enum class Kind { custom, bsm, prospect, file };

struct Spectral {
    std::string name;
    Kind kind = Kind::custom;
    std::vector<float> r, t;
    float cab = 40.0f, cw = 0.01f, cdm = 0.01f, cs = 0.0f, n = 1.5f;
    float smc = 25.0f, brightness = 0.5f, lat = 25.0f, lon = 45.0f;
    std::string path;
    float tau_tir = 0.0f, refl_tir = 0.0f;
};

float bounded(float v, float fallback) { return std::clamp(std::isfinite(v) ? v : fallback, 0.0f, 1.0f); }
float to_um(float w) { return w > 50.0f ? w / 1000.0f : w; }
float to_nm(float w) { return w > 0.0f && w <= 50.0f ? w * 1000.0f : w; }

std::vector<float> spectrum_row(std::string line)
{
    std::replace(line.begin(), line.end(), ',', ' ');
    std::replace(line.begin(), line.end(), ';', ' ');
    std::vector<float> out;
    std::istringstream in(line);
    float v = 0.0f;
    while (in >> v)
        if (std::isfinite(v)) out.push_back(v);
    return out;
}

void read_spectrum_file(const std::string& path, std::vector<float>& wl, std::vector<float>& r,
                        std::vector<float>& t)
{
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Cannot open imported spectrum: " + path);
    std::vector<std::vector<float>> rows;
    std::string line;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.erase(hash);
        auto v = spectrum_row(line);
        if (!v.empty()) rows.push_back(std::move(v));
    }
    if (rows.size() < 2 || rows.size() > 3 || rows[0].size() < 2 || rows[1].size() != rows[0].size() ||
        (rows.size() == 3 && rows[2].size() != rows[0].size()))
        throw std::runtime_error(
            "Imported spectrum must contain wavelength and reflectance rows, plus optional "
            "transmittance row: " + path);
    std::vector<std::pair<float, size_t>> order;
    for (size_t i = 0; i < rows[0].size(); ++i) order.emplace_back(to_nm(rows[0][i]), i);
    std::sort(order.begin(), order.end());
    wl.clear();
    r.clear();
    t.clear();
    for (const auto& e : order) {
        if (!wl.empty() && e.first <= wl.back())
            throw std::runtime_error("Imported spectrum wavelengths must be unique: " + path);
        wl.push_back(e.first);
        r.push_back(rows[1][e.second]);
        t.push_back(rows.size() == 3 ? rows[2][e.second] : 0.0f);
    }
}

float interpolate(const std::vector<float>& wl, const std::vector<float>& v, float w, float fallback)
{
    if (v.empty()) return fallback;
    if (v.size() == 1 || wl.size() != v.size()) return v.front();
    const float x = to_nm(w);
    if (x <= wl.front()) return v.front();
    if (x >= wl.back()) return v.back();
    const size_t right = size_t(std::upper_bound(wl.begin(), wl.end(), x) - wl.begin());
    const size_t left = right - 1;
    const float span = wl[right] - wl[left];
    const float weight = span > 0.0f ? (x - wl[left]) / span : 0.0f;
    return v[left] + (v[right] - v[left]) * weight;
}

// Mean transmissivity of a dielectric surface at incidence alfa (degrees),
// Stern's formula as the PROSPECT family uses it (calctav).
float tav(float alfa, float nr)
{
    const float pi = 3.1415926f;
    const float rd = pi / 180;
    const float n2 = nr * nr, np = n2 + 1, nm = n2 - 1;
    const float a = (nr + 1) * (nr + 1) / 2;
    const float k = -(n2 - 1) * (n2 - 1) / 4;
    const float sa = float(std::sin(double(alfa * rd)));
    float b1 = 0;
    if (alfa != 90) b1 = float(std::sqrt(double((sa * sa - np / 2) * (sa * sa - np / 2) + k)));
    const float b2 = sa * sa - np / 2;
    const float b = b1 - b2;
    const float b3 = b * b * b, a3 = a * a * a;
    const float ts = (k * k / (6 * b3) + k / b - b / 2) - (k * k / (6 * a3) + k / a - a / 2);
    const float tp1 = -2 * n2 * (b - a) / (np * np);
    const float tp2 = float(double(-2 * n2 * np) * std::log(double(b / a)) / double(nm * nm));
    const float tp3 = n2 * (1 / b - 1 / a) / 2;
    const float tp4 = float(double(16 * n2 * n2 * (n2 * n2 + 1)) *
                            std::log(double((2 * np * b - nm * nm) / (2 * np * a - nm * nm))) /
                            double(np * np * np * nm * nm));
    const float tp5 = 16 * n2 * n2 * n2 * (1 / (2 * np * b - nm * nm) - 1 / (2 * np * a - nm * nm)) /
                      (np * np * np);
    const float tp = tp1 + tp2 + tp3 + tp4 + tp5;
    return (ts + tp) / (2 * sa * sa);
}

// The exponential integral E1(x) as the reference's trapezoid-free Riemann
// sum over [1, 100) in steps of 0.001 (Utils::expint).
float expint(float x)
{
    double sum = 0.0;
    for (int i = 1000; i < 100000; ++i) {
        const double ii = i / 1000.0;
        sum = sum + std::exp(double(-x) * ii) / ii * 0.001;
    }
    return float(sum);
}

// PROSPECT leaf model (fluspect): N layers of a plate with absorption from
// chlorophyll, dry matter, water and senescent material.
void prospect(const Coefficients& c, const Spectral& m, std::vector<float>& r, std::vector<float>& t)
{
    r.clear();
    t.clear();
    for (int i = 0; i < kSamples; ++i) {
        const float nr = c.nr[i], kdm = c.kdm[i], kab = c.kab[i], kw = c.kw[i], ks = c.ks[i];
        const float kall = (m.cab * kab + m.cdm * kdm + m.cw * kw + m.cs * ks) / m.n;
        const float t1 = float(double(1 - kall) * std::exp(double(-kall)));
        const float t2 = kall * kall * expint(kall);
        float tau = 1;
        if (kall > 0) tau = t1 + t2;
        const float talf = tav(59, nr), ralf = 1 - talf;
        const float t12 = tav(90, nr), r12 = 1 - t12;
        const float t21 = t12 / (nr * nr), r21 = 1 - t21;
        float denom = 1 - r21 * r21 * tau * tau;
        const float ta = talf * tau * t21 / denom;
        const float ra = ralf + r21 * tau * ta;
        const float tt = t12 * tau * t21 / denom;
        const float rr = r12 + r21 * tau * tt;
        const float d = float(std::sqrt(double((1 + rr + tt) * (1 + rr - tt) * (1 - rr + tt) *
                                               (1 - rr - tt))));
        const float rq = rr * rr, tq = tt * tt;
        const float a = (1 + rq - tq + d) / (2 * rr);
        const float b = (1 - rq + tq + d) / (2 * tt);
        const float bnm1 = float(std::pow(double(b), double(m.n - 1)));
        const float bn2 = bnm1 * bnm1;
        const float a2 = a * a;
        denom = a2 * bn2 - 1;
        float rsub = a * (bn2 - 1) / denom;
        float tsub = bnm1 * (a2 - 1) / denom;
        if (rr + tt >= 1) {
            tsub = tt / (tt + (1 - tt) * (m.n - 1));
            rsub = 1 - tsub;
        }
        denom = 1 - rsub * rr;
        t.push_back(ta * tsub / denom);
        r.push_back(ra + ta * rsub * tt / denom);
    }
}

// BSM soil model: dry soil from three spectral vectors, a water film of
// moisture SMC.
void bsm(const Coefficients& c, const Spectral& m, std::vector<float>& r, std::vector<float>& t)
{
    const float B = m.brightness, lat = m.lat, lon = m.lon;
    float smc = m.smc > 1.0f ? m.smc / 100.0f : m.smc;
    smc = std::clamp(smc, 0.0f, 1.0f);
    const float smcp = 0.25f, film = 0.015f;
    const float rd = float(3.1415926 / 180.0);
    const float f1 = float(double(B) * std::sin(double(lat * rd)));
    const float f2 = float(double(B) * std::cos(double(lat * rd)) * std::sin(double(lon * rd)));
    const float f3 = float(double(B) * std::cos(double(lat * rd)) * std::cos(double(lon * rd)));
    r.clear();
    t.clear();
    std::vector<float> dry;
    for (size_t k = 0; k < c.gsv1.size(); ++k) dry.push_back(c.gsv1[k] * f1 + c.gsv2[k] * f2 + c.gsv3[k] * f3);
    for (size_t k = 0; k < c.gsv1.size(); ++k) {
        const float rdry = dry[k];
        const float tw = float(std::exp(double(-c.kw[k] * film)));
        const float rbac = 1 - (1 - dry[k]) * (dry[k] * tav(90, float(2.0 / c.nw[k])) / tav(90, 2.0f) +
                                               1 - dry[k]);
        const float p = 1 - tav(90, c.nw[k]) / c.nw[k] / c.nw[k];
        const float rw = 1 - tav(40, c.nw[k]);
        const float radd = (1 - rw) * (1 - p) * rbac / (1 - p * rbac);
        const float mu = float((double(smc) - 0.05) / double(smcp));
        const float fdry = float(std::exp(double(-mu)));
        const float fmul = float((std::exp(double(tw * mu)) - 1) * double(fdry));
        r.push_back(rdry * fdry + rw * (1 - fdry) + radd * fmul);
        t.push_back(0.0f);
    }
}

// Compo::resolveSpectrals: a material's reflectance/transmittance on the
// requested wavelengths (thermal ones take the TIR values).
void resolve_spectral(const Spectral& m, const std::vector<float>& out_wl,
                      const std::vector<float>& custom_wl, const Coefficients& c,
                      std::vector<float>& r_out, std::vector<float>& t_out)
{
    std::vector<float> wl, r, t;
    if (m.kind == Kind::prospect || m.kind == Kind::bsm) {
        const size_t N = kSamples;
        const bool prospect_ready = c.wl.size() >= N && c.nr.size() >= N && c.kdm.size() >= N &&
                                    c.kab.size() >= N && c.kw.size() >= N && c.ks.size() >= N &&
                                    c.phi1.size() >= N && c.phi2.size() >= N;
        const bool bsm_ready = c.wl.size() >= N && c.gsv1.size() >= N && c.gsv2.size() >= N &&
                               c.gsv3.size() >= N && c.kw.size() >= N && c.nw.size() >= N;
        if ((m.kind == Kind::prospect && !prospect_ready) || (m.kind == Kind::bsm && !bsm_ready))
            throw std::runtime_error("Optical model coefficients are unavailable for material: " +
                                     m.name);
        std::vector<float> mr, mt;
        if (m.kind == Kind::prospect)
            prospect(c, m, mr, mt);
        else
            bsm(c, m, mr, mt);
        const size_t n = std::min(mr.size(), c.wl.size());
        for (size_t i = 0; i < n; ++i) {
            wl.push_back(to_nm(c.wl[i]));
            r.push_back(mr[i]);
            t.push_back(mt[i]);
        }
    } else if (m.kind == Kind::file) {
        if (m.path.empty())
            throw std::runtime_error("Imported spectrum path is empty for material: " + m.name);
        read_spectrum_file(m.path, wl, r, t);
    } else {
        for (float w : custom_wl) wl.push_back(to_nm(w));
        r = m.r;
        t = m.t;
    }
    r_out.clear();
    t_out.clear();
    for (float w : out_wl) {
        if (to_um(w) > 2.5f) {
            const float rr = bounded(m.refl_tir, 0.05f);
            r_out.push_back(rr);
            t_out.push_back(std::min(bounded(m.tau_tir, 0.0f), 1.0f - rr));
            continue;
        }
        const float rr = bounded(interpolate(wl, r, w, 0.2f), 0.2f);
        r_out.push_back(rr);
        t_out.push_back(std::min(bounded(interpolate(wl, t, w, 0.0f), 0.0f), 1.0f - rr));
    }
}

// The 18-column optipar.txt beside the sun spectrum file.
Coefficients load_coefficients(const std::string& xml, const std::filesystem::path& input)
{
    Coefficients c;
    const std::string esun = trim(first_tag(xml, "esunFileName"));
    if (esun.empty()) return c;
    std::ifstream in(resolve(input, esun).parent_path() / "optipar.txt");
    if (!in) return c;
    // wl nr kab kca ks kw kdm phiI phiII kcaV kcaZ kcant kcaV2 phi gsv1 gsv2 gsv3 nw
    std::vector<float>* cols[18] = {&c.wl, &c.nr, &c.kab, nullptr, &c.ks, &c.kw, &c.kdm, &c.phi1,
                                    &c.phi2, nullptr, nullptr, nullptr, nullptr, nullptr, &c.gsv1,
                                    &c.gsv2, &c.gsv3, &c.nw};
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream row(line);
        std::array<float, 18> v{};
        bool ok = true;
        for (float& x : v) ok = ok && static_cast<bool>(row >> x);
        if (!ok) continue;
        for (size_t i = 0; i < 18; ++i)
            if (cols[i]) cols[i]->push_back(v[i]);
    }
    return c;
}

void load_surface(const std::string& xml, const std::string& spectral_name,
                  const std::string& thermal_name, const std::vector<float>& wavelengths,
                  const Coefficients& c, const std::filesystem::path& input, Surface& s)
{
    const std::string sp = named_block(xml, "spectral", spectral_name);
    if (!sp.empty()) {
        const size_t opening_end = sp.find('>');
        const std::string opening = opening_end == std::string::npos ? std::string{}
                                                                     : sp.substr(0, opening_end + 1);
        const std::string type = attribute(opening, "type");
        Spectral m;
        m.name = spectral_name;
        m.kind = iequal(type, "Prospect") ? Kind::prospect
                 : iequal(type, "BSM")    ? Kind::bsm
                 : iequal(type, "file")   ? Kind::file
                                          : Kind::custom;
        m.r = number_list(first_tag(sp, "reflectance"));
        m.t = number_list(first_tag(sp, "transmittance"));
        m.refl_tir = xml_float(sp, "ref_TIR", s.tir_r);
        m.tau_tir = xml_float(sp, "tau_TIR", s.tir_t);
        m.cab = xml_float(sp, "Cab", 40.0f);
        m.cw = xml_float(sp, "Cw", 0.01f);
        m.cdm = xml_float(sp, "Cdm", 0.01f);
        m.cs = xml_float(sp, "Cs", 0.0f);
        m.n = xml_float(sp, "N", 1.5f);
        m.smc = xml_float(sp, "SMC", 25.0f);
        m.brightness = xml_float(sp, "BSMBrightness", 0.5f);
        m.lat = xml_float(sp, "BSMlat", 25.0f);
        m.lon = xml_float(sp, "BSMlon", 45.0f);
        if (m.kind == Kind::file) m.path = resolve(input, trim(first_tag(sp, "spectral_file"))).string();
        resolve_spectral(m, wavelengths, wavelengths, c, s.r, s.t);
        std::vector<float> energy_wl;
        energy_wl.reserve(kSamples);
        for (int i = 0; i < kSamples; ++i) energy_wl.push_back(400.0f + float(i));
        resolve_spectral(m, energy_wl, wavelengths, c, s.er, s.et);
        s.tir_r = xml_float(sp, "ref_TIR", s.tir_r);
        s.tir_t = xml_float(sp, "tau_TIR", s.tir_t);
        s.tex_strength = 0.0f;
        s.tex_repeat = 1.0f;
        const std::string tex = trim(first_tag(sp, "physicalTextureEnabled"));
        if (tex == "1" || iequal(tex, "true") || iequal(tex, "yes") || iequal(tex, "on")) {
            const std::string file = trim(first_tag(sp, "physicalTextureFile"));
            if (file.empty())
                throw std::runtime_error("Physical texture is enabled but has no file: " +
                                         spectral_name);
            s.tex_strength = std::clamp(xml_float(sp, "physicalTextureStrength", 0.2f), 0.0f, 1.0f);
            s.tex_repeat = std::max(0.01f, xml_float(sp, "physicalTextureRepeatSize", 2.0f));
            s.texture = load_texture(resolve(input, file));
        }
    }
    const std::string th = named_block(xml, "thermal", thermal_name);
    if (!th.empty()) {
        s.t_sun = xml_float(th, "sunlitTemperature", s.t_sun);
        s.t_shade = xml_float(th, "shadedTemperature", s.t_shade);
    }
}

void load_soil(const std::string& xml, const std::string& name, Surface& s)
{
    const std::string soil = named_block(xml, "soilSet", name);
    if (soil.empty()) return;
    s.soil_method = std::clamp(int(std::lround(xml_float(soil, "method", 1.0f))), 0, 2);
    s.rs = std::max(0.0f, xml_float(soil, "rss", s.rs));
    s.c = std::max(1.0f, xml_float(soil, "cs", s.c));
    s.density = std::max(1.0f, xml_float(soil, "rhos", s.density));
    s.k = std::max(0.001f, xml_float(soil, "lambdas", s.k));
    const float moisture = xml_float(soil, "SMC", s.moisture);
    s.moisture = std::clamp(moisture > 1.0f ? moisture * 0.01f : moisture, 0.0f, 1.0f);
}

Parameters parameters_from_input(const std::string& xml, const std::filesystem::path& input)
{
    Parameters p;
    p.wavelengths = number_list(first_tag(xml, "controlBand"));
    p.wavelengths.erase(std::remove_if(p.wavelengths.begin(), p.wavelengths.end(),
                                       [](float w) { return !std::isfinite(w) || w <= 0.0f; }),
                        p.wavelengths.end());
    if (p.wavelengths.empty()) p.wavelengths.push_back(550.0f);
    p.sky_temperature = std::clamp(xml_float(xml, "skyTemperature", 250.0f), 100.0f, 400.0f);
    p.accelerated = trim(first_tag(xml, "radiationSolver")) == "accelerated";
    const Coefficients c = load_coefficients(xml, input);
    const std::vector<std::string> objects = object_blocks(xml);
    if (!objects.empty())
        load_surface(xml, first_list_name(first_tag(objects.front(), "spectralNames")),
                     first_list_name(first_tag(objects.front(), "thermalNames")), p.wavelengths,
                     c, input, p.object);
    load_surface(xml, trim(first_tag(xml, "bgSpectral")), trim(first_tag(xml, "bgThermal")),
                 p.wavelengths, c, input, p.ground);
    load_soil(xml, trim(first_tag(xml, "bgBioName")), p.ground);
    return p;
}

// ---- geometry --------------------------------------------------------------
struct Geometry {
    std::vector<V3> positions;
    std::vector<std::array<int, 3>> triangles;
    std::vector<std::string> groups;
};

Geometry read_obj(const std::filesystem::path& path)
{
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Cannot open scene OBJ: " + path.string());
    Geometry g;
    std::string group, line;
    while (std::getline(in, line)) {
        std::istringstream fields(line);
        std::string kind;
        fields >> kind;
        if (kind == "g" || kind == "o") {
            std::string name;
            if (fields >> name) group = name;
        } else if (kind == "usemtl" && group.empty()) {
            fields >> group;
        } else if (kind == "v") {
            V3 p{};
            if (!(fields >> p[0] >> p[1] >> p[2]))
                throw std::runtime_error("Invalid OBJ vertex in " + path.string());
            g.positions.push_back(p);
        } else if (kind == "f") {
            std::vector<int> face;
            std::string token;
            while (fields >> token) face.push_back(host::obj_position(token, g.positions.size()));
            for (size_t i = 1; i + 1 < face.size(); ++i) {
                g.triangles.push_back({face[0], face[i], face[i + 1]});
                g.groups.push_back(group);
            }
        }
    }
    if (g.positions.empty() || g.triangles.empty())
        throw std::runtime_error("Scene OBJ contains no usable geometry: " + path.string());
    float low = std::numeric_limits<float>::max();
    for (const V3& p : g.positions) low = std::min(low, p[1]);
    for (V3& p : g.positions) p[1] -= low;
    return g;
}

struct Placement {
    float x = 0, y = 0, z = 0, scale = 1, rotation = 0;
};

std::vector<Placement> read_placements(const std::filesystem::path& input, const std::string& obj,
                                       float width, float depth)
{
    std::vector<Placement> out;
    const std::string file = trim(first_tag(obj, "objectPosition"));
    if (!file.empty()) {
        const std::filesystem::path path = resolve(input, file);
        std::ifstream in(path);
        if (!in) throw std::runtime_error("Cannot open object positions: " + path.string());
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream fields(line);
            Placement p;
            if (!(fields >> p.x >> p.y >> p.z)) continue;
            if (!(fields >> p.scale)) {
                p.scale = 1.0f;
                fields.clear();
            }
            if (!(fields >> p.rotation)) p.rotation = 0.0f;
            if (std::isfinite(p.x) && std::isfinite(p.y) && std::isfinite(p.z) &&
                std::isfinite(p.scale) && std::isfinite(p.rotation) && p.scale > 0.0f)
                out.push_back(p);
        }
    }
    if (out.empty()) out.push_back({width * 0.5f, depth * 0.5f, 0.0f, 1.0f, 0.0f});
    return out;
}

V3 place(const V3& p, const Placement& pl, float width, float depth)
{
    const float radians = -pl.rotation * kPi / 180.0f;
    const float c = std::cos(radians), s = std::sin(radians);
    const float x = p[0] * pl.scale, y = p[1] * pl.scale, z = p[2] * pl.scale;
    return {c * x + s * z + pl.x - width * 0.5f, y + pl.z, -s * x + c * z + pl.y - depth * 0.5f};
}

std::vector<V3> clip(const std::vector<V3>& src, size_t axis, float plane, bool keep_greater)
{
    std::vector<V3> out;
    if (src.empty()) return out;
    auto inside = [&](const V3& p) {
        return keep_greater ? p[axis] >= plane - 1.0e-6f : p[axis] <= plane + 1.0e-6f;
    };
    V3 prev = src.back();
    bool prev_in = inside(prev);
    for (const V3& cur : src) {
        const bool cur_in = inside(cur);
        if (cur_in != prev_in) {
            const float den = cur[axis] - prev[axis];
            if (std::abs(den) > 1.0e-8f) {
                const float amount = std::clamp((plane - prev[axis]) / den, 0.0f, 1.0f);
                V3 x{};
                for (size_t a = 0; a < 3; ++a) x[a] = prev[a] + amount * (cur[a] - prev[a]);
                out.push_back(x);
            }
        }
        if (cur_in) out.push_back(cur);
        prev = cur;
        prev_in = cur_in;
    }
    return out;
}

void push_inside(host::HostScene& sc, const V3& a, const V3& b, const V3& c, const V3& lo,
                 const V3& hi, uint32_t material)
{
    std::vector<V3> poly{a, b, c};
    for (size_t axis = 0; axis < 3 && poly.size() >= 3; ++axis) {
        poly = clip(poly, axis, lo[axis], true);
        poly = clip(poly, axis, hi[axis], false);
    }
    for (size_t i = 1; i + 1 < poly.size(); ++i) host::push_triangle(sc, poly[0], poly[i], poly[i + 1], material);
}

struct Binding {
    std::string mesh;
    uint32_t material = 0;
};

void append_geometry(host::HostScene& sc, const Geometry& g, const Placement& pl, float width,
                     float depth, float height, const std::vector<Binding>& bindings)
{
    const V3 lo{-width * 0.5f, 0.0f, -depth * 0.5f}, hi{width * 0.5f, height, depth * 0.5f};
    for (size_t i = 0; i < g.triangles.size(); ++i) {
        const auto& tri = g.triangles[i];
        uint32_t material = bindings.empty() ? 0u : bindings.front().material;
        const std::string group = i < g.groups.size() ? g.groups[i] : std::string{};
        for (const Binding& b : bindings)
            if (!b.mesh.empty() && iequal(b.mesh, group)) {
                material = b.material;
                break;
            }
        push_inside(sc, place(g.positions[tri[0]], pl, width, depth),
                    place(g.positions[tri[1]], pl, width, depth),
                    place(g.positions[tri[2]], pl, width, depth), lo, hi, material);
    }
}

Geometry cube(const std::string& obj)
{
    float length = 1.0f, width = 1.0f, height = 1.0f;
    std::istringstream values(first_tag(obj, "shapes"));
    char sep = 0;
    values >> length >> sep >> width >> sep >> height;
    if (!(length > 0.0f) || !(width > 0.0f) || !(height > 0.0f)) length = width = height = 1.0f;
    const float hx = length * 0.5f, hz = width * 0.5f;
    Geometry g;
    g.positions = {{-hx, 0.0f, -hz}, {hx, 0.0f, -hz}, {hx, 0.0f, hz}, {-hx, 0.0f, hz},
                   {-hx, height, -hz}, {hx, height, -hz}, {hx, height, hz}, {-hx, height, hz}};
    g.triangles = {{0, 2, 1}, {0, 3, 2}, {4, 5, 6}, {4, 6, 7}, {0, 1, 5}, {0, 5, 4},
                   {1, 2, 6}, {1, 6, 5}, {2, 3, 7}, {2, 7, 6}, {3, 0, 4}, {3, 4, 7}};
    g.groups.assign(g.triangles.size(), std::string{});
    return g;
}

void append_ground(host::HostScene& sc, float width, float depth, float voxel, uint32_t max_grid,
                   uint32_t material, const dem::HeightField& dem)
{
    const float x0 = -width * 0.5f, z0 = -depth * 0.5f;
    const uint32_t want_cols = std::max(1u, uint32_t(std::ceil(width / voxel)));
    const uint32_t want_rows = std::max(1u, uint32_t(std::ceil(depth / voxel)));
    const uint32_t cols = std::clamp(want_cols, 1u, max_grid);
    const uint32_t rows = std::clamp(want_rows, 1u, max_grid);
    const float cw = width / float(cols), cd = depth / float(rows);
    // the whole DEM is stretched over the domain, 1 cm below its height
    for (uint32_t r = 0; r < rows; ++r) {
        const float za = z0 + cd * float(r);
        const float zb = r + 1 == rows ? z0 + depth : z0 + cd * float(r + 1);
        for (uint32_t c = 0; c < cols; ++c) {
            const float xa = x0 + cw * float(c);
            const float xb = c + 1 == cols ? x0 + width : x0 + cw * float(c + 1);
            const float sxa = xa + width * 0.5f, sxb = xb + width * 0.5f;
            const float sza = za + depth * 0.5f, szb = zb + depth * 0.5f;
            const float haa = dem.above_minimum(sxa, sza, width, depth) - 0.01f;
            const float hab = dem.above_minimum(sxa, szb, width, depth) - 0.01f;
            const float hba = dem.above_minimum(sxb, sza, width, depth) - 0.01f;
            const float hbb = dem.above_minimum(sxb, szb, width, depth) - 0.01f;
            host::push_triangle(sc, {xa, haa, za}, {xb, hbb, zb}, {xb, hba, za}, material);
            host::push_triangle(sc, {xa, haa, za}, {xa, hab, zb}, {xb, hbb, zb}, material);
        }
    }
}

// facetArea (facetrtcore.cpp:704-716).
float facet_area(const host::HostScene& sc, uint32_t f)
{
    const float* a = sc.vertices[3 * f].position;
    const float* b = sc.vertices[3 * f + 1].position;
    const float* c = sc.vertices[3 * f + 2].position;
    const V3 ea{b[0] - a[0], b[1] - a[1], b[2] - a[2]}, eb{c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const V3 n = host::cross3(ea, eb);
    return 0.5f * std::sqrt(host::dot3(n, n));
}

// sampledReflectanceVariance (:718-741): the texture on the three axis
// planes through the facet's centre, weighted by |normal|.
float sampled_variance(const host::HostScene& sc, uint32_t f, const Surface& s)
{
    if (!s.texture) return 0.0f;
    const facetcu_vertex &a = sc.vertices[3 * f], &b = sc.vertices[3 * f + 1],
                         &c = sc.vertices[3 * f + 2];
    const V3 centre{(a.position[0] + b.position[0] + c.position[0]) / 3.0f,
                    (a.position[1] + b.position[1] + c.position[1]) / 3.0f,
                    (a.position[2] + b.position[2] + c.position[2]) / 3.0f};
    const V3 n{std::abs(a.normal[0]), std::abs(a.normal[1]), std::abs(a.normal[2])};
    const float weight = std::max(1.0e-6f, n[0] + n[1] + n[2]);
    const float inv = 1.0f / std::max(0.01f, s.tex_repeat);
    const Texture& t = *s.texture;
    return (n[0] * t.sample(centre[2] * inv, centre[1] * inv) +
            n[1] * t.sample(centre[0] * inv, centre[2] * inv) +
            n[2] * t.sample(centre[0] * inv, centre[1] * inv)) / weight;
}

// maximumMeanPreservingFactor (:743-762).
float max_mean_preserving_factor(const Surface& s)
{
    float m = std::numeric_limits<float>::infinity();
    const auto bands = [&m](const std::vector<float>& r, const std::vector<float>& t) {
        for (size_t band = 0; band < r.size(); ++band) {
            const float base = std::clamp(r[band], 0.0f, 1.0f);
            if (!(base > 1.0e-6f)) continue;
            const float tau =
                t.empty() ? 0.0f : std::clamp(t[std::min(band, t.size() - 1)], 0.0f, 1.0f - base);
            m = std::min(m, (1.0f - tau) / base);
        }
    };
    bands(s.r, s.t);
    bands(s.er, s.et);
    return m;
}

// finalizeReflectanceTextureFactors (:764-846): per textured material the
// area-weighted mean sample is removed and the deviations are scaled so the
// factors stay positive and below the mean-preserving bound.
std::vector<float> texture_factors(const host::HostScene& sc, const std::vector<Surface>& mats)
{
    const uint32_t F = sc.facets();
    std::vector<float> factors(F, 1.0f);
    if (F == 0 || mats.empty()) return factors;
    struct Stats {
        double area = 0.0, weighted = 0.0;
        float min_dev = 0.0f, max_dev = 0.0f, scale = 0.0f;
        double weighted_factor = 0.0;
        float min_factor = std::numeric_limits<float>::infinity();
        float max_factor = std::numeric_limits<float>::lowest();
    };
    std::vector<Stats> st(mats.size());
    std::vector<float> samples(F, 0.0f), areas(F, 0.0f);
    for (uint32_t f = 0; f < F; ++f) {
        if (f >= sc.material.size()) continue;
        const uint32_t m = sc.material[f];
        if (m >= mats.size()) continue;
        const Surface& s = mats[m];
        if (!s.texture || !(s.tex_strength > 0.0f)) continue;
        areas[f] = facet_area(sc, f);
        samples[f] = sampled_variance(sc, f, s);
        st[m].area += areas[f];
        st[m].weighted += double(areas[f]) * samples[f];
    }
    for (uint32_t f = 0; f < F; ++f) {
        if (f >= sc.material.size() || !(areas[f] > 0.0f)) continue;
        Stats& x = st[sc.material[f]];
        const float mean = x.area > 0.0 ? float(x.weighted / x.area) : 0.0f;
        const float dev = samples[f] - mean;
        samples[f] = dev;
        x.min_dev = std::min(x.min_dev, dev);
        x.max_dev = std::max(x.max_dev, dev);
    }
    for (size_t m = 0; m < mats.size(); ++m) {
        Stats& x = st[m];
        if (!(x.area > 0.0)) continue;
        float scale = std::clamp(mats[m].tex_strength, 0.0f, 1.0f);
        if (x.min_dev < 0.0f) scale = std::min(scale, 0.999f / -x.min_dev);
        const float bound = max_mean_preserving_factor(mats[m]);
        if (x.max_dev > 0.0f && std::isfinite(bound))
            scale = std::min(scale, std::max(0.0f, bound - 1.0f) / x.max_dev);
        x.scale = scale;
    }
    for (uint32_t f = 0; f < F; ++f) {
        if (f >= sc.material.size() || !(areas[f] > 0.0f)) continue;
        Stats& x = st[sc.material[f]];
        const float factor = 1.0f + x.scale * samples[f];
        factors[f] = factor;
        x.weighted_factor += double(areas[f]) * factor;
        x.min_factor = std::min(x.min_factor, factor);
        x.max_factor = std::max(x.max_factor, factor);
    }
    for (size_t m = 0; m < st.size(); ++m)
        if (st[m].area > 0.0)
            std::cout << "facetrt: physical texture material " << m
                      << ", area-weighted factor mean=" << st[m].weighted_factor / st[m].area
                      << ", range=[" << st[m].min_factor << ',' << st[m].max_factor << "]"
                      << std::endl;
    return factors;
}

uint32_t adaptive_layers(uint32_t facets, uint32_t periodic, uint32_t raster, uint32_t layers)
{
    const double pixels = double(raster) * raster;
    if (pixels <= 0.0) return layers;
    const double avg = double(facets) * double(periodic + 1u) / pixels;
    const uint32_t estimated = uint32_t(std::ceil(std::max(1.0, avg * 16.0)));
    while (layers < estimated && layers < 64u) layers = std::min(64u, layers * 2u);
    return layers;
}

}  // namespace

Project load(const std::string& path)
{
    const std::filesystem::path input(path);
    const std::string xml = read_text(path);
    const float width = std::max(0.01f, xml_float(xml, "sceneSizeX", 8.0f));
    const float depth = std::max(0.01f, xml_float(xml, "sceneSizeY", 8.0f));
    const float height = std::max(0.01f, xml_float(xml, "Height", 4.0f));
    const float voxel = std::max(0.01f, xml_float(xml, "voxelSize", 1.0f));
    dem::HeightField dem;  // readDemHeightField (facetrtcore.cpp:2652-2697)
    const std::string dem_enabled = trim(first_tag(xml, "isDEM"));
    if (dem_enabled.empty() || dem_enabled == "1") {
        const std::string file = trim(first_tag(xml, "DEM"));
        if (!file.empty()) dem = dem::read_height_field(resolve(input, file));
    }
    Project P;
    P.periodic = uint32_t(
        std::clamp(int(std::lround(xml_float(xml, "periodicNeighborCount", 0.0f))), 0, 20));
    P.periodic_x = width;
    P.periodic_z = depth;
    if (std::max(width, depth) >= 1000.0f) {
        P.raster = 2048;
        P.layers = 16;
    }
    P.params = parameters_from_input(xml, input);
    P.strength = std::clamp(xml_float(xml, "backgroundAngularStrength", 0.0f), 0.0f, 1.0f);
    const std::string model = trim(first_tag(xml, "backgroundHeterogeneity"));
    if (!model.empty() && model != "Hapke" && model != "hapke") P.strength = 0.0f;
    const Coefficients coefficients = load_coefficients(xml, input);
    std::string angles = first_tag(xml, "lightAngle");
    const size_t nested = angles.find('>');
    if (nested != std::string::npos) angles = angles.substr(nested + 1);
    std::istringstream av(angles);
    char sep = 0;
    if (!(av >> P.sun_zenith >> sep >> P.sun_azimuth)) {
        P.sun_zenith = 30.0f;
        P.sun_azimuth = 135.0f;
    }
    host::HostScene& sc = P.scene;
    for (const std::string& obj : object_blocks(xml)) {
        const auto meshes = name_list(first_tag(obj, "meshNames"));
        const auto spectral = name_list(first_tag(obj, "spectralNames"));
        const auto thermal = name_list(first_tag(obj, "thermalNames"));
        const auto physical = name_list(first_tag(obj, "bioNames"));
        const size_t count = std::max<size_t>(1, std::max(meshes.size(), std::max(spectral.size(), thermal.size())));
        std::vector<Binding> bindings;
        for (size_t i = 0; i < count; ++i) {
            Surface m = P.params.object;
            const std::string type = trim(first_tag(obj, "componentType"));
            m.component = type == "Soil" ? 1 : type == "Vegetation" ? 2 : type == "Building" ? 3
                          : type == "Water"                          ? 5
                                                                     : 0;
            auto pick = [i](const std::vector<std::string>& v) {
                return v.empty() ? std::string{} : v[std::min(i, v.size() - 1)];
            };
            load_surface(xml, pick(spectral), pick(thermal), P.params.wavelengths, coefficients,
                         input, m);
            const std::string phys_name = pick(physical);
            const std::string phys = named_block(xml, "surfaceEnergy", phys_name);
            if (!phys.empty()) {
                m.pv = xml_float(phys, "photovoltaic", 0) > 0.5f;
                m.vegetation = xml_float(phys, "vegetation", 1) > 0.5f && !m.pv;
                m.eta25 = xml_float(phys, "eta25", .22f);
                m.gamma = xml_float(phys, "gamma", -.0035f);
                m.bif = xml_float(phys, "bifaciality", 0);
                m.hcap = xml_float(phys, "heatCapacityPerArea", 60000);
                m.conv = xml_float(phys, "convectiveScale", 1);
                if (m.pv && (!(m.eta25 >= 0 && m.eta25 <= .5f) || !(m.gamma >= -.02f && m.gamma <= 0) ||
                             !(m.bif >= 0 && m.bif <= 1) || !(m.hcap >= 0) || !(m.conv > 0)))
                    throw std::runtime_error("Invalid photovoltaic material parameters: " + phys_name);
                if (m.pv && (m.tir_t > 1e-6f || std::any_of(m.et.begin(), m.et.end(),
                                                            [](float x) { return x > 1e-6f; })))
                    throw std::runtime_error("Photovoltaic surface must be opaque: " + phys_name);
            }
            const uint32_t index = uint32_t(P.materials.size());
            if (m.pv) m.component = 4;
            P.materials.push_back(std::move(m));
            bindings.push_back({pick(meshes), index});
        }
        std::string file = trim(first_tag(obj, "fileName"));
        if (file.empty()) file = trim(first_tag(obj, "objectfile"));
        const Geometry g = file.empty() ? cube(obj) : read_obj(resolve(input, file));
        for (Placement pl : read_placements(input, obj, width, depth)) {
            pl.z += dem.above_minimum(pl.x, pl.y, width, depth);
            append_geometry(sc, g, pl, width, depth, height, bindings);
        }
    }
    sc.leaf = sc.facets();
    const uint32_t ground = uint32_t(P.materials.size());
    P.materials.push_back(P.params.ground);
    append_ground(sc, width, depth, voxel, P.raster / 4u, ground, dem);
    const uint32_t initial = P.layers;
    P.layers = adaptive_layers(sc.facets(), P.periodic, P.raster, P.layers);
    if (P.layers != initial)
        std::cout << "facetrt: automatically increased A-buffer layers from " << initial << " to "
                  << P.layers << " for " << sc.facets() << " facets" << std::endl;
    const float big = std::numeric_limits<float>::max(), low = std::numeric_limits<float>::lowest();
    sc.lo = {big, big, big};
    sc.hi = {low, low, low};
    for (const facetcu_vertex& v : sc.vertices)
        for (int a = 0; a < 3; ++a) {
            sc.lo[a] = std::min(sc.lo[a], v.position[a]);
            sc.hi[a] = std::max(sc.hi[a], v.position[a]);
        }
    P.texture = texture_factors(sc, P.materials);
    // C views
    auto view = [](const Surface& s) {
        facetcu_surface_parameters v{};
        v.reflectance = s.r.empty() ? nullptr : s.r.data();
        v.reflectance_count = uint32_t(s.r.size());
        v.transmittance = s.t.empty() ? nullptr : s.t.data();
        v.transmittance_count = uint32_t(s.t.size());
        v.tir_reflectance = s.tir_r;
        v.tir_transmittance = s.tir_t;
        v.sunlit_temperature = s.t_sun;
        v.shaded_temperature = s.t_shade;
        return v;
    };
    for (const Surface& s : P.materials) P.optics_view.push_back(view(s));
    P.object_view = view(P.params.object);
    P.ground_view = view(P.params.ground);
    return P;
}

void spectral_view(const Project& P, facetcu_spectral_parameters* parameters)
{
    *parameters = facetcu_spectral_parameters{};
    parameters->wavelengths = P.params.wavelengths.data();
    parameters->band_count = uint32_t(P.params.wavelengths.size());
    parameters->object = P.object_view;
    parameters->ground = P.ground_view;
    parameters->materials = P.optics_view.data();
    parameters->material_count = uint32_t(P.optics_view.size());
    parameters->material_indices = P.scene.material.data();
    parameters->texture_factors = P.texture.data();
    parameters->leaf_facet_count = P.scene.leaf;
    parameters->background_angular_strength = P.strength;
    parameters->sky_temperature = P.params.sky_temperature;
    parameters->accelerated_solver = P.params.accelerated ? 1u : 0u;
}

void energy_view(const Surface& s, const facetcu_surface_parameters& optics,
                 facetcu_energy_surface* out)
{
    *out = facetcu_energy_surface{};
    out->optics = optics;
    out->energy_reflectance = s.er.empty() ? nullptr : s.er.data();
    out->energy_reflectance_count = uint32_t(s.er.size());
    out->energy_transmittance = s.et.empty() ? nullptr : s.et.data();
    out->energy_transmittance_count = uint32_t(s.et.size());
    out->surface_resistance = s.rs;
    out->specific_heat = s.c;
    out->density = s.density;
    out->thermal_conductivity = s.k;
    out->soil_moisture = s.moisture;
    out->heat_capacity_per_area = s.hcap;
    out->soil_temperature_method = s.soil_method;
    out->photovoltaic = s.pv ? 1u : 0u;
    out->vegetation = s.vegetation ? 1u : 0u;
    out->pv_eta25 = s.eta25;
    out->pv_gamma = s.gamma;
    out->pv_bifaciality = s.bif;
    out->convective_scale = s.conv;
}

}  // namespace project
}  // namespace facetcu

struct facetcu_project {
    facetcu::project::Project p;
};

extern "C" {

int facetcu_project_load(const char* path, facetcu_project** project)
{
    facetcu_set_host_error("");
    if (!path || !project) {
        facetcu_set_host_error("path and project are required");
        return FACETCU_INVALID_ARGUMENT;
    }
    *project = nullptr;
    try {
        auto* p = new facetcu_project{facetcu::project::load(path)};
        *project = p;
        return FACETCU_OK;
    } catch (const std::exception& e) {
        facetcu_set_host_error(e.what());
        return FACETCU_RUNTIME_ERROR;
    }
}

void facetcu_project_release(facetcu_project* project) { delete project; }

int facetcu_project_get_info(const facetcu_project* project, facetcu_project_info* info)
{
    if (!project || !info) return FACETCU_INVALID_ARGUMENT;
    const auto& P = project->p;
    *info = facetcu_project_info{};
    info->facet_count = P.scene.facets();
    info->leaf_facet_count = P.scene.leaf;
    info->material_count = uint32_t(P.materials.size());
    info->band_count = uint32_t(P.params.wavelengths.size());
    info->sun_zenith = P.sun_zenith;
    info->sun_azimuth = P.sun_azimuth;
    info->periodic_neighbor_count = P.periodic;
    info->periodic_size_x = P.periodic_x;
    info->periodic_size_z = P.periodic_z;
    info->raster_size = P.raster;
    info->raster_layers = P.layers;
    info->background_angular_strength = P.strength;
    for (int a = 0; a < 3; ++a) {
        info->minimum[a] = P.scene.lo[a];
        info->maximum[a] = P.scene.hi[a];
    }
    info->sky_temperature = P.params.sky_temperature;
    info->accelerated_solver = P.params.accelerated ? 1u : 0u;
    return FACETCU_OK;
}

int facetcu_project_get_geometry(const facetcu_project* project, facetcu_vertex* vertices,
                                 uint32_t* material_indices, float* texture_factors)
{
    if (!project) return FACETCU_INVALID_ARGUMENT;
    const auto& P = project->p;
    if (vertices) std::memcpy(vertices, P.scene.vertices.data(), P.scene.vertices.size() * sizeof(facetcu_vertex));
    if (material_indices) std::memcpy(material_indices, P.scene.material.data(), P.scene.material.size() * 4);
    if (texture_factors) std::memcpy(texture_factors, P.texture.data(), P.texture.size() * 4);
    return FACETCU_OK;
}

int facetcu_project_get_material(const facetcu_project* project, uint32_t index,
                                 facetcu_energy_surface* surface, uint32_t* output_component)
{
    if (!project || !surface) return FACETCU_INVALID_ARGUMENT;
    const auto& P = project->p;
    const uint32_t M = uint32_t(P.materials.size());
    if (index > M + 1) return FACETCU_INVALID_ARGUMENT;
    const facetcu::project::Surface& s =
        index < M ? P.materials[index] : (index == M ? P.params.object : P.params.ground);
    const facetcu_surface_parameters& v =
        index < M ? P.optics_view[index] : (index == M ? P.object_view : P.ground_view);
    facetcu::project::energy_view(s, v, surface);
    if (output_component) *output_component = s.component;
    return FACETCU_OK;
}

int facetcu_project_spectral_parameters(const facetcu_project* project,
                                        facetcu_spectral_parameters* parameters)
{
    if (!project || !parameters) return FACETCU_INVALID_ARGUMENT;
    facetcu::project::spectral_view(project->p, parameters);
    return FACETCU_OK;
}

}  // extern "C"

namespace facetcu {
namespace project {

void run_facetrt(const std::string& input, const std::string& result_file)
{
    using namespace host;
    const Project P = load(input);
    const HostScene& sc = P.scene;
    RunOutput r;
    const auto t0 = Clock::now();
    progress(3, "Creating CUDA context and device buffers");
    Context c;
    facetcu_config cfg{};
    cfg.raster_width = P.raster;
    cfg.raster_height = P.raster;
    cfg.max_fragments_per_pixel = P.layers;
    cfg.periodic_neighbor_count = P.periodic;
    cfg.periodic_size_x = P.periodic_x;
    cfg.periodic_size_z = P.periodic_z;
    c.check(facetcu_initialize(c.ctx, &cfg));
    c.check(facetcu_set_geometry(c.ctx, sc.vertices.data(), sc.vertices.size()));
    progress(10, "GPU visibility graph: 40 directions at " + std::to_string(P.raster) + " x " +
                     std::to_string(P.raster));
    const auto t_vis = Clock::now();
    std::vector<facetcu_direction> dirs(40);
    facetcu_hemisphere_directions(40, dirs.data());
    c.check(facetcu_build_visibility_graph(c.ctx, dirs.data(), 40, &r.graph));
    const auto t_vis_end = Clock::now();
    r.visibility_ms = ms_between(t_vis, t_vis_end);
    progress(72, "GPU sunlight visibility raster");
    const uint32_t S = sc.facets() * 2;
    const facetcu_direction sun = facetcu_sun_direction(P.sun_zenith, P.sun_azimuth);
    r.sunlit.resize(S);
    c.check(facetcu_compute_sunlit_fraction(c.ctx, &sun, r.sunlit.data()));
    const auto t_sun = Clock::now();
    r.sunlight_ms = ms_between(t_vis_end, t_sun);
    progress(82, std::string(P.params.accelerated ? "GPU accelerated" : "GPU traditional") +
                     " spectral solve of " + std::to_string(P.params.wavelengths.size()) + " bands");
    facetcu_spectral_parameters sp{};
    spectral_view(P, &sp);
    const uint32_t nb = sp.band_count;
    std::vector<float> bands(size_t(nb) * S);
    r.enhancement.resize(S);
    facetcu_band_result br{};
    c.check(facetcu_solve_bands(c.ctx, &sp, r.sunlit.data(), &sun, bands.data(),
                                r.enhancement.data(), &br));
    r.wavelengths = P.params.wavelengths;
    r.radiosity.assign(bands.begin(), bands.begin() + S);
    if (nb > 1) r.band_radiosity = std::move(bands);
    r.iterations = br.iterations;
    r.max_delta = br.max_delta;
    if (br.thermal_bands == nb) {
        r.quantity = "spectral radiance";
        r.units = "W m-2 sr-1 um-1";
    } else if (br.thermal_bands == 0) {
        r.quantity = "reflectance";
        r.units = "1";
    } else {
        r.quantity = "reflectance and spectral radiance";
        r.units = "band-dependent";
    }
    const auto t_end = Clock::now();
    r.solve_ms = ms_between(t_sun, t_end);
    r.total_ms = ms_between(t0, t_end);
    progress(100, "CUDA GPU complete");
    const std::filesystem::path parent = std::filesystem::path(result_file).parent_path();
    if (!parent.empty()) std::filesystem::create_directories(parent);
    write_web_result(result_file, sc, r);
}

}  // namespace project
}  // namespace facetcu
