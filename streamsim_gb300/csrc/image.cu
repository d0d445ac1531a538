// image.cu — sensor images of per-side values (the reference's
// writeRadiosityTiffForAngle, server.mjs:1127-1600, a JavaScript routine of
// its Node backend that runs on the host, pixel loop by pixel loop).
//
// Here the raster runs on the device:
//   k_prepare   per facet: its three vertices projected to the sensor
//               (viewVertex :1295-1307) and the side it shows (:1309-1317)
//   k_depth     a warp per facet over its pixel box: the barycentric test at
//               pixel centres (:1335-1347) and atomicMax of the depth, as an
//               order-preserving 64-bit key of the double
//   k_index     the same traversal: the smallest facet index among those at
//               the nearest depth, i.e. the facet the reference's sequential
//               loop keeps (it replaces a pixel only for a strictly nearer
//               depth)
//   k_observed  facet -> observed side index image
//   k_nadir     a parallel sensor's output grid mapped back into the
//               observed image (:1363-1387)
//   k_fill      per band and pixel: the side's value, else for a
//               perspective sensor the analytic sky (skyOutputValue
//               :1229-1255, no atmosphere table), else NaN
// Every coordinate is a double, computed in the reference's operation order
// (this file is compiled with -fmad=false), so the side index image is the
// reference's arithmetic exactly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "internal.h"

namespace facetcu {
namespace image {
namespace {

__device__ __forceinline__ double ddot(const double* a, const double* b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

struct Proj {
    double x, y, depth;
    int valid;
};

__device__ Proj project(const Camera& c, const double* p)
{
    Proj r;
    if (!c.perspective) {
        r.x = (ddot(p, c.right) - c.min_x) / c.range_x * double(c.width);
        r.y = (c.max_y - ddot(p, c.up)) / c.range_y * double(c.height);
        r.depth = ddot(p, c.out);
        r.valid = 1;
        return r;
    }
    const double rel[3] = {p[0] - c.cam_pos[0], p[1] - c.cam_pos[1], p[2] - c.cam_pos[2]};
    const double depth = ddot(rel, c.forward);
    const double half_w = c.tan_half * double(c.width) / double(c.height);
    r.x = (0.5 + ddot(rel, c.right) / (2.0 * depth * half_w)) * double(c.width);
    r.y = (0.5 - ddot(rel, c.up) / (2.0 * depth * c.tan_half)) * double(c.height);
    r.depth = -depth;
    r.valid = depth > 1e-6 ? 1 : 0;
    return r;
}

__device__ __forceinline__ double edge_fn(const Proj& a, const Proj& b, double x, double y)
{
    return (x - a.x) * (b.y - a.y) - (y - a.y) * (b.x - a.x);
}

__device__ __forceinline__ unsigned long long depth_key(double d)
{
    const long long b = __double_as_longlong(d);
    return b >= 0 ? (static_cast<unsigned long long>(b) | 0x8000000000000000ull)
                  : ~static_cast<unsigned long long>(b);
}

__global__ void k_prepare(uint32_t F, const facetcu_vertex* __restrict__ V, Camera c,
                          Proj* __restrict__ proj, int32_t* __restrict__ side)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    double p[3][3];
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) p[k][a] = double(V[3 * size_t(f) + k].position[a]);
    const double e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    const double e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
    const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                         e1[0] * e2[1] - e1[1] * e2[0]};
    double d[3];
    if (c.perspective) {
        for (int a = 0; a < 3; ++a) d[a] = c.cam_pos[a] - (p[0][a] + p[1][a] + p[2][a]) / 3.0;
    } else {
        for (int a = 0; a < 3; ++a) d[a] = c.out[a];
    }
    side[f] = int32_t(2 * f + (ddot(n, d) >= 0.0 ? 0 : 1));
    for (int k = 0; k < 3; ++k) proj[3 * size_t(f) + k] = project(c, p[k]);
}

// The pixel box of facet f and its barycentric test; calls visit(pixel,
// depth) for every covered pixel, the warp's lanes striding the box.
template <typename Visit>
__device__ __forceinline__ void cover(const Camera& c, const Proj* __restrict__ proj, uint32_t f,
                                      uint32_t lane, Visit visit)
{
    const Proj a = proj[3 * size_t(f)], b = proj[3 * size_t(f) + 1], cc = proj[3 * size_t(f) + 2];
    if (!a.valid || !b.valid || !cc.valid) return;
    const double area = edge_fn(a, b, cc.x, cc.y);
    if (fabs(area) < 1e-10) return;
    const double W = double(c.width), H = double(c.height);
    const double x0 = fmax(0.0, floor(fmin(fmin(a.x, b.x), cc.x)));
    const double x1 = fmin(W - 1.0, ceil(fmax(fmax(a.x, b.x), cc.x)) - 1.0);
    const double y0 = fmax(0.0, floor(fmin(fmin(a.y, b.y), cc.y)));
    const double y1 = fmin(H - 1.0, ceil(fmax(fmax(a.y, b.y), cc.y)) - 1.0);
    if (!(x1 >= x0) || !(y1 >= y0)) return;
    const long long bx = (long long)(x1 - x0) + 1, by = (long long)(y1 - y0) + 1;
    const long long n = bx * by;
    for (long long i = lane; i < n; i += 32) {
        const double x = x0 + double(i % bx), y = y0 + double(i / bx);
        const double sx = x + 0.5, sy = y + 0.5;
        const double wa = edge_fn(b, cc, sx, sy) / area;
        const double wb = edge_fn(cc, a, sx, sy) / area;
        const double wc = 1.0 - wa - wb;
        if (wa < -1e-7 || wb < -1e-7 || wc < -1e-7) continue;
        const double depth = wa * a.depth + wb * b.depth + wc * cc.depth;
        visit(size_t(y) * c.width + size_t(x), depth);
    }
}

__global__ void k_depth(uint32_t F, Camera c, const Proj* __restrict__ proj,
                        unsigned long long* __restrict__ zbuf)
{
    const uint32_t f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (f >= F) return;
    cover(c, proj, f, threadIdx.x & 31u,
          [&](size_t px, double depth) { atomicMax(zbuf + px, depth_key(depth)); });
}

__global__ void k_index(uint32_t F, Camera c, const Proj* __restrict__ proj,
                        const unsigned long long* __restrict__ zbuf, int32_t* __restrict__ index)
{
    const uint32_t f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (f >= F) return;
    cover(c, proj, f, threadIdx.x & 31u, [&](size_t px, double depth) {
        if (depth_key(depth) == zbuf[px]) atomicMin(index + px, int32_t(f));
    });
}

constexpr int32_t kEmpty = 0x7f7f7f7f;  // the index buffer's fill: above any facet index

__global__ void k_observed(size_t n, const int32_t* __restrict__ side, int32_t* __restrict__ img,
                           uint32_t* __restrict__ count)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t f = img[i];
    const bool seen = f != kEmpty;
    img[i] = seen ? side[f] : -1;
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, seen);
    if ((threadIdx.x & 31u) == unsigned(__ffs(active) - 1)) atomicAdd(count, unsigned(__popc(m)));
}

__global__ void k_nadir(Camera c, const int32_t* __restrict__ observed, int32_t* __restrict__ out,
                        uint32_t* __restrict__ count)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t n = size_t(c.width) * c.height;
    if (i >= n) return;
    const uint32_t x = uint32_t(i % c.width), y = uint32_t(i / c.width);
    const double rw = double(c.width > 1 ? c.width - 1 : 1);
    const double rh = double(c.height > 1 ? c.height - 1 : 1);
    int32_t s = -1;
    const double wx = c.orth_max_x - double(y) / rh * c.orth_north;
    const double wz = c.orth_min_z + double(x) / rw * c.orth_east;
    if (!(wx < -c.scene_w / 2.0 || wx > c.scene_w / 2.0 || wz < -c.scene_d / 2.0 ||
          wz > c.scene_d / 2.0)) {
        const double p[3] = {wx, 0.0, wz};
        const Proj src = project(c, p);
        if (src.valid) {
            const double tx = trunc(src.x), ty = trunc(src.y);
            if (tx >= 0.0 && tx < double(c.width) && ty >= 0.0 && ty < double(c.height))
                s = observed[size_t(ty) * c.width + size_t(tx)];
        }
    }
    out[i] = s;
    if (s >= 0) atomicAdd(count, 1u);
}

__device__ double planck_js(double wl_nm, double temperature)
{
    const double um = wl_nm > 50.0 ? wl_nm / 1000.0 : wl_nm;
    return 1.19104e8 / (pow(um, 5.0) * expm1(14387.7 / (temperature * um)));
}

__device__ double inverse_planck_js(double wl_nm, double radiance)
{
    const double um = wl_nm > 50.0 ? wl_nm / 1000.0 : wl_nm;
    return 14387.7 / (um * log(1.19104e8 / (radiance * pow(um, 5.0)) + 1.0));
}

constexpr double kPiD = 3.141592653589793;

__device__ double sky_value(double wl_nm, double zenith_deg, bool as_temperature, double sky_t)
{
    const double wl = (wl_nm > 0.0 && wl_nm <= 50.0) ? wl_nm * 1000.0 : wl_nm;
    const double zr = fmax(0.0, fmin(89.5, zenith_deg)) * kPiD / 180.0;
    const double visibility = 23.0;
    if (wl <= 2500.0) {
        const double weight = fmax(0.06, fmin(2.0, pow(550.0 / fmax(350.0, fmin(2500.0, wl)), 1.8)));
        const double aerosol = fmax(0.4, fmin(2.3, 23.0 / visibility));
        const double cz = fmax(0.12, cos(zr));
        const double air_mass = 1.0 / cz;
        const double trans = exp(-(0.10 * weight + 0.025 * aerosol) * air_mass);
        const double boost = 1.0 + 0.55 * (1.0 - cz);
        return fmax(0.002, fmin(0.85, (1.0 - trans) * 0.55 * weight * boost + 0.008 * aerosol * boost));
    }
    const double cz = fmax(0.05, cos(zr));
    const double emis = 0.72;
    const double frac = fmax(emis, fmin(1.0, 1.0 - (1.0 - emis) * cz));
    const double radiance = planck_js(wl, sky_t) * frac;
    return as_temperature ? inverse_planck_js(wl, radiance) : radiance;
}

__global__ void k_fill(Camera c, uint32_t nb, size_t S, const int32_t* __restrict__ sides,
                       const float* __restrict__ values, const float* __restrict__ wavelengths,
                       int as_temperature, double sky_t, float* __restrict__ image)
{
    const size_t n = size_t(c.width) * c.height;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n * nb) return;
    const uint32_t b = uint32_t(i / n);
    const size_t px = i % n;
    const int32_t s = sides[px];
    float v = __int_as_float(0x7fc00000);  // NaN
    if (s >= 0) {
        v = values[size_t(b) * S + size_t(s)];
    } else if (c.perspective) {
        const uint32_t x = uint32_t(px % c.width), y = uint32_t(px / c.width);
        const double vs = c.tan_half, hs = c.tan_half * double(c.width) / double(c.height);
        const double sy = (1.0 - 2.0 * (double(y) + 0.5) / double(c.height)) * vs;
        const double sx = (2.0 * (double(x) + 0.5) / double(c.width) - 1.0) * hs;
        double ray[3];
        for (int a = 0; a < 3; ++a) ray[a] = c.forward[a] + c.right[a] * sx + c.up[a] * sy;
        const double len = sqrt(ray[0] * ray[0] + ray[1] * ray[1] + ray[2] * ray[2]);
        if (len > 1e-9) {
            for (int a = 0; a < 3; ++a) ray[a] = ray[a] / len;
        } else {
            for (int a = 0; a < 3; ++a) ray[a] = c.forward[a];
        }
        if (ray[1] > 0.0) {
            // the sky image holds the zenith angle as a float
            const float zen = float(acos(fmax(0.0, fmin(1.0, ray[1]))) * 180.0 / kPiD);
            const double wl = double(wavelengths[b]);
            const double wl_nm = (wl > 0.0 && wl <= 50.0) ? wl * 1000.0 : wl;
            v = float(sky_value(wl_nm, double(zen), as_temperature != 0, sky_t));
        }
    }
    image[i] = v;
}

inline unsigned blocks(size_t n, unsigned b) { return unsigned((n + b - 1) / b); }

}  // namespace

namespace {
double hdot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double hlen(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
void hnormalize(double* v, const double* fallback)
{
    const double n = hlen(v);
    for (int a = 0; a < 3; ++a) v[a] = n > 1e-9 ? v[a] / n : fallback[a];
}
void hcross(const double* a, const double* b, double* r)
{
    const double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2],
                 z = a[0] * b[1] - a[1] * b[0];
    r[0] = x;
    r[1] = y;
    r[2] = z;
}
}  // namespace

Camera camera(const facetcu_sensor& s, double* naming_zenith, double* naming_azimuth)
{
    // server.mjs:1134-1301 in the same operation order
    const double pi = 3.141592653589793;
    Camera c{};
    c.width = s.width ? s.width : 512;
    c.height = s.height ? s.height : 512;
    c.perspective = s.perspective ? 1 : 0;
    c.scene_w = std::max(1e-6, s.scene_x != 0.0 && std::isfinite(s.scene_x) ? s.scene_x : 1.0);
    c.scene_d = std::max(1e-6, s.scene_y != 0.0 && std::isfinite(s.scene_y) ? s.scene_y : 1.0);
    const bool placed = std::isfinite(s.position[0]) && std::isfinite(s.position[1]) &&
                        std::isfinite(s.position[2]);
    const double world[3] = {placed ? s.position[0] : c.scene_w / 2,
                             placed ? s.position[1] : c.scene_d / 2, placed ? s.position[2] : 3000.0};
    c.cam_pos[0] = world[0] - c.scene_w / 2;
    c.cam_pos[1] = std::max(0.01, world[2]);
    c.cam_pos[2] = world[1] - c.scene_d / 2;
    const double z = (std::isfinite(s.view_zenith) ? s.view_zenith : 0.0) * pi / 180;
    const double a = (std::isfinite(s.view_azimuth) ? s.view_azimuth : 0.0) * pi / 180;
    c.out[0] = std::sin(z) * std::cos(a);
    c.out[1] = std::cos(z);
    c.out[2] = std::sin(z) * std::sin(a);
    for (int k = 0; k < 3; ++k) c.forward[k] = -c.out[k];
    // cameraBasis: north-up for a parallel sensor, world-up for a perspective one
    const double north[3] = {1, 0, 0}, world_up[3] = {0, 1, 0};
    const double* preferred = c.perspective ? world_up : north;
    const double* fallback = c.perspective ? north : world_up;
    double up[3];
    const double pp = hdot(preferred, c.forward);
    for (int k = 0; k < 3; ++k) up[k] = preferred[k] - pp * c.forward[k];
    if (hlen(up) <= 1e-9) {
        const double q = hdot(fallback, c.forward);
        for (int k = 0; k < 3; ++k) up[k] = fallback[k] - q * c.forward[k];
    }
    const double fx[3] = {1, 0, 0}, fz[3] = {0, 0, 1};
    hnormalize(up, fx);
    hcross(c.forward, up, c.right);
    hnormalize(c.right, fz);
    double up2[3];
    hcross(c.right, c.forward, up2);
    hnormalize(up2, up);
    for (int k = 0; k < 3; ++k) c.up[k] = up2[k];
    c.tan_half = 1.0;
    if (c.perspective) {
        const double fov = std::max(0.1, std::min(120.0, s.fov != 0.0 && std::isfinite(s.fov) ? s.fov : 60.0));
        c.tan_half = std::tan(fov * 0.5 * pi / 180);
    }
    const double W = c.width, H = c.height, aspect = W / H;
    double mnx, mxx, mny, mxy;
    if (c.perspective) {
        mnx = -1;
        mxx = 1;
        mny = -1;
        mxy = 1;
    } else {
        mnx = INFINITY;
        mxx = -INFINITY;
        mny = INFINITY;
        mxy = -INFINITY;
        const double corners[4][3] = {{-c.scene_w / 2, 0, -c.scene_d / 2},
                                      {-c.scene_w / 2, 0, c.scene_d / 2},
                                      {c.scene_w / 2, 0, -c.scene_d / 2},
                                      {c.scene_w / 2, 0, c.scene_d / 2}};
        for (const auto& p : corners) {
            const double px = hdot(p, c.right), py = hdot(p, c.up);
            mnx = std::min(mnx, px);
            mxx = std::max(mxx, px);
            mny = std::min(mny, py);
            mxy = std::max(mxy, py);
        }
    }
    double rx = std::max(1e-6, mxx - mnx), ry = std::max(1e-6, mxy - mny);
    const double cx = (mnx + mxx) / 2, cy = (mny + mxy) / 2;
    if (rx / ry > aspect)
        ry = rx / aspect;
    else
        rx = ry * aspect;
    rx *= 1 + 0.5 / W;
    ry *= 1 + 0.5 / H;
    c.range_x = rx;
    c.range_y = ry;
    c.min_x = cx - rx / 2;
    c.max_y = cy + ry / 2;
    double east = c.scene_d, northr = c.scene_w;
    if (east / northr > aspect)
        northr = east / aspect;
    else
        east = northr * aspect;
    c.orth_east = east / 1.0;
    c.orth_north = northr / 1.0;
    c.orth_min_z = -c.orth_east / 2;
    c.orth_max_x = c.orth_north / 2;
    if (naming_zenith && naming_azimuth) {
        if (c.perspective) {
            const double h = std::hypot(c.out[0], c.out[2]);
            *naming_zenith = std::acos(std::max(-1.0, std::min(1.0, c.out[1]))) * 180 / pi;
            *naming_azimuth =
                h < 1e-9 ? 0.0 : std::fmod(std::atan2(c.out[2], c.out[0]) * 180 / pi + 360, 360.0);
        } else {
            *naming_zenith = s.view_zenith;
            *naming_azimuth = s.view_azimuth;
        }
    }
    return c;
}

void render(const Camera& c, uint32_t F, const facetcu_vertex* V, const float* values,
            uint32_t nb, size_t S, const float* wavelengths, bool as_temperature, double sky_t,
            Scratch& w, float* image, int32_t* sides, uint32_t* counts, cudaStream_t s)
{
    const size_t n = size_t(c.width) * c.height;
    FCU_CHECK(cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), s));
    FCU_CHECK(cudaMemsetAsync(w.zbuf, 0, n * sizeof(unsigned long long), s));
    FCU_CHECK(cudaMemsetAsync(w.index, 0x7f, n * sizeof(int32_t), s));
    if (F) {
        k_prepare<<<blocks(F, 128), 128, 0, s>>>(F, V, c, reinterpret_cast<Proj*>(w.proj), w.side);
        FCU_LAUNCH("k_prepare");
        k_depth<<<blocks(size_t(F) * 32, 256), 256, 0, s>>>(F, c, reinterpret_cast<Proj*>(w.proj),
                                                            w.zbuf);
        FCU_LAUNCH("k_depth");
        k_index<<<blocks(size_t(F) * 32, 256), 256, 0, s>>>(F, c, reinterpret_cast<Proj*>(w.proj),
                                                            w.zbuf, w.index);
        FCU_LAUNCH("k_index");
    }
    k_observed<<<blocks(n, 256), 256, 0, s>>>(n, w.side, w.index, counts);
    FCU_LAUNCH("k_observed");
    int32_t* out = w.index;
    if (!c.perspective) {
        k_nadir<<<blocks(n, 256), 256, 0, s>>>(c, w.index, sides, counts + 1);
        FCU_LAUNCH("k_nadir");
        out = sides;
    } else {
        FCU_CHECK(cudaMemcpyAsync(sides, w.index, n * 4, cudaMemcpyDeviceToDevice, s));
        FCU_CHECK(cudaMemcpyAsync(counts + 1, counts, 4, cudaMemcpyDeviceToDevice, s));
        out = sides;
    }
    if (nb) {
        k_fill<<<blocks(n * nb, 256), 256, 0, s>>>(c, nb, S, out, values, wavelengths,
                                                   as_temperature ? 1 : 0, sky_t, image);
        FCU_LAUNCH("k_fill");
    }
}

}  // namespace image
}  // namespace facetcu
