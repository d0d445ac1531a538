"""image_oracle.py — TEST INFRASTRUCTURE ONLY.

A restatement, in Python doubles, of the reference's sensor-image synthesis
(writeRadiosityTiffForAngle, server.mjs:1127-1420, StreamSim's Node
backend): the camera of a parallel or perspective sensor, the observed side
of every facet, the z-buffered raster of side indices (barycentric test at
pixel centres, the nearest depth wins, the first facet among equal depths),
the nadir remap of a parallel view, the sky zenith image of a perspective
view, and the per-band fill with the analytic sky (no atmosphere table).

The reference is JavaScript and no JavaScript runtime is available here, so
parity is unpinned: this restatement follows the source line by line (the
same double-precision operations in the same order; Math.hypot is taken as
sqrt(x*x + y*y + z*z), which agrees with it to the last bit or one unit in
the last place).  Only tests import it.
"""
import math

import numpy as np


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _sub(a, b):
    return [a[0] - b[0], a[1] - b[1], a[2] - b[2]]


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def _length(v):
    return math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])


def _normalize(v, fallback):
    n = _length(v)
    return [c / n for c in v] if n > 1e-9 else list(fallback)


def _basis(forward, perspective):
    north, world_up = [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]
    preferred = world_up if perspective else north
    fallback = north if perspective else world_up
    p = _dot(preferred, forward)
    up = [c - p * forward[i] for i, c in enumerate(preferred)]
    if _length(up) <= 1e-9:
        q = _dot(fallback, forward)
        up = [c - q * forward[i] for i, c in enumerate(fallback)]
    up = _normalize(up, [1.0, 0.0, 0.0])
    right = _normalize(_cross(forward, up), [0.0, 0.0, 1.0])
    return right, _normalize(_cross(right, forward), up)


def _direction(zenith, azimuth):
    z = (zenith if math.isfinite(zenith) else 0.0) * math.pi / 180
    a = (azimuth if math.isfinite(azimuth) else 0.0) * math.pi / 180
    return [math.sin(z) * math.cos(a), math.cos(z), math.sin(z) * math.sin(a)]


class Camera:
    """The sensor's camera (server.mjs:1134-1301)."""

    def __init__(self, width=512, height=512, perspective=False, vza=0.0, vaa=0.0, fov=60.0,
                 scene_x=1.0, scene_y=1.0, position=(math.nan, math.nan, math.nan)):
        self.width, self.height = int(width), int(height)
        self.perspective = bool(perspective)
        self.scene_w = max(1e-6, scene_x or 1.0)
        self.scene_d = max(1e-6, scene_y or 1.0)
        pos = list(position)
        world = pos if all(math.isfinite(v) for v in pos) else \
            [self.scene_w / 2, self.scene_d / 2, 3000.0]
        self.cam_pos = [world[0] - self.scene_w / 2, max(0.01, world[2]), world[1] - self.scene_d / 2]
        self.out = _direction(vza, vaa)
        self.forward = [-c for c in self.out]
        self.right, self.up = _basis(self.forward, self.perspective)
        self.tan_half = 1.0
        if self.perspective:
            fov_v = max(0.1, min(120.0, fov or 60.0))
            self.tan_half = math.tan(fov_v * 0.5 * math.pi / 180)
        W, H = self.width, self.height
        aspect = W / H
        if self.perspective:
            mnx, mxx, mny, mxy = -1.0, 1.0, -1.0, 1.0
        else:
            mnx, mxx, mny, mxy = math.inf, -math.inf, math.inf, -math.inf
            for c in ([-self.scene_w / 2, 0.0, -self.scene_d / 2],
                      [-self.scene_w / 2, 0.0, self.scene_d / 2],
                      [self.scene_w / 2, 0.0, -self.scene_d / 2],
                      [self.scene_w / 2, 0.0, self.scene_d / 2]):
                px, py = _dot(c, self.right), _dot(c, self.up)
                mnx, mxx = min(mnx, px), max(mxx, px)
                mny, mxy = min(mny, py), max(mxy, py)
        rx = max(1e-6, mxx - mnx)
        ry = max(1e-6, mxy - mny)
        cx, cy = (mnx + mxx) / 2, (mny + mxy) / 2
        if rx / ry > aspect:
            ry = rx / aspect
        else:
            rx = ry * aspect
        rx *= 1 + 0.5 / W
        ry *= 1 + 0.5 / H
        self.range_x, self.range_y = rx, ry
        self.min_x = cx - rx / 2
        self.max_y = cy + ry / 2
        east, north = self.scene_d, self.scene_w
        if east / north > aspect:
            north = east / aspect
        else:
            east = north * aspect
        self.orth_east, self.orth_north = east / 1.0, north / 1.0
        self.orth_min_z = -self.orth_east / 2
        self.orth_max_x = self.orth_north / 2

    def project(self, p):
        """viewVertex: (x, y, depth, valid)."""
        if not self.perspective:
            return ((_dot(p, self.right) - self.min_x) / self.range_x * self.width,
                    (self.max_y - _dot(p, self.up)) / self.range_y * self.height,
                    _dot(p, self.out), True)
        rel = _sub(p, self.cam_pos)
        depth = _dot(rel, self.forward)
        half_w = self.tan_half * self.width / self.height
        return ((0.5 + _dot(rel, self.right) / (2 * depth * half_w)) * self.width,
                (0.5 - _dot(rel, self.up) / (2 * depth * self.tan_half)) * self.height,
                -depth, depth > 1e-6)

    def naming_angles(self, vza, vaa):
        if not self.perspective:
            return vza, vaa
        o = self.out
        h = math.hypot(o[0], o[2])
        return (math.acos(max(-1.0, min(1.0, o[1]))) * 180 / math.pi,
                0.0 if h < 1e-9 else (math.atan2(o[2], o[0]) * 180 / math.pi + 360) % 360)


def _edge(a, b, x, y):
    return (x - a[0]) * (b[1] - a[1]) - (y - a[1]) * (b[0] - a[0])


def side_image(cam, positions):
    """(output side-index image (H, W) int32, observed image) for facet
    positions (F, 3, 3) (server.mjs:1319-1400)."""
    P = np.asarray(positions, np.float64).reshape(-1, 3, 3)
    F = len(P)
    W, H = cam.width, cam.height
    sides = np.empty(F, np.int64)
    proj = []
    for f in range(F):
        a, b, c = [list(map(float, P[f, k])) for k in range(3)]
        n = _cross(_sub(b, a), _sub(c, a))
        centroid = [(a[i] + b[i] + c[i]) / 3 for i in range(3)]
        d = _sub(cam.cam_pos, centroid) if cam.perspective else cam.out
        sides[f] = 2 * f + (0 if _dot(n, d) >= 0 else 1)
        proj.append([cam.project(a), cam.project(b), cam.project(c)])
    depth = np.full(W * H, -math.inf)
    index = np.full(W * H, -1, np.int64)
    for f in range(F):
        a, b, c = proj[f]
        if not (a[3] and b[3] and c[3]):
            continue
        area = _edge(a, b, c[0], c[1])
        if abs(area) < 1e-10:
            continue
        x0 = max(0, math.floor(min(a[0], b[0], c[0])))
        x1 = min(W - 1, math.ceil(max(a[0], b[0], c[0])) - 1)
        y0 = max(0, math.floor(min(a[1], b[1], c[1])))
        y1 = min(H - 1, math.ceil(max(a[1], b[1], c[1])) - 1)
        for y in range(y0, y1 + 1):
            for x in range(x0, x1 + 1):
                sx, sy = x + 0.5, y + 0.5
                wa = _edge(b, c, sx, sy) / area
                wb = _edge(c, a, sx, sy) / area
                wc = 1 - wa - wb
                if wa < -1e-7 or wb < -1e-7 or wc < -1e-7:
                    continue
                z = wa * a[2] + wb * b[2] + wc * c[2]
                px = y * W + x
                if z <= depth[px]:
                    continue
                depth[px] = z
                index[px] = sides[f]
    observed = index.reshape(H, W)
    if cam.perspective:
        return observed.astype(np.int32), observed.astype(np.int32)
    out = np.full((H, W), -1, np.int64)
    rw, rh = max(1, W - 1), max(1, H - 1)
    for y in range(H):
        wx = cam.orth_max_x - y / rh * cam.orth_north
        if wx < -cam.scene_w / 2 or wx > cam.scene_w / 2:
            continue
        for x in range(W):
            wz = cam.orth_min_z + x / rw * cam.orth_east
            if wz < -cam.scene_d / 2 or wz > cam.scene_d / 2:
                continue
            sx, sy, _, valid = cam.project([wx, 0.0, wz])
            if not valid:
                continue
            ix, iy = math.trunc(sx), math.trunc(sy)
            if ix < 0 or ix >= W or iy < 0 or iy >= H:
                continue
            s = observed[iy, ix]
            if s >= 0:
                out[y, x] = s
    return out.astype(np.int32), observed.astype(np.int32)


def sky_zenith(cam):
    """Degrees from the zenith of each perspective pixel's upward ray, NaN
    elsewhere (server.mjs:1402-1419)."""
    W, H = cam.width, cam.height
    out = np.full((H, W), np.nan, np.float32)
    if not cam.perspective:
        return out
    vs = cam.tan_half
    hs = cam.tan_half * W / H
    f, r, u = cam.forward, cam.right, cam.up
    for y in range(H):
        sy = (1 - 2 * (y + 0.5) / H) * vs
        for x in range(W):
            sx = (2 * (x + 0.5) / W - 1) * hs
            ray = _normalize([f[0] + r[0] * sx + u[0] * sy, f[1] + r[1] * sx + u[1] * sy,
                              f[2] + r[2] * sx + u[2] * sy], f)
            if ray[1] > 0:
                out[y, x] = math.acos(max(0.0, min(1.0, ray[1]))) * 180 / math.pi
    return out


def planck(wavelength_nm, temperature):
    um = wavelength_nm / 1000 if wavelength_nm > 50 else wavelength_nm
    return 1.19104e8 / (math.pow(um, 5) * math.expm1(14387.7 / (temperature * um)))


def inverse_planck(wavelength_nm, radiance):
    um = wavelength_nm / 1000 if wavelength_nm > 50 else wavelength_nm
    return 14387.7 / (um * math.log(1.19104e8 / (radiance * math.pow(um, 5)) + 1))


def sky_value(wavelength_nm, zenith_deg, as_temperature, sky_temperature=250.0, visibility=23.0):
    """skyOutputValue without an atmosphere table (server.mjs:1229-1255)."""
    wl = wavelength_nm * 1000 if 0 < wavelength_nm <= 50 else wavelength_nm
    zr = max(0.0, min(89.5, zenith_deg)) * math.pi / 180
    if wl <= 2500:
        weight = max(0.06, min(2.0, math.pow(550 / max(350.0, min(2500.0, wl)), 1.8)))
        aerosol = max(0.4, min(2.3, 23 / visibility))
        cz = max(0.12, math.cos(zr))
        air_mass = 1 / cz
        trans = math.exp(-(0.10 * weight + 0.025 * aerosol) * air_mass)
        boost = 1 + 0.55 * (1 - cz)
        return max(0.002, min(0.85, (1 - trans) * 0.55 * weight * boost + 0.008 * aerosol * boost))
    cz = max(0.05, math.cos(zr))
    emis = 0.72
    frac = max(emis, min(1.0, 1 - (1 - emis) * cz))
    radiance = planck(wl, sky_temperature) * frac
    return inverse_planck(wl, radiance) if as_temperature else radiance


def band_images(cam, side_index, values, wavelengths, temperature_output=False,
                sky_temperature=250.0):
    """Float32 images (bands, H, W): the side values where a side is seen,
    the sky where a perspective ray looks up, NaN elsewhere."""
    values = np.asarray(values, np.float32)
    zen = sky_zenith(cam)
    out = np.full((len(values),) + side_index.shape, np.nan, np.float32)
    for b in range(len(values)):
        seen = side_index >= 0
        out[b][seen] = values[b][side_index[seen]]
        wl = wavelengths[b] if b < len(wavelengths) else 1.0
        wl_nm = wl * 1000 if 0 < wl <= 50 else wl
        for y, x in zip(*np.nonzero(~seen & np.isfinite(zen))):
            out[b, y, x] = np.float32(sky_value(wl_nm, float(zen[y, x]), temperature_output,
                                                sky_temperature))
    return out
