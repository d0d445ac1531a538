"""Sensor-image products on the host (no GPU): the float TIFF writer's
layout (server.mjs:1907-1975), file names (:706-717), band labels
(:1140-1153), and the image oracle (a restatement of server.mjs:1127-1420)
on scenes whose images are known."""
import math
import struct

import numpy as np

from oracle import image_oracle as io
from streamsim_gb300 import sensor_image as si


def test_tiff_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.uniform(0, 1, (3, 5, 7)).astype(np.float32)
    img[1, 2, 3] = np.inf
    names = si.band_names([450.0, 0.65, 10000.0])
    p = si.write_float_tiff(str(tmp_path / "a.tif"), img, names)
    raw = open(p, "rb").read()
    assert raw[:4] == b"II*\x00" and struct.unpack_from("<I", raw, 4)[0] == 8
    n = struct.unpack_from("<H", raw, 8)[0]
    tags = [struct.unpack_from("<HHII", raw, 10 + 12 * i) for i in range(n)]
    assert n == 13 and [t[0] for t in tags] == [256, 257, 258, 259, 262, 270, 273, 277, 278,
                                                279, 284, 338, 339]
    assert tags[0][3] == 7 and tags[1][3] == 5 and tags[7][3] == 3
    assert tags[9][3] == 3 * 5 * 7 * 4 and tags[6][3] % 4 == 0
    bits = struct.unpack_from("<3H", raw, tags[2][3])
    assert bits == (32, 32, 32)
    back, desc = si.read_float_tiff(p)
    assert desc == ("HiStream image bands: {Reflectance [-] @ 450 nm, Reflectance [-] @ 0.65 nm, "
                    "Spectral radiance [W m-2 sr-1 um-1] @ 10000 nm}")
    expect = img.copy()
    expect[1, 2, 3] = np.nan
    assert np.array_equal(back, expect, equal_nan=True)
    # one band: 12 entries, BitsPerSample inline
    p1 = si.write_float_tiff(str(tmp_path / "b.tif"), img[0], ["温度 [K]"])
    raw1 = open(p1, "rb").read()
    assert struct.unpack_from("<H", raw1, 8)[0] == 12
    assert struct.unpack_from("<HHII", raw1, 10 + 12 * 2)[3] == 32
    b1, d1 = si.read_float_tiff(p1)
    assert np.array_equal(b1[0], img[0]) and d1.endswith(")\xa6 [K]}")  # low bytes of the label


def test_output_names():
    assert si.output_tiff_name("eFacetRT", 30, 135, 0, 0) == \
        "SZA=30.00_SAA=135.00_VZA=0.00_VAA=0.00_f.tif"
    assert si.output_tiff_name("eFacetEB", vza=12.345, vaa=7, time_token="DOY172_12-00") == \
        "T=DOY172_12-00_VZA=12.35_VAA=7.00_f.tif"
    assert si.output_tiff_name("eFacetRT", 1, 2, 3, 4, atmosphere=True).endswith("_f_a.tif")


def _quad(x0, x1, z0, z1, y=0.0):
    a, b, c, d = [x0, y, z0], [x1, y, z0], [x1, y, z1], [x0, y, z1]
    return np.array([[a, d, c], [a, c, b]], np.float64)  # normals +y


def test_oracle_nadir_sees_the_ground_grid():
    # a 4 x 4 m ground plane seen from nadir by a parallel 16 x 16 sensor:
    # every output pixel sees it, from above (side 0)
    cam = io.Camera(16, 16, False, 0.0, 0.0, scene_x=4.0, scene_y=4.0)
    idx, observed = io.side_image(cam, _quad(-2.0, 2.0, -2.0, 2.0))
    assert np.all(idx >= 0) and set(np.unique(idx)) <= {0, 2}
    # a smaller raised square occludes the ground over its own extent
    geo = np.concatenate([_quad(-2.0, 2.0, -2.0, 2.0), _quad(-0.5, 0.5, -0.5, 0.5, 1.0)])
    idx2, _ = io.side_image(cam, geo)
    assert np.any(idx2 >= 4) and np.all(idx2[idx2 >= 4] % 2 == 0)
    frac = np.mean(idx2 >= 4)
    assert abs(frac - 1.0 / 16.0) < 0.05


def test_oracle_perspective_sky():
    cam = io.Camera(24, 16, True, 80.0, 0.0, fov=60.0, scene_x=10.0, scene_y=10.0,
                    position=(5.0, 5.0, 1.5))
    zen = io.sky_zenith(cam)
    assert np.isfinite(zen[0]).all() and np.isnan(zen[-1]).all()  # top rows see the sky
    v = io.sky_value(550.0, 45.0, False)
    assert 0.002 <= v <= 0.85
    t = io.sky_value(11000.0, 30.0, True, 250.0)
    assert 230.0 < t < 250.0  # brightness temperature below the sky temperature
    assert math.isclose(io.inverse_planck(11000.0, io.planck(11000.0, 300.0)), 300.0,
                        rel_tol=1e-12)
