"""Sensor images on the device against the image oracle (a restatement of
the reference's writeRadiosityTiffForAngle, server.mjs:1127-1420; parity
unpinned: the reference is JavaScript and cannot run here).

The side-index images are compared exactly (the same double-precision
operations in the same order); band values are the sides' own values where a
side is seen, and the analytic sky of perspective views within 1e-6
relative (CUDA's double pow/exp/cos against the C library's)."""
import numpy as np
import pytest

from oracle import image_oracle as io
from streamsim_gb300 import facetcu, scenes, sensor_image
from tests.gpu_helpers import model_for, require_gpu

pytestmark = pytest.mark.gpu

WAVELENGTHS = [450.0, 0.865, 11000.0]


@pytest.fixture(scope="module")
def site():
    require_gpu()
    sc, _, _ = scenes.energy_site(seed=2, leaves=700, soil_cells=10)
    m = model_for(sc.vertices, 256, 64)
    rng = np.random.default_rng(3)
    values = rng.uniform(0.0, 1.0, (len(WAVELENGTHS), sc.surface_count)).astype(np.float32)
    positions = sc.vertices.reshape(-1, 3, 6)[:, :, :3]
    yield dict(scene=sc, model=m, values=values, positions=positions)
    m.close()


CASES = [
    dict(width=96, height=80, perspective=False, vza=0.0, vaa=0.0, scene_x=12.0, scene_y=12.0),
    dict(width=90, height=64, perspective=False, vza=35.0, vaa=45.0, scene_x=12.0, scene_y=12.0),
    dict(width=64, height=96, perspective=False, vza=60.0, vaa=250.0, scene_x=12.0, scene_y=10.0),
    dict(width=96, height=72, perspective=True, vza=70.0, vaa=200.0, fov=50.0, scene_x=12.0,
         scene_y=12.0, position=(9.0, 10.0, 2.5)),
    dict(width=80, height=80, perspective=True, vza=10.0, vaa=0.0, fov=40.0, scene_x=12.0,
         scene_y=12.0, position=(6.0, 6.0, 25.0)),
]


def _oracle(case, positions):
    kw = {k: v for k, v in case.items() if k != "position"}
    cam = io.Camera(position=case.get("position", (np.nan,) * 3), **kw)
    return cam, io.side_image(cam, positions)[0]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_side_index_images_match_the_oracle(site, case):
    c = CASES[case]
    s = facetcu.sensor(c["width"], c["height"], c["perspective"], c["vza"], c["vaa"],
                       c.get("fov", 0.0), c["scene_x"], c["scene_y"],
                       c.get("position", (np.nan,) * 3))
    img, idx, info = site["model"].renderSensorImage(s, site["values"], WAVELENGTHS)
    cam, want = _oracle(c, site["positions"])
    assert np.array_equal(idx, want), f"{np.sum(idx != want)} pixels differ"
    assert info["output_pixels"] == int(np.sum(want >= 0)) > 0
    expect = io.band_images(cam, want, site["values"], WAVELENGTHS)
    seen = want >= 0
    assert np.array_equal(img[:, seen], expect[:, seen])
    sky = ~seen & np.isfinite(expect[0])
    if c["perspective"] and c["vza"] > 45.0:  # a low view sees the sky
        assert sky.any()
    assert np.allclose(img[:, sky], expect[:, sky], rtol=1e-6, atol=0)
    assert np.all(np.isnan(img[:, ~seen & ~sky]))


def test_temperature_image_with_thermal_sky(site):
    c = CASES[3]
    T = np.random.default_rng(4).uniform(285.0, 320.0, (1, site["scene"].surface_count))
    s = facetcu.sensor(c["width"], c["height"], True, c["vza"], c["vaa"], c["fov"], c["scene_x"],
                       c["scene_y"], c["position"], sky_temperature=255.0, temperature_output=True)
    img, idx, _ = site["model"].renderSensorImage(s, T.astype(np.float32), [11000.0])
    cam, want = _oracle(c, site["positions"])
    expect = io.band_images(cam, want, T, [11000.0], temperature_output=True,
                            sky_temperature=255.0)
    sky = (want < 0) & np.isfinite(expect[0])
    assert sky.any() and np.all(expect[0][sky] < 255.0)
    assert np.allclose(img[0][sky], expect[0][sky], rtol=1e-6)
    assert np.array_equal(img[0][want >= 0], expect[0][want >= 0])


def test_faceteb_step_record_to_tiff(site, tmp_path):
    sc, m = site["scene"], site["model"]
    S = sc.surface_count
    rec = np.random.default_rng(6).uniform(0, 1, (S, 9 + len(WAVELENGTHS))).astype("<f4")
    rec[:, 0] = 290.0 + 20.0 * rec[:, 0]
    path = tmp_path / "energy_T=DOY172_12-00.bin"
    rec.tofile(path)
    s = facetcu.sensor(64, 48, False, 20.0, 90.0, 0.0, 12.0, 12.0)
    img, idx, info = sensor_image.faceteb_images(m, s, str(path), WAVELENGTHS)
    seen = idx >= 0
    assert np.array_equal(img[:, seen], rec[idx[seen], 9:].T)
    name = sensor_image.output_tiff_name("eFacetEB", vza=info["naming_zenith"],
                                         vaa=info["naming_azimuth"], time_token="DOY172_12-00")
    out = sensor_image.write_float_tiff(str(tmp_path / name), img,
                                        sensor_image.band_names(WAVELENGTHS))
    back, _ = sensor_image.read_float_tiff(out)
    assert np.array_equal(back, img, equal_nan=True)
    timg, tidx, _ = sensor_image.faceteb_images(m, facetcu.sensor(64, 48, False, 20.0, 90.0, 0.0,
                                                                  12.0, 12.0), str(path),
                                                WAVELENGTHS, temperature_output=True)
    assert timg.shape[0] == 1 and np.array_equal(timg[0][tidx >= 0], rec[tidx[tidx >= 0], 0])


def test_rejects_bad_arguments(site):
    m = site["model"]
    with pytest.raises(ValueError):
        m.renderSensorImage(facetcu.sensor(8, 8), site["values"], WAVELENGTHS[:1])
    with pytest.raises(ValueError):
        m.renderSensorImage(facetcu.sensor(8, 8), site["values"][:1], [np.nan])
