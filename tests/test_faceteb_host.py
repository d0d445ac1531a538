"""Host arithmetic of the FacetEB node (no GPU): the shortwave spectrum's
spectral-acceleration windows and per-band irradiances against the
reference's own ShortwaveSpectrum (oracle/_ref), bit for bit, and the
SurfaceParameters defaults (models/histream/src/facetrt/facetrtcore.cpp
:113-138, :2458-2541, :3485-3536)."""
import numpy as np
import pytest

from streamsim_gb300 import facetcu

WAVELENGTHS = [400.0, 450.0, 0.65, 1000.0, 1650.0, 2399.0, 2500.0, 3000.0, 10000.0]


def _spectra():
    rng = np.random.default_rng(11)
    d = rng.uniform(0.0, 2.0, 1500).astype(np.float32)
    f = rng.uniform(0.0, 1.0, 1700).astype(np.float32)
    d[5] = np.nan
    f[7] = -3.0
    d[900:950] = 0.0
    f[900:950] = 0.0
    solar = np.exp(-((np.arange(2001) - 150.0) / 700.0) ** 2).astype(np.float32)
    return [(None, None), (d, f), (solar, 0.2 * solar), (d[:1], f[:1]),
            (np.zeros(50, np.float32), np.zeros(50, np.float32)),
            (np.full(2500, 1.0, np.float32), np.full(2600, 0.5, np.float32))]


@pytest.mark.parametrize("width", [1, 7, 100, 333, 1000])
def test_windows_match_reference_bit_for_bit(reference, width):
    for spectrum in _spectra():
        for total, cosz in ((800.0, 0.866), (300.0, 0.05), (0.0, 0.8), (650.0, 5e-5),
                            (-10.0, 0.5), (1200.0, 0.2)):
            w0, bd0, bf0 = reference.shortwave_windows(total, cosz, spectrum[0], spectrum[1], 0.8,
                                                       width, WAVELENGTHS)
            w1, _, bd1, bf1 = facetcu.shortwave_windows(total, cosz, spectrum[0], spectrum[1],
                                                        0.8, width, WAVELENGTHS)
            assert w0.shape == w1.shape, (width, total, cosz)
            assert np.array_equal(w0.astype(np.float32).view(np.uint32),
                                  w1.astype(np.float32).view(np.uint32))
            assert np.array_equal(bd0.view(np.uint32), bd1.view(np.uint32))
            assert np.array_equal(bf0.view(np.uint32), bf1.view(np.uint32))


def test_windows_direct_fraction_of_the_flat_spectrum(reference):
    for fraction in (0.0, 0.35, 1.0):
        w0, bd0, bf0 = reference.shortwave_windows(700.0, 0.7, None, None, fraction, 100,
                                                   WAVELENGTHS)
        w1, _, bd1, bf1 = facetcu.shortwave_windows(700.0, 0.7, None, None, fraction, 100,
                                                    WAVELENGTHS)
        assert np.array_equal(w0, w1) and np.array_equal(bd0, bd1) and np.array_equal(bf0, bf1)


def test_windows_cover_the_spectrum():
    # 2001 flat samples, width 100: 20 windows centred on 50, 150, ..., 1950;
    # the direct normal beam is scaled so that its horizontal part is the
    # direct share of the total, capped at 1400 W m-2 normal
    w, arr, _, _ = facetcu.shortwave_windows(800.0, 0.5, direct_fraction=0.8, window_width=100)
    assert len(w) == 20 and list(w[:, 2]) == [50 + 100 * i for i in range(20)]
    horizontal = (w[:, 0] * 0.5).sum() + w[:, 1].sum()
    assert abs(horizontal - 800.0) < 0.1
    capped, _, _, _ = facetcu.shortwave_windows(800.0, 0.2, direct_fraction=0.8)
    assert abs(capped[:, 0].sum() - 1400.0) < 0.1


def test_windows_errors():
    lib = facetcu.load()
    spec = facetcu.ShortwaveSpectrum(None, None, 0, 0.8, 0)
    count = facetcu.C.c_uint32(0)
    assert lib.facetcu_shortwave_windows(facetcu.C.byref(spec), 800.0, 0.5, None, 0, None, 0,
                                         facetcu.C.byref(count), None, None) == facetcu.INVALID_ARGUMENT
    spec.window_width = 100
    assert lib.facetcu_shortwave_windows(facetcu.C.byref(spec), 800.0, 0.5, None, 0, None, 0,
                                         facetcu.C.byref(count), None, None) == facetcu.OVERFLOW_ERROR
    assert count.value == 20
    assert lib.facetcu_shortwave_windows(None, 800.0, 0.5, None, 0, None, 0,
                                         facetcu.C.byref(count), None, None) == facetcu.INVALID_ARGUMENT


def test_energy_surface_defaults_are_the_reference_defaults():
    s = facetcu.EnergySurfaceParameters()
    facetcu.load().facetcu_energy_surface_defaults(facetcu.C.byref(s))
    py = facetcu.EnergySurface()
    for name, _ in facetcu.EnergySurfaceParameters._fields_:
        if name.startswith(("optics", "energy_")):
            continue
        assert np.isclose(float(getattr(s, name)), float(getattr(py, name))), name
    assert s.optics.reflectance_count == 1 and s.optics.transmittance_count == 1
    assert np.isclose(s.optics.tir_reflectance, 0.03) and s.optics.tir_transmittance == 0.0
    assert (s.surface_resistance, s.soil_temperature_method, s.vegetation) == (120.0, 1, 1)


def test_time_tokens_and_default_meteorology():
    from streamsim_gb300 import faceteb
    assert faceteb.time_token(1.0) == "DOY1_00-00"
    assert faceteb.time_token(172.5) == "DOY172_12-00"
    assert faceteb.time_token(10.99999) == "DOY11_00-00"  # 1439.99 min round up to the next day
    assert faceteb.time_token(3.0208333) == "DOY3_00-30"
    rows = faceteb.default_meteorology(4, 1800.0)
    assert [r["node"] for r in rows] == [0, 1, 2, 3]
    assert np.float32(rows[3]["julian_time"]) == np.float32(1.0) + np.float32(3 * 1800.0 / 86400.0)
    assert rows[0]["pressure"] == 839.0 and rows[0]["longwave"] == 320.0


def test_read_meteorology(tmp_path):
    from streamsim_gb300 import faceteb
    p = tmp_path / "meteo.txt"
    p.write_text("julian T e p u sw lw\n"
                 "172.25 18.5 12.0 1000 1.5 120 330\n"
                 "bad row here\n"
                 "172.5 24 15 1001 2.0 800 350\n"
                 "172.75 22 14\n")
    rows = faceteb.read_meteorology(str(p))
    assert [r["node"] for r in rows] == [0, 2]
    assert rows[1]["shortwave"] == 800.0 and rows[1]["air_temperature"] == 24.0
