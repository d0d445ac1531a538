"""The eFacetRT run on an XML project (runFacetRTCore with loadProjectScene,
facetRTParametersFromInput and runGpu's spectral band loop,
models/histream/src/facetrt/facetrtcore.cpp:1621-1780, 2880-3025,
3116-3161) through facetcu_run_facetrt_core, against the reference's own
makeSpectralOptics and solveCpu (oracle/_ref) run band by band on the same
scene, graph and sun raster; on flat ground and on a DEM (a GeoTIFF hill).

Tolerances: band radiosity within 1e-5 relative (FP32 gather vs the
reference's FP64-accumulated gather), the integer graph and the sunlit
fractions identical."""
import json

import numpy as np
import pytest

from oracle.pyoracle import Graph
from streamsim_gb300 import facetcu, scenes
from tests import tiff_writer
from tests.gpu_helpers import model_for, require_gpu
from tests.test_project_host import _write_project

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["flat", "dem"])
def project(tmp_path_factory, request):
    require_gpu()
    root = tmp_path_factory.mktemp("project")
    control, scene = "<periodicNeighborCount>4</periodicNeighborCount>", ""
    if request.param == "dem":  # a hill under the ground grid and the objects
        y, x = np.mgrid[0:21, 0:17] / np.array([20.0, 16.0])[:, None, None]
        z = 80.0 + 1.5 * np.exp(-((x - 0.3) ** 2 + (y - 0.6) ** 2) / 0.08)
        tiff_writer.write(str(root / "hill.tif"), z.astype(np.float32), compression=8,
                          predictor=3, tile=(16, 16))
        control += "<isDEM>1</isDEM>"
        scene = "<DEM>hill.tif</DEM>"
    path = _write_project(root, coefficients=False, bands="450,550,0.865,1650,10500",
                          extra_control=control, extra_scene=scene)
    return path, facetcu.Project(path)


def test_efacetrt_run_on_an_xml_project(reference, project, tmp_path):
    path, p = project
    out = str(tmp_path / "facetrt.json")
    assert facetcu.run_facetrt_core(path, out) == 0
    doc = json.load(open(out))
    info = p.info
    S = 2 * info["facet_count"]
    assert doc["facetCount"] == info["facet_count"]
    assert doc["leafFacetCount"] == info["leaf_facet_count"]
    assert doc["quantity"] == "reflectance and spectral radiance"
    assert doc["units"] == "band-dependent"
    assert np.allclose(doc["wavelengths"], [450, 550, 0.865, 1650, 10500])
    band = np.array(doc["bandRadiosity"], np.float32).reshape(5, S)
    assert np.array_equal(np.array(doc["radiosity"], np.float32), band[0])

    # the same scene, graph and sun raster by hand
    m = model_for(p.vertices, info["raster_size"], info["raster_layers"],
                  periodic=(info["periodic_neighbor_count"], info["periodic_size_x"],
                            info["periodic_size_z"]))
    diag = m.buildVisibilityGraph(scenes.hemisphere_directions())
    assert doc["graph"]["directedEdges"] == diag["directed_edge_count"]
    sun = facetcu.sun_direction(info["sun_zenith"], info["sun_azimuth"])
    lit = m.computeSunlitFraction(sun)
    assert np.array_equal(np.array(doc["sunlit"], np.float32), lit)
    g = Graph(*m.graph())
    surfaces = []
    for i in range(info["material_count"] + 2):
        d = p.material(i)
        surfaces.append(facetcu.Surface(d["reflectance"], d["transmittance"],
                                        d["tir_reflectance"], d["tir_transmittance"],
                                        d["sunlit_temperature"], d["shaded_temperature"]))
    M = info["material_count"]
    wl = [450.0, 550.0, 0.865, 1650.0, 10500.0]
    ref_irr = np.float32(700.0 * max(0.0, float(sun[1])) + 50.0)
    for b, w in enumerate(wl):
        o = reference.make_spectral_optics(
            p.vertices, info["leaf_facet_count"], lit, info["sun_zenith"], info["sun_azimuth"],
            wl, b, surfaces[M], surfaces[M + 1], surfaces[:M], p.material_indices,
            p.texture_factors, info["background_angular_strength"], info["sky_temperature"])
        optical = (w * 1000.0 if w <= 2.5 else w) <= 2500.0
        sky = 50.0 if optical else reference.planck(w, info["sky_temperature"])
        B, _ = reference.solve(g, o, sky, 64)
        if optical:
            B = np.clip(B / ref_irr, 0.0, 1.0)
        scale = np.maximum(np.abs(B), 1e-6 * np.abs(B).max())
        assert np.max(np.abs(band[b] - B) / scale) < 1e-5, w
    m.close()
