"""One FacetEB time node on the device against the reference's own CPU
functions (oracle/_ref: makeEnergyShortwaveOptics, solveCpu,
incidentIrradianceCpu, makeEnergyLongwaveOptics, latentHeatFlux, ...,
called in runFacetEBCore's order, models/histream/src/facetrt/
facetrtcore.cpp:3462-3908).

The site has vegetation, a building, a PV array, soils with each storage
method, a dry soil, facets without a material (the reference's fallbacks),
texture factors and a per-sample energy reflectance spectrum.

Tolerances: temperatures within 2e-3 K; each flux field within 1e-4 of its
largest magnitude (the device gathers in FP32 where solveCpu accumulates in
FP64, ~1e-6 relative per solve, and CUDA's powf/exp10 may differ from the C
library's in the last place); the same number of coupling rounds."""
import numpy as np
import pytest

from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import model_for, require_gpu

pytestmark = pytest.mark.gpu

ZENITH, AZIMUTH = 35.0, 120.0
BANDS = [450.0, 0.65, 865.0, 1650.0, 10000.0, 11000.0]
FIELDS = ("radiosity", "shortwave_radiosity", "diffuse_radiosity", "longwave_radiosity",
          "absorbed_shortwave", "incident_shortwave", "net_radiation", "sensible_heat",
          "latent_heat", "storage_heat", "photovoltaic_power")


def _materials():
    red_edge = np.where(np.arange(2001) < 300, 0.06, 0.46).astype(np.float32)
    return [
        facetcu.EnergySurface([0.05, 0.08, 0.45, 0.30, 0.22], [0.04, 0.06, 0.40], 0.02, 0.01,
                              energy_reflectance=red_edge, energy_transmittance=0.8 * red_edge,
                              surface_resistance=150.0, heat_capacity_per_area=1500.0),
        facetcu.EnergySurface([0.25, 0.35], [0.0], 0.08, 0.0, vegetation=False,
                              heat_capacity_per_area=150000.0, convective_scale=1.3),
        facetcu.EnergySurface([0.06, 0.05, 0.08, 0.12, 0.15], [0.0], 0.12, 0.0,
                              vegetation=False, photovoltaic=True, heat_capacity_per_area=12000.0,
                              pv_eta25=0.21, pv_gamma=-0.004, pv_bifaciality=0.1),
        facetcu.EnergySurface([0.15], [0.0], 0.05, 0.0, soil_moisture=0.22,
                              soil_temperature_method=1),
        facetcu.EnergySurface([0.20], [0.0], 0.04, 0.0, soil_temperature_method=0),
        facetcu.EnergySurface([0.30], [0.0], 0.06, 0.0, soil_moisture=0.01,
                              soil_temperature_method=2, specific_heat=800.0,
                              thermal_conductivity=0.3),
    ]


def _spectrum():
    nm = np.arange(2001, dtype=np.float64)
    direct = np.exp(-((nm - 150.0) / 600.0) ** 2) * (1.0 - 0.6 * np.exp(-((nm - 540) / 30) ** 2))
    diffuse = 0.35 * np.exp(-((nm - 20.0) / 300.0) ** 2)
    return direct.astype(np.float32), diffuse.astype(np.float32)


@pytest.fixture(scope="module")
def site():
    require_gpu()
    sc, mi, _ = scenes.energy_site(seed=3)
    m = model_for(sc.vertices, 512, 64)
    m.buildVisibilityGraph(scenes.hemisphere_directions())
    sun = scenes.sun_direction(ZENITH, AZIMUTH)
    lit = m.computeSunlitFraction(sun)
    rows, nb, cnt, den, sky = m.graph()
    rng = np.random.default_rng(5)
    tex = rng.uniform(0.85, 1.15, sc.facet_count).astype(np.float32)
    yield dict(scene=sc, model=m, mi=mi, tex=tex, sun=sun, lit=lit,
               graph=(rows, np.stack([nb, cnt], 1), den, sky), materials=_materials(),
               spectrum=_spectrum())
    m.close()


def _run(reference, site, meteo, temperature, width=150, bands=BANDS, strength=0.0,
         **settings):
    sc = site["scene"]
    cosz = max(0.0, float(site["sun"][1]))
    direct, diffuse = site["spectrum"]
    _, windows, bd, bf = facetcu.shortwave_windows(meteo["shortwave"], cosz, direct, diffuse,
                                                   0.8, width, bands)
    nwin = len(facetcu.shortwave_windows(meteo["shortwave"], cosz, direct, diffuse, 0.8,
                                         width)[0])
    tol = settings.get("temperature_tolerance", 0.05)
    p, keep = facetcu.energy_parameters(
        sc.leaf_count, site["materials"], site["mi"], site["tex"], strength, bands,
        coupling_iterations=settings.get("coupling_iterations", 20), temperature_tolerance=tol,
        vegetation_temperature_method=settings.get("vegetation_method", 0),
        solver_tolerance=settings.get("solver_tolerance", 0.0),
        precision=settings.get("precision", facetcu.PRECISION_FP32))
    ours, res = site["model"].facetebNode(p, meteo, site["sun"], site["lit"],
                                          windows if nwin else None, temperature, bd, bf)
    m = meteo
    theirs, summary = reference.faceteb_node(
        sc.vertices, sc.leaf_count, site["graph"], site["lit"], ZENITH, AZIMUTH,
        (m["air_temperature"], m["vapor_pressure"], m["pressure"], m["wind_speed"],
         m["shortwave"], m["longwave"]), temperature, site["materials"], site["mi"], site["tex"],
        strength, site["spectrum"], 0.8, width, tolerance=tol, wavelengths=bands,
        coupling_iterations=settings.get("coupling_iterations", 20),
        vegetation_method=settings.get("vegetation_method", 0))
    return ours, res, theirs, summary, nwin


def _compare(ours, theirs, t_tol=2e-3, rel=1e-4):
    dT = np.max(np.abs(ours["temperature"] - theirs["temperature"]))
    assert dT <= t_tol, f"temperature differs by {dT} K"
    for k in FIELDS:
        a, b = ours[k].astype(np.float64), theirs[k].astype(np.float64)
        scale = max(np.max(np.abs(b)), 1e-3)
        err = np.max(np.abs(a - b)) / scale
        assert err <= rel, f"{k}: {err:.3g} of its scale {scale:.4g}"
    if "band_output" in theirs and theirs["band_output"].size:
        a, b = ours["band_output"].astype(np.float64), theirs["band_output"].astype(np.float64)
        for i in range(len(b)):
            scale = max(np.max(np.abs(b[i])), 1e-6)
            assert np.max(np.abs(a[i] - b[i])) / scale <= rel, f"band {i}"


DAY = dict(air_temperature=24.0, vapor_pressure=15.0, pressure=1000.0, wind_speed=2.0,
           shortwave=750.0, longwave=330.0)
NIGHT = dict(air_temperature=14.0, vapor_pressure=11.0, pressure=1002.0, wind_speed=0.5,
             shortwave=0.0, longwave=0.0)


def _seed(site, meteo):
    return np.full(site["scene"].surface_count,
                   np.clip(meteo["air_temperature"] + 273.15, 220.0, 340.0), np.float32)


def test_node_fixed_rounds_matches_reference(reference, site):
    T0 = _seed(site, DAY)
    ours, res, theirs, summary, nwin = _run(reference, site, DAY, T0, coupling_iterations=5,
                                            temperature_tolerance=1e-7)
    assert nwin > 10
    assert res["coupling_iterations"] == summary["coupling_iterations"] == 5
    assert res["solves"] == 2 * nwin + 6 + len(BANDS)
    _compare(ours, theirs)
    # the PV array produced power, the leaves transpired, the building stored heat
    S_obj = 2 * site["scene"].leaf_count
    assert ours["photovoltaic_power"][:S_obj].max() > 10.0
    assert ours["latent_heat"][:S_obj].max() > 1.0
    assert np.abs(ours["temperature"] - T0).max() > 1.0
    assert np.isclose(res["max_energy_residual"], summary["max_energy_residual"],
                      rtol=1e-3, atol=1e-3)


def test_node_default_settings_converge_like_reference(reference, site):
    T0 = _seed(site, DAY)
    ours, res, theirs, summary, _ = _run(reference, site, DAY, T0)
    assert res["coupling_iterations"] == summary["coupling_iterations"]
    assert res["converged"] == summary["converged"]
    _compare(ours, theirs)


def test_day_then_night_with_farquhar(reference, site):
    T0 = _seed(site, DAY)
    day, _, day_ref, _, _ = _run(reference, site, DAY, T0, vegetation_method=1,
                                 coupling_iterations=6, temperature_tolerance=1e-7)
    _compare(day, day_ref)
    # the next node starts from each side's own solved state; no sun at night
    night, res, night_ref, summary, nwin = _run(reference, site, NIGHT, day_ref["temperature"],
                                                vegetation_method=1, coupling_iterations=6,
                                                temperature_tolerance=1e-7)
    assert nwin == 0 and res["shortwave_sweeps"] == 0
    assert not np.any(night["absorbed_shortwave"])
    _compare(night, night_ref)


def test_accelerated_solves_agree_and_sweep_less(reference, site):
    T0 = _seed(site, DAY)
    fixed, r_fixed, theirs, _, _ = _run(reference, site, DAY, T0, coupling_iterations=5,
                                        temperature_tolerance=1e-7)
    fast, r_fast, _, _, _ = _run(reference, site, DAY, T0, coupling_iterations=5,
                                 temperature_tolerance=1e-7, solver_tolerance=1e-6)
    _compare(fast, theirs)
    # fixed-sweep solves also end early once the FP32 iterate stops changing
    # (the result of the remaining sweeps); warm starts cut the longwave ones
    assert r_fast["longwave_sweeps"] < r_fixed["longwave_sweeps"]
    assert r_fast["shortwave_sweeps"] <= r_fixed["shortwave_sweeps"]


def test_mixed_precision_windows(reference, site):
    # 64-sample windows give more than 32 window columns: the MIXED solver's
    # int8 panel takes them
    T0 = _seed(site, DAY)
    ours, res, theirs, _, nwin = _run(reference, site, DAY, T0, width=60, coupling_iterations=4,
                                      temperature_tolerance=1e-7, solver_tolerance=1e-6,
                                      precision=facetcu.PRECISION_MIXED)
    assert 2 * nwin >= 64
    _compare(ours, theirs, t_tol=5e-3, rel=5e-4)


def test_node_with_angular_ground(reference, site):
    T0 = _seed(site, DAY)
    ours, _, theirs, _, _ = _run(reference, site, DAY, T0, strength=0.5, coupling_iterations=3,
                                 temperature_tolerance=1e-7)
    _compare(ours, theirs)


def test_node_rejects_bad_arguments(site):
    sc, m = site["scene"], site["model"]
    T0 = _seed(site, DAY)
    for bad in (dict(coupling_iterations=0), dict(temperature_relaxation=0.0),
                dict(precision=facetcu.PRECISION_MIXED), dict(time_step=0.5),
                dict(solver_iterations=0), dict(precision=facetcu.PRECISION_FP64)):
        p, keep = facetcu.energy_parameters(sc.leaf_count, site["materials"], site["mi"], **bad)
        with pytest.raises(ValueError):
            m.facetebNode(p, DAY, site["sun"], site["lit"], None, T0)
    p, keep = facetcu.energy_parameters(sc.leaf_count + sc.facet_count, site["materials"])
    with pytest.raises(ValueError):
        m.facetebNode(p, DAY, site["sun"], site["lit"], None, T0)
    p, keep = facetcu.energy_parameters(sc.leaf_count, site["materials"], wavelengths=[550.0])
    with pytest.raises(ValueError):  # bands without their spectral irradiances
        m.facetebNode(p, DAY, site["sun"], site["lit"], None, T0)


def test_node_sequence_writes_the_reference_records(reference, site, tmp_path):
    """Three nodes through the FacetEB caller (morning, noon, night): each
    node starts from the previous node's temperatures, the sun is rastered
    per node, and the step records and faceteb.json are written."""
    from streamsim_gb300 import faceteb
    sc, m = site["scene"], site["model"]
    rows = [dict(DAY, node=0, julian_time=172.375, shortwave=420.0, air_temperature=20.0),
            dict(DAY, node=1, julian_time=172.5),
            dict(NIGHT, node=2, julian_time=172.875)]
    suns = {0: (60.0, 95.0), 1: (25.0, 170.0), 2: (100.0, 300.0)}
    run = faceteb.Run(m, sc.leaf_count, site["materials"], site["mi"], site["tex"],
                      wavelengths=BANDS, spectrum=site["spectrum"], window_width=150,
                      coupling_iterations=6, temperature_tolerance=1e-7)
    results, last = run.run(rows, lambda r: suns[r["node"]], output_dir=str(tmp_path),
                            vertices=sc.vertices, progress=None)
    assert [r["token"] for r in results] == ["DOY172_09-00", "DOY172_12-00", "DOY172_21-00"]
    # the reference's chain on the same rasters
    T = np.full(sc.surface_count, np.float32(20.0 + 273.15), np.float32)
    for r in rows:
        zen, az = suns[r["node"]]
        lit = m.computeSunlitFraction(facetcu.sun_direction(zen, az))
        theirs, _ = reference.faceteb_node(
            sc.vertices, sc.leaf_count, site["graph"], lit, zen, az,
            (r["air_temperature"], r["vapor_pressure"], r["pressure"], r["wind_speed"],
             r["shortwave"], r["longwave"]), T, site["materials"], site["mi"], site["tex"], 0.0,
            site["spectrum"], 0.8, 150, tolerance=1e-7, wavelengths=BANDS, coupling_iterations=6)
        T = theirs["temperature"]
        rec = np.fromfile(tmp_path / ".facet_steps" / f"energy_T={faceteb.time_token(r['julian_time'])}.bin",
                          "<f4").reshape(sc.surface_count, 9 + len(BANDS))
        assert np.max(np.abs(rec[:, 0] - theirs["temperature"])) <= 5e-3
        assert np.array_equal(rec[:, 8], lit)
    _compare(last, theirs, t_tol=5e-3)
    comp = np.fromfile(tmp_path / ".facet_steps" / "components.bin", np.uint8)
    assert comp.size == sc.facet_count and np.all(comp[sc.leaf_count:] == 1)
    import json
    doc = json.loads((tmp_path / "faceteb.json").read_text())
    assert doc["time"] == "DOY172_21-00" and len(doc["temperature"]) == sc.surface_count
    assert len(doc["vertexPositions"]) == 9 * sc.facet_count


def test_node_sequence_places_the_sun_by_date(site, tmp_path):
    """Without a caller's sun, each node's sun is updateSolarPosition's for
    the row's date and local time at the site (facetcu_faceteb_sun): the
    step records' sunlit column is the raster of that sun."""
    from streamsim_gb300 import faceteb
    sc, m = site["scene"], site["model"]
    rows = [dict(DAY, node=0, julian_time=172.375), dict(DAY, node=1, julian_time=172.5)]
    run = faceteb.Run(m, sc.leaf_count, site["materials"], site["mi"], site["tex"],
                      spectrum=site["spectrum"], coupling_iterations=3)
    results, _ = run.run(rows, output_dir=str(tmp_path), progress=None, latitude=35.0,
                         longitude=110.0)
    assert len(results) == 2
    for r in rows:
        zen, az = facetcu.faceteb_sun(r["julian_time"], 35.0, 110.0, r["pressure"],
                                      r["air_temperature"])
        assert 0.0 < zen < 80.0
        lit = m.computeSunlitFraction(facetcu.sun_direction(zen, az))
        rec = np.fromfile(tmp_path / ".facet_steps" /
                          f"energy_T={faceteb.time_token(r['julian_time'])}.bin",
                          "<f4").reshape(sc.surface_count, 9)
        assert np.array_equal(rec[:, 8], lit) and lit.max() > 0.0


def test_faceteb_process_entry_on_an_xml_project(tmp_path):
    """runFacetEBCore's process entry (faceteb.run_faceteb_core) on an XML
    project: its settings, meteorology file and site, one shared graph,
    two nodes; the records, components and faceteb.json are written, and
    every node's sunlit column is the raster of that node's dated sun."""
    import json
    from streamsim_gb300 import faceteb
    from tests.test_project_host import _write_project
    require_gpu()
    (tmp_path / "met.txt").write_text("julian Ta ea Pa u Rs Rl\n"
                                      "172.375 22 14 1005 2.0 520 340\n"
                                      "172.5 26 15 1003 2.5 800 350\n")
    path = _write_project(tmp_path, coefficients=False, bands="550,865,11000",
                          extra_control="<endTimeNode>2</endTimeNode><dTime>10800</dTime>"
                                        "<filePath>met.txt</filePath><Latitude>35</Latitude>"
                                        "<Longitude>110</Longitude>"
                                        "<couplingIterations>6</couplingIterations>"
                                        "<isRadiationProcess>1</isRadiationProcess>"
                                        "<isEnergyProcess>1</isEnergyProcess>")
    out = faceteb.run_faceteb_core(path, str(tmp_path / "out" / "faceteb.json"), progress=None)
    doc = json.load(open(out))
    p = facetcu.Project(path)
    info = p.info
    F = info["facet_count"]
    assert doc["facetCount"] == F and doc["leafFacetCount"] == info["leaf_facet_count"]
    assert doc["time"] == faceteb.time_token(172.5) and len(doc["temperature"]) == 2 * F
    steps = tmp_path / "out" / ".facet_steps"
    comp = np.fromfile(steps / "components.bin", np.uint8)
    assert comp.size == F and np.all(comp[info["leaf_facet_count"]:] == 1)
    pv = [i for i in range(info["material_count"]) if p.material(i)["photovoltaic"]]
    assert pv and np.any(comp == 4)  # the project's PV panel
    m = facetcu.FacetrtCuda()
    m.initialize(info["raster_size"], info["raster_size"], info["raster_layers"], 0,
                 info["periodic_neighbor_count"], info["periodic_size_x"],
                 info["periodic_size_z"])
    m.setGeometry(p.vertices)
    for jt, ta, pa in ((172.375, 22.0, 1005.0), (172.5, 26.0, 1003.0)):
        rec = np.fromfile(steps / f"energy_T={faceteb.time_token(jt)}.bin",
                          "<f4").reshape(2 * F, 9 + 3)
        zen, az = facetcu.faceteb_sun(jt, 35.0, 110.0, pa, ta)
        assert np.array_equal(rec[:, 8], m.computeSunlitFraction(facetcu.sun_direction(zen, az)))
        assert np.all(np.isfinite(rec)) and 250.0 < rec[:, 0].min() and rec[:, 0].max() < 360.0
    m.close()
    # the project's PV panel: a node table per node and one summary row per node
    summary = (tmp_path / "out" / "photovoltaic_summary.csv").read_text().splitlines()
    assert summary[0].startswith("node,time,area_m2") and len(summary) == 3
    assert [r.split(",")[1] for r in summary[1:]] == [faceteb.time_token(172.375),
                                                      faceteb.time_token(172.5)]
    node = (tmp_path / "out" / "photovoltaic_node_1.csv").read_text().splitlines()
    pv_facets = int(np.sum(comp == 4))
    assert len(node) == pv_facets + 1
    area = sum(float(r.split(",")[0]) for r in node[1:])
    assert abs(area - float(summary[2].split(",")[2])) <= 1e-4 * area
    assert float(summary[2].split(",")[-1]) > float(summary[1].split(",")[-1]) > 0.0
    index = json.loads((tmp_path / "out" / "faceteb_run.json").read_text())
    assert index["status"] in ("completed", "non_converged") and len(index["completed"]) == 2
    assert [c["token"] for c in index["completed"]] == [faceteb.time_token(172.375),
                                                        faceteb.time_token(172.5)]
    assert index["products"][:2] == ["photovoltaic_summary.csv", ".facet_steps/components.bin"]
    assert index["products"][-1] == "faceteb.json" and index["convergence"]["iterationBudget"] == 6
    # process records of the last node: the same fields as its step record
    tok = faceteb.time_token(172.5)
    rec = np.fromfile(steps / f"energy_T={tok}.bin", "<f4").reshape(2 * F, 12)
    proc = tmp_path / "out" / "process"
    rad = np.fromfile(proc / f"facetrt_T={tok}.bin", "<f4").reshape(2 * F, 3)
    eng = np.fromfile(proc / f"faceteb_T={tok}.bin", "<f4").reshape(2 * F, 5)
    pvr = np.fromfile(proc / f"faceteb_pv_T={tok}.bin", "<f4").reshape(2 * F, 3)
    assert np.array_equal(rad, rec[:, [2, 3, 4]])        # shortwave, longwave, net
    assert np.array_equal(eng, rec[:, [6, 5, 7, 0, 4]])  # latent, sensible, storage, T, net
    assert np.array_equal(pvr[:, 1], rec[:, 0])
    meta = json.loads((proc / f"faceteb_T={tok}.json").read_text(encoding="utf-8"))
    assert meta["kind"] == "facet-energy-process" and meta["recordFloats"] == 5
    assert meta["surfaceCount"] == 2 * F and meta["time"] == tok and meta["node"] == 1
    assert [f["id"] for f in meta["fields"]] == ["latentHeat", "sensibleHeat", "surfaceHeatFlux",
                                                 "temperature", "netRadiation"]
    zen, az = facetcu.faceteb_sun(172.5, 35.0, 110.0, 1003.0, 26.0)
    assert abs(meta["solarZenith"] - float(zen)) < 1e-5 and abs(meta["solarAzimuth"] - float(az)) < 1e-4
    assert f"process/facetrt_T={tok}.bin" in index["products"]
