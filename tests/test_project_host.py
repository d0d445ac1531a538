"""XML project ingestion (no GPU): the library's facetcu_project_load
against the reference's own loadProjectScene and facetRTParametersFromInput
(models/histream/src/facetrt/facetrtcore.cpp:2038-3025 with Compo's
spectral models, compiled into oracle/_ref/libproject_ref.so), bit for bit:
geometry (placements, rotations, scales, domain clipping, cubes, the ground
grid), material bindings by mesh name, custom / file / PROSPECT / BSM
spectra on the sensor bands and on the 2001 energy samples, thermal, soil
and surface-energy blocks, raster settings, and the error messages."""
import os
import shutil

import numpy as np
import pytest

from oracle.build_ref import REFERENCE  # the reference tree the oracle recipe reads
from streamsim_gb300 import facetcu

OPTIPAR = os.path.join(REFERENCE, "models", "bin_x64", "Release", "defined", "optipar.txt")

HOUSE_OBJ = """# a house: walls and a roof in their own groups
o body
v 0 0.2 0
v 2 0.2 0
v 2 0.2 1
v 0 0.2 1
v 0 1.7 0
v 2 1.7 0
v 2 1.7 1
v 0 1.7 1
v 1 2.4 0.5
g WALL
f 1 2 6 5
f 2 3 7 6
f 3/1 4/1 8/1 7/1
f -6 -9 -5 -2
g roof
f 5 6 9
f 6 7 9
f 7 8 9
f 8 5 9
"""

TREE_OBJ = """usemtl crown
v 0 1 0
v 0.5 1.5 0.1
v -0.2 1.8 0.4
v 0.3 2.2 -0.3
f 1 2 3
f 2 3 4
f 1 3 4
"""

SPECTRUM = """# rows: wavelength (um, unsorted), reflectance, transmittance
0.9, 0.45 0.7 1.5   # near infrared first
0.45 0.05; 0.2 0.3
0.4 0.03 0.1 0.2
"""


def _spectra(coefficients):
    model = """<spectral name="soil" type="BSM"><ref_TIR>0.04</ref_TIR><SMC>20</SMC>
<BSMBrightness>0.4</BSMBrightness><BSMlat>30</BSMlat><BSMlon>50</BSMlon></spectral>
<spectral name="green_leaf" type="Prospect"><Cab>45</Cab><Cw>0.012</Cw><Cdm>0.008</Cdm>
<Cs>0.1</Cs><N>1.6</N><ref_TIR>0.02</ref_TIR><tau_TIR>0.01</tau_TIR></spectral>"""
    plain = """<spectral name="soil" type="custom"><reflectance>0.18, 0.25 0.3</reflectance>
<ref_TIR>0.04</ref_TIR></spectral>
<spectral name="green_leaf" type="custom"><reflectance>0.05;0.45</reflectance>
<transmittance>0.04;0.40</transmittance><ref_TIR>0.02</ref_TIR></spectral>"""
    return (model if coefficients else plain) + """
<spectral name="panel" type="custom"><reflectance>0.05,0.06,0.08,0.1</reflectance>
<transmittance>0</transmittance><ref_TIR>0.1</ref_TIR><tau_TIR>0</tau_TIR></spectral>
<spectral name="concrete" type="custom"><reflectance>0.25;0.3 0.35</reflectance>
<transmittance>0</transmittance><ref_TIR>0.08</ref_TIR></spectral>
<spectral name="bark" type="file"><spectral_file>spectra/bark.txt</spectral_file>
<ref_TIR>0.06</ref_TIR></spectral>"""


def _write_project(root, *, bands="450,550,0.865,1650,10500", size=(8.0, 6.0), voxel=0.5,
                   coefficients=True, extra_control="", heterogeneity="Hapke", objects=None,
                   extra_spectral="", extra_scene=""):
    root = str(root)
    for d in ("models", "positions", "spectra", "defined"):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    open(os.path.join(root, "models", "house.obj"), "w").write(HOUSE_OBJ)
    open(os.path.join(root, "models", "tree.obj"), "w").write(TREE_OBJ)
    open(os.path.join(root, "spectra", "bark.txt"), "w").write(SPECTRUM)
    # x y z [scale [rotation]]: a bad line, a negative scale (dropped), a
    # house across the domain edge (clipped), a rotated and scaled one
    open(os.path.join(root, "positions", "house.txt"), "w").write(
        "3 4 0\n6.5 2 0.5 1.2 30\nbad line\n1 1 1 -1\n7.6 5.5 0 1 75\n2 1.5 0.1 0.8\n")
    open(os.path.join(root, "positions", "trees.txt"), "w").write(
        "1.5 4.5 0 1.3 10\n4 1 0 0.7 200\n5.5 3 0 x\n")
    if coefficients:
        shutil.copy(OPTIPAR, os.path.join(root, "defined", "optipar.txt"))
    esun = "<esunFileName>defined/Esun_.dat</esunFileName>"
    objects = objects if objects is not None else """
<object objName="House"><componentType>Building</componentType><meshNames>wall, Roof</meshNames>
<spectralNames>concrete;panel</spectralNames><thermalNames>building_temperature</thermalNames>
<bioNames>wallset,pvset</bioNames><fileName>models/house.obj</fileName>
<objectPosition>positions/house.txt</objectPosition></object>
<object objName="Trees"><componentType>Vegetation</componentType><meshNames>crown</meshNames>
<spectralNames>green_leaf</spectralNames><thermalNames>vegetation_temperature</thermalNames>
<bioNames>leafset</bioNames><objectfile>models/tree.obj</objectfile>
<objectPosition>positions/trees.txt</objectPosition></object>
<object objName="Box"><componentType>Water</componentType><spectralNames>bark</spectralNames>
<bioNames>leafset</bioNames><shapes>1.5,2,0.5</shapes></object>"""
    xml = f"""<?xml version="1.0"?>
<HiStreamProject><Control>{extra_control}</Control>
<Geometry><Light><light name="Solar"><lightAngle><lightAngle>35,120</lightAngle></lightAngle>
<skyTemperature>255</skyTemperature>{esun}</light></Light>
<Sensor><sensor name="S"><controlBand>{bands}</controlBand></sensor></Sensor></Geometry>
<Scene><sceneSizeX>{size[0]}</sceneSizeX><sceneSizeY>{size[1]}</sceneSizeY><Height>5</Height>
<voxelSize>{voxel}</voxelSize><bgSpectral>soil</bgSpectral><bgThermal>soil_temperature</bgThermal>
<bgBioName>soilset</bgBioName><backgroundHeterogeneity>{heterogeneity}</backgroundHeterogeneity>
<backgroundAngularStrength>0.4</backgroundAngularStrength>{extra_scene}
<Object>{objects}</Object></Scene>
<Attribute><Optical>{_spectra(coefficients)}{extra_spectral}</Optical><Thermal>
<thermal name="building_temperature"><sunlitTemperature>310</sunlitTemperature>
<shadedTemperature>298</shadedTemperature></thermal>
<thermal name="soil_temperature"><sunlitTemperature>315</sunlitTemperature></thermal></Thermal>
<Biochemistry><property><soilSet name="soilset"><method>2</method><rss>1500</rss><cs>1100</cs>
<rhos>1700</rhos><lambdas>1.2</lambdas><SMC>30</SMC></soilSet></property>
<surfaceEnergy name="pvset"><photovoltaic>1</photovoltaic><vegetation>0</vegetation>
<eta25>0.2</eta25><gamma>-0.004</gamma><bifaciality>0.1</bifaciality>
<heatCapacityPerArea>12000</heatCapacityPerArea><convectiveScale>1</convectiveScale></surfaceEnergy>
<surfaceEnergy name="leafset"><photovoltaic>0</photovoltaic><vegetation>1</vegetation>
<heatCapacityPerArea>1500</heatCapacityPerArea></surfaceEnergy>
<surfaceEnergy name="wallset"><photovoltaic>0</photovoltaic><vegetation>0</vegetation>
<heatCapacityPerArea>90000</heatCapacityPerArea><convectiveScale>1.3</convectiveScale>
</surfaceEnergy></Biochemistry></Attribute></HiStreamProject>"""
    path = os.path.join(root, "Input.xml")
    open(path, "w").write(xml)
    return path


@pytest.fixture(scope="module")
def ref_project(reference):
    from oracle import pyoracle
    if not os.path.exists(pyoracle.PROJECT_LIB):
        pytest.skip("project loader oracle not built (no reference tree)")
    return pyoracle.ReferenceProject()


def _same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                                                 b.view(np.uint32) if b.dtype == np.float32 else b)


def _compare(ours, theirs):
    info = ours.info
    for k, v in theirs["info"].items():
        got = info[k]
        assert np.allclose(np.float32(got), np.float32(v), rtol=0, atol=0), k
    assert _same(ours.vertices, theirs["vertices"])
    assert _same(ours.material_indices, theirs["material_indices"])
    M = info["material_count"]
    surfaces = theirs["materials"] + [theirs["object"], theirs["ground"]]
    for i, want in enumerate(surfaces):
        got = ours.material(i)
        for k in ("reflectance", "transmittance", "energy_reflectance", "energy_transmittance"):
            assert _same(np.asarray(got[k], np.float32), np.asarray(want[k], np.float32)), (i, k)
        for k in ("tir_reflectance", "tir_transmittance", "sunlit_temperature",
                  "shaded_temperature", "surface_resistance", "specific_heat", "density",
                  "thermal_conductivity", "soil_moisture", "heat_capacity_per_area",
                  "pv_eta25", "pv_gamma", "pv_bifaciality", "convective_scale"):
            assert np.float32(got[k]) == np.float32(want[k]), (i, k)
        assert got["soil_temperature_method"] == int(want["soil_temperature_method"])
        assert got["photovoltaic"] == int(want["photovoltaic"])
        assert got["vegetation"] == int(want["vegetation"])
        if i < M:
            assert got["output_component"] == int(want["output_component"]), i
    p = ours.spectral_parameters()
    wl = np.ctypeslib.as_array(facetcu.C.cast(p.wavelengths, facetcu.C.POINTER(facetcu.C.c_float)),
                               (p.band_count,))
    assert _same(np.asarray(wl, np.float32), theirs["wavelengths"])
    if theirs["texture_factors"].size:
        assert _same(ours.texture_factors, theirs["texture_factors"])


@pytest.mark.slow
def test_project_with_spectral_models_matches_reference(tmp_path, ref_project):
    if not os.path.exists(OPTIPAR):
        pytest.skip("optipar.txt not in the reference tree")
    path = _write_project(tmp_path)
    theirs = ref_project.load(path)
    ours = facetcu.Project(path)
    _compare(ours, theirs)
    info = ours.info
    assert info["leaf_facet_count"] > 0 and info["material_count"] == 5  # 2 + 1 + 1 + ground
    # the house across the east edge is clipped to the domain
    assert np.max(ours.vertices[:, 0]) <= 4.0 + 1e-5 and np.max(ours.vertices[:, 2]) <= 3.0 + 1e-5
    pv = [i for i in range(info["material_count"]) if ours.material(i)["photovoltaic"]]
    assert pv and ours.material(pv[0])["output_component"] == 4


def test_custom_spectra_large_periodic_scene(tmp_path, ref_project):
    path = _write_project(tmp_path, size=(1200.0, 900.0), voxel=40.0, coefficients=False,
                          heterogeneity="Lambert", bands="0.55;0.65, 0.85 1.6 11",
                          extra_control="<periodicNeighborCount>8</periodicNeighborCount>"
                                        "<radiationSolver>accelerated</radiationSolver>")
    theirs = ref_project.load(path)
    ours = facetcu.Project(path)
    _compare(ours, theirs)
    info = ours.info
    assert (info["raster_size"], info["periodic_neighbor_count"]) == (2048, 8)
    assert info["background_angular_strength"] == 0.0 and info["accelerated_solver"] == 1


def test_objects_without_positions_or_bindings(tmp_path, ref_project):
    objects = """
<object objName="Lone"><spectralNames>concrete</spectralNames><fileName>models/house.obj</fileName></object>
<object objName="Cube"><shapes>-1,2,3</shapes></object>"""
    path = _write_project(tmp_path, coefficients=False, objects=objects, bands="")
    theirs = ref_project.load(path)
    ours = facetcu.Project(path)
    _compare(ours, theirs)
    assert ours.info["band_count"] == 1  # the 550 nm default


@pytest.mark.parametrize("case", ["dem", "texture", "pv_transmits", "pv_eta", "missing_obj",
                                  "no_coefficients", "json"])
def test_errors_match_reference(tmp_path, ref_project, case):
    kw = dict(coefficients=False)
    if case == "dem":
        kw["extra_control"] = "<isDEM>1</isDEM>"
        kw["objects"] = "<object objName=\"a\"><shapes>1,1,1</shapes></object><DEM>terrain/d.tif</DEM>"
    elif case == "texture":
        kw["extra_spectral"] = ""
        kw["objects"] = """<object objName="a"><spectralNames>tex</spectralNames></object>"""
        kw["extra_spectral"] = ("<spectral name=\"tex\" type=\"custom\"><reflectance>0.2</reflectance>"
                                "<physicalTextureEnabled>true</physicalTextureEnabled>"
                                "<physicalTextureFile>t/a.tif</physicalTextureFile></spectral>")
    elif case == "pv_transmits":
        kw["objects"] = """<object objName="a"><spectralNames>green_leaf</spectralNames>
<bioNames>pvset</bioNames><shapes>1,1,1</shapes></object>"""
    elif case == "pv_eta":
        kw["objects"] = """<object objName="a"><spectralNames>panel</spectralNames>
<bioNames>bad</bioNames><shapes>1,1,1</shapes></object>"""
        kw["extra_spectral"] = ""
    elif case == "missing_obj":
        kw["objects"] = """<object objName="a"><fileName>models/none.obj</fileName></object>"""
    elif case == "no_coefficients":
        kw["objects"] = """<object objName="a"><spectralNames>green_leaf</spectralNames></object>"""
        kw["extra_spectral"] = "<spectral name=\"green_leaf\" type=\"Prospect\"><Cab>40</Cab></spectral>"
    path = _write_project(tmp_path, **kw)
    if case == "pv_eta":
        text = open(path).read().replace(
            "<surfaceEnergy name=\"pvset\">",
            "<surfaceEnergy name=\"bad\"><photovoltaic>1</photovoltaic><eta25>0.9</eta25>"
            "</surfaceEnergy><surfaceEnergy name=\"pvset\">")
        open(path, "w").write(text)
    if case == "no_coefficients":
        text = open(path).read().replace("<spectral name=\"green_leaf\" type=\"custom\">",
                                         "<spectral name=\"unused\" type=\"custom\">")
        open(path, "w").write(text)
    if case == "json":
        path = str(tmp_path / "project.json")
        open(path, "w").write("{}")
    with pytest.raises(RuntimeError) as want:
        ref_project.load(path)
    with pytest.raises(RuntimeError) as got:
        facetcu.Project(path)
    if case == "json":  # the oracle has no JSON reader; ProjectJson::load's message
        assert str(got.value) == "project.json has no configuration object"
    else:
        assert str(got.value) == str(want.value)


def _project_json(root, **over):
    import json
    cfg = {
        "outDir": "output",
        "scene": {"x": 8, "y": 6, "height": 5, "voxel": 0.5,
                  "background": {"spectralName": "soil", "thermalName": "soil_temperature",
                                 "materialName": "soilset", "heterogeneityEnabled": True,
                                 "angularEffectStrength": 0.3}},
        "light": {"zenith": 35, "azimuth": "120", "direct": 0.8, "skyTemperature": 255},
        "sensor": {"bands": "550;450, 10500 550", "continuousBands": True, "bandStart": 1000,
                   "bandEnd": 1040, "bandStep": 20},
        "control": {"periodicBoundary": True, "periodicNeighborCount": 4, "radiationSolver": "accelerated",
                    "soilTemperatureMethod": 0},
        "objects": {"items": [
            {"name": "House", "type": "Building", "fileName": "models/house.obj",
             "positionFile": "positions/house.txt", "materialName": "wallset",
             "meshes": [{"name": "wall", "spectralName": "concrete", "thermalName": "building_temperature",
                         "materialName": "wallset"},
                        {"name": "Roof", "spectralName": "panel", "materialName": "pvset"}]},
            {"name": "Trees", "type": "Vegetation", "fileName": "models/tree.obj",
             "positionFile": "positions/trees.txt", "spectralName": "green_leaf",
             "materialName": "leafset"},
            {"name": "Smoke", "type": "Fire"},
            {"name": "Fogbank", "type": "Building", "medium": {}},
            {"name": "Box", "type": "Water", "spectralName": "bark", "materialName": "leafset",
             "dimensions": [1.5, 2, 0.5]}]},
        "spectra": [
            {"name": "soil", "model": "BSM", "refTir": 0.04,
             "params": {"SMC": 20, "BSMBrightness": 0.4, "BSMlat": 30, "BSMlon": 50}},
            {"name": "green_leaf", "model": "Prospect", "refTir": 0.02, "tauTir": 0.01,
             "params": {"Cab": 45, "Cw": 0.012, "Cdm": 0.008, "Cs": 0.1, "N": 1.6}},
            {"name": "panel", "reflectance": "0.05,0.06,0.08,0.1", "transmittance": 0, "refTir": 0.1},
            {"name": "concrete", "reflectance": "0.25;0.3 0.35", "refTir": 0.08},
            {"name": "bark", "model": "file", "fileName": "spectra/bark.txt", "refTir": 0.06}],
        "thermals": [{"name": "building_temperature", "sunlitTemperature": 310,
                      "shadedTemperature": 298}],
        "materials": [
            {"name": "soilset", "type": "Soil", "params": {"method": 2, "rss": 1500, "cs": 1100,
                                                           "rhos": 1700, "lambdas": 1.2, "SMC": 30}},
            {"name": "pvset", "type": "Building", "energyModel": "photovoltaic",
             "params": {"eta25": 0.2, "gamma": -0.004, "bifaciality": 0.1}},
            {"name": "leafset", "type": "Vegetation", "params": {"heatCapacityPerArea": 1500}},
            {"name": "wallset", "type": "Building", "params": {"heatCapacityPerArea": 90000,
                                                               "convectiveScale": 1.3}}],
        "meteo": {"start": 0, "end": 2, "dTime": 1800},
    }
    cfg.update(over)
    doc = {"schemaVersion": 2, "format": "streamsim-project", "name": "t", "configuration": cfg}
    path = os.path.join(str(root), "project.json")
    with open(path, "w") as f:
        json.dump(doc, f)
    return path


@pytest.mark.slow
def test_project_json_through_its_xml_view(tmp_path, ref_project, monkeypatch):
    if not os.path.exists(OPTIPAR):
        pytest.skip("optipar.txt not in the reference tree")
    _write_project(tmp_path)  # models, positions, spectra, defined/optipar.txt
    monkeypatch.chdir(tmp_path)  # the runtime "defined" folder is ./defined
    path = _project_json(tmp_path)
    view = facetcu.project_xml_view(path)
    assert "<controlBand>450,550,1000,1020,1040,10500</controlBand>" in view
    assert "<periodicNeighborCount>4</periodicNeighborCount>" in view
    assert "<backgroundHeterogeneity>Hapke</backgroundHeterogeneity>" in view
    assert "Smoke" not in view and "Fogbank" not in view
    assert "<meshNames>wall,Roof</meshNames>" in view and "<method>0</method>" in view
    xml_path = str(tmp_path / "view.xml")
    open(xml_path, "w").write(view)
    theirs = ref_project.load(xml_path)  # the reference's loader on the same view
    ours = facetcu.Project(path)
    _compare(ours, theirs)
    assert ours.info["periodic_neighbor_count"] == 4 and ours.info["accelerated_solver"] == 1


@pytest.mark.parametrize("case,message", [
    ("name", "HiStream accepts project.json only"),
    ("format", "Unsupported project format: other"),
    ("version", "Unsupported project schemaVersion; expected 1-6"),
    ("configuration", "project.json has no configuration object"),
    ("pv_ground", "Photovoltaic panels must be scene objects, not background ground"),
    ("syntax", "Invalid project.json"),
])
def test_project_json_errors(tmp_path, case, message):
    import json
    path = _project_json(tmp_path)
    doc = json.load(open(path))
    if case == "name":
        os.rename(path, str(tmp_path / "scene.json"))
        path = str(tmp_path / "scene.json")
    elif case == "format":
        doc["format"] = "other"
    elif case == "version":
        doc["schemaVersion"] = 7
    elif case == "configuration":
        doc["configuration"] = {}
    elif case == "pv_ground":
        doc["configuration"]["scene"]["background"]["materialName"] = "pvset"
    if case in ("format", "version", "configuration", "pv_ground"):
        json.dump(doc, open(path, "w"))
    if case == "syntax":
        open(path, "w").write('{"configuration": {"scene": [1, 2,, 3]}}')
    with pytest.raises((ValueError, RuntimeError)) as e:
        facetcu.project_xml_view(path)
    assert str(e.value).startswith(message)
