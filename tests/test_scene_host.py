"""Host-side pieces of the eFacetRT seam (no GPU): the OBJ scene loader,
makeOptics and planckRadiance against the reference's own functions
(oracle/_ref), bit for bit, and the `facetcu` executable's argument
handling and exit codes (models/histream/src/main.cpp:56-80)."""
import os
import subprocess

import numpy as np
import pytest

from streamsim_gb300 import facetcu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CLI = os.path.join(os.path.dirname(facetcu.LIB_PATH), "facetcu")

QUAD_OBJ = """# quads, negative indices, texture/normal tokens, a degenerate face
o leaf_block
v 0 1.5 0
v 1 1.25 0
v 1 1.75 1
v 0 2.0 1
v 0.5 3 0.5
vt 0 0
vn 0 1 0
f 1/1/1 2/1/1 3/1/1 4/1/1
f -5 -3 -1
f 1 1 2
v 2 1 2
v 3 1 2
v 2 1 3
f 6 7 8
"""

TERRAIN_OBJ = """o tree
v 0 1 0
v 1 1 0
v 0 1 1
f 1 2 3
o STREAMSIM_TERRAIN
v -2 0 -2
v 2 0 -2
v 2 0 2
v -2 0 2
f 4 5 6 7
o STREAMSIM_TERRAIN
v 0 2 0
v 1 2 1
v 0 2.5 1
f 8 9 10
"""


def _scene_files(tmp_path):
    files = [os.path.join(GOLDEN, n) for n in ("urban_tree_building.obj",
                                                "urban_dem_building.obj")]
    for name, text in (("quads.obj", QUAD_OBJ), ("terrain.obj", TERRAIN_OBJ)):
        p = tmp_path / name
        p.write_text(text)
        files.append(str(p))
    return files


def test_load_tree_with_soil_matches_reference(reference, tmp_path):
    for path in _scene_files(tmp_path):
        v, m, leaf, lo, hi = facetcu.load_tree_with_soil(path)
        rv, rm, rleaf, rlo, rhi = reference.load_tree_with_soil(path)
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32)), path
        assert np.array_equal(m, rm) and leaf == rleaf, path
        assert np.array_equal(lo, rlo) and np.array_equal(hi, rhi), path


def test_load_tree_with_soil_errors_match_reference(reference, tmp_path):
    cases = {"missing.obj": None, "bad_index.obj": "v 0 0 0\nv 1 0 0\nv 0 0 1\nf 1 2 7\n",
             "empty.obj": "# nothing\n", "bad_vertex.obj": "v 0 zero 0\n",
             "no_index.obj": "v 0 0 0\nv 1 0 0\nv 0 0 1\nf /1 2 3\n"}
    for name, text in cases.items():
        p = tmp_path / name
        if text is not None:
            p.write_text(text)
        with pytest.raises(RuntimeError) as ours:
            facetcu.load_tree_with_soil(str(p))
        with pytest.raises(RuntimeError) as theirs:
            reference.load_tree_with_soil(str(p))
        assert str(ours.value) == str(theirs.value), name


def test_make_optics_matches_reference(reference):
    path = os.path.join(GOLDEN, "urban_tree_building.obj")
    v, _, leaf, _, _ = facetcu.load_tree_with_soil(path)
    rng = np.random.default_rng(1)
    lit = rng.uniform(0, 1, 2 * (len(v) // 3)).astype(np.float32)
    lit[::7] = 0.0
    for zen, az in ((30.0, 135.0), (0.0, 0.0), (75.0, 300.0)):
        ours = facetcu.make_optics(v, leaf, lit, facetcu.sun_direction(zen, az))
        theirs = reference.make_optics(v, leaf, lit, zen, az)
        assert np.array_equal(ours.view(np.uint32), theirs.view(np.uint32))


def test_planck_matches_reference(reference):
    for wl in (400.0, 550.0, 865.0, 1600.0, 2500.0, 8000.0, 10000.0, 14000.0, 0.55, 10.0, 2.0):
        for t in (0.5, 250.0, 296.0, 305.0, 5800.0):
            assert facetcu.planck_radiance(wl, t) == reference.planck(wl, t), (wl, t)


def _cli(*args):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=120)


def test_cli_argument_handling():
    assert os.path.exists(CLI), "build() makes streamsim_gb300/facetcu"
    r = _cli("eUnknown")
    assert r.returncode == 2 and r.stderr.startswith("Usage: facetcu [eVoxelEB|eFacetEB|eFacetRT")
    r = _cli("eVoxelEB", "x.json")  # not built on this backend
    assert r.returncode == 3 and "Failed to create engine resources for eVoxelEB" in r.stderr
    # eFacetEB runs the FacetEB entry (python -m streamsim_gb300.faceteb)
    r = _cli("eFacetEB", "/nonexistent/Input.xml")
    assert r.returncode == 1 and r.stderr.startswith("faceteb: ")
    r = subprocess.run([CLI, "eFacetEB", "x.xml"], capture_output=True, text=True, timeout=60,
                       env=dict(os.environ, FACETCU_PYTHON="/nonexistent/python"))
    assert r.returncode == 3 and "cannot start /nonexistent/python" in r.stderr
    r = _cli("eFacetRT")
    assert r.returncode == 1 and "facetrt: FacetRT requires project.json" in r.stderr
    r = _cli("eFacetRT", "/nonexistent/project.json")  # read through its XML view
    assert r.returncode == 1 and r.stderr.startswith("facetrt: Cannot open project.json: ")
    r = _cli("eFacetRT", "/nonexistent/Input.xml")
    assert r.returncode == 1 and "facetrt: Cannot open HiStream input: /nonexistent/Input.xml" in r.stderr
    r = _cli("eFacetRT", "/nonexistent/scene.obj")
    assert r.returncode == 1
    assert "facetrt: Cannot open tree OBJ: /nonexistent/scene.obj" in r.stderr
