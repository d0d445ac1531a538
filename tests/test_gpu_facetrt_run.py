"""The eFacetRT process seam end to end on the GPU: facetcu_run_facetrt_core
and the `facetcu` executable on the reference's own validation scene,
against the reference's CPU backend run on the same OBJ (runCpu,
oracle/_ref) and against the reference's shipped Vulkan output
(tests/golden/urban_tree_building_vulkan.npz).

The graph and sunlit fractions must be identical to the CPU backend's;
radiosity within 1e-5 relative (64 FP32 sweeps against the CPU's FP64
gather).  Against the shipped Vulkan output the raster edge rule differs
(inclusive on the CPU path this library follows, top-left in the Vulkan
shaders), so the comparison there is statistical, as for the CPU backend:
median relative difference, 99th percentile and the scene sum."""
import json
import os
import subprocess

import numpy as np
import pytest

from streamsim_gb300 import facetcu
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
OBJ = os.path.join(GOLDEN, "urban_tree_building.obj")
CLI = os.path.join(os.path.dirname(facetcu.LIB_PATH), "facetcu")
KEYS = ["backend", "quantity", "units", "facetCount", "leafFacetCount", "vertexPositions",
        "graph", "timing", "iterations", "maxDelta", "wavelengths", "sunlit", "radiosity",
        "lightEnhancement"]


def _check_result(doc, ref=None):
    assert list(doc.keys()) == KEYS
    assert doc["backend"] == "CUDA GPU" and doc["quantity"] == "hemispherical radiosity"
    assert doc["units"] == "W m-2" and doc["iterations"] == 64 and doc["wavelengths"] == []
    assert list(doc["graph"].keys()) == ["directedEdges", "closureError", "fragmentOverflow",
                                         "hashOverflow"]
    assert list(doc["timing"].keys()) == ["totalMs", "visibilityMs", "sunlightMs", "solveMs"]
    v, _, leaf, _, _ = facetcu.load_tree_with_soil(OBJ)
    F = len(v) // 3
    assert doc["facetCount"] == F and doc["leafFacetCount"] == leaf
    pos = np.array(doc["vertexPositions"], np.float32).reshape(-1, 3)
    assert np.array_equal(pos, v[:, :3])  # 9 significant digits round-trip float32
    for k in ("sunlit", "radiosity", "lightEnhancement"):
        assert len(doc[k]) == 2 * F
    assert doc["graph"]["fragmentOverflow"] == 0 and doc["graph"]["hashOverflow"] == 0
    if ref is not None:
        rad = np.array(doc["radiosity"], np.float32)
        assert doc["graph"]["directedEdges"] == ref["directedEdges"]
        assert doc["graph"]["closureError"] == pytest.approx(ref["closureError"], abs=0)
        assert np.array_equal(np.array(doc["sunlit"], np.float32), ref["sunlit"])
        scale = np.maximum(np.abs(ref["radiosity"]), 1e-6 * np.abs(ref["radiosity"]).max())
        assert np.max(np.abs(rad - ref["radiosity"]) / scale) < 1e-5
        enh = np.array(doc["lightEnhancement"], np.float32)
        assert np.max(np.abs(enh - ref["lightEnhancement"])) < 1e-5 * np.abs(ref["radiosity"]).max()


def test_run_facetrt_core_matches_reference_cpu_backend(reference, tmp_path, capfd):
    require_gpu()
    out = tmp_path / "sub" / "facetrt.json"
    assert facetcu.run_facetrt_core(OBJ, str(out)) == 0
    stdout = capfd.readouterr().out.splitlines()
    assert stdout[-1] == f"RESULT\t{out}"
    progress = [int(line.split("\t")[1]) for line in stdout if line.startswith("PROGRESS\t")]
    assert progress == sorted(progress) and progress[-1] == 100
    doc = json.loads(out.read_text())
    _check_result(doc, reference.run_cpu_obj(OBJ))


def test_run_matches_shipped_vulkan_output_statistically(tmp_path):
    require_gpu()
    out = tmp_path / "facetrt.json"
    assert facetcu.run_facetrt_core(OBJ, str(out)) == 0
    doc = json.loads(out.read_text())
    g = np.load(os.path.join(GOLDEN, "urban_tree_building_vulkan.npz"))
    rad = np.array(doc["radiosity"], np.float64)
    ref = g["radiosity"].astype(np.float64)
    rel = np.abs(rad - ref) / np.maximum(np.abs(ref), 1e-6 * np.abs(ref).max())
    assert doc["facetCount"] == int(g["facetCount"])
    assert np.median(rel) < 1e-5 and np.percentile(rel, 99) < 0.2
    assert abs(rad.sum() / ref.sum() - 1.0) < 1e-3
    lit = np.array(doc["sunlit"], np.float32)
    assert np.mean(lit == g["sunlit"]) > 0.95


def test_cli_executable_end_to_end(tmp_path):
    require_gpu()
    scene = tmp_path / "scene.obj"
    scene.write_bytes(open(OBJ, "rb").read())
    r = subprocess.run([CLI, "eFacetRT", str(scene)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    default_out = tmp_path / "facetrt.json"
    assert r.stdout.splitlines()[-1] == f"RESULT\t{default_out}"
    _check_result(json.loads(default_out.read_text()))


def test_module_seam_runs_the_scene(tmp_path):
    """include/facetcu_module.hpp: setup, upload, create and run of the
    reference's Facetrt on the validation scene write the same facetrt.json
    layout (command.cpp:16-24: runFacetRTCore(...) == 0)."""
    require_gpu()
    from tests.test_abi import _build_module_check
    exe = _build_module_check(tmp_path)
    out = tmp_path / "module.json"
    r = subprocess.run([exe, OBJ, str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"RESULT\t{out}" in r.stdout and "module seam ok" in r.stdout
    _check_result(json.load(open(out)))
