"""The CPU oracle against the reference's own CPU backend and golden vectors.

Reference behaviour pinned here:
  * buildCpuGraph / computeCpuSunlit / solveCpu (facetrtcore.cpp:1348-1529),
    compiled in place by oracle/build_ref.py: bit-exact equality;
  * radiosity_gpu.json shipped in validation/*/output (Vulkan backend, Windows):
    statistical agreement (the Vulkan raster uses top-left fill rules while
    the CPU uses inclusive edges, facetrtcore.cpp:1317-1318, so edge pixels
    differ; medians agree to 1e-7 / 1e-3).
"""
import numpy as np
import pytest

from oracle.pyoracle import raster_config

SCENES = ["urban_tree_building", "urban_dem_building"]


def _cfg(oracle, scene, raster):
    F = len(scene["vertices"]) // 3
    layers = oracle.adaptive_layers(F, 0, raster)
    return raster_config(raster, layers, scene["bmin"], scene["bmax"])


def _graph_equal(a, b):
    b = b.sorted_rows()
    for name in ("row_offsets", "neighbors", "counts", "denominators", "sky_counts"):
        if not np.array_equal(getattr(a, name), getattr(b, name)):
            return name
    return None


def test_directions_and_sun_match_reference(oracle, reference):
    assert np.array_equal(oracle.hemisphere_directions().view(np.uint32),
                          reference.hemisphere_directions().view(np.uint32))
    for zen, az in [(30, 135), (0, 0), (75, 290), (45.5, 12.25)]:
        assert np.array_equal(oracle.sun_direction(zen, az), reference.sun_direction(zen, az))
    for F, P, raster in [(4746, 0, 1024), (200_000, 0, 1024), (2_000_000, 0, 1024),
                         (500_000, 8, 2048), (10, 0, 1)]:
        assert oracle.adaptive_layers(F, P, raster, 64) == reference.adaptive_layers(F, P, raster, 64)
        assert oracle.adaptive_layers(F, P, raster, 16) == reference.adaptive_layers(F, P, raster, 16)


@pytest.mark.parametrize("name", SCENES)
def test_load_tree_with_soil_matches_reference(oracle, reference, golden_scene, name):
    s = golden_scene(name)
    v, m, leaf, bmin, bmax = reference.load_tree_with_soil(s["path"])
    assert np.array_equal(v.view(np.uint32), s["vertices"].view(np.uint32))
    assert np.array_equal(m, s["materials"])
    assert leaf == s["leaf"]
    assert np.array_equal(bmin, s["bmin"]) and np.array_equal(bmax, s["bmax"])
    assert len(v) // 3 == int(s["golden"]["facetCount"])
    assert leaf == int(s["golden"]["leafFacetCount"])


@pytest.mark.parametrize("name,raster", [("urban_tree_building", 256),
                                         ("urban_dem_building", 256),
                                         ("urban_tree_building", 1024)])
def test_graph_sunlit_solve_bit_exact_vs_reference(oracle, reference, golden_scene, name, raster):
    s = golden_scene(name)
    cfg = _cfg(oracle, s, raster)
    g = oracle.build_graph(s["vertices"], cfg, oracle.hemisphere_directions())
    r = reference.build_graph(s["vertices"], raster, cfg.layers, s["bmin"], s["bmax"])
    assert _graph_equal(g, r) is None
    assert g.max_closure_error == r.max_closure_error == 0.0
    sun = oracle.sun_direction(30, 135)
    lit, rc = oracle.sunlit(s["vertices"], cfg, sun)
    assert rc == 0
    lit_ref = reference.sunlit(s["vertices"], raster, cfg.layers, s["bmin"], s["bmax"], 30, 135)
    assert np.array_equal(lit, lit_ref)
    optics = oracle.make_optics(s["vertices"], s["leaf"], lit, sun)
    assert np.array_equal(optics, reference.make_optics(s["vertices"], s["leaf"], lit, 30, 135))
    b, md = oracle.solve(g, optics, 100.0, 64)
    b_ref, md_ref = reference.solve(r, optics, 100.0, 64)
    # The reference gathers in unordered_map order, the oracle in neighbour
    # order; the FP64 sums then round to the same float.
    assert np.array_equal(b, b_ref)
    h = oracle.incident(g, b, optics, 100.0)
    assert np.array_equal(h, reference.incident(r, b, optics, 100.0))


def _stacked_scene(seed=1):
    rng = np.random.default_rng(seed)
    base = np.array([(0, 0, 0), (1, 0, 0.2), (0.3, 1, 0.1)], np.float64)
    tris = [base] * 40
    tris += [base + rng.normal(size=3) * 0.01 for _ in range(30)]
    tris += [base + (0, 0, 0.05 * (k % 5)) for k in range(30)]
    out = []
    for t in tris:
        n = np.cross(t[1] - t[0], t[2] - t[0])
        n /= np.linalg.norm(n)
        out += [np.r_[p, n] for p in t]
    return np.array(out, np.float32)


def test_equal_depth_chains_follow_reference_sort(oracle, reference):
    """100 fragments per pixel, 40 of them at identical depth: the order of
    equal-depth fragments is that of the reference's std::sort."""
    v = _stacked_scene()
    bmin, bmax = v[:, :3].min(0), v[:, :3].max(0)
    cfg = raster_config(64, 128, bmin, bmax)
    g = oracle.build_graph(v, cfg, oracle.hemisphere_directions())
    assert g.max_depth == 100
    r = reference.build_graph(v, 64, 128, bmin, bmax)
    assert _graph_equal(g, r) is None
    lit, _ = oracle.sunlit(v, cfg, oracle.sun_direction(30, 135))
    assert np.array_equal(lit, reference.sunlit(v, 64, 128, bmin, bmax, 30, 135))


def test_periodic_tiles_match_reference(oracle, reference):
    v = _stacked_scene(2)
    bmin, bmax = v[:, :3].min(0), v[:, :3].max(0)
    cfg = raster_config(64, 512, bmin, bmax, 4, 1.3, 1.1)
    g = oracle.build_graph(v, cfg, oracle.hemisphere_directions())
    r = reference.build_graph(v, 64, 512, bmin, bmax, 4, 1.3, 1.1)
    assert _graph_equal(g, r) is None
    assert g.max_closure_error == pytest.approx(r.max_closure_error, abs=0)


def test_overflow_is_reported(oracle, reference):
    v = _stacked_scene()
    bmin, bmax = v[:, :3].min(0), v[:, :3].max(0)
    cfg = raster_config(64, 16, bmin, bmax)
    g = oracle.build_graph(v, cfg, oracle.hemisphere_directions())
    assert g.fragment_overflow > 0
    with pytest.raises(RuntimeError, match="overflow"):
        reference.build_graph(v, 64, 16, bmin, bmax)


@pytest.mark.parametrize("name,median_tol", [("urban_tree_building", 1e-6),
                                             ("urban_dem_building", 2e-3)])
def test_oracle_vs_shipped_vulkan_result(oracle, golden_scene, name, median_tol):
    s = golden_scene(name)
    gold = s["golden"]
    cfg = _cfg(oracle, s, 1024)
    g = oracle.build_graph(s["vertices"], cfg, oracle.hemisphere_directions())
    assert g.fragment_overflow == int(gold["fragmentOverflow"]) == 0
    assert g.max_closure_error == float(gold["closureError"]) == 0.0
    sun = oracle.sun_direction(30, 135)
    lit, _ = oracle.sunlit(s["vertices"], cfg, sun)
    optics = oracle.make_optics(s["vertices"], s["leaf"], lit, sun)
    b, _ = oracle.solve(g, optics, 100.0, 64)
    diffuse = optics.copy()
    diffuse[:, 3] = 0.0
    b0, _ = oracle.solve(g, diffuse, 100.0, 64)
    ref = gold["radiosity"]
    rel = np.abs(b - ref) / np.maximum(np.abs(ref), 1e-6)
    assert np.median(rel) < median_tol
    assert np.percentile(rel, 99) < 0.2
    assert abs(b.sum() / ref.sum() - 1.0) < 2e-4
    assert abs(b.max() / ref.max() - 1.0) < 1e-4
    assert np.mean(lit == gold["sunlit"]) > 0.9
    enh = np.maximum(0.0, b - b0)
    assert abs(enh.sum() / gold["lightEnhancement"].sum() - 1.0) < 5e-4


def test_fp64_solve_energy_closure(oracle, golden_scene):
    s = golden_scene("urban_tree_building")
    cfg = _cfg(oracle, s, 256)
    g = oracle.build_graph(s["vertices"], cfg, oracle.hemisphere_directions())
    sun = oracle.sun_direction(30, 135)
    lit, _ = oracle.sunlit(s["vertices"], cfg, sun)
    optics = oracle.make_optics(s["vertices"], s["leaf"], lit, sun)
    b64, it = oracle.solve_f64(g, optics, 100.0, 500, 1e-15)
    lhs, rhs = oracle.energy_closure(g, optics, 100.0, b64)
    assert abs(lhs - rhs) / abs(lhs) < 1e-10
    b32, _ = oracle.solve(g, optics, 100.0, 64)
    assert np.max(np.abs(b32 - b64) / np.maximum(np.abs(b64), 1e-6)) < 1e-5


def test_limit_cases(oracle):
    """Theory-manual limit scenes (docs/theory-manual.md:920-929)."""
    # isolated horizontal plane: sees only sky, H = L + D, B = rho (L + D)
    a, b_, c = (0, 0, 0), (0, 0, 1), (1, 0, 0)
    n = np.cross(np.subtract(b_, a), np.subtract(c, a)).astype(np.float64)
    n /= np.linalg.norm(n)
    v = np.array([np.r_[p, n] for p in (a, b_, c)], np.float32)
    cfg = raster_config(64, 8, v[:, :3].min(0), v[:, :3].max(0))
    g = oracle.build_graph(v, cfg, oracle.hemisphere_directions())
    assert g.nnz == 0
    optics = np.array([[0.3, 0.0, 0.0, 500.0], [0.2, 0.0, 0.0, 0.0]], np.float32)
    b, _ = oracle.solve(g, optics, 100.0, 8)
    np.testing.assert_allclose(b, [0.3 * 600.0, 0.2 * 100.0], rtol=1e-6)
    # blackbody: rho = tau = 0 gives B = e
    optics = np.array([[0.0, 0.0, 7.0, 500.0], [0.0, 0.0, 3.0, 0.0]], np.float32)
    b, _ = oracle.solve(g, optics, 100.0, 4)
    np.testing.assert_allclose(b, [7.0, 3.0])
