"""Raster visibility graph and sunlit fraction on the GPU, through the C ABI,
against the CPU oracle (itself bit-exact with the reference's CPU backend,
tests/test_oracle.py).  Integer counts must be identical."""
import numpy as np
import pytest

from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import graphs_equal, model_for, oracle_cfg, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


@pytest.mark.parametrize("name,raster", [("urban_tree_building", 256),
                                         ("urban_tree_building", 1024),
                                         ("urban_dem_building", 512)])
def test_validation_scene_graph_bit_exact(oracle, golden_scene, name, raster):
    s = golden_scene(name)
    F = len(s["vertices"]) // 3
    layers = oracle.adaptive_layers(F, 0, raster)
    bounds = (s["bmin"], s["bmax"])  # the CPU backend rasterises in the Scene bounds
    m = model_for(s["vertices"], raster, layers, bounds)
    dirs = scenes.hemisphere_directions()
    diag = m.buildVisibilityGraph(dirs)
    g = oracle.build_graph(s["vertices"], oracle_cfg(s["vertices"], raster, layers, bounds), dirs)
    assert graphs_equal(m.graph(), g) is None
    assert diag["directed_edge_count"] == g.nnz
    assert diag["fragment_overflow"] == 0 and diag["hash_overflow"] == 0
    assert diag["max_closure_error"] == g.max_closure_error == 0.0
    sun = scenes.sun_direction(30, 135)
    lit = m.computeSunlitFraction(sun)
    lit_o, _ = oracle.sunlit(s["vertices"], oracle_cfg(s["vertices"], raster, layers, bounds), sun)
    assert np.array_equal(lit, lit_o)
    m.close()


def test_single_directions_and_repeated_direction(oracle, golden_scene):
    """Each direction alone is exact, and 40 copies of one direction give
    exactly 40 times its counts (exercises the multi-tile pair sort)."""
    s = golden_scene("urban_tree_building")
    bounds = (s["bmin"], s["bmax"])
    m = model_for(s["vertices"], 256, 64, bounds)
    dirs = scenes.hemisphere_directions()
    cfg = oracle_cfg(s["vertices"], 256, 64, bounds)
    for d in (0, 7, 19, 33):
        m.buildVisibilityGraph(dirs[d:d + 1])
        assert graphs_equal(m.graph(), oracle.build_graph(s["vertices"], cfg, dirs[d:d + 1])) is None
    m.buildVisibilityGraph(dirs[5:6])
    rows1, nb1, cnt1, den1, sky1 = m.graph()
    m.buildVisibilityGraph(np.repeat(dirs[5:6], 40, axis=0))
    rows, nb, cnt, den, sky = m.graph()
    assert np.array_equal(rows, rows1) and np.array_equal(nb, nb1)
    assert np.array_equal(cnt, 40 * cnt1) and np.array_equal(den, 40 * den1)
    assert np.array_equal(sky, 40 * sky1)
    m.close()


def test_vertex_bounds_frame_matches_oracle(oracle):
    """Default frame = vertex bounds (FacetrtVulkan::setGeometry)."""
    sc = scenes.config1(seed=0)
    m = model_for(sc.vertices, 512, 64)
    dirs = scenes.hemisphere_directions()
    m.buildVisibilityGraph(dirs)
    g = oracle.build_graph(sc.vertices, oracle_cfg(sc.vertices, 512, 64), dirs)
    assert graphs_equal(m.graph(), g) is None
    sun = scenes.sun_direction(30, 135)
    assert np.array_equal(m.computeSunlitFraction(sun),
                          oracle.sunlit(sc.vertices, oracle_cfg(sc.vertices, 512, 64), sun)[0])
    m.close()


def _stacked(seed):
    from tests.test_oracle import _stacked_scene
    return _stacked_scene(seed)


def test_equal_depth_chains_and_deep_pixels(oracle):
    """100-fragment chains with exact depth ties: the GPU replays the
    reference's std::sort order (chains > 64 take the deep-chain kernel)."""
    v = _stacked(1)
    m = model_for(v, 64, 128)
    dirs = scenes.hemisphere_directions()
    m.buildVisibilityGraph(dirs)
    g = oracle.build_graph(v, oracle_cfg(v, 64, 128), dirs)
    assert g.max_depth == 100
    assert graphs_equal(m.graph(), g) is None
    sun = scenes.sun_direction(30, 135)
    assert np.array_equal(m.computeSunlitFraction(sun), oracle.sunlit(v, oracle_cfg(v, 64, 128), sun)[0])
    m.close()


def test_periodic_tiles(oracle):
    v = _stacked(2)
    per = (4, 1.3, 1.1)
    m = model_for(v, 64, 512, periodic=per)
    dirs = scenes.hemisphere_directions()
    diag = m.buildVisibilityGraph(dirs)
    g = oracle.build_graph(v, oracle_cfg(v, 64, 512, periodic=per), dirs)
    assert graphs_equal(m.graph(), g) is None
    assert diag["max_closure_error"] == pytest.approx(g.max_closure_error, abs=0)
    m.close()


def test_overflow_raises_like_the_reference():
    v = _stacked(1)
    m = model_for(v, 64, 16)
    with pytest.raises(RuntimeError, match="A-buffer overflow"):
        m.buildVisibilityGraph(scenes.hemisphere_directions())
    assert m.diagnostics["fragment_overflow"] > 0
    with pytest.raises(RuntimeError, match="Direct-light A-buffer overflow"):
        m.computeSunlitFraction(scenes.sun_direction(30, 135))
    m.close()


def test_call_order_and_validation():
    m = facetcu.FacetrtCuda()
    with pytest.raises(facetcu.LogicError):
        m.setGeometry(np.zeros((3, 6), np.float32))
    m.initialize(64, 64, 8)
    with pytest.raises(facetcu.LogicError):
        m.buildVisibilityGraph(scenes.hemisphere_directions())
    bad = scenes.config1().vertices.copy()
    bad[0, 3:] = [0, 0, 0]
    with pytest.raises(ValueError, match="normalized"):
        m.setGeometry(bad)
    bad = scenes.config1().vertices.copy()
    bad[4, 0] = np.nan
    with pytest.raises(ValueError, match="non-finite"):
        m.setGeometry(bad)
    with pytest.raises(ValueError, match="triangle list"):
        m.setGeometry(np.zeros((4, 6), np.float32))
    m.setGeometry(scenes.config1().vertices)
    with pytest.raises(facetcu.LogicError):
        m.solve(np.zeros((8192, 4), np.float32), 100.0)
    with pytest.raises(ValueError, match="direction"):
        m.buildVisibilityGraph(np.zeros((1, 3), np.float32))
    m.close()


def test_no_samples_raises():
    # a facet seen exactly edge-on by the only direction covers no pixel centre
    v = np.array([[0, 0, 0, 0, 1, 0], [0, 0, 1, 0, 1, 0], [1, 0, 0, 0, 1, 0]], np.float32)
    m = model_for(v, 16, 8)
    with pytest.raises(RuntimeError, match="no surface samples"):
        m.buildVisibilityGraph(np.array([[1.0, 0.0, 0.0]], np.float32))
    m.close()


def test_graph_round_trip_and_determinism():
    sc = scenes.config1(seed=3)
    m = model_for(sc.vertices, 256, 64)
    m.buildVisibilityGraph(scenes.hemisphere_directions())
    g1 = m.graph()
    m.buildVisibilityGraph(scenes.hemisphere_directions())
    g2 = m.graph()
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
    # symmetric counts: (s -> n, c) implies (n -> s, c)
    rows, nb, cnt, den, sky = g1
    src = np.repeat(np.arange(len(den)), np.diff(rows.astype(np.int64)))
    fwd = set(zip(src.tolist(), nb.tolist(), cnt.tolist()))
    assert all((n, s, c) in fwd for s, n, c in list(fwd)[:5000])
    m.setGraph(*g1)
    for a, b in zip(m.graph(), g1):
        assert np.array_equal(a, b)
    m.close()
