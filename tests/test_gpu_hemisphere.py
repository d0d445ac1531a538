"""Hemisphere ray-cast view factors and sun visibility (LBVH traversal on the
GPU) against the oracle's brute-force caster over all facets: same sample
tables, same arithmetic, same tie rules, so the integer counts must be
identical."""
import numpy as np
import pytest

from oracle.pyoracle import Graph
from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import graphs_equal, rel_err, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _model(v):
    m = facetcu.FacetrtCuda()
    m.initialize(64, 64, 64)
    m.setGeometry(v)
    return m


@pytest.mark.parametrize("rays,top_k", [(64, 64), (64, 8), (96, 32)])
def test_hemisphere_graph_bit_exact(oracle, rays, top_k):
    sc = scenes.config1(seed=1, leaves=300, grid=6)
    uv, dirs = scenes.hemisphere_samples(rays, 8, seed=3)
    m = _model(sc.vertices)
    diag, dropped = m.buildHemisphereGraph(uv, dirs, rays, top_k, 8)
    g, dropped_o = oracle.hemisphere_graph(sc.vertices, uv, dirs, rays, 8, top_k)
    assert graphs_equal(m.graph(), g) is None
    assert dropped == dropped_o
    if top_k >= rays:
        assert dropped == 0
    assert diag["directed_edge_count"] == g.nnz
    assert diag["max_closure_error"] == 0.0  # rows are renormalised over kept + sky
    m.close()


def test_hemisphere_on_validation_scene(oracle, golden_scene):
    """Buildings, trunks and a ground grid: coplanar facets and shared edges."""
    s = golden_scene("urban_tree_building")
    v = s["vertices"]
    rays = 32
    uv, dirs = scenes.hemisphere_samples(rays, 4, seed=9)
    m = _model(v)
    m.buildHemisphereGraph(uv, dirs, rays, 16, 4)
    g, _ = oracle.hemisphere_graph(v, uv, dirs, rays, 4, 16)
    assert graphs_equal(m.graph(), g) is None
    suv, _ = scenes.hemisphere_samples(16, 4, seed=10)
    sun = scenes.sun_direction(30, 135)
    lit = m.hemisphereSunlit(sun, suv, 16, 4)
    assert np.array_equal(lit, oracle.hemisphere_sunlit(v, suv, 16, 4, sun))
    m.close()


def test_hemisphere_sunlit_bit_exact(oracle):
    sc = scenes.config1(seed=2, leaves=300, grid=6)
    uv, _ = scenes.hemisphere_samples(48, 8, seed=5)
    sun = scenes.sun_direction(35, 200)
    m = _model(sc.vertices)
    lit = m.hemisphereSunlit(sun, uv, 48, 8)
    ref = oracle.hemisphere_sunlit(sc.vertices, uv, 48, 8, sun)
    assert np.array_equal(lit, ref)
    # sides facing away from the sun are 0, soil tops are mostly lit
    n = sc.normals()
    facing = (n @ sun) > 0
    assert np.all(lit[1::2][facing] == 0) and np.all(lit[0::2][~facing] == 0)
    assert lit[0::2][sc.leaf_count:].mean() > 0.5
    m.close()


def test_hemisphere_view_factors_statistics(oracle):
    """Against geometry: downward soil sides see only sky; reciprocity
    A_i F_ij ~ A_j F_ji holds in aggregate between panels and soil (Monte
    Carlo; large panels keep the hit counts high)."""
    rng = np.random.default_rng(4)
    n = 40
    centres = np.stack([rng.uniform(-3, 3, n), rng.uniform(0.5, 2.0, n), rng.uniform(-3, 3, n)], 1)
    normals = scenes.uniform_sphere(n, rng)
    panels = scenes._triangles_to_vertices(*scenes.equilateral(centres, normals, 1.2, rng))
    soil = scenes._triangles_to_vertices(*scenes.soil_grid(-5, 5, -5, 5, 8, 8))
    sc = scenes.Scene(np.concatenate([panels, soil]), len(panels) // 3, "panels")
    rays = 512
    uv, dirs = scenes.hemisphere_samples(rays, 16, seed=11)
    m = _model(sc.vertices)
    m.buildHemisphereGraph(uv, dirs, rays, rays, 16)
    rows, nb, cnt, den, sky = m.graph()
    S = len(den)
    F = np.zeros((S, S))
    src = np.repeat(np.arange(S), np.diff(rows.astype(np.int64)))
    F[src, nb] = cnt / den[src]
    v = sc.vertices.reshape(-1, 3, 6)[:, :, :3].astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), axis=1)
    A = np.repeat(area, 2)
    obj = np.zeros(S, bool)
    obj[:2 * sc.leaf_count] = True
    to_soil = (A[obj, None] * F[np.ix_(obj, ~obj)]).sum()
    to_obj = (A[~obj, None] * F[np.ix_(~obj, obj)]).sum()
    assert abs(to_soil - to_obj) / to_soil < 0.05
    # downward soil sides see nothing: all sky
    soil_bottom = np.arange(2 * sc.leaf_count + 1, S, 2)
    assert np.all(sky[soil_bottom] == den[soil_bottom])
    m.close()


def test_batched_solve_on_hemisphere_graph(oracle):
    sc = scenes.config1(seed=5, leaves=500, grid=8)
    rays = 128
    uv, dirs = scenes.hemisphere_samples(rays, 8, seed=12)
    m = _model(sc.vertices)
    m.buildHemisphereGraph(uv, dirs, rays, 64, 8)
    suv, _ = scenes.hemisphere_samples(64, 8, seed=13)
    sun = scenes.sun_direction(30, 135)
    lit = m.hemisphereSunlit(sun, suv, 64, 8)
    g = Graph(*m.graph())
    rho, tau = scenes.band_optics(sc, 4)
    dgeo = scenes.direct_geometry(sc, lit, sun)[None, :]
    sky = np.full(4, 100.0, np.float32)
    beam = np.full(4, 800.0, np.float32)
    for precision in (facetcu.PRECISION_FP32, facetcu.PRECISION_MIXED):
        out, res = m.solveBatched(rho, tau, sky, beam, dgeo, precision=precision, tolerance=1e-6)
        for b in range(4):
            o = np.zeros((sc.surface_count, 4), np.float32)
            o[:, 0], o[:, 1], o[:, 3] = rho[b], tau[b], dgeo[0] * beam[b]
            truth, _ = oracle.solve_f64(g, o, 100.0, 3000, 1e-14)
            assert rel_err(out[b], truth) < 1e-4
    m.close()


def test_hemisphere_argument_validation():
    sc = scenes.config1(seed=1, leaves=50, grid=2)
    m = _model(sc.vertices)
    uv, dirs = scenes.hemisphere_samples(64, 8)
    with pytest.raises(ValueError):
        m.buildHemisphereGraph(uv, dirs, 64, 16, 4)  # tables sized for 8 sets
    big_uv, big_dirs = scenes.hemisphere_samples(1024, 1)
    with pytest.raises(ValueError, match="rays_per_side"):
        m.buildHemisphereGraph(big_uv, big_dirs, 1024, 16, 1)
    m.close()


@pytest.mark.parametrize("neighbours", [4, 8, 20])
def test_hemisphere_periodic_tiles_bit_exact(oracle, neighbours):
    """Periodic tiling in the hemisphere mode: rays see the scene and its
    copies in the raster mode's neighbour tiles (offsets of the tile size,
    here the 10 m field), against the oracle's brute-force caster over the
    same tiles.  Low grazing rays from the soil now hit leaves of the copies
    instead of the sky."""
    sc = scenes.config1(seed=4, leaves=250, grid=6)
    rays = 64
    uv, dirs = scenes.hemisphere_samples(rays, 8, seed=6)
    m = facetcu.FacetrtCuda()
    m.initialize(64, 64, 64, 0, neighbours, 10.0, 10.0)
    m.setGeometry(sc.vertices)
    m.buildHemisphereGraph(uv, dirs, rays, 32, 8)
    g, _ = oracle.hemisphere_graph(sc.vertices, uv, dirs, rays, 8, 32,
                                   periodic=(neighbours, 10.0, 10.0))
    assert graphs_equal(m.graph(), g) is None
    flat, _ = oracle.hemisphere_graph(sc.vertices, uv, dirs, rays, 8, 32)
    assert g.sky_counts.sum() < flat.sky_counts.sum()  # the copies block sky
    suv, _ = scenes.hemisphere_samples(32, 8, seed=7)
    sun = scenes.sun_direction(70.0, 30.0)
    lit = m.hemisphereSunlit(sun, suv, 32, 8)
    assert np.array_equal(lit, oracle.hemisphere_sunlit(sc.vertices, suv, 32, 8, sun,
                                                        periodic=(neighbours, 10.0, 10.0)))
    m.close()


def test_hemisphere_graph_config2_scale_bit_exact(oracle):
    """The bench's view factors at full size: the 60-tree forest (203,840
    facets, 407,680 sides), 512 rays per side, top-K 256, against the
    oracle's BVH caster on the host cores (the brute force's rules; its
    equality with the brute force is a CPU test).  Every row, count,
    denominator and sky count must match, as must the 256-sample sun pass."""
    sc = scenes.config2(seed=0)
    uv, dirs = scenes.hemisphere_samples(512, 32, seed=7)
    m = facetcu.FacetrtCuda()
    m.initialize(1024, 1024, 1024)
    m.setGeometry(sc.vertices)
    diag, dropped = m.buildHemisphereGraph(uv, dirs, 512, 256, 32)
    suv, _ = scenes.hemisphere_samples(256, 32, seed=8)
    sun = scenes.sun_direction(30.0, 135.0)
    lit = m.hemisphereSunlit(sun, suv, 256, 32)
    gpu_graph = m.graph()
    m.close()
    g, dropped_o = oracle.hemisphere_graph_bvh(sc.vertices, uv, dirs, 512, 32, 256)
    assert g.nnz == diag["directed_edge_count"]
    assert graphs_equal(gpu_graph, g) is None
    assert dropped == dropped_o
    assert np.array_equal(lit, oracle.hemisphere_sunlit_bvh(sc.vertices, suv, 256, 32, sun))
