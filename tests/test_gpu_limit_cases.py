"""Limit cases of the reference's validation rules (docs/theory-manual.md,
section 15.1: black body, perfect reflector, unoccluded plane, single facet;
exchange creates no energy; periodic copies count no energy twice) on the
GPU path, through the C ABI, with both view-factor modes.

Tolerances: exact (bitwise) where the arithmetic is exact (a black body's
radiosity is its emission); 1e-6 relative for analytic radiosities of the
FP32 solvers; 1e-7 for energy identities of the FP64 batched solve (its
output is rounded to float32, which bounds the identity at a few 1e-9); 1e-5
for the same identities of the MIXED solve at a 1e-7 stop rule."""
import numpy as np
import pytest

from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _scene(a, b, c, name):
    v = scenes._triangles_to_vertices(a, b, c)
    return scenes.Scene(v, len(v) // 3, name)


def _model(sc, mode, periodic=(0, 1.0, 1.0)):
    m = facetcu.FacetrtCuda()
    m.initialize(256, 256, 64, 0, periodic[0], periodic[1], periodic[2])
    m.setGeometry(sc.vertices)
    sun = scenes.sun_direction(30.0, 135.0)
    if mode == "raster":
        m.buildVisibilityGraph(scenes.hemisphere_directions())
        lit = m.computeSunlitFraction(sun)
    else:
        uv, dirs = scenes.hemisphere_samples(128, 8, seed=7)
        m.buildHemisphereGraph(uv, dirs, 128, 128, 8)
        suv, _ = scenes.hemisphere_samples(64, 8, seed=8)
        lit = m.hemisphereSunlit(sun, suv, 64, 8)
    return m, sun, lit


def _optics(rho, tau, emis, direct):
    o = np.zeros((len(rho), 4), np.float32)
    o[:, 0], o[:, 1], o[:, 2], o[:, 3] = rho, tau, emis, direct
    return o


def _plane(size=2.0137, cells=1, y=1.013):
    # generic coordinates: no pixel centre of the raster lands on a shared edge
    return _scene(*scenes.quad_grid((-size / 2 + 0.0071, y, -size / 2 - 0.0043), (0, 0, size),
                                    (size, 0, 0), cells, cells), "plane")


def _closed_box(w=2.013, d=3.017, h=1.507, cell=0.75):
    a, b, c = scenes.box(0.0, 0.0, w, d, h, cell)
    fa, fb, fc = scenes.quad_grid((0.0, 0.0, 0.0), (w, 0, 0), (0, 0, d),
                                  int(np.ceil(w / cell)), int(np.ceil(d / cell)))  # floor, -y
    return _scene(np.concatenate([a, fa]), np.concatenate([b, fb]), np.concatenate([c, fc]),
                  "closed box")


@pytest.mark.parametrize("mode", ["raster", "hemisphere"])
def test_black_body_radiosity_is_its_emission(mode):
    """rho = tau = 0: B = e exactly, whatever the graph, in every solver."""
    sc = scenes.forest(2, 10.0, 200, seed=4, leaves_per_crown=300, name="bb")
    m, sun, lit = _model(sc, mode)
    S = sc.surface_count
    rng = np.random.default_rng(1)
    e = rng.uniform(0.0, 50.0, S).astype(np.float32)
    zero = np.zeros(S, np.float32)
    direct = scenes.direct_geometry(sc, lit, sun) * 800.0
    r = m.solve(_optics(zero, zero, e, direct), 100.0, 64)
    assert np.array_equal(r["radiosity"], e)
    for prec in (facetcu.PRECISION_FP64, facetcu.PRECISION_FP32, facetcu.PRECISION_MIXED):
        out, res = m.solveBatched(np.stack([zero] * 40), np.stack([zero] * 40),
                                  np.full(40, 100.0, np.float32), np.full(40, 800.0, np.float32),
                                  scenes.direct_geometry(sc, lit, sun)[None, :],
                                  emission=np.stack([e] * 40), precision=prec, tolerance=1e-7)
        assert np.array_equal(out, np.stack([e] * 40)), prec
    m.close()


@pytest.mark.parametrize("mode", ["raster", "hemisphere"])
@pytest.mark.parametrize("cells", [1, 3])
def test_unoccluded_plane_sees_only_sky(mode, cells):
    """A horizontal plane in empty space (one quad of two facets, or 3 x 3
    quads): every side sees only sky, so H = L + D and
    B_s = rho (L + D_s) + tau (L + D_(s^1)); the top is fully sunlit."""
    sc = _plane(cells=cells)
    m, sun, lit = _model(sc, mode)
    rows, _, _, den, sky = m.graph()
    assert rows[-1] == 0 and np.array_equal(den, sky) and np.all(sky > 0)
    assert np.all(lit[0::2] == 1.0) and np.all(lit[1::2] == 0.0)
    S = sc.surface_count
    L, beam = 100.0, 800.0
    D = scenes.direct_geometry(sc, lit, sun) * beam
    rho = np.full(S, 0.3, np.float32)
    tau = np.full(S, 0.1, np.float32)
    pair = np.arange(S) ^ 1
    expect = rho.astype(np.float64) * (L + D) + tau.astype(np.float64) * (L + D[pair])
    r = m.solve(_optics(rho, tau, np.zeros(S, np.float32), D), L, 64)
    assert np.max(np.abs(r["radiosity"] - expect) / expect) < 1e-6
    out, _ = m.solveBatched(rho[None, :], tau[None, :], np.array([L], np.float32),
                            np.array([beam], np.float32), scenes.direct_geometry(sc, lit, sun)[None, :],
                            precision=facetcu.PRECISION_FP64, tolerance=1e-13)
    assert np.max(np.abs(out[0] - expect) / expect) < 1e-6
    m.close()


def test_single_facet():
    """One triangle: both sides see only sky in both modes, and the solve is
    the unoccluded-plane formula."""
    tri = _scene(np.array([[0.0, 1.0, 0.0]]), np.array([[0.0, 1.0, 1.0]]),
                 np.array([[1.0, 1.0, 0.0]]), "one facet")
    for mode in ("raster", "hemisphere"):
        m, sun, lit = _model(tri, mode)
        rows, _, _, den, sky = m.graph()
        assert rows.tolist() == [0, 0, 0] and np.array_equal(den, sky) and np.all(sky > 0)
        D = scenes.direct_geometry(tri, lit, sun) * 700.0
        r = m.solve(_optics(np.array([0.2, 0.2], np.float32), np.zeros(2, np.float32),
                            np.zeros(2, np.float32), D), 50.0, 64)
        assert np.allclose(r["radiosity"], 0.2 * (50.0 + D), rtol=1e-6)
        m.close()


def _raster_balance(m, rho, tau, e, D, L, B):
    """Both sides of the count-form energy balance of the raster graph
    (symmetric counts, equal denominators on a facet's two sides), FP64:
    sum w (D + e) + sum sky L  vs  sum w (1 - rho - tau_(s^1)) H + sum sky B,
    w = denominators."""
    rows, nb, cnt, den, sky = m.graph()
    S = len(den)
    B = np.asarray(B, np.float64)
    src = np.repeat(np.arange(S), np.diff(rows.astype(np.int64)))
    G = np.bincount(src, weights=cnt.astype(np.float64) * B[nb], minlength=S)
    w = den.astype(np.float64)
    H = np.where(w > 0, (sky * L + G) / np.maximum(w, 1.0), L) + D
    pair = np.arange(S) ^ 1
    lhs = float((w * (D + e)).sum() + (sky * L).sum())
    rhs = float((w * (1.0 - rho - tau[pair]) * H).sum() + (sky * B).sum())
    return lhs, rhs


def test_perfect_reflector_sends_everything_to_the_sky():
    """rho = 1, tau = 0 everywhere in an open scene: nothing is absorbed, so
    at convergence all direct and sky input leaves to the sky:
    sum w D + sum sky L = sum sky B (raster graph: exact in count units)."""
    sc = scenes.config1(seed=5, leaves=150, grid=4)
    m, sun, lit = _model(sc, "raster")
    S = sc.surface_count
    rho = np.ones(S, np.float32)
    tau = np.zeros(S, np.float32)
    geo = scenes.direct_geometry(sc, lit, sun)
    for prec, tol, bar in ((facetcu.PRECISION_FP64, 1e-14, 1e-7),
                           (facetcu.PRECISION_MIXED, 1e-7, 1e-5)):
        out, res = m.solveBatched(np.stack([rho] * 32), np.stack([tau] * 32),
                                  np.full(32, 100.0, np.float32), np.full(32, 800.0, np.float32),
                                  geo[None, :], precision=prec, tolerance=tol,
                                  maximum_iterations=20000)
        assert res["converged"] == 1
        lhs, rhs = _raster_balance(m, rho.astype(np.float64), tau.astype(np.float64),
                                   np.zeros(S), geo.astype(np.float64) * 800.0, 100.0, out[0])
        assert abs(lhs - rhs) / lhs < bar, (prec, lhs, rhs)
    m.close()


def test_closed_box_absorbs_what_it_emits():
    """A closed box (walls, roof and floor) with an emitting floor inside and
    rho = 0.6 on every inner side: no sky reaches the inside, so the inner
    sides absorb exactly what the floor emits, and the outer sides (no sky,
    no sun) stay dark.  Raster graph, FP64 and MIXED."""
    sc = _closed_box()
    m, sun, lit = _model(sc, "raster")
    rows, nb, cnt, den, sky = m.graph()
    S = sc.surface_count
    n = sc.normals()
    centre = sc.vertices.reshape(-1, 3, 6)[:, :, :3].mean(1)
    inward = ((np.array([1.0, 0.75, 1.5]) - centre) * n).sum(1) > 0  # the normal side faces in
    inner = np.empty(S, bool)
    inner[0::2] = inward
    inner[1::2] = ~inward
    # closed: light leaves the inside only through rasterised cracks between
    # facets (the count-form balance below counts that leak as sky)
    assert sky[inner].sum() <= 1e-3 * den[inner].sum() and np.all(den[inner] > 0)
    floor = np.zeros(S, bool)
    floor_f = np.abs(centre[:, 1]) < 1e-6
    floor[0::2] = floor_f & inward
    floor[1::2] = floor_f & ~inward
    e = np.where(floor, 40.0, 0.0).astype(np.float32)
    rho = np.where(inner, 0.6, 0.0).astype(np.float32)
    tau = np.zeros(S, np.float32)
    for prec, tol, bar in ((facetcu.PRECISION_FP64, 1e-14, 1e-7),
                           (facetcu.PRECISION_MIXED, 1e-7, 1e-5)):
        out, res = m.solveBatched(np.stack([rho] * 32), np.stack([tau] * 32),
                                  np.zeros(32, np.float32), np.zeros(32, np.float32), None,
                                  emission=np.stack([e] * 32), precision=prec, tolerance=tol,
                                  maximum_iterations=20000)
        assert res["converged"] == 1
        B = out[0].astype(np.float64)
        assert np.all(B[~inner] == 0.0)
        lhs, rhs = _raster_balance(m, rho.astype(np.float64), tau.astype(np.float64),
                                   e.astype(np.float64), np.zeros(S), 0.0, B)
        assert abs(lhs - rhs) / lhs < bar, (prec, lhs, rhs)
    m.close()


@pytest.mark.parametrize("mode", ["raster", "hemisphere"])
def test_periodic_copies_count_no_energy_twice(mode):
    """A plane and its 8 periodic copies (coplanar, tiling the ground): no
    side sees another copy (no edges), so every side sees only sky and the
    radiosity equals the single plane's.  (The raster samples the plane
    with slightly different fragment counts once copies share its frame;
    with no edges the view factors are still all sky.)"""
    sc = _plane(cells=2)
    m0, sun, lit0 = _model(sc, mode)
    m8, _, lit8 = _model(sc, mode, periodic=(8, 2.0137, 2.0137))
    assert np.array_equal(lit0, lit8)
    g0, g8 = m0.graph(), m8.graph()
    assert g0[0][-1] == 0 and g8[0][-1] == 0
    assert np.array_equal(g8[3], g8[4]) and np.all(g8[4] > 0)
    S = sc.surface_count
    D = scenes.direct_geometry(sc, lit0, sun) * 800.0
    o = _optics(np.full(S, 0.25, np.float32), np.full(S, 0.05, np.float32),
                np.zeros(S, np.float32), D)
    assert np.array_equal(m0.solve(o, 100.0, 64)["radiosity"], m8.solve(o, 100.0, 64)["radiosity"])
    m0.close()
    m8.close()
