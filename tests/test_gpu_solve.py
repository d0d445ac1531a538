"""Solves on the GPU through the C ABI against the CPU oracle.

Tolerances (floating point):
  * facetcu_solve / _accelerated (FP32 gather, reference radiosity.comp) vs
    the reference CPU solve (FP64 gather): max relative error 1e-5;
  * incident irradiance (FP64 gather on both sides): 1e-6;
  * batched FP64 vs the oracle's FP64 Jacobi: 1e-9;
  * batched FP32 and MIXED (BF16 defect + FP32 residual correction) vs FP64
    truth of the same graph: 1e-4 (the bar of the headline metric).
"""
import numpy as np
import pytest

from oracle.pyoracle import Graph
from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import model_for, oracle_cfg, rel_err, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


@pytest.fixture(scope="module")
def c1(oracle):
    sc = scenes.config1(seed=0)
    m = model_for(sc.vertices, 512, 64)
    m.buildVisibilityGraph(scenes.hemisphere_directions())
    sun = scenes.sun_direction(30, 135)
    lit = m.computeSunlitFraction(sun)
    g = Graph(*m.graph())
    yield dict(scene=sc, model=m, sun=sun, lit=lit, graph=g)
    m.close()


def test_solve_matches_reference_cpu_solver(oracle, c1):
    optics = scenes.reference_optics(c1["scene"], c1["lit"], c1["sun"])
    r = c1["model"].solve(optics, 100.0, 64, 1.0)
    b_ref, md_ref = oracle.solve(c1["graph"], optics, 100.0, 64)
    assert r["iterations"] == 64
    assert rel_err(r["radiosity"], b_ref) < 1e-5
    assert r["maxDelta"] <= 1e-3
    # diffuse-only baseline and light enhancement (facetrtcore.cpp:1561-1583)
    diffuse = optics.copy()
    diffuse[:, 3] = 0
    r0 = c1["model"].solve(diffuse, 100.0)
    b0, _ = oracle.solve(c1["graph"], diffuse, 100.0, 64)
    enh = np.maximum(0, r["radiosity"] - r0["radiosity"])
    enh_ref = np.maximum(0, b_ref - b0)
    assert np.max(np.abs(enh - enh_ref)) < 1e-5 * np.max(b_ref)


def test_solve_relaxation_and_validation(oracle, c1):
    optics = scenes.reference_optics(c1["scene"], c1["lit"], c1["sun"])
    r = c1["model"].solve(optics, 100.0, 200, 0.5)
    b_ref, _ = oracle.solve(c1["graph"], optics, 100.0, 200, 0.5)
    assert rel_err(r["radiosity"], b_ref) < 1e-5
    bad = optics.copy()
    bad[5, 0] = 0.9
    bad[5, 1] = 0.2
    with pytest.raises(ValueError, match="reflectance\\+transmittance"):
        c1["model"].solve(bad, 100.0)
    with pytest.raises(ValueError, match="relaxation"):
        c1["model"].solve(optics, 100.0, 8, 0.0)
    with pytest.raises(ValueError, match="skyRadiosity"):
        c1["model"].solve(optics, -1.0)
    with pytest.raises(ValueError):
        c1["model"].solve(optics[:-2], 100.0)


def test_solve_accelerated_semantics(oracle, c1):
    optics = scenes.reference_optics(c1["scene"], c1["lit"], c1["sun"])
    r = c1["model"].solveAccelerated(optics, 100.0, None, 64, 8, 1e-4, 1.0)
    assert r["iterations"] % 8 == 0 and r["iterations"] < 64
    assert r["maxDelta"] <= 1e-4
    b_ref, _ = oracle.solve(c1["graph"], optics, 100.0, r["iterations"])
    assert rel_err(r["radiosity"], b_ref) < 1e-5
    # warm start from the converged answer stops after the first batch
    w = c1["model"].solveAccelerated(optics, 100.0, r["radiosity"], 64, 8, 1e-4, 1.0)
    assert w["iterations"] == 8
    with pytest.raises(ValueError, match="Initial radiosity"):
        bad = r["radiosity"].copy()
        bad[0] = -1
        c1["model"].solveAccelerated(optics, 100.0, bad)


def test_incident_irradiance(oracle, c1):
    optics = scenes.reference_optics(c1["scene"], c1["lit"], c1["sun"])
    b, _ = oracle.solve(c1["graph"], optics, 100.0, 64)
    h = c1["model"].incidentIrradiance(b, optics, 100.0)
    h_ref = oracle.incident(c1["graph"], b, optics, 100.0)
    assert rel_err(h, h_ref) < 1e-6


def _bands(sc, lit, sun, bands):
    rho, tau = scenes.band_optics(sc, bands)
    dgeo = scenes.direct_geometry(sc, lit, sun)[None, :]
    sky = np.full(bands, 100.0, np.float32)
    beam = np.full(bands, 800.0, np.float32)
    return rho, tau, dgeo, sky, beam


def test_batched_fp64_matches_oracle_fp64(oracle, c1):
    sc = c1["scene"]
    rho, tau, dgeo, sky, beam = _bands(sc, c1["lit"], c1["sun"], 2)
    out, res = c1["model"].solveBatched(rho, tau, sky, beam, dgeo,
                                        precision=facetcu.PRECISION_FP64, tolerance=1e-13)
    assert res["converged"] == 1
    for b in range(2):
        optics = np.zeros((sc.surface_count, 4), np.float32)
        optics[:, 0] = rho[b]
        optics[:, 1] = tau[b]
        optics[:, 3] = dgeo[0] * beam[b]
        truth, _ = oracle.solve_f64(c1["graph"], optics, float(sky[b]), 2000, 1e-14)
        assert rel_err(out[b], truth) < 1e-6  # output rounded to float32


@pytest.mark.parametrize("precision", [facetcu.PRECISION_FP32, facetcu.PRECISION_MIXED])
@pytest.mark.parametrize("bands,suns", [(2, 1), (64, 1), (5, 3)])
def test_batched_meets_1e4_vs_fp64(c1, precision, bands, suns):
    sc = c1["scene"]
    rho, tau, _, sky, beam = _bands(sc, c1["lit"], c1["sun"], bands)
    sky = np.linspace(50, 150, bands).astype(np.float32)
    dgeo = np.stack([scenes.direct_geometry(sc, c1["lit"], scenes.sun_direction(z, 135))
                     for z in np.linspace(10, 60, suns)])
    truth, rt = c1["model"].solveBatched(rho, tau, sky, beam, dgeo,
                                         precision=facetcu.PRECISION_FP64, tolerance=1e-12)
    out, res = c1["model"].solveBatched(rho, tau, sky, beam, dgeo, precision=precision,
                                        tolerance=1e-6)
    assert res["converged"] == 1
    assert out.shape == (bands * suns, sc.surface_count)
    assert rel_err(out, truth) < 1e-4
    if precision == facetcu.PRECISION_MIXED:
        assert res["residual_corrections"] >= 1


def test_batched_column_layout_matches_single_solves(c1):
    """Column r = sun * bands + band equals the single-RHS solve of that band/sun."""
    sc = c1["scene"]
    bands, suns = 3, 2
    rho, tau, _, sky, beam = _bands(sc, c1["lit"], c1["sun"], bands)
    dgeo = np.stack([scenes.direct_geometry(sc, c1["lit"], scenes.sun_direction(z, 90))
                     for z in (20, 50)])
    out, _ = c1["model"].solveBatched(rho, tau, sky, beam, dgeo, tolerance=1e-7)
    for k in range(suns):
        for b in range(bands):
            single, _ = c1["model"].solveBatched(rho[b:b + 1], tau[b:b + 1], sky[b:b + 1],
                                                 beam[b:b + 1], dgeo[k:k + 1], tolerance=1e-7)
            assert rel_err(out[k * bands + b], single[0]) < 1e-5


def test_batched_warm_start_given(c1):
    sc = c1["scene"]
    rho, tau, dgeo, sky, beam = _bands(sc, c1["lit"], c1["sun"], 4)
    out, res = c1["model"].solveBatched(rho, tau, sky, beam, dgeo, tolerance=1e-6)
    out2, res2 = c1["model"].solveBatched(rho, tau, sky, beam, dgeo, tolerance=1e-6, initial=out)
    assert res2["iterations"] < res["iterations"] / 3
    assert rel_err(out2, out) < 1e-5


def test_mixed_graph_replay_matches_per_sweep_launches(c1):
    """The int8 phase run as one graph launch (a conditional WHILE node the
    device ends) gives the same bits as launching every step and check one
    by one (the sweep-timing mode), on a wide panel and on two panels of
    different widths."""
    sc = c1["scene"]
    for bands, suns in ((64, 1), (32, 3)):
        rho, tau, _, sky, beam = _bands(sc, c1["lit"], c1["sun"], bands)
        dgeo = np.stack([scenes.direct_geometry(sc, c1["lit"], scenes.sun_direction(z, 135))
                         for z in np.linspace(10, 60, suns)])
        kw = dict(precision=facetcu.PRECISION_MIXED, tolerance=1e-7, maximum_iterations=400,
                  raise_on_nonconvergence=False)
        a, ra = c1["model"].solveBatched(rho, tau, sky, beam, dgeo, **kw)
        b, rb = c1["model"].solveBatched(rho, tau, sky, beam, dgeo,
                                         flags=facetcu.BATCH_TIME_SWEEPS, **kw)
        assert ra["graph_launches"] > 0 and rb["graph_launches"] == 0
        assert ra["iterations"] == rb["iterations"]
        assert np.array_equal(a, b)


@pytest.mark.parametrize("limit", [4, 5, 9])
def test_mixed_loop_graph_stops_at_the_iteration_limit(c1, monkeypatch, limit):
    """A MIXED solve that cannot converge within maximum_iterations: the
    device loop stops at the limit (an odd budget leaves one step for the
    host to launch alone), reports it, and gives the same bits as launching
    every step one by one and as the steps launched without the loop graph
    (the path taken where conditional graph nodes are unavailable)."""
    sc = c1["scene"]
    rho, tau, dgeo, sky, beam = _bands(sc, c1["lit"], c1["sun"], 64)
    kw = dict(precision=facetcu.PRECISION_MIXED, tolerance=1e-9, maximum_iterations=limit,
              raise_on_nonconvergence=False)
    a, ra = c1["model"].solveBatched(rho, tau, sky, beam, dgeo, **kw)
    assert ra["converged"] == 0 and ra["iterations"] == limit
    b, rb = c1["model"].solveBatched(rho, tau, sky, beam, dgeo,
                                     flags=facetcu.BATCH_TIME_SWEEPS, **kw)
    assert rb["iterations"] == limit and np.array_equal(a, b)
    fresh = model_for(sc.vertices, 512, 64)
    fresh.setGraph(*c1["model"].graph())
    monkeypatch.setenv("FACETCU_TEST_NO_LOOP_GRAPH", "1")
    c, rc = fresh.solveBatched(rho, tau, sky, beam, dgeo, **kw)
    fresh.close()
    assert rc["graph_launches"] == 0 and rc["iterations"] == limit
    assert np.array_equal(a, c)


def test_scene_batch_matches_scenes_solved_alone():
    """facetcu_scene_batch: three scenes of uneven size (crops, urban, a
    config-1 field) as one block-diagonal graph.  Its FP64 solve equals each
    scene's own FP64 solve, and the MIXED solve of the batch (one launch per
    step over all three) meets the 1e-4 bar against it, with a thermal band
    as a 65th column (panels of 64 + 1)."""
    parts = [scenes.row_crops(6000, 3), scenes.urban(9000, 4), scenes.config1(5, 700, 10)]
    uv, dirs = scenes.hemisphere_samples(128, 8, seed=7)
    suv, _ = scenes.hemisphere_samples(64, 8, seed=8)
    models, rho, tau, emis, dgeo = [], [], [], [], []
    rng = np.random.default_rng(0)
    for i, sc in enumerate(parts):
        m = model_for(sc.vertices, 256, 64)
        m.buildHemisphereGraph(uv, dirs, 128, 64, 8)
        sun = scenes.sun_direction(20.0 + 15 * i, 40.0 * i)
        dgeo.append(scenes.direct_geometry(sc, m.hemisphereSunlit(sun, suv, 64, 8), sun))
        r, t = scenes.band_optics(sc, 64)
        tr, tt, te = scenes.thermal_optics(sc, rng.uniform(280, 320, sc.facet_count))
        rho.append(np.vstack([r, tr]))
        tau.append(np.vstack([t, tt]))
        emis.append(np.vstack([np.zeros_like(r), te]))
        models.append(m)
    sky = np.append(np.full(64, 100.0), facetcu.planck_radiance(11000.0, 250.0)).astype(np.float32)
    beam = np.append(np.full(64, 800.0), 0.0).astype(np.float32)
    batch = facetcu.FacetrtCuda()
    batch.initialize(16, 16, 8)
    offsets, diag = batch.sceneBatch(models)
    assert list(np.diff(offsets)) == [2 * sc.facet_count for sc in parts]
    cat = lambda xs: np.ascontiguousarray(np.concatenate(xs, axis=-1))
    args = (cat(rho), cat(tau), sky, beam, cat(dgeo)[None, :])
    truth, _ = batch.solveBatched(*args, emission=cat(emis), precision=facetcu.PRECISION_FP64,
                                  tolerance=1e-12, maximum_iterations=4000)
    for i, m in enumerate(models):
        alone, _ = m.solveBatched(rho[i], tau[i], sky, beam, dgeo[i][None, :], emission=emis[i],
                                  precision=facetcu.PRECISION_FP64, tolerance=1e-12,
                                  maximum_iterations=4000)
        # both FP64 to 1e-12, written as float32: equal to the last bits
        assert rel_err(truth[:, offsets[i]:offsets[i + 1]], alone) < 1e-6
    out, res = batch.solveBatched(*args, emission=cat(emis), precision=facetcu.PRECISION_MIXED,
                                  tolerance=1e-6)
    assert res["converged"] and rel_err(out, truth) < 1e-4
    # the pipelined scene step equals the register-gather one bit for bit
    reg, rres = batch.solveBatched(*args, emission=cat(emis), precision=facetcu.PRECISION_MIXED,
                                   tolerance=1e-6, flags=facetcu.BATCH_LEGACY_STEP)
    assert np.array_equal(out, reg) and res["iterations"] == rres["iterations"]
    for m in models + [batch]:
        m.close()


def test_batched_input_checks_on_host_and_device_paths(c1):
    """The optics, sky and beam checks of the batched solve (the reference's
    solve-time validation) run on the device for both entry points: a NaN,
    a negative value or rho + tau > 1 anywhere in bands x sides, a negative
    sky or beam, each raise the reference's message; valid inputs still
    solve afterwards."""
    torch = pytest.importorskip("torch")
    sc = c1["scene"]
    m = c1["model"]
    rho, tau, dgeo, sky, beam = _bands(sc, c1["lit"], c1["sun"], 8)
    cases = []
    r = rho.copy(); r[5, 123] = np.nan; cases.append((r, tau, sky, beam, "Optical values"))
    t = tau.copy(); t[7, -1] = -0.1; cases.append((rho, t, sky, beam, "Optical values"))
    r = rho.copy(); r[2, 77] = 0.9; t = tau.copy(); t[2, 77] = 0.2
    cases.append((r, t, sky, beam, "Optical values"))
    k = sky.copy(); k[3] = -1.0; cases.append((rho, tau, k, beam, "skyRadiosity"))
    b = beam.copy(); b[6] = np.inf; cases.append((rho, tau, sky, b, "beam irradiance"))
    dev = torch.device("cuda")
    S = sc.surface_count
    out = torch.empty((8, S), dtype=torch.float32, device=dev)
    for r, t, k, b, msg in cases:
        with pytest.raises(ValueError, match=msg):
            m.solveBatched(r, t, k, b, dgeo)
        d = {n: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
             for n, v in (("r", r), ("t", t), ("k", k), ("b", b), ("g", dgeo))}
        torch.cuda.synchronize()
        cfg = facetcu.BatchConfig(8, 1, facetcu.PRECISION_MIXED, facetcu.WARM_NONE, 200, 1e-5, 0, 0)
        with pytest.raises(ValueError, match=msg):
            m.solveBatchedDevice(cfg, d["r"].data_ptr(), d["t"].data_ptr(), None,
                                 d["k"].data_ptr(), d["b"].data_ptr(), d["g"].data_ptr(), None,
                                 out.data_ptr())
    ok, res = m.solveBatched(rho, tau, sky, beam, dgeo, tolerance=1e-5)
    assert res["converged"] and np.all(np.isfinite(ok))


def test_autotune_panel_width_and_cache(c1, tmp_path):
    """facetcu_autotune_batched times the panel widths (and the pipelined
    step's CTAs per SM) on short solves, keeps the fastest (one of 32/64/128
    not wider than the columns), writes it to
    the JSON-lines cache, and later solves with panel_width = 0 use it: the
    same bits as a solve with that width given explicitly, also in a fresh
    context that only reads the cache."""
    torch = pytest.importorskip("torch")
    sc = c1["scene"]
    m = c1["model"]
    rho, tau, _, sky, beam = _bands(sc, c1["lit"], c1["sun"], 32)
    dgeo = np.stack([scenes.direct_geometry(sc, c1["lit"], scenes.sun_direction(z, 135))
                     for z in (20, 40, 60)])
    dev = torch.device("cuda")
    d = {n: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for n, v in (("r", rho), ("t", tau), ("k", sky), ("b", beam), ("g", dgeo))}
    out = torch.empty((96, sc.surface_count), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    ptrs = (d["r"].data_ptr(), d["t"].data_ptr(), None, d["k"].data_ptr(), d["b"].data_ptr(),
            d["g"].data_ptr())
    cache = tmp_path / "tune.jsonl"
    cfg = facetcu.BatchConfig(32, 3, facetcu.PRECISION_MIXED, facetcu.WARM_NONE, 500, 1e-5, 0, 0)
    best = m.autotuneBatched(cfg, *ptrs, out.data_ptr(), str(cache))
    assert best in (32, 64)  # 96 columns: 128 would only pad
    text = cache.read_text()
    assert f'"panel_width": {best}' in text and "|R=96|precision=1" in text

    def solve(model, width):
        c = facetcu.BatchConfig(32, 3, facetcu.PRECISION_MIXED, facetcu.WARM_NONE, 500, 1e-5,
                                width, 0)
        model.solveBatchedDevice(c, *ptrs, None, out.data_ptr())
        return out.cpu().numpy()

    tuned = solve(m, 0)
    assert np.array_equal(tuned, solve(m, best))
    fresh = model_for(sc.vertices, 512, 64)
    fresh.setGraph(*m.graph())
    assert fresh.autotuneBatched(cfg, *ptrs, out.data_ptr(), str(cache)) == best  # from the cache
    assert np.array_equal(solve(fresh, 0), tuned)
    fresh.close()
    # the pipelined step's CTAs per SM (the tuner's second parameter) change
    # the time, not the bits: a cached choice of 64 columns at 1 CTA per SM
    # equals the explicit 64-column solve at the occupancy limit
    import json
    key = json.loads(text.splitlines()[0])["key"]
    assert '"step_ctas_per_sm": ' in text
    one = tmp_path / "tune_one_cta.jsonl"
    one.write_text(json.dumps({"key": key, "panel_width": 64, "step_ctas_per_sm": 1}) + "\n")
    slow = model_for(sc.vertices, 512, 64)
    slow.setGraph(*m.graph())
    assert slow.autotuneBatched(cfg, *ptrs, out.data_ptr(), str(one)) == 64
    assert np.array_equal(solve(slow, 0), solve(slow, 64))
    slow.close()


@pytest.mark.parametrize("kind,suns", [("forest", 1), ("coarse_soil", 1), ("forest", 2),
                                       ("coarse_soil", 2)])
def test_pipelined_int8_step_bit_identical(kind, suns):
    """The 64-column int8 step runs as an asynchronous-copy pipeline (rows
    staged in shared memory by cp.async); FACETCU_BATCH_LEGACY_STEP runs the
    register-gather kernel instead.  Both sum exactly in int32, so the
    radiosity must be the same bits and the sweep counts the same; the
    result meets the 1e-4 bar against FP64.  With two suns the 128 columns
    run as one 128-column panel (the pipelined kernel's 4-group layout).
    Both graphs have empty rows
    (downward soil sides); the coarse soil (2.5 m quads under low leaves)
    has counts above 255, which the solver's copy of the graph splits into
    edges of at most 255 (the pipelined step takes every count as one
    byte; the register-gather kernel, run on the same copy, adds high bytes
    when a count has them)."""
    if kind == "forest":
        sc = scenes.forest(6, 20.0, 2000, 3, name="step")
    else:
        sc = scenes.config1(seed=3, leaves=2048, grid=4)
    m = facetcu.FacetrtCuda()
    m.initialize(512, 512, 1024)
    m.setGeometry(sc.vertices)
    sun = scenes.sun_direction(30.0, 135.0)
    uv, dirs = scenes.hemisphere_samples(512, 32, seed=7)
    m.buildHemisphereGraph(uv, dirs, 512, 256, 32)
    suv, _ = scenes.hemisphere_samples(256, 32, seed=8)
    lit = m.hemisphereSunlit(sun, suv, 256, 32)
    rows, _, counts, _, _ = m.graph()
    assert np.any(np.diff(rows) == 0)  # empty rows
    if kind == "coarse_soil":
        assert 255 < counts.max() < 1024  # packed graph, counts above one byte
    rho, tau, dgeo, sky, beam = _bands(sc, lit, sun, 64)
    if suns == 2:
        sun2 = scenes.sun_direction(55.0, 250.0)
        lit2 = m.hemisphereSunlit(sun2, suv, 256, 32)
        dgeo = np.vstack([dgeo, scenes.direct_geometry(sc, lit2, sun2)[None, :]])
    a, ra = m.solveBatched(rho, tau, sky, beam, dgeo, precision=facetcu.PRECISION_MIXED,
                           tolerance=1e-6)
    b, rb = m.solveBatched(rho, tau, sky, beam, dgeo, precision=facetcu.PRECISION_MIXED,
                           tolerance=1e-6, flags=facetcu.BATCH_LEGACY_STEP)
    assert ra["iterations"] == rb["iterations"]
    assert ra["kernel_launches"] == rb["kernel_launches"]
    assert np.array_equal(a, b)
    truth, _ = m.solveBatched(rho, tau, sky, beam, dgeo, precision=facetcu.PRECISION_FP64,
                              tolerance=1e-12, maximum_iterations=4000)
    assert rel_err(a, truth) < 1e-4
    m.close()


def test_pipelined_scene_step_128_columns_bit_identical():
    """A scene batch solved on 128-column panels (64 bands x 2 suns): the
    pipelined step with per-scene scales and stops gives the same bits as
    the register-gather kernel, and meets the 1e-4 bar against FP64."""
    parts = [scenes.row_crops(5000, 7), scenes.urban(8000, 8), scenes.config1(9, 600, 10)]
    uv, dirs = scenes.hemisphere_samples(128, 8, seed=7)
    suv, _ = scenes.hemisphere_samples(64, 8, seed=8)
    models, rho, tau, dgeo = [], [], [], []
    for i, sc in enumerate(parts):
        m = model_for(sc.vertices, 256, 64)
        m.buildHemisphereGraph(uv, dirs, 128, 64, 8)
        rows = []
        for sun in (scenes.sun_direction(25.0 + 10 * i, 30.0 * i),
                    scenes.sun_direction(50.0, 200.0 + 20 * i)):
            rows.append(scenes.direct_geometry(sc, m.hemisphereSunlit(sun, suv, 64, 8), sun))
        dgeo.append(np.stack(rows))
        r, t = scenes.band_optics(sc, 64)
        rho.append(r)
        tau.append(t)
        models.append(m)
    batch = facetcu.FacetrtCuda()
    batch.initialize(16, 16, 8)
    batch.sceneBatch(models)
    cat = lambda xs: np.ascontiguousarray(np.concatenate(xs, axis=-1))
    args = (cat(rho), cat(tau), np.full(64, 100.0, np.float32), np.full(64, 800.0, np.float32),
            cat(dgeo))
    out, res = batch.solveBatched(*args, precision=facetcu.PRECISION_MIXED, tolerance=1e-6,
                                  panel_width=128)
    reg, rres = batch.solveBatched(*args, precision=facetcu.PRECISION_MIXED, tolerance=1e-6,
                                   panel_width=128, flags=facetcu.BATCH_LEGACY_STEP)
    assert res["converged"] and res["iterations"] == rres["iterations"]
    assert np.array_equal(out, reg)
    truth, _ = batch.solveBatched(*args, precision=facetcu.PRECISION_FP64, tolerance=1e-12,
                                  maximum_iterations=4000)
    assert rel_err(out, truth) < 1e-4
    for m in models + [batch]:
        m.close()
