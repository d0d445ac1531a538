"""The library's MLP kernels (forward, backward, Adam) through the C ABI
against the float64 CPU oracle (oracle/mlp_oracle.py).

Tolerances: forward outputs 1e-4 relative to the output scale (FP32
activations vs float64); gradients 2e-3 relative in the L2 norm and per
parameter tensor (FP32 accumulation over the batch)."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from streamsim_gb300 import facetcu, scenes
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    require_gpu()
    m = facetcu.FacetrtCuda()
    m.initialize(16, 16, 8)
    m.mlpReset(7)
    yield m
    m.close()


def test_parameter_round_trip(model):
    p = model.mlpParameters()
    assert p.size == M.COUNT == facetcu.MLP_PARAMETERS
    assert np.all(np.isfinite(p)) and np.abs(p).max() < 1.0
    q = p * 0.5
    model.mlpSetParameters(q)
    assert np.array_equal(model.mlpParameters(), q)
    model.mlpSetParameters(p)


@pytest.mark.parametrize("n", [5, 300, 4096])
def test_forward_and_gradient_match_cpu_oracle(model, n):
    rng = np.random.default_rng(n)
    params = rng.normal(scale=0.15, size=M.COUNT).astype(np.float32)
    model.mlpSetParameters(params)
    x = rng.normal(size=(n, 12)).astype(np.float32)
    t = rng.normal(size=(n, 64)).astype(np.float32)
    y = model.mlpForward(x)
    y_ref, _ = M.forward(params, x)
    assert np.max(np.abs(y - y_ref)) <= 1e-4 * max(1.0, np.abs(y_ref).max())
    loss, g = model.mlpLossAndGradient(x, t)
    loss_ref, g_ref = M.loss_and_grad(params, x, t)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    assert np.linalg.norm(g - g_ref) <= 2e-3 * np.linalg.norm(g_ref)
    off = 0
    for name, shape in M.SIZES:
        k = int(np.prod(shape))
        a, b = g[off:off + k], g_ref[off:off + k]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b) + 1e-12, name
        off += k


@pytest.mark.parametrize("n", [5, 300, 4096, 100003])
def test_tensor_core_forward(model, n):
    """facetcu_mlp_forward_tensor (tcgen05.mma on 128-row tiles, BF16
    operands from TMA, FP32 accumulation in tensor memory; partial last
    tiles at 5, 300 and 100,003 rows): against the oracle with the same BF16
    roundings of inputs and hidden activations (5e-3 of the output scale:
    the FP32 accumulation order can move an activation across a BF16
    rounding boundary), and against the FP32-activation path (3e-2, the
    BF16 activations' own effect)."""
    rng = np.random.default_rng(n + 1)
    params = rng.normal(scale=0.15, size=M.COUNT).astype(np.float32)
    model.mlpSetParameters(params)
    x = rng.normal(size=(n, 12)).astype(np.float32)
    y = model.mlpForwardTensor(x)
    scale = max(1.0, float(np.abs(y).max()))
    ref = M.forward_bf16_activations(params, x)
    assert np.all(np.isfinite(y))
    assert np.max(np.abs(y - ref)) <= 5e-3 * scale
    assert np.max(np.abs(y - model.mlpForward(x))) <= 3e-2 * scale
    # a second call reuses the buffers and gives the same bits
    assert np.array_equal(model.mlpForwardTensor(x), y)


def test_training_reduces_loss_on_a_learnable_map(model):
    """Adam on device data: fit y = tanh(x A) for a fixed A."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    A = rng.normal(scale=0.5, size=(12, 64))
    x = rng.normal(size=(20000, 12)).astype(np.float32)
    t = np.tanh(x @ A).astype(np.float32)
    model.mlpReset(11)
    loss0, _ = model.mlpLossAndGradient(x[:2048], t[:2048])
    dx = torch.from_numpy(x).cuda()
    dt = torch.from_numpy(t).cuda()
    torch.cuda.synchronize()
    final = model.mlpTrainDevice(dx.data_ptr(), dt.data_ptr(), len(x), 300, 1024, 3e-3, 5)
    loss1, _ = model.mlpLossAndGradient(x[:2048], t[:2048])
    assert final < 0.5 * loss0 and loss1 < 0.3 * loss0


# ---- the warm start inside the batched solver --------------------------------
@pytest.fixture(scope="module")
def small_scene():
    from streamsim_gb300 import scenes
    from tests.gpu_helpers import model_for
    require_gpu()
    sc = scenes.config1(seed=3, leaves=1024, grid=16)
    m = model_for(sc.vertices, 256, 64)
    m.buildVisibilityGraph(scenes.hemisphere_directions())
    sun = scenes.sun_direction(30, 135)
    lit = m.computeSunlitFraction(sun)
    rho, tau = scenes.band_optics(sc, 64)
    case = dict(scene=sc, model=m, rho=rho, tau=tau,
                dgeo=scenes.direct_geometry(sc, lit, sun)[None, :],
                sky=np.linspace(80, 120, 64).astype(np.float32),
                beam=np.linspace(700, 900, 64).astype(np.float32))
    yield case
    m.close()


def test_samples_are_first_sweep_features_and_scaled_remainder(small_scene):
    """facetcu_mlp_samples_device: features from the first FP32 sweep B1,
    targets (B - B1) / (sky + beam), checked against host recomputation."""
    torch = pytest.importorskip("torch")
    c = small_scene
    m = c["model"]
    S = c["scene"].surface_count
    args = (c["rho"], c["tau"], c["sky"], c["beam"], c["dgeo"])
    b1, _ = m.solveBatched(*args, precision=facetcu.PRECISION_FP32, maximum_iterations=1,
                           tolerance=0.0, raise_on_nonconvergence=False)
    truth, _ = m.solveBatched(*args, precision=facetcu.PRECISION_FP64, tolerance=1e-12,
                              maximum_iterations=4000)
    dev = torch.device("cuda")
    t = {k: torch.from_numpy(np.ascontiguousarray(c[k])).to(dev)
         for k in ("rho", "tau", "sky", "beam", "dgeo")}
    conv = torch.from_numpy(truth).to(dev)
    x = torch.zeros((S, 12), dtype=torch.float32, device=dev)
    y = torch.zeros((S, 64), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    cfg = facetcu.BatchConfig(64, 1, facetcu.PRECISION_FP32, facetcu.WARM_NONE, 1, 0.0, 0, 0)
    m.mlpSamplesDevice(cfg, t["rho"].data_ptr(), t["tau"].data_ptr(), None, t["sky"].data_ptr(),
                       t["beam"].data_ptr(), t["dgeo"].data_ptr(), conv.data_ptr(), x.data_ptr(),
                       y.data_ptr())
    x = x.cpu().numpy()
    y = y.cpu().numpy()
    ref = (c["sky"] + c["beam"]).astype(np.float32)
    for g in range(8):
        b = 9 * g
        assert np.allclose(x[:, g], b1[b] / ref[b], rtol=1e-6, atol=0)
    assert np.array_equal(x[:, 8], c["rho"][32]) and np.array_equal(x[:, 9], c["tau"][32])
    _, _, _, den, skyc = m.graph()
    frac = np.where(den > 0, skyc / np.maximum(den, 1), 1.0).astype(np.float32)
    assert np.allclose(x[:, 10], frac, rtol=1e-6, atol=0)
    ny = c["scene"].normals()[:, 1].astype(np.float32)
    side_ny = np.empty(S, np.float32)
    side_ny[0::2] = ny
    side_ny[1::2] = -ny
    assert np.allclose(x[:, 11], side_ny, atol=1e-6)
    assert np.allclose(y, ((truth - b1) / ref[:, None]).T, rtol=1e-5, atol=1e-7)


def test_warm_start_argument_checks(small_scene):
    c = small_scene
    args = (c["rho"], c["tau"], c["sky"], c["beam"], c["dgeo"])
    fresh = facetcu.FacetrtCuda()
    fresh.initialize(256, 256, 64)
    fresh.setGeometry(c["scene"].vertices)
    fresh.buildVisibilityGraph(scenes.hemisphere_directions())
    with pytest.raises(facetcu.LogicError):
        fresh.solveBatched(*args, warm_start=facetcu.WARM_MLP)
    fresh.mlpReset(2)
    with pytest.raises(ValueError):
        fresh.solveBatched(c["rho"][:32], c["tau"][:32], c["sky"][:32], c["beam"][:32], c["dgeo"],
                           warm_start=facetcu.WARM_MLP)
    fresh.close()


def test_mlp_warm_start_converges_to_the_same_answer(small_scene):
    """Any parameters (here untrained) give a start the solver converges
    from to the FP64 answer within the 1e-4 bar."""
    c = small_scene
    m = c["model"]
    m.mlpReset(4)
    args = (c["rho"], c["tau"], c["sky"], c["beam"], c["dgeo"])
    truth, _ = m.solveBatched(*args, precision=facetcu.PRECISION_FP64, tolerance=1e-12,
                              maximum_iterations=4000)
    for prec in (facetcu.PRECISION_FP32, facetcu.PRECISION_MIXED):
        out, res = m.solveBatched(*args, precision=prec, tolerance=1e-6, maximum_iterations=2000,
                                  warm_start=facetcu.WARM_MLP)
        scale = np.maximum(np.abs(truth), 1e-6 * np.abs(truth).max())
        assert np.max(np.abs(out - truth) / scale) <= 1e-4
        assert res["converged"]


def test_trained_warm_start_on_an_unseen_forest():
    """The shipped weights (trained by streamsim_gb300/train_mlp.py on other
    forest seeds and random optics) against the cold start on the
    benchmark's forest family at an unseen seed.  Both meet the 1e-4 bar
    against FP64.  On this family the solve from zero already reaches the
    1e-6 stop rule in about 19 sweeps, and the learned start (one FP32 sweep
    plus the network) lands within one sweep of it: the bound below is a
    regression check, not a claimed gain."""
    import os

    from streamsim_gb300 import train_mlp
    require_gpu()
    assert os.path.exists(facetcu.WARM_START_WEIGHTS), "trained warm-start weights missing"
    args = train_mlp.parse([])
    case = train_mlp.make_case(facetcu, scenes, 10005, train_mlp.fixed_optics(), args)
    truth = train_mlp.solve_truth(facetcu, case)
    row = train_mlp.evaluate(facetcu, case, truth, np.load(facetcu.WARM_START_WEIGHTS), 1e-6)
    case["model"].close()
    assert row["cold"]["max_rel_err"] <= 1e-4 and row["mlp"]["max_rel_err"] <= 1e-4
    assert row["mlp"]["iterations"] <= row["cold"]["iterations"] + 1, row


def test_tensor_core_wait_times_out_and_context_survives(model, monkeypatch):
    """A bounded wait that runs out: with the test switch set, the tensor
    kernels' load barrier expects more bytes than arrive, each CTA's wait
    gives up after 1 s, frees its tensor memory and raises the error flag,
    and the call returns FACETCU_DEVICE_TIMEOUT; the next call, without the
    switch, computes the right answer in the same context."""
    rng = np.random.default_rng(11)
    params = rng.normal(scale=0.15, size=M.COUNT).astype(np.float32)
    model.mlpSetParameters(params)
    x = rng.normal(size=(5, 12)).astype(np.float32)  # one CTA per layer
    monkeypatch.setenv("FACETCU_TEST_STALL_TENSOR_WAIT", "1")
    with pytest.raises(facetcu.FacetcuError) as err:
        model.mlpForwardTensor(x)
    assert err.value.code == facetcu.DEVICE_TIMEOUT
    monkeypatch.delenv("FACETCU_TEST_STALL_TENSOR_WAIT")
    y = model.mlpForwardTensor(x)
    assert np.max(np.abs(y - M.forward_bf16_activations(params, x))) <= 5e-3 * max(1.0, np.abs(y).max())
