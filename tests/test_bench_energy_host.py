"""bench.py's FP64 energy accounting (no GPU): on a random graph with
symmetric counts and equal side denominators, the closure it reports is
zero for the exact solution and equals the relative defect of the energy
balance sum w D + sum sky L + sum w e = sum w (1 - rho - tau_(s^1)) H +
sum sky B for any other."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
import bench  # noqa: E402


def _system(seed=0, F=200, bands=3):
    rng = np.random.default_rng(seed)
    S = 2 * F
    C = np.zeros((S, S))
    for _ in range(3000):
        a, b = rng.integers(0, S, 2)
        if a // 2 != b // 2:
            C[a, b] += 1
            C[b, a] += 1
    C[6:8, :] = 0.0  # facet 3 sees nothing: denominator 0 on both sides
    C[:, 6:8] = 0.0
    sky = rng.integers(0, 20, S).astype(np.float64)
    sky[6:8] = 0.0
    den = C.sum(1) + sky
    top = np.maximum(den[0::2], den[1::2])  # equal samples on both sides
    sky[0::2] += top - den[0::2]
    sky[1::2] += top - den[1::2]
    den = C.sum(1) + sky
    rows = np.concatenate([[0], np.cumsum((C > 0).sum(1))]).astype(np.uint32)
    nbrs = np.concatenate([np.nonzero(C[i])[0] for i in range(S)]).astype(np.uint32)
    cnts = np.concatenate([C[i][C[i] > 0] for i in range(S)]).astype(np.uint32)

    class Model:
        def graph(self):
            return rows, nbrs, cnts, den.astype(np.uint32), sky.astype(np.uint32)

    verts = rng.uniform(0, 1, (F, 3, 6)).reshape(-1, 6)
    rho = rng.uniform(0.05, 0.5, (bands, S))
    tau = 0.3 * rho
    emis = rng.uniform(0, 20, (bands, S)) * (rng.random((1, S)) < 0.3)
    L = np.array([100.0, 50.0, 80.0][:bands])
    beam = np.array([800.0, 600.0, 0.0][:bands])
    dgeo = rng.uniform(0, 1, S)
    pair = np.arange(S) ^ 1
    Wn = np.where(den[:, None] > 0, C / np.maximum(den, 1)[:, None], 0.0)
    exact = []
    for b in range(bands):
        H0 = np.where(den > 0, sky * L[b] / np.maximum(den, 1), L[b]) + beam[b] * dgeo
        M = np.diag(rho[b]) @ Wn + np.diag(tau[b]) @ np.eye(S)[pair] @ Wn
        E = emis[b] + rho[b] * H0 + tau[b] * H0[pair]
        exact.append(np.linalg.solve(np.eye(S) - M, E))
    return Model(), verts, rho, tau, emis, L, beam, dgeo, np.array(exact), C, den, sky


def test_closure_is_the_energy_balance_defect():
    model, verts, rho, tau, emis, L, beam, dgeo, exact, C, den, sky = _system()
    pert = exact * (1 + 1e-4 * np.random.default_rng(1).standard_normal(exact.shape))
    got = bench.energy_metrics(model, verts, rho, tau, L, beam, dgeo, [exact, pert],
                               torch.device("cpu"), emission=emis)
    assert got[0]["closure"] < 1e-14
    pair = np.arange(len(den)) ^ 1
    defects = []
    for b in range(len(L)):
        B = pert[b]
        H = np.where(den > 0, (sky * L[b] + C @ B) / np.maximum(den, 1), L[b]) + beam[b] * dgeo
        src = (den * (beam[b] * dgeo + emis[b])).sum() + (sky * L[b]).sum()
        sink = (den * (1 - rho[b] - tau[b][pair]) * H).sum() + (sky * B).sum()
        defects.append(abs(src - sink) / src)
    assert got[1]["closure"] == pytest.approx(max(defects), rel=1e-9)
    assert got[1]["closure"] > 1e-7


def test_report_compares_with_the_fp64_solution():
    model, verts, rho, tau, emis, L, beam, dgeo, exact, *_ = _system(seed=2)
    rep = bench.energy_report(model, verts, rho, tau, L, beam, dgeo[None, :], exact.copy(),
                              exact, torch.device("cpu"), emission=emis)
    assert rep["absorbed_rel_err_vs_fp64"] == 0.0 and rep["rel_err_per_side"]["max"] == 0.0
    assert rep["closure_residual"] < 1e-14
