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
    assert rep["fixed_point_defect"] < 1e-14


def _equal_area_graph(rng, facets=6, denom=100):
    """Right triangles of area 0.5 and a symmetric count matrix with equal
    denominators: A_s F_sn = 0.5 c_sn / denom is symmetric (exact
    reciprocity)."""
    verts = np.zeros((facets * 3, 6), np.float32)
    for f in range(facets):
        verts[3 * f] = [f * 2.0, 0, 0, 0, 1, 0]
        verts[3 * f + 1] = [f * 2.0 + 1.0, 0, 0, 0, 1, 0]
        verts[3 * f + 2] = [f * 2.0, 0, 1.0, 0, 1, 0]
    S = 2 * facets
    c = rng.integers(0, 9, (S, S))
    c = np.triu(c, 1)
    c = c + c.T
    rows, nbrs, counts = [0], [], []
    for s in range(S):
        for n in range(S):
            if c[s, n]:
                nbrs.append(n)
                counts.append(c[s, n])
        rows.append(len(nbrs))
    den = np.full(S, denom, np.uint32)
    return verts, [np.array(rows, np.uint32), np.array(nbrs, np.uint32),
                   np.array(counts, np.uint32), den, den - np.array([c[s].sum() for s in range(S)],
                                                                    np.uint32)]


def test_exchange_metrics_reciprocity_and_conservation():
    """Exact reciprocity gives zero reciprocity error and a zero conservation
    residual for any radiosity; breaking one count's symmetry shows in both."""
    rng = np.random.default_rng(3)
    verts, g = _equal_area_graph(rng)
    B = [rng.uniform(1, 5, len(g[3])) for _ in range(3)]
    rec, cons = bench.exchange_metrics(g, verts, B, torch.device("cpu"))
    assert rec["weighted"] < 1e-15 and rec["reverse_edge_share"] == 1.0
    assert cons["max_over_bands"] < 1e-14
    g[2] = g[2].copy()
    g[2][0] += 3  # one directed count without its reverse change
    rec, cons = bench.exchange_metrics(g, verts, B, torch.device("cpu"))
    assert rec["weighted"] > 1e-3 and cons["max_over_bands"] > 1e-4
