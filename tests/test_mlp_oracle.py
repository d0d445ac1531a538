"""The CPU MLP oracle's hand-written backprop against central finite
differences in float64 (the check that makes it usable as the reference
for the device gradients)."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_backprop_matches_finite_differences():
    rng = np.random.default_rng(0)
    params = rng.normal(scale=0.2, size=M.COUNT).astype(np.float32)
    x = rng.normal(size=(7, 12))
    t = rng.normal(size=(7, 64))
    _, g = M.loss_and_grad(params, x, t)
    eff = M.effective(params)
    flat = M.pack(eff)
    h = 1e-6
    for i in rng.choice(M.COUNT, 60, replace=False):
        plus, minus = flat.copy(), flat.copy()
        plus[i] += h
        minus[i] -= h
        fd = (M.loss_only(M.unpack(plus), x, t) - M.loss_only(M.unpack(minus), x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd)


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, 3.1415926, -2.5e-3], np.float32)
    r = M.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway rounds to even
    assert r[2] == 1.0078125
    assert abs(r[3] - 3.140625) < 1e-12
