"""The scorer's CPU oracle itself: its analytic gradient against central
finite differences of its loss (BF16 roundings off, so the loss is smooth),
and its BF16 rounding."""
import numpy as np


def test_oracle_gradient_matches_finite_differences():
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(0)
    nf, h = 16, 64
    npar = h * nf + h + h * h + h + h + 1
    params = rng.normal(0, 0.3, npar)
    mean = np.zeros(16, np.float32)
    inv_std = np.ones(16, np.float32)
    X = rng.normal(0, 1, (64, 16)).astype(np.float32)
    y = (rng.random(64) < 0.3).astype(np.float64)
    g, _ = M.gradient(params, mean, inv_std, X, y, 2.0, exact=True)
    picks = [5, 300, h * nf + 3, h * nf + h + 17, h * nf + h + 2000, h * nf + h + h * h + 9,
             h * nf + h + h * h + h + 30, npar - 1]
    for i in picks:
        e = 1e-5
        pp, pm = params.copy(), params.copy()
        pp[i] += e
        pm[i] -= e
        fd = (M.gradient(pp, mean, inv_std, X, y, 2.0, exact=True)[1] -
              M.gradient(pm, mean, inv_std, X, y, 2.0, exact=True)[1]) / (2 * e)
        assert abs(fd - g[i]) < 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_round_is_nearest_even():
    from oracle import mlp_oracle as M
    x = np.array([1.0, 1.00390625, 1.0078125, 1.01171875, -2.5], np.float32)
    r = M.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == 1.015625 and r[4] == -2.5
