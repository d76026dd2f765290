"""The FP64 oracle of the admissibility network (hidden width 64 and 128):
its backward pass against central finite differences of its own forward
pass (pins the oracle the GPU kernels are checked against)."""
import numpy as np
import pytest


@pytest.mark.parametrize("width", [64, 128])
def test_oracle_gradient_matches_finite_differences(oracle_mod, width):
    rng = np.random.default_rng(5)
    oracle_mod.mlp_set_width(width)
    try:
        _check(oracle_mod, rng, width)
    finally:
        oracle_mod.mlp_set_width(64)


def _check(oracle_mod, rng, w):
    n = oracle_mod.mlp_param_count()
    assert n == 8 * w + w + 2 * (w * w + w) + w + 1
    p = (rng.standard_normal(n) * 0.2).astype(np.float32)
    X = rng.standard_normal((6, 8)).astype(np.float32)
    y = rng.standard_normal(6).astype(np.float32)
    loss, g = oracle_mod.mlp_grad(p, X, y)
    pred = oracle_mod.mlp_forward(p, X)
    assert abs(loss - np.mean((pred - y) ** 2)) < 1e-12 * max(1.0, loss)
    # finite differences in FP64 need parameters exactly representable after
    # the step: perturb by powers of two on float32 parameters
    idx = rng.choice(n, 40, replace=False)
    worst = 0.0
    for k in idx:
        h = 2.0 ** -12
        pp = p.copy()
        pm = p.copy()
        pp[k] += np.float32(h)
        pm[k] -= np.float32(h)
        lp, _ = oracle_mod.mlp_grad(pp, X, y)
        lm, _ = oracle_mod.mlp_grad(pm, X, y)
        fd = (lp - lm) / (float(pp[k]) - float(pm[k]))
        worst = max(worst, abs(fd - g[k]) / max(1e-3, abs(g[k])))
    assert worst < 1e-3, worst
