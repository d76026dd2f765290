"""The FP64 oracle of the admissibility network: its backward pass against
central finite differences of its own forward pass (pins the oracle the GPU
kernels are checked against)."""
import numpy as np


def test_oracle_gradient_matches_finite_differences(oracle_mod):
    rng = np.random.default_rng(5)
    n = oracle_mod.mlp_param_count()
    assert n == 8 * 64 + 64 + 2 * (64 * 64 + 64) + 64 + 1
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
