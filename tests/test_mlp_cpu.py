"""CPU tests of the learned tuner's oracle: the numpy network's analytic gradient against
central finite differences, and the soft-target construction."""
import numpy as np

from oracle import mlp_oracle
from benchmark_spmv_using_csr_gb300 import mlp


def test_numpy_gradient_matches_finite_differences():
    I, H, K, B = 16, 8, 5, 7
    rng = np.random.default_rng(0)
    p = mlp.init_params(I, H, K, seed=3).astype(np.float64)
    p[H * I:H * I + H] = rng.standard_normal(H) * 0.1  # non-zero biases
    f = rng.standard_normal((B, I))
    t = mlp.soft_targets(rng.uniform(1, 2, (B, K))).astype(np.float64)
    mean, std = f.mean(0), f.std(0)
    loss, g = mlp_oracle.loss_and_grad(p, f, t, mean, std, I, H, K)
    eps = 1e-6
    for j in rng.choice(p.size, 40, replace=False):
        e = np.zeros_like(p)
        e[j] = eps
        lp, _ = mlp_oracle.loss_and_grad(p + e, f, t, mean, std, I, H, K)
        lm, _ = mlp_oracle.loss_and_grad(p - e, f, t, mean, std, I, H, K)
        assert abs((lp - lm) / (2 * eps) - g[j]) <= 1e-6 * max(1.0, abs(g[j]))


def test_soft_targets():
    ms = np.array([[1.0, 1.01, 2.0, 1.5]])
    t = mlp.soft_targets(ms, 0.05)
    assert abs(t.sum() - 1) < 1e-6 and t[0, 0] > t[0, 1] > t[0, 3] > t[0, 2]
    assert t[0, 0] / t[0, 1] < 1.3  # near-ties share mass
