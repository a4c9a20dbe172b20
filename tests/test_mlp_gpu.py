"""GPU tests of the learned tuner's CUDA kernels (bhsp_mlp_*) through the C ABI: forward
probabilities and gradients against the numpy oracle, and training that learns a toy mapping.
If the committed GB300 model and timing tables are present, their held-out evaluation is
recomputed and must reach >= 95 % of the autotuner-best time."""
import os

import numpy as np
import pytest

from oracle import mlp_oracle
from benchmark_spmv_using_csr_gb300 import mlp

pytestmark = pytest.mark.gpu


def test_forward_and_gradients_match_oracle(cuda_ok):
    I, H, K, B = 16, 64, 18, 300
    rng = np.random.default_rng(1)
    net = mlp.MLP(I, H, K, max_batch=512, seed=5)
    p = net.get_params().astype(np.float64)
    p += rng.standard_normal(p.size) * 0.01
    net.set_params(p.astype(np.float32))
    f = rng.standard_normal((B, I)).astype(np.float32) * 3 + 1
    mean, std = f.mean(0), f.std(0)
    net.set_normalization(mean, std)
    t = mlp.soft_targets(rng.uniform(1, 3, (B, K)))
    probs = net.forward(f)
    ref = mlp_oracle.forward(net.get_params(), f, mean, std, I, H, K)["p"]
    np.testing.assert_allclose(probs, ref, rtol=2e-4, atol=1e-6)
    g, loss = net.gradients(f, t)
    loss_ref, g_ref = mlp_oracle.loss_and_grad(net.get_params(), f, t, mean, std, I, H, K)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref)
    err = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert err <= 1e-4, err
    net.close()


def test_training_learns_a_toy_rule(cuda_ok):
    rng = np.random.default_rng(2)
    n, K = 1500, 6
    f = rng.standard_normal((n, 16)).astype(np.float32)
    best = (np.floor((f[:, 0] + 3) / 1.0).clip(0, K - 1)).astype(int)  # class from feature 0
    ms = np.ones((n, K), np.float32) * 2.0
    ms[np.arange(n), best] = 1.0
    tuner = mlp.LearnedTuner(n_out=K, seed=1)
    hist = tuner.fit(f[:1200], ms[:1200], epochs=120, batch=128, lr=3e-3)
    assert hist[-1] < 0.5 * hist[0]
    ev = tuner.evaluate(f[1200:], ms[1200:])
    assert ev["mean_frac_without_fallback"] >= 0.9, ev


DATA = os.path.join(os.path.dirname(mlp.__file__), "tuner_data")


@pytest.mark.skipif(not os.path.exists(os.path.join(DATA, "gb300_fp32_tuner.npz")),
                    reason="no trained model committed")
def test_committed_model_held_out(cuda_ok):
    d = np.load(os.path.join(DATA, "gb300_fp32_timings.npz"))
    done = int(d["done"])
    f, ms = d["features"][:done], d["ms"][:done]
    tuner = mlp.LearnedTuner.load(os.path.join(DATA, "gb300_fp32_tuner.npz"))
    ev = tuner.evaluate(f[2000:], ms[2000:])
    assert ev["mean_frac_of_best"] >= 0.95, ev
