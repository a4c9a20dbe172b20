"""GPU tests of the learned tuner's CUDA kernels (bhsp_mlp_*) through the C ABI: forward
probabilities and gradients against the numpy oracle, and training that learns a toy mapping.
If the committed GB300 model and timing tables are present, their held-out evaluation is
recomputed and must reach >= 95 % of the autotuner-best time."""
import os

import numpy as np
import pytest

import oracle
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
NAMES = ["f64", "f32", "mixed_f32", "mixed_bf16"]


def _net_path(name):
    return os.path.join(DATA, f"gb300_{name}_tuner.bin")


@pytest.mark.parametrize("name", NAMES)
def test_committed_network_on_device_kernels(cuda_ok, name):
    """The committed network, run by the CUDA forward kernel, reproduces its held-out
    evaluation: picks (with the sweep below the threshold) within 5 % of the autotuner-best
    time on average."""
    if not os.path.exists(_net_path(name)):
        pytest.skip("no trained network committed")
    from benchmark_spmv_using_csr_gb300.tuner_data import train
    d = np.load(os.path.join(DATA, f"gb300_{name}_timings.npz"))
    done = int(d["done"])
    f, ms = d["features"][:done], d["ms"][:done]
    _, te = train.split(done)
    tuner = mlp.LearnedTuner.load(_net_path(name))
    ev = tuner.evaluate(f[te], ms[te])
    assert ev["mean_frac_of_best"] >= 0.95, ev
    ref = mlp_oracle.forward(tuner.net.get_params(), f[te], tuner.net.mean, tuner.net.std,
                             16, tuner.net.hidden, tuner.n_out)["p"]
    np.testing.assert_allclose(tuner.net.forward(f[te]), ref, rtol=2e-4, atol=1e-6)


def _write_with_threshold(src, dst, threshold, risk_threshold=None):
    """A copy of a network file with its confidence threshold (and its risk network's
    threshold, when given) replaced."""
    d = mlp.read_network(src)
    risk = d["risk"]
    if risk is not None and risk_threshold is not None:
        risk = dict(risk, threshold=risk_threshold)
    mlp.write_network(dst, d["value_type"], d["hidden"], threshold, d["mean"], d["std"],
                      d["candidates"], d["params"], risk)
    return d


def _prepare(vt, a, x, tuner=None):
    import benchmark_spmv_using_csr_gb300 as sp
    dt = sp.host_dtype(vt)
    h = sp.BhsparseSpmvCuda(vt)
    if tuner is not None:
        assert h.set_tuner(tuner) == 0
    y = np.zeros(a.m, dt)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val.astype(dt), x.astype(dt), y) == 0, \
        h.last_error
    return h, y


@pytest.mark.parametrize("vt", [0, 1, 2, 3])
def test_prepare_mem_takes_the_networks_pick(cuda_ok, tmp_path, vt):
    """Without bhsp_set_config, prepare_mem runs the learned network on the matrix's features
    (forward kernel on the device) and takes its most probable schedule when the network is
    confident: with both thresholds opened (confidence 0, risk 1) the schedule equals the argmax
    of the numpy restatement of the network on the same features."""
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen, tune
    name = sp.VALUE_NAMES[vt]
    if not os.path.exists(_net_path(name)):
        pytest.skip("no trained network committed")
    path = str(tmp_path / "net.bin")
    d = _write_with_threshold(_net_path(name), path, 0.0, risk_threshold=1.0)
    for a in (gen.powerlaw(200_000, seed=3), gen.stencil3d(50, 40, 30, seed=4)):
        x = gen.uniform(a.n, 5)
        h, y = _prepare(vt, a, x, path)
        src, conf = h.schedule_source()
        assert src == sp.SCHEDULE_LEARNED
        f = tune.row_features(torch.from_numpy(a.row_ptr).cuda(), a.n)
        p = mlp_oracle.forward(d["params"], f[None], d["mean"], d["std"], 16, d["hidden"],
                               d["n_out"])["p"][0]
        assert tuple(h.get_config()) == tuple(int(v) for v in d["candidates"][p.argmax()])
        assert abs(conf - p.max()) <= 1e-3
        # the schedule only changes speed: y is the oracle's
        assert h.run_benchmark() == 0 and h.get_y() == 0
        if vt <= 1:
            ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val.astype(y.dtype).astype(np.float64),
                                    x.astype(y.dtype).astype(np.float64))
            scale = oracle.csr_absrow(a.row_ptr, a.col, a.val.astype(y.dtype).astype(np.float64),
                                      x.astype(y.dtype).astype(np.float64))
            assert oracle.componentwise_error(y, ystar, scale) <= (1e-12 if vt == 0 else 1e-5)
        h.close()


def test_low_confidence_takes_the_sweep(cuda_ok, tmp_path):
    """Below the network's confidence threshold prepare_mem runs the full autotune sweep; with
    the threshold above any probability every matrix takes it."""
    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen, tune
    if not os.path.exists(_net_path("f64")):
        pytest.skip("no trained network committed")
    path = str(tmp_path / "net.bin")
    _write_with_threshold(_net_path("f64"), path, 2.0)
    a = gen.powerlaw(100_000, seed=6)
    x = gen.uniform(a.n, 7)
    h, y = _prepare(sp.VALUE_F64, a, x, path)
    src, conf = h.schedule_source()
    assert src == sp.SCHEDULE_SWEEP and 0.0 < conf <= 1.0
    assert tuple(h.get_config()) in tune.candidates()
    # the sweep ran SpMVs into the device y; the caller's initial y is still what get_y returns
    # before any run_benchmark, and run_benchmark gives the oracle's y
    assert h.get_y() == 0 and not np.any(y)
    assert h.run_benchmark() == 0 and h.get_y() == 0
    ystar = oracle.csr_dot2(a.row_ptr, a.col, a.val, x)
    scale = oracle.csr_absrow(a.row_ptr, a.col, a.val, x)
    assert oracle.componentwise_error(y, ystar, scale) <= 1e-12
    h.close()


def test_schedule_sources(cuda_ok):
    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen
    a = gen.stencil2d(60, 50)
    x = gen.uniform(a.n, 1)
    h, _ = _prepare(sp.VALUE_F64, a, x, "")  # no network: the fixed default
    assert h.schedule_source() == (sp.SCHEDULE_DEFAULT, 0.0)
    assert tuple(h.get_config()) == sp.DEFAULT_CONFIG
    h.close()
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert h.set_config(8, 4, 4, 0) == 0
    y = np.zeros(a.m)
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x, y) == 0
    assert h.schedule_source()[0] == sp.SCHEDULE_CALLER and h.get_config() == (8, 4, 4, 0)
    h.close()
    h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
    assert h.set_tuner("/nonexistent/net.bin") == 0
    assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x, y) == \
        sp.BHSPARSE_INVALID_ARGUMENT
    h.close()


@pytest.mark.parametrize("name", NAMES)
def test_risk_network_decides_the_fallback(cuda_ok, tmp_path, name):
    """The C path runs the file's risk network on the features and the schedule network's
    output: with the risk threshold at 0 (every pick rated slow) the matrix goes to the sweep,
    with it at 1 it takes the network's pick; the numpy restatement of both networks gives the
    risk the device computes."""
    import torch

    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen, tune
    if not os.path.exists(_net_path(name)):
        pytest.skip("no trained network committed")
    d = mlp.read_network(_net_path(name))
    if d["risk"] is None:
        pytest.skip("network file without a risk network")
    vt = {"f64": 0, "f32": 1, "mixed_f32": 2, "mixed_bf16": 3}[name]
    a = gen.powerlaw(150_000, seed=12)
    x = gen.uniform(a.n, 13)
    sweep, learned = str(tmp_path / "sweep.bin"), str(tmp_path / "learned.bin")
    _write_with_threshold(_net_path(name), sweep, 0.0, risk_threshold=0.0)
    _write_with_threshold(_net_path(name), learned, 0.0, risk_threshold=1.0)
    h, _ = _prepare(vt, a, x, sweep)
    assert h.schedule_source()[0] == sp.SCHEDULE_SWEEP
    h.close()
    h, _ = _prepare(vt, a, x, learned)
    assert h.schedule_source()[0] == sp.SCHEDULE_LEARNED
    h.close()
    f = tune.row_features(torch.from_numpy(a.row_ptr).cuda(), a.n)
    p = mlp_oracle.forward(d["params"], f[None], d["mean"], d["std"], 16, d["hidden"],
                           d["n_out"])["p"]
    r = d["risk"]
    risk = mlp_oracle.forward(r["params"], mlp.risk_inputs(f[None], p), r["mean"], r["std"],
                              r["n_in"], r["hidden"], 2)["p"][0, 1]
    tuner = mlp.LearnedTuner.load(_net_path(name))
    _, fb, _, r_dev = tuner.fallback(f[None])
    assert abs(float(r_dev[0]) - risk) <= 1e-4
    assert bool(fb[0]) == (risk > r["threshold"])


def test_malformed_or_mismatched_network_files_are_refused(cuda_ok, tmp_path):
    """prepare_mem refuses a network file that is truncated, has trailing bytes, or was trained
    for another value type, instead of reading a schedule out of it."""
    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import gen
    if not os.path.exists(_net_path("f64")):
        pytest.skip("no trained network committed")
    raw = open(_net_path("f64"), "rb").read()
    a = gen.stencil2d(40, 30)
    x = gen.uniform(a.n, 2)
    bad = {"truncated.bin": raw[:-7], "trailing.bin": raw + b"junk", "empty.bin": b"",
           "f32.bin": open(_net_path("f32"), "rb").read()}
    for name, data in bad.items():
        path = tmp_path / name
        path.write_bytes(data)
        h = sp.BhsparseSpmvCuda(sp.VALUE_F64)
        assert h.set_tuner(str(path)) == 0
        y = np.zeros(a.m)
        assert h.prepare_mem(a.m, a.n, a.nnz, a.row_ptr, a.col, a.val, x, y) == \
            sp.BHSPARSE_INVALID_ARGUMENT, name
        h.close()
