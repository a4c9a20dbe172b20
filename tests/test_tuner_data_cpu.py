"""The committed learned tuners (one network per value type, trained on GB300 timing tables by
the library's CUDA kernels), evaluated on the CPU with the numpy restatement of the network on
the 220 held-out matrices of each committed timing table (tuner_data.train.split):

* the picks, with the sweep standing in below the network's confidence threshold, reach >= 95 %
  of the autotuner-best time on average (the benchmark's target for the learned tuner);
* they gain over the methods without a network: >= 1.08x the best single fixed schedule and
  >= 1.3x the library's fixed default schedule;
* the fallback is real: the threshold sends a share of the held-out matrices to the sweep, and
  that raises both the mean and the worst case over the network's picks alone.
"""
import os

import numpy as np
import pytest

from oracle import mlp_oracle
from benchmark_spmv_using_csr_gb300 import mlp
from benchmark_spmv_using_csr_gb300.tuner_data import train

DATA = os.path.join(os.path.dirname(mlp.__file__), "tuner_data")
NAMES = ["f64", "f32", "mixed_f32", "mixed_bf16"]
DEFAULTS = {"f64": (16, 8, 4, 0), "f32": (16, 8, 4, 0), "mixed_f32": (16, 8, 4, 0),
            "mixed_bf16": (16, 8, 4, 2)}
VT = {"f64": 0, "f32": 1, "mixed_f32": 2, "mixed_bf16": 3}


@pytest.mark.parametrize("name", NAMES)
def test_committed_network_held_out(name):
    net = mlp.read_network(os.path.join(DATA, f"gb300_{name}_tuner.bin"))
    d = np.load(os.path.join(DATA, f"gb300_{name}_timings.npz"))
    assert net["value_type"] == VT[name] and int(d["value_type"]) == VT[name]
    cands = [tuple(int(v) for v in c) for c in net["candidates"]]
    assert cands == [tuple(int(v) for v in c) for c in d["candidates"]]
    done = int(d["done"])
    assert done == 2400
    f, ms = d["features"][:done], d["ms"][:done].astype(np.float64)
    p = mlp_oracle.forward(net["params"], f, net["mean"], net["std"], 16, net["hidden"],
                           net["n_out"])["p"]
    pick, conf = p.argmax(1), p.max(1)
    frac = ms.min(1) / ms[np.arange(done), pick]
    tr, te = train.split(done)
    fb = conf[te] < net["threshold"]
    r = net["risk"]
    if r is not None:  # the risk network decides the fallback
        risk = mlp_oracle.forward(r["params"], mlp.risk_inputs(f[te], p[te]), r["mean"],
                                  r["std"], r["n_in"], r["hidden"], 2)["p"][:, 1]
        fb = fb | (risk > r["threshold"])
    with_fb = np.where(fb, 1.0, frac[te])
    assert with_fb.mean() >= 0.95
    ftr = ms[tr].min(1, keepdims=True) / ms[tr]
    fixed = int(ftr.mean(0).argmax())
    frac_fixed = ms[te].min(1) / ms[te][:, fixed]
    frac_default = ms[te].min(1) / ms[te][:, cands.index(DEFAULTS[name])]
    assert with_fb.mean() >= 1.08 * frac_fixed.mean()
    assert with_fb.mean() >= 1.3 * frac_default.mean()
    assert 0.05 <= fb.mean() <= 0.3
    assert with_fb.mean() > frac[te].mean() and with_fb.min() >= frac[te].min()
