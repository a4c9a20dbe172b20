"""Train the learned tuner on the GB300 timing tables with the library's CUDA kernels, calibrate
its confidence threshold on the training matrices, and evaluate it on the 200 held-out ones:
mean / min fraction of the autotuner-best time, fallback rate, and the gain over the best
fixed schedule (the one schedule with the best mean fraction on the training matrices).

    python -m benchmark_spmv_using_csr_gb300.tuner_data.train [timings.npz] [out_prefix]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

N_TRAIN = 2000
EPOCHS, LR, WD = 300, 2e-3, 3e-4


def main(data_path: str, out_prefix: str) -> dict:
    from benchmark_spmv_using_csr_gb300 import mlp
    d = np.load(data_path)
    done = int(d["done"])
    f, ms = d["features"][:done], d["ms"][:done]
    ntr = min(N_TRAIN, done - max(done // 11, 1))
    ftr, mtr, fte, mte = f[:ntr], ms[:ntr], f[ntr:], ms[ntr:]
    # the confidence threshold is calibrated on matrices the network was not fitted on: fit on
    # 85 % of the training set, calibrate on the other 15 %, then refit on all of it
    nfit = int(0.85 * ntr)
    cands = d["candidates"] if "candidates" in d.files else None
    probe = mlp.LearnedTuner(n_out=ms.shape[1], seed=0, candidates=cands)
    probe.fit(ftr[:nfit], mtr[:nfit], epochs=EPOCHS, batch=256, lr=LR, weight_decay=WD)
    threshold = probe.calibrate_threshold(ftr[nfit:], mtr[nfit:], target=0.97, max_fallback=0.25)
    tuner = mlp.LearnedTuner(n_out=ms.shape[1], seed=0, candidates=cands)
    hist = tuner.fit(ftr, mtr, epochs=EPOCHS, batch=256, lr=LR, weight_decay=WD)
    tuner.threshold = threshold
    ev_te = tuner.evaluate(fte, mte)
    ev_tr = tuner.evaluate(ftr, mtr)
    frac_tr = mtr.min(1, keepdims=True) / mtr
    fixed = int(frac_tr.mean(0).argmax())
    frac_fixed_te = mte.min(1) / mte[:, fixed]
    report = {"train_matrices": int(ntr), "held_out_matrices": int(done - ntr),
              "final_train_loss": hist[-1], "first_train_loss": hist[0],
              "held_out": ev_te, "train": ev_tr,
              "best_fixed_schedule": int(fixed),
              "held_out_fixed_mean_frac_of_best": float(frac_fixed_te.mean()),
              "held_out_fixed_min_frac_of_best": float(frac_fixed_te.min()),
              "gain_over_fixed": float(ev_te["mean_frac_of_best"] / frac_fixed_te.mean())}
    tuner.save(out_prefix + "_tuner.npz")
    with open(out_prefix + "_report.json", "w") as fh:
        json.dump(report, fh, indent=1)
    return report


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    data = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "gb300_fp32_timings.npz")
    prefix = sys.argv[2] if len(sys.argv) > 2 else os.path.join(here, "gb300_fp32")
    print(json.dumps(main(data, prefix), indent=1))
