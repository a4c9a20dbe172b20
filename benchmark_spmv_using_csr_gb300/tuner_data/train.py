"""Train the learned tuners on the GB300 timing tables with the library's CUDA kernels, one
network per value type, calibrate each network's confidence threshold, and evaluate it on the
220 held-out matrices (see split): mean / min fraction of the autotuner-best time, fallback rate, and the
gain over the two methods without a network -- the best single fixed schedule (the one with
the best mean fraction on the training matrices) and the library's fixed default schedule.

The threshold comes from matrices the network was not fitted on: a probe network is fitted on
6 of every 7 training matrices and the threshold set on the 7th so that every probe pick below
95 % of the best time falls back to the sweep (with at most 25 % of matrices falling back); the
final network is then fitted on all training matrices.

    python -m benchmark_spmv_using_csr_gb300.tuner_data.train [data_dir] [value type name ...]

Writes gb300_<name>_tuner.bin (the network file the C library reads) and
gb300_<name>_report.json next to the timing files.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

EPOCHS, LR, WD = 300, 2e-3, 3e-4


def split(done: int):
    """(train, held-out) row indices of a timing table: matrices 0-1999 and 2200-2379 train,
    2000-2199 and 2380-2399 (the last 20 of the large stratum) are held out."""
    idx = np.arange(done)
    held = ((idx >= 2000) & (idx < 2200)) | (idx >= 2380)
    return idx[~held], idx[held]


def _frac(ms, idx):
    return ms.min(1) / ms[np.arange(len(ms)), idx]


def train_one(data_dir: str, value_type: int) -> dict:
    import benchmark_spmv_using_csr_gb300 as sp
    from benchmark_spmv_using_csr_gb300 import mlp
    name = sp.VALUE_NAMES[value_type]
    d = np.load(os.path.join(data_dir, f"gb300_{name}_timings.npz"))
    done = int(d["done"])
    f, ms = d["features"][:done], d["ms"][:done].astype(np.float64)
    cands = [tuple(int(v) for v in c) for c in d["candidates"]]
    tr, te = split(done)
    ftr, mtr, fte, mte = f[tr], ms[tr], f[te], ms[te]
    ntr = len(tr)
    # the probe network's fit / calibration split: every 7th training matrix calibrates
    cal = np.zeros(ntr, bool)
    cal[::7] = True
    probe = mlp.LearnedTuner(n_out=ms.shape[1], seed=0, candidates=cands)
    probe.fit(ftr[~cal], mtr[~cal], epochs=EPOCHS, batch=256, lr=LR, weight_decay=WD)
    threshold = probe.calibrate_threshold(ftr[cal], mtr[cal], floor=0.95, max_fallback=0.25)
    validation = probe.evaluate(ftr[cal], mtr[cal])
    tuner = mlp.LearnedTuner(n_out=ms.shape[1], seed=0, candidates=cands)
    hist = tuner.fit(ftr, mtr, epochs=EPOCHS, batch=256, lr=LR, weight_decay=WD)
    tuner.threshold = threshold
    ev_te = tuner.evaluate(fte, mte)
    ev_tr = tuner.evaluate(ftr, mtr)
    large = te >= 2200
    ev_large = tuner.evaluate(fte[large], mte[large]) if large.any() else None
    fixed = int(np.nan_to_num(mtr.min(1, keepdims=True) / mtr).mean(0).argmax())
    default = cands.index(tuple(sp.BhsparseSpmvCuda(value_type).get_config()))
    frac_fixed = _frac(mte, np.full(len(mte), fixed))
    frac_default = _frac(mte, np.full(len(mte), default))
    report = {"value_type": name, "candidates": len(cands), "train_matrices": int(ntr),
              "held_out_matrices": int(done - ntr),
              "final_train_loss": hist[-1], "first_train_loss": hist[0],
              "validation_of_threshold": validation,
              "held_out": ev_te, "held_out_large_stratum": ev_large, "train": ev_tr,
              "best_fixed_schedule": list(cands[fixed]),
              "held_out_fixed_mean_frac_of_best": float(frac_fixed.mean()),
              "held_out_fixed_min_frac_of_best": float(frac_fixed.min()),
              "default_schedule": list(cands[default]),
              "held_out_default_mean_frac_of_best": float(frac_default.mean()),
              "gain_over_fixed": float(ev_te["mean_frac_of_best"] / frac_fixed.mean()),
              "gain_over_default": float(ev_te["mean_frac_of_best"] / frac_default.mean())}
    tuner.save(os.path.join(data_dir, f"gb300_{name}_tuner.bin"), value_type)
    with open(os.path.join(data_dir, f"gb300_{name}_report.json"), "w") as fh:
        json.dump(report, fh, indent=1)
    return report


def main(data_dir: str, names=None) -> dict:
    import benchmark_spmv_using_csr_gb300 as sp
    by_name = {v: k for k, v in sp.VALUE_NAMES.items()}
    names = list(sp.VALUE_NAMES.values()) if not names else names
    return {n: train_one(data_dir, by_name[n]) for n in names}


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    data = sys.argv[1] if len(sys.argv) > 1 else here
    print(json.dumps(main(data, sys.argv[2:]), indent=1))
