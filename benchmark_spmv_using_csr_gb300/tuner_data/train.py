"""Train the learned tuners on the GB300 timing tables with the library's CUDA kernels, one
network per value type, calibrate each network's confidence threshold, and evaluate it on the
220 held-out matrices (see split): mean / min fraction of the autotuner-best time, fallback rate, and the
gain over the two methods without a network -- the best single fixed schedule (the one with
the best mean fraction on the training matrices) and the library's fixed default schedule.

The fallback is decided by a second, small network (the risk network: the 16 features and the
schedule network's top two probabilities and entropy -> 32 -> 32 -> 2).  Its labels are the
schedule network's out-of-fold picks on the training matrices (5 folds): slow where the pick is
below 95 % of the best time.  It is fitted on 6 of every 7 of them and its threshold set on the
7th: the largest that sends every slow pick there to the sweep, or, if that would send more than
25 % of the matrices, the one that sends 25 %.  The schedule network itself is fitted on all
training matrices.

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
FOLDS = 5              # out-of-fold picks for the risk network's training labels
FLOOR = 0.95           # a pick slower than this fraction of the best time is a slow pick
MAX_FALLBACK = 0.25    # at most this share of matrices go to the sweep


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
    # out-of-fold picks: the schedule network fitted on 4 of 5 folds predicts the 5th, so that the
    # risk network learns from picks made on matrices the schedule network has not seen
    folds = np.arange(ntr) % FOLDS
    probs = np.zeros((ntr, ms.shape[1]), np.float32)
    for k in range(FOLDS):
        t = mlp.LearnedTuner(n_out=ms.shape[1], seed=k, candidates=cands)
        t.fit(ftr[folds != k], mtr[folds != k], epochs=EPOCHS, batch=256, lr=LR, weight_decay=WD)
        probs[folds == k] = t.net.forward(ftr[folds == k])
        t.net.close()
    pick = probs.argmax(1)
    bad = mtr.min(1) / mtr[np.arange(ntr), pick] < FLOOR
    # the final schedule network on every training matrix; its risk network on 6 of every 7
    # out-of-fold picks, the risk threshold set on the 7th
    tuner = mlp.LearnedTuner(n_out=ms.shape[1], seed=0, candidates=cands)
    hist = tuner.fit(ftr, mtr, epochs=EPOCHS, batch=256, lr=LR, weight_decay=WD)
    cal = np.zeros(ntr, bool)
    cal[::7] = True
    tuner.fit_risk(ftr[~cal], probs[~cal], bad[~cal])
    # threshold on the calibration seventh, scored with its out-of-fold probabilities
    r_cal = tuner.risk.forward(mlp.risk_inputs(ftr[cal], probs[cal]))[:, 1]
    order = np.sort(r_cal)[::-1]
    cap = int(np.floor(MAX_FALLBACK * cal.sum()))
    bc = bad[cal]
    need = int(np.searchsorted(-order, -r_cal[bc].min(), side="right")) if bc.any() else 0
    k = min(need, cap)
    tuner.risk_threshold = float(order[k] if k < len(order) else 0.0)
    tuner.threshold = 0.0  # the risk network decides the fallback
    cal_fb = r_cal > tuner.risk_threshold
    validation = {"matrices": int(cal.sum()), "fallback_rate": float(cal_fb.mean()),
                  "slow_picks": int(bc.sum()), "slow_picks_sent_to_sweep": int((bc & cal_fb).sum()),
                  "risk_auc": _auc(r_cal, bc)}
    ev_te = tuner.evaluate(fte, mte)
    ev_tr = tuner.evaluate(ftr, mtr)
    large = te >= 2200
    ev_large = tuner.evaluate(fte[large], mte[large]) if large.any() else None
    _, _, conf_te, r_te = tuner.fallback(fte)
    pick_te = tuner.predict(fte)[0]
    bad_te = mte.min(1) / mte[np.arange(len(te)), pick_te] < FLOOR
    fixed = int(np.nan_to_num(mtr.min(1, keepdims=True) / mtr).mean(0).argmax())
    default = cands.index(tuple(sp.BhsparseSpmvCuda(value_type).get_config()))
    frac_fixed = _frac(mte, np.full(len(mte), fixed))
    frac_default = _frac(mte, np.full(len(mte), default))
    report = {"value_type": name, "candidates": len(cands), "train_matrices": int(ntr),
              "held_out_matrices": int(len(te)),
              "final_train_loss": hist[-1], "first_train_loss": hist[0],
              "out_of_fold_slow_picks": int(bad.sum()),
              "validation_of_risk_threshold": validation,
              "held_out": ev_te, "held_out_large_stratum": ev_large, "train": ev_tr,
              "held_out_risk_auc": _auc(r_te, bad_te),
              "held_out_max_probability_auc": _auc(-conf_te, bad_te),
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


def _auc(score: np.ndarray, positive: np.ndarray) -> float | None:
    """Probability that a positive (a slow pick) scores above a negative (ties count half)."""
    pos, neg = score[positive], score[~positive]
    if len(pos) == 0 or len(neg) == 0:
        return None
    gt = (pos[:, None] > neg[None, :]).mean()
    eq = (pos[:, None] == neg[None, :]).mean()
    return float(gt + 0.5 * eq)


def main(data_dir: str, names=None) -> dict:
    import benchmark_spmv_using_csr_gb300 as sp
    by_name = {v: k for k, v in sp.VALUE_NAMES.items()}
    names = list(sp.VALUE_NAMES.values()) if not names else names
    return {n: train_one(data_dir, by_name[n]) for n in names}


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    data = sys.argv[1] if len(sys.argv) > 1 else here
    print(json.dumps(main(data, sys.argv[2:]), indent=1))
