"""The learned schedule tuner: a small MLP (16 row-length features -> 64 -> 64 -> one logit per
candidate schedule) trained on the autotuner's own timing tables by the library's CUDA kernels
(bhsp_mlp_*), with the full autotune sweep as its fallback below a confidence threshold.

It only chooses a schedule: whichever schedule it picks, y = A.x is computed by the same
kernels and arithmetic.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import tune
from ._lib import lib

HIDDEN = 64
RISK_HIDDEN = 32


def soft_targets(ms: np.ndarray, temperature: float = 0.05) -> np.ndarray:
    """Training targets from a timing table: probability mass on every schedule within a few
    per cent of the best, p_k ~ exp(-(ms_k / ms_best - 1) / temperature)."""
    ms = np.asarray(ms, np.float64)
    rel = ms / ms.min(axis=-1, keepdims=True) - 1.0
    w = np.exp(-rel / temperature)
    return (w / w.sum(axis=-1, keepdims=True)).astype(np.float32)


def init_params(n_in: int, hidden: int, n_out: int, seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases, in the network's flat layout."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((hidden, n_in)) * np.sqrt(2.0 / n_in)
    W2 = rng.standard_normal((hidden, hidden)) * np.sqrt(2.0 / hidden)
    W3 = rng.standard_normal((n_out, hidden)) * np.sqrt(1.0 / hidden)
    return np.concatenate([W1.ravel(), np.zeros(hidden), W2.ravel(), np.zeros(hidden),
                           W3.ravel(), np.zeros(n_out)]).astype(np.float32)


class MLP:
    """Device network (bhsp_mlp) with host-side parameter and normalisation access."""

    def __init__(self, n_in: int = tune.NUM_FEATURES, hidden: int = HIDDEN, n_out: int = 18,
                 max_batch: int = 4096, seed: int = 0):
        self.n_in, self.hidden, self.n_out, self.max_batch = n_in, hidden, n_out, max_batch
        self._m = ctypes.c_void_p()
        rc = lib().bhsp_mlp_create(ctypes.byref(self._m), n_in, hidden, n_out, max_batch)
        if rc != 0:
            raise RuntimeError(f"bhsp_mlp_create failed ({rc})")
        self.mean = np.zeros(n_in, np.float32)
        self.std = np.ones(n_in, np.float32)
        self.set_params(init_params(n_in, hidden, n_out, seed))

    @property
    def num_params(self) -> int:
        return int(lib().bhsp_mlp_num_params(self._m))

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if lib().bhsp_mlp_set_params(self._m, p.ctypes.data_as(ctypes.c_void_p), p.size) != 0:
            raise RuntimeError("bhsp_mlp_set_params failed")

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        if lib().bhsp_mlp_get_params(self._m, p.ctypes.data_as(ctypes.c_void_p), p.size) != 0:
            raise RuntimeError("bhsp_mlp_get_params failed")
        return p

    def set_normalization(self, mean, std) -> None:
        self.mean = np.ascontiguousarray(mean, np.float32)
        self.std = np.ascontiguousarray(np.maximum(std, 1e-6), np.float32)
        rc = lib().bhsp_mlp_set_normalization(self._m, self.mean.ctypes.data_as(ctypes.c_void_p),
                                              self.std.ctypes.data_as(ctypes.c_void_p))
        if rc != 0:
            raise RuntimeError("bhsp_mlp_set_normalization failed")

    def _dev(self, a):
        import torch
        return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()

    def forward(self, feats: np.ndarray) -> np.ndarray:
        import torch
        f = self._dev(np.atleast_2d(feats))
        out = np.zeros((f.shape[0], self.n_out), np.float32)
        for s in range(0, f.shape[0], self.max_batch):
            fb = f[s:s + self.max_batch]
            p = torch.empty((fb.shape[0], self.n_out), dtype=torch.float32, device="cuda")
            rc = lib().bhsp_mlp_forward(self._m, fb.data_ptr(), fb.shape[0], p.data_ptr(),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            if rc != 0:
                raise RuntimeError("bhsp_mlp_forward failed")
            out[s:s + fb.shape[0]] = p.cpu().numpy()
        return out

    def gradients(self, feats: np.ndarray, targets: np.ndarray) -> tuple[np.ndarray, float]:
        import torch
        f, t = self._dev(feats), self._dev(targets)
        g = torch.empty(self.num_params, dtype=torch.float32, device="cuda")
        loss = ctypes.c_float()
        rc = lib().bhsp_mlp_gradients(self._m, f.data_ptr(), t.data_ptr(), f.shape[0], g.data_ptr(),
                                      ctypes.byref(loss),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc != 0:
            raise RuntimeError("bhsp_mlp_gradients failed")
        return g.cpu().numpy(), float(loss.value)

    def train_step(self, f_dev, t_dev, lr: float, weight_decay: float = 0.0) -> float:
        import torch
        loss = ctypes.c_float()
        rc = lib().bhsp_mlp_train_step(self._m, f_dev.data_ptr(), t_dev.data_ptr(), f_dev.shape[0],
                                       ctypes.c_float(lr), ctypes.c_float(weight_decay),
                                       ctypes.byref(loss),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc != 0:
            raise RuntimeError("bhsp_mlp_train_step failed")
        return float(loss.value)

    def close(self) -> None:
        if self._m:
            lib().bhsp_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LearnedTuner:
    """Features -> schedule, trained on autotuner timing tables; falls back to the sweep."""

    def __init__(self, n_out: int | None = None, hidden: int = HIDDEN, seed: int = 0,
                 candidates=None):
        # the schedules the network's outputs stand for (the timing table's columns); a network
        # with another number of outputs and no list is a plain classifier (no choose())
        if candidates is None:
            live = tune.candidates()
            candidates = live if n_out is None or n_out == len(live) else None
        self.candidates = (None if candidates is None else
                           [tuple(int(v) for v in c) for c in candidates])
        self.n_out = len(self.candidates) if n_out is None else n_out
        if self.candidates is not None and self.n_out != len(self.candidates):
            raise ValueError("one network output per candidate schedule")
        self.net = MLP(tune.NUM_FEATURES, hidden, self.n_out, seed=seed)
        self.threshold = 0.0
        # the optional risk network and its threshold (fallback where its P(slow pick) exceeds it)
        self.risk = None
        self.risk_threshold = 1.0

    def fit(self, feats: np.ndarray, ms: np.ndarray, epochs: int = 400, batch: int = 256,
            lr: float = 3e-3, weight_decay: float = 1e-4, temperature: float = 0.05,
            seed: int = 0) -> list:
        """Train on (features, timing table) pairs with the device kernels; returns the
        per-epoch mean loss."""
        return train_net(self.net, feats, soft_targets(ms, temperature), epochs, batch, lr,
                         weight_decay, seed)

    def fit_risk(self, feats: np.ndarray, probs: np.ndarray, bad: np.ndarray,
                 hidden: int = RISK_HIDDEN, epochs: int = 300, batch: int = 256,
                 lr: float = 2e-3, weight_decay: float = 3e-4, seed: int = 1) -> list:
        """Train the risk network: from the features and the schedule network's output
        distribution (its picks made on matrices it was not fitted on) to whether the pick is
        slow (`bad`, e.g. below 95 % of the best time).  The sweep is the fallback where the
        risk is above risk_threshold."""
        x = risk_inputs(feats, probs)
        self.risk = MLP(x.shape[1], hidden, 2, seed=seed)
        b = np.asarray(bad, np.float32)
        return train_net(self.risk, x, np.stack([1.0 - b, b], 1), epochs, batch, lr,
                         weight_decay, seed)

    def predict(self, feats: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """(picked candidate index, confidence = its probability) per row of features."""
        p = self.net.forward(np.atleast_2d(feats))
        return p.argmax(1), p.max(1)

    def fallback(self, feats: np.ndarray):
        """(picks, whether each goes to the sweep, confidence, risk): the sweep decides where
        the risk network's P(slow pick) exceeds risk_threshold, or, without a risk network,
        where the confidence is below the threshold."""
        feats = np.atleast_2d(feats)
        p = self.net.forward(feats)
        pick, conf = p.argmax(1), p.max(1)
        if self.risk is not None:
            r = self.risk.forward(risk_inputs(feats, p))[:, 1]
            return pick, r > self.risk_threshold, conf, r
        return pick, conf < self.threshold, conf, np.zeros_like(conf)

    def calibrate_threshold(self, feats, ms, floor: float = 0.95, max_fallback: float = 0.25) -> float:
        """Confidence threshold from matrices the network was not fitted on: the smallest one
        below which every pick slower than `floor` of the best time falls back to the sweep,
        or, if that would send more than `max_fallback` of the matrices to the sweep, the
        largest threshold within that budget."""
        pick, conf = self.predict(feats)
        frac = ms.min(1) / ms[np.arange(len(pick)), pick]
        self.threshold = 0.0
        for th in np.concatenate([[0.0], np.sort(np.unique(conf)) + 1e-7]):
            keep = conf >= th
            if (~keep).mean() > max_fallback:
                break
            self.threshold = float(th)
            if not np.any(keep & (frac < floor)):
                break
        return self.threshold

    def evaluate(self, feats, ms) -> dict:
        """Fraction of the autotuner's best time per matrix (best_ms / picked_ms), with the
        sweep standing in below the confidence threshold."""
        pick, fb, _, _ = self.fallback(feats)
        frac = ms.min(1) / ms[np.arange(len(pick)), pick]
        frac_with_fb = np.where(fb, 1.0, frac)
        return {"mean_frac_of_best": float(frac_with_fb.mean()),
                "min_frac_of_best": float(frac_with_fb.min()),
                "mean_frac_without_fallback": float(frac.mean()),
                "min_frac_without_fallback": float(frac.min()),
                "picks_below_95pct_kept": int(np.sum((frac < 0.95) & ~fb)),
                "picks_below_95pct_without_fallback": int(np.sum(frac < 0.95)),
                "fallback_rate": float(fb.mean()), "threshold": self.threshold,
                "risk_threshold": self.risk_threshold if self.risk is not None else None}

    def choose(self, value_type: int, row_ptr, col_idx, val, x, y, n: int | None = None) -> dict:
        """Pick a schedule for a device matrix: the network if confident, else the sweep."""
        if self.candidates is None:
            raise ValueError("this network's outputs are not tied to candidate schedules")
        n = x.numel() if n is None else n
        f = tune.row_features(row_ptr, n)
        pick, fb, conf, _ = self.fallback(f)
        if not fb[0]:
            return {"index": int(pick[0]), "confidence": float(conf[0]), "fallback": False,
                    "config": self.candidates[int(pick[0])]}
        ms, best = tune.autotune(value_type, row_ptr, col_idx, val, x, y, n=n)
        return {"index": best, "confidence": float(conf[0]), "fallback": True,
                "config": tune.candidates()[best], "ms": ms}

    def save(self, path: str, value_type: int) -> None:
        """Write the network file the C library reads (csrc/learned.cu): magic, value type,
        sizes, threshold, input standardisation, candidate schedules, parameters."""
        if self.candidates is None:
            raise ValueError("only a network tied to candidate schedules can be saved")
        risk = None
        if self.risk is not None:
            risk = {"hidden": self.risk.hidden, "threshold": self.risk_threshold,
                    "mean": self.risk.mean, "std": self.risk.std, "params": self.risk.get_params()}
        write_network(path, value_type, self.net.hidden, self.threshold, self.net.mean,
                      self.net.std, np.array(self.candidates, np.int32), self.net.get_params(),
                      risk)

    @classmethod
    def load(cls, path: str) -> "LearnedTuner":
        d = read_network(path)
        t = cls(n_out=d["n_out"], hidden=d["hidden"], candidates=d["candidates"])
        t.net.set_params(d["params"])
        t.net.set_normalization(d["mean"], d["std"])
        t.threshold = d["threshold"]
        t.value_type = d["value_type"]
        r = d.get("risk")
        if r is not None:
            t.risk = MLP(r["n_in"], r["hidden"], 2)
            t.risk.set_params(r["params"])
            t.risk.set_normalization(r["mean"], r["std"])
            t.risk_threshold = r["threshold"]
        return t


MAGIC = b"BHSPTUN1"
RISK_MAGIC = b"BHSPRSK1"


def risk_inputs(feats: np.ndarray, probs: np.ndarray) -> np.ndarray:
    """The risk network's inputs: the 16 row features, then the schedule network's largest and
    second-largest probability and the entropy of its distribution."""
    f = np.atleast_2d(np.asarray(feats, np.float32))
    p = np.atleast_2d(np.asarray(probs, np.float64))
    top = np.sort(p, 1)
    ent = -(p * np.log(np.maximum(p, 1e-30))).sum(1)
    return np.concatenate([f, top[:, -1:], top[:, -2:-1], ent[:, None]], 1).astype(np.float32)


def train_net(net: "MLP", x: np.ndarray, targets: np.ndarray, epochs: int, batch: int,
              lr: float, weight_decay: float, seed: int) -> list:
    """Mini-batch Adam with cosine decay over (inputs, target distributions), all in the device
    kernels; standardises the inputs first.  Returns the per-epoch mean loss."""
    import torch
    x = np.asarray(x, np.float32)
    mean, std = x.mean(0), x.std(0)
    std[std < 1e-6] = 1.0
    net.set_normalization(mean, std)
    f_dev, t_dev = net._dev(x), net._dev(np.asarray(targets, np.float32))
    rng = np.random.default_rng(seed)
    hist = []
    n = x.shape[0]
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        step_lr = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))
        losses = []
        for s in range(0, n, batch):
            idx = perm[s:s + batch]
            losses.append(net.train_step(f_dev[idx].contiguous(), t_dev[idx].contiguous(),
                                         step_lr, weight_decay))
        hist.append(float(np.mean(losses)))
    return hist


def write_network(path: str, value_type: int, hidden: int, threshold: float, mean, std,
                  candidates: np.ndarray, params: np.ndarray, risk: dict | None = None) -> None:
    """The little-endian network file of csrc/learned.cu, with the optional risk section."""
    cands = np.ascontiguousarray(candidates, "<i4").reshape(-1, 4)
    mean = np.ascontiguousarray(mean, "<f4")
    std = np.ascontiguousarray(std, "<f4")
    params = np.ascontiguousarray(params, "<f4")
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.array([value_type, mean.size, hidden, cands.shape[0]], "<i4").tobytes())
        f.write(np.array([threshold], "<f4").tobytes())
        f.write(mean.tobytes())
        f.write(std.tobytes())
        f.write(cands.tobytes())
        f.write(np.array([params.size], "<i4").tobytes())
        f.write(params.tobytes())
        if risk is not None:
            rm = np.ascontiguousarray(risk["mean"], "<f4")
            rs = np.ascontiguousarray(risk["std"], "<f4")
            rp = np.ascontiguousarray(risk["params"], "<f4")
            f.write(RISK_MAGIC)
            f.write(np.array([rm.size, risk["hidden"], 2], "<i4").tobytes())
            f.write(np.array([risk["threshold"]], "<f4").tobytes())
            f.write(rm.tobytes())
            f.write(rs.tobytes())
            f.write(np.array([rp.size], "<i4").tobytes())
            f.write(rp.tobytes())


def read_network(path: str) -> dict:
    raw = open(path, "rb").read()
    if raw[:8] != MAGIC:
        raise ValueError(f"{path}: not a network file")
    vt, n_in, hidden, n_out = (int(v) for v in np.frombuffer(raw, "<i4", 4, 8))
    o = 24
    threshold = float(np.frombuffer(raw, "<f4", 1, o)[0])
    o += 4
    mean = np.frombuffer(raw, "<f4", n_in, o).copy()
    o += 4 * n_in
    std = np.frombuffer(raw, "<f4", n_in, o).copy()
    o += 4 * n_in
    cands = np.frombuffer(raw, "<i4", 4 * n_out, o).reshape(n_out, 4).copy()
    o += 16 * n_out
    npar = int(np.frombuffer(raw, "<i4", 1, o)[0])
    o += 4
    params = np.frombuffer(raw, "<f4", npar, o).copy()
    o += 4 * npar
    risk = None
    if o < len(raw):
        if raw[o:o + 8] != RISK_MAGIC:
            raise ValueError(f"{path}: unknown section after the parameters")
        o += 8
        r_in, r_hidden, r_out = (int(v) for v in np.frombuffer(raw, "<i4", 3, o))
        o += 12
        r_th = float(np.frombuffer(raw, "<f4", 1, o)[0])
        o += 4
        r_mean = np.frombuffer(raw, "<f4", r_in, o).copy()
        o += 4 * r_in
        r_std = np.frombuffer(raw, "<f4", r_in, o).copy()
        o += 4 * r_in
        r_np = int(np.frombuffer(raw, "<i4", 1, o)[0])
        o += 4
        r_params = np.frombuffer(raw, "<f4", r_np, o).copy()
        o += 4 * r_np
        risk = {"n_in": r_in, "hidden": r_hidden, "n_out": r_out, "threshold": r_th,
                "mean": r_mean, "std": r_std, "params": r_params}
    if o != len(raw):
        raise ValueError(f"{path}: trailing or missing bytes")
    return {"value_type": vt, "n_in": n_in, "hidden": hidden, "n_out": n_out,
            "threshold": threshold, "mean": mean, "std": std, "candidates": cands,
            "params": params, "risk": risk}
