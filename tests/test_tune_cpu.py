"""CPU tests of the tuning host logic: the candidate table and the feature arithmetic."""
import numpy as np

from benchmark_spmv_using_csr_gb300 import gen, tune


def test_candidate_table():
    """24 direct-load schedules and 8 TMA-staged ones (stages 2 and 3 at S = 8 and 16)."""
    c = tune.candidates()
    assert len(c) == 32
    assert len(set(c)) == len(c)
    for seg, tpw, warps, stages in c:
        assert seg in (8, 16, 32) and tpw >= 1 and warps in (4, 8) and stages in (0, 2, 3)
    staged = [x for x in c if x[3]]
    assert len(staged) == 8 and {x[0] for x in staged} == {8, 16}
    # the handle's default schedules are candidates (the trainer reports the gain over them)
    assert (16, 8, 4, 0) in c and (16, 8, 4, 2) in c


def _features_numpy(rp, n):
    L = np.diff(rp.astype(np.int64))
    m = L.size
    mean = L.mean()
    std = np.sqrt(max((L.astype(np.float64) ** 2).mean() - mean * mean, 0.0))
    f = [np.log2(m + 1), np.log2(n + 1), np.log2(L.sum() + 1), np.log2(1 + mean),
         np.log2(1 + std), np.log2(1 + L.max()), (L == 0).mean()]
    edges = [(1, 1), (2, 3), (4, 7), (8, 15), (16, 31), (32, 63), (64, 255), (256, 4095),
             (4096, 1 << 40)]
    f += [((L >= lo) & (L <= hi)).mean() for lo, hi in edges]
    return np.array(f, np.float32)


def test_features_match_numpy():
    for a in (gen.powerlaw(20000, seed=3), gen.stencil2d(50, 40),
              gen.mixed_rows(5000, 9000, dense_row=7, mean_len=3, empty_frac=0.9, seed=2)):
        c = tune.feature_counts(a.row_ptr)
        f = tune.features_from_counts(a.m, a.n, c)
        np.testing.assert_allclose(f, _features_numpy(a.row_ptr, a.n), rtol=1e-5, atol=1e-6)
        assert abs(f[7:].sum() + f[6] - 1.0) < 1e-5  # bins + empty cover every row


def test_tune_cache_roundtrip(tmp_path):
    p = str(tmp_path / "t.json")
    cache = tune.TuneCache(p)
    f = np.arange(16, dtype=np.float32)
    k = len(tune.candidates())
    cache.put(0, f, np.ones(k, np.float32) * 2, 5)
    cache.save()
    again = tune.TuneCache(p)
    ms, best = again.get(0, f)
    assert best == 5 and ms.shape == (k,) and again.get(1, f) is None
