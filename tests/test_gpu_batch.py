"""scamp_gb300_join_batch: many independent mixed self-joins in one call must
each match the oracle's self-join (1e-5 in r, indices equal or near-ties),
for series of uneven length, window, scale and offset (the batched workload's
distributions, scaled down), including NaN windows and series too short to
hold any cell."""
import numpy as np
import pytest

from parity import TOL_MIXED, check_1nn

pytestmark = pytest.mark.gpu


def _batch(seed, count):
    rng = np.random.default_rng(seed)
    series, windows = [], []
    for _ in range(count):
        n = int(round(2 ** rng.uniform(10, 13)))
        m = int(rng.choice([32, 64, 128]))
        x = np.cumsum(rng.standard_normal(n)) * 10 ** rng.uniform(-3, 3) + rng.uniform(-1e4, 1e4)
        series.append(x)
        windows.append(m)
    series[3][100:110] = np.nan  # NaN windows
    series[5] = series[5][: windows[5] + 5]  # fewer windows than the exclusion zone
    return series, windows


def test_batch_matches_oracle(gpu_engine, oracle_mod):
    series, windows = _batch(42, 48)
    out = gpu_engine.join_batch(series, windows, precision="mixed", return_corr=True)
    assert len(out) == len(series)
    for k, (x, m, r) in enumerate(zip(series, windows, out)):
        want = oracle_mod.join(x, None, m, "1NN_INDEX", exact_flat=True)
        _, gi = gpu_engine.unpack_profile(r["profile_a"])
        check_1nn("batch%d" % k, r["corr_a"], gi, want["corr_a"], want["idx_a"], TOL_MIXED,
                  x, x, m)
    # one launch per stage for the whole batch (the block-averaged pre-pass
    # that seeds it adds six)
    assert out[0]["gpu_launches"] <= 13


def test_batch_equals_single_joins(gpu_engine):
    series, windows = _batch(7, 12)
    out = gpu_engine.join_batch(series, windows, precision="mixed", return_corr=True)
    for x, m, r in zip(series, windows, out):
        single = gpu_engine.join(x, None, m, "1NN_INDEX", "mixed", return_corr=True)
        ok = single["corr_a"] >= -1
        assert np.array_equal(ok, r["corr_a"] >= -1)
        assert np.max(np.abs(single["corr_a"][ok] - r["corr_a"][ok]), initial=0.0) <= TOL_MIXED


def _close(x, y):
    ok = x["corr_a"] >= -1
    assert np.array_equal(ok, y["corr_a"] >= -1)
    assert np.max(np.abs(x["corr_a"][ok] - y["corr_a"][ok]), initial=0.0) <= TOL_MIXED


def test_batch_graph_replay(gpu_engine):
    """The device part of a batch is one captured graph, replayed while the
    layout repeats: a repeated call gives the same profiles (within the
    mixed tolerance: which cells take the exact path depends on timing),
    the band kernel's events inside the graph time it, and another layout
    captures a new graph."""
    series, windows = _batch(9, 16)
    a = gpu_engine.join_batch(series, windows, return_corr=True)
    b = gpu_engine.join_batch(series, windows, return_corr=True)
    for r in (a[0], b[0]):
        assert 0 < r["join_kernel_ms"] <= r["elapsed_ms"]
        assert r["counters"]["steps"] > 0
    for x, y in zip(a, b):
        _close(x, y)
    c = gpu_engine.join_batch(series[:10], windows[:10], return_corr=True)
    for x, y in zip(a[:10], c):
        _close(x, y)


def test_batch_autotune(gpu_engine, oracle_mod):
    """tune_batch picks each window's segment length among the cold-start
    anchor interval (8 m within [1024, 4096]), half and a quarter of it,
    capped for short series as the rule is; batches joined after tuning
    still match the oracle."""
    series, windows = _batch(21, 24)
    seg = gpu_engine.tune_batch(series, windows, retune=True)
    assert len(seg) == len(series)
    by_m = {}
    for x, m, K in zip(series, windows, seg):
        rule = min(max(4096, 2 * m), max(1024, 8 * m))
        half = max(128, ((len(x) - m + 1) // 2 // 128) * 128)
        assert K in {min(c, half) for c in (rule, rule // 2, rule // 4)}, (len(x), m, K)
        if (len(x) - m + 1) // 2 >= rule:
            by_m.setdefault(m, set()).add(int(K))
    assert all(len(v) == 1 for v in by_m.values())  # one choice per window
    out = gpu_engine.join_batch(series, windows, precision="mixed", return_corr=True,
                                autotune=True)
    for k, (x, m, r) in enumerate(zip(series, windows, out)):
        want = oracle_mod.join(x, None, m, "1NN_INDEX", exact_flat=True)
        _, gi = gpu_engine.unpack_profile(r["profile_a"])
        check_1nn("tuned%d" % k, r["corr_a"], gi, want["corr_a"], want["idx_a"], TOL_MIXED,
                  x, x, m)


def test_batch_rejects_unsupported(gpu_engine):
    with pytest.raises(ValueError):
        gpu_engine.join_batch([np.arange(500.0)], [600])
    with pytest.raises(ValueError):
        gpu_engine.join_batch([np.cumsum(np.ones(500))], [50], precision="double")
