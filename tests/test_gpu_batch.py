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
    assert out[0]["gpu_launches"] <= 8  # one launch per stage for the whole batch


def test_batch_equals_single_joins(gpu_engine):
    series, windows = _batch(7, 12)
    out = gpu_engine.join_batch(series, windows, precision="mixed", return_corr=True)
    for x, m, r in zip(series, windows, out):
        single = gpu_engine.join(x, None, m, "1NN_INDEX", "mixed", return_corr=True)
        ok = single["corr_a"] >= -1
        assert np.array_equal(ok, r["corr_a"] >= -1)
        assert np.max(np.abs(single["corr_a"][ok] - r["corr_a"][ok]), initial=0.0) <= TOL_MIXED


def test_batch_rejects_unsupported(gpu_engine):
    with pytest.raises(ValueError):
        gpu_engine.join_batch([np.arange(500.0)], [600])
    with pytest.raises(ValueError):
        gpu_engine.join_batch([np.cumsum(np.ones(500))], [50], precision="double")
