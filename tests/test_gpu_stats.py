"""GPU: the window statistics kernel against exact brute-force statistics.

The engine's statistics (scamp_gb300_window_stats, the kernel every join
runs; the reference's compute_statistics_cpu, src/cpu_stats.cpp:123-160) are
compared with statistics computed exactly in rational arithmetic from prefix
sums of the cleaned samples, then rounded once: mean and inverse norm within
1e-13 relative, df bit-equal to its one-rounding formula, dg within 1e-13 of
the operands' scale.  Non-finite samples count as 0 and make their windows'
inverse norms NaN; flat windows are NaN (src/cpu_stats.cpp:140-152).
"""
import math
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-13


def exact_stats(x, m):
    """Mean, inverse norm, df, dg of every window, from exact prefix sums."""
    bad = ~np.isfinite(x)
    c = np.where(bad, 0.0, x)
    n = len(c)
    ns = n - m + 1
    p1 = [Fraction(0)] * (n + 1)
    p2 = [Fraction(0)] * (n + 1)
    for i, v in enumerate(c.tolist()):
        f = Fraction(v)
        p1[i + 1] = p1[i] + f
        p2[i + 1] = p2[i] + f * f
    nb = np.concatenate([[0], np.cumsum(bad)])
    mean_q = [(p1[w + m] - p1[w]) / m for w in range(ns)]
    mean = np.array([float(q) for q in mean_q])
    inv = np.empty(ns)
    flat = np.zeros(ns, dtype=bool)
    for w in range(ns):
        s = p1[w + m] - p1[w]
        ssd = (p2[w + m] - p2[w]) - s * s / m
        if nb[w + m] - nb[w] > 0 or ssd <= Fraction(1e-13):
            inv[w] = np.nan
            flat[w] = nb[w + m] - nb[w] == 0
        else:
            inv[w] = 1.0 / math.sqrt(float(ssd))
    df = np.zeros(ns)
    dg = np.zeros(ns)
    scale = np.zeros(ns)
    a, b = c[: ns - 1], c[m : m + ns - 1]
    df[: ns - 1] = (b - a) / 2.0
    dg_q = [(Fraction(float(b[i])) - mean_q[i + 1]) + (Fraction(float(a[i])) - mean_q[i])
            for i in range(ns - 1)]
    dg[: ns - 1] = [float(q) for q in dg_q]
    scale[: ns - 1] = np.abs(a) + np.abs(b) + np.abs(mean[1:]) + np.abs(mean[:-1])
    # a mean's rounding scale: the window's largest |sample|
    mscale = np.lib.stride_tricks.sliding_window_view(np.abs(c), m).max(axis=1)
    return mean, inv, df, dg, scale, mscale, flat


def check(engine, x, m, ultra=False):
    mean, inv, df, dg = engine.window_stats(x, m, high_precision_norms=ultra)
    tm, ti, tdf, tdg, scale, mscale, _ = exact_stats(x, m)
    assert np.all(np.abs(mean - tm) <= REL * mscale)
    nan = np.isnan(ti)
    assert np.array_equal(np.isnan(inv), nan)
    assert np.all(np.abs(inv[~nan] - ti[~nan]) <= REL * ti[~nan])
    assert np.array_equal(df, tdf)
    assert np.all(np.abs(dg - tdg) <= REL * scale + 1e-300)
    assert df[-1] == 0 and dg[-1] == 0


@pytest.mark.parametrize("n,m", [(4000, 100), (3000, 8), (5000, 1024), (2050, 2048)])
def test_stats_random_walk(gpu_engine, n, m):
    rng = np.random.default_rng(n + m)
    check(gpu_engine, np.cumsum(rng.standard_normal(n)), m)


def test_stats_offset_series(gpu_engine):
    # a batch member's regime: unit noise on a large offset
    rng = np.random.default_rng(7)
    check(gpu_engine, 1e4 + rng.standard_normal(6000), 64)
    check(gpu_engine, -3e5 + np.cumsum(rng.standard_normal(6000)) * 1e-2, 200)


def test_stats_nan_and_flat(gpu_engine):
    rng = np.random.default_rng(11)
    x = np.cumsum(rng.standard_normal(5000))
    x[700] = np.nan
    x[1900:1903] = np.inf
    x[3000] = -np.inf
    x[3500:3800] = 2.5       # flat stretch: windows inside it are flat
    x[4200:4400] = 0.1
    mean, inv, df, dg = gpu_engine.window_stats(x, 50)
    tm, ti, tdf, tdg, scale, mscale, flat = exact_stats(x, 50)
    assert flat.sum() > 300
    assert np.array_equal(np.isnan(inv), np.isnan(ti))
    ok = ~np.isnan(ti)
    assert np.all(np.abs(inv[ok] - ti[ok]) <= REL * ti[ok])
    assert np.all(np.abs(mean - tm) <= REL * mscale)
    assert np.array_equal(df, tdf)
    assert np.all(np.abs(dg - tdg) <= REL * scale + 1e-300)


def test_stats_ultra(gpu_engine):
    rng = np.random.default_rng(3)
    check(gpu_engine, np.cumsum(rng.standard_normal(3000)), 77, ultra=True)


def test_stats_arguments(gpu_engine):
    with pytest.raises(ValueError):
        gpu_engine.window_stats(np.zeros(10), 2)
    with pytest.raises(ValueError):
        gpu_engine.window_stats(np.zeros(10), 11)
