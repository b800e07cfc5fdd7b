"""Seeded synthetic series for the benchmark configurations.

No public dataset is named for this path; these generators produce series
with the shapes, sizes and value distributions of the five benchmark
configurations (numpy PCG64, fixed seeds).  ``n`` can be scaled down for
tests while keeping the distribution.
"""
import numpy as np


def random_walk(rng, n):
    """x[0] = 0, x[t] = x[t-1] + N(0, 1)."""
    x = np.empty(n)
    x[0] = 0.0
    x[1:] = np.cumsum(rng.standard_normal(n - 1))
    return x


def walk_selfjoin(n=131072, seed=1):
    """Self-join, m=100: one seeded random walk."""
    rng = np.random.default_rng(seed)
    return random_walk(rng, n), 100


def motif_abjoin(na=1 << 20, nb=1 << 19, m=256, motifs=64, motif_len=256,
                nan_frac=0.001, seed=2):
    """AB-join, m=256: two random walks sharing 64 planted sinusoid motifs
    (sin(2 pi t / P) + 0.1 N(0,1), P ~ U[20, 200], length 256) at seeded
    non-overlapping positions, with 0.1% of the samples set to NaN."""
    rng = np.random.default_rng(seed)
    a = random_walk(rng, na)
    b = random_walk(rng, nb)
    motif_len = min(motif_len, na // (2 * motifs), nb // (2 * motifs))
    for s, n in ((a, na), (b, nb)):
        slots = n // motif_len
        pos = rng.choice(slots, size=motifs, replace=False) * motif_len
        rng_m = np.random.default_rng(seed + 1000)  # same motif shapes in A and B
        for p in sorted(pos):
            period = rng_m.uniform(20, 200)
            t = np.arange(motif_len)
            s[p:p + motif_len] = np.sin(2 * np.pi * t / period) + 0.1 * rng_m.standard_normal(motif_len)
    for s, n in ((a, na), (b, nb)):
        k = int(round(nan_frac * n))
        s[rng.choice(n, size=k, replace=False)] = np.nan
    return a, b, m


def noisy_walk_selfjoin(n=1 << 24, m=1024, seed=3):
    """Self-join: random walk plus 0.5 N(0,1) noise."""
    rng = np.random.default_rng(seed)
    return random_walk(rng, n) + 0.5 * rng.standard_normal(n), m


def walk_batch(count=4096, lo=10, hi=16, seed=4):
    """Independent series: lengths round(2^U[lo,hi]), random walks scaled by
    LogU(1e-3, 1e3) and offset by U(-1e4, 1e4), windows from {32, 64, 128}."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(round(2 ** rng.uniform(lo, hi)))
        s = 10 ** rng.uniform(-3, 3)
        o = rng.uniform(-1e4, 1e4)
        m = int(rng.choice([32, 64, 128]))
        out.append((random_walk(rng, n) * s + o, m))
    return out


def gapped_walk_selfjoin(n=1 << 27, m=4096, gap_frac=0.01, seed=5):
    """Self-join: random walk with 1% of samples in NaN gaps of length
    U[1, 500]."""
    rng = np.random.default_rng(seed)
    x = random_walk(rng, n)
    target = int(gap_frac * n)
    covered = 0
    while covered < target:
        L = int(rng.integers(1, 501))
        p = int(rng.integers(0, n - L))
        x[p:p + L] = np.nan
        covered += L
    return x, m
