"""Pins the CPU oracle (oracle/scamp_oracle.c) before it is trusted.

1. Against the golden outputs shipped with the reference
   (test/SampleOutput/mp_*, mpi_*; tolerances of test/difference.py:24 and
   test/run_tests.sh:36), and against the reference's compiled CPU path run
   on its static stress inputs and its earthquake series -- both from the
   committed fixtures of tests/golden/reference_data
   (tests/golden/make_reference_fixtures.py) -- always.
2. Against the reference's own CPU path compiled from its sources
   (oracle/_ref/libscampref.so) on seeded inputs, including 40 randomized
   configurations of profile type, geometry and edge cases -- where it was
   built.
3. Against the committed fixtures tests/golden/*.npz, produced by that same
   compiled reference (tests/golden/make_golden.py) -- always.
4. Against a brute-force compensated-dot evaluation of every cell and
   against numpy's corrcoef (the reference's distance_matrix_np,
   test/distance_matrix_fast.py) -- always.
"""
import glob
import os

import numpy as np
import pytest

from parity import check_sum, pair_corr

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
REFDATA = os.path.join(GOLDEN, "reference_data")


def _refdata(kind):
    """The committed fixtures of the reference's test data: 'inputs',
    'goldens' (its shipped outputs) or 'compiled' (its CPU path's outputs)."""
    return np.load(os.path.join(REFDATA, kind + ".npz"), allow_pickle=False)


def _distance(oracle, packed, m):
    c, i = oracle.unpack(packed)
    return oracle.to_distance(c, m), i


@pytest.mark.parametrize("name", ["randomwalk8K", "randomwalk16K", "randomwalk32K",
                                  "randomwalk64K", "randomwalk64K_nan"])
def test_oracle_vs_reference_goldens_selfjoin(oracle_mod, name):
    a = _refdata("inputs")[name]
    g = _refdata("goldens")
    gd = g["mp_" + name].astype(np.float64)
    gi = g["mpi_" + name].astype(np.int64)
    d, i = _distance(oracle_mod, oracle_mod.join(a, None, 100)["packed_a"], 100)
    assert np.array_equal(np.isnan(d), np.isnan(gd))
    ok = ~np.isnan(gd)
    assert np.max(np.abs(d[ok] - gd[ok])) <= 0.01
    assert np.max(np.abs(d[ok] - gd[ok])) <= 1e-5  # observed ~2e-6
    assert np.sum(i != gi) <= len(gi) // 100


@pytest.mark.parametrize("na,nb", [("randomwalk16K", "randomwalk32K"),
                                   ("randomwalk32K", "randomwalk16K")])
def test_oracle_vs_reference_goldens_abjoin(oracle_mod, na, nb):
    inp = _refdata("inputs")
    a, b = inp[na], inp[nb]
    g = _refdata("goldens")
    gd = g["mp_%s_%s" % (na, nb)].astype(np.float64)
    gi = g["mpi_%s_%s" % (na, nb)].astype(np.int64)
    d, i = _distance(oracle_mod, oracle_mod.join(a, b, 100, computing_rows=False)["packed_a"], 100)
    assert np.max(np.abs(d - gd)) <= 1e-5
    assert np.sum(i != gi) <= len(gi) // 100


def test_oracle_aligned_self_as_ab_vs_reference_golden(oracle_mod):
    """test/run_tests.sh:49-77: an aligned AB-join of a series with itself
    reproduces its self-join golden."""
    a = _refdata("inputs")["randomwalk8K"]
    g = _refdata("goldens")
    gd = g["mp_randomwalk8K"].astype(np.float64)
    gi = g["mpi_randomwalk8K"].astype(np.int64)
    d, i = _distance(oracle_mod, oracle_mod.join(a, a.copy(), 100, aligned=True,
                                                 computing_rows=False)["packed_a"], 100)
    assert np.max(np.abs(d - gd)) <= 1e-5
    assert np.sum(i != gi) <= len(gi) // 100


def test_oracle_keep_rows_global_offsets_vs_reference_goldens(oracle_mod):
    """test/run_tests.sh:137-206: an AB-join with keep_rows and global
    offsets (not aligned, so they change nothing) reproduces both
    directions' goldens."""
    inp = _refdata("inputs")
    a, b = inp["randomwalk32K"], inp["randomwalk16K"]
    r = oracle_mod.join(a, b, 100, keep_rows=True, start_row=9000000000, start_col=100000)
    g = _refdata("goldens")
    for side, name in (("a", "randomwalk32K_randomwalk16K"), ("b", "randomwalk16K_randomwalk32K")):
        gd = g["mp_" + name].astype(np.float64)
        gi = g["mpi_" + name].astype(np.int64)
        d, i = _distance(oracle_mod, r["packed_" + side], 100)
        assert np.max(np.abs(d - gd)) <= 1e-5, side
        assert np.sum(i != gi) <= len(gi) // 100, side


@pytest.mark.parametrize("name", ["poorly_conditioned_test", "randomwalk1K_nan"])
def test_oracle_vs_compiled_reference_static_inputs(oracle_mod, name):
    """test/run_tests.py:12-17: the static inputs (a quantized, poorly
    conditioned series and a walk with NaN samples) at every window the
    reference tests, 1NN_INDEX and SUM_THRESH at its thresholds, against
    the reference's compiled CPU path (its outputs committed as fixtures):
    the same values at float32 resolution and NaN pattern; index
    differences only at float32 ties; sums equal up to whole multiples of
    the threshold (cells whose r is the threshold itself, frequent in
    quantized data, fall on either side by one rounding: the reference's own
    rule, test/test_common.py:25-49)."""
    x = _refdata("inputs")[name]
    comp = _refdata("compiled")
    for m in (5, 7, 13, 25, 33, 78, 92, 100, 189, 339, 500):
        if m > len(x) // 2:
            continue
        got = oracle_mod.join(x, None, m)
        wc, wi = oracle_mod.unpack(comp["%s_m%d_1nn" % (name, m)])
        gc, gi = oracle_mod.unpack(got["packed_a"])
        assert np.array_equal(wc < -1, gc < -1), m
        ok = wc >= -1
        assert np.max(np.abs(wc[ok].astype(np.float64) - gc[ok]), initial=0.0) <= 2.5e-7, m
        mism = ok & (wi != gi)
        assert np.all(np.abs(wc[mism].astype(np.float64) - gc[mism]) <= 2.5e-7), m
        for thr in (0.0, 0.125, 0.5):
            ws = comp["%s_m%d_sum%g" % (name, m, thr)].astype(np.float64)
            gs = oracle_mod.join(x, None, m, profile="SUM_THRESH", threshold=thr)
            check_sum("%s m=%d thr=%g" % (name, m, thr), gs["sum_a"], ws, thr, 1e-6)


@pytest.mark.parametrize("m", [100, 1000])
def test_oracle_vs_compiled_reference_earthquake(oracle_mod, m):
    """The series the reference's documentation names as the one that breaks
    its reduced-precision modes (docs/source/cli.rst:127): the oracle's
    DOUBLE join equals the reference's compiled CPU path (fixture) at
    float32 resolution, indices differing only at float32 ties."""
    x = _refdata("inputs")["earthquake_precision_test100K"]
    wc, wi = oracle_mod.unpack(_refdata("compiled")["earthquake_precision_test100K_m%d_1nn" % m])
    gc, gi = oracle_mod.unpack(oracle_mod.join(x, None, m)["packed_a"])
    assert np.array_equal(wc < -1, gc < -1)
    ok = wc >= -1
    assert np.max(np.abs(wc[ok].astype(np.float64) - gc[ok])) <= 2.5e-7
    mism = ok & (wi != gi)
    assert np.all(np.abs(wc[mism].astype(np.float64) - gc[mism]) <= 2.5e-7)


def test_reference_fixtures_match_reference_tree():
    """Where the reference tree is present (SCAMP_REFERENCE_TREE), the
    committed fixtures hold exactly its sample inputs and golden outputs."""
    from conftest import REFERENCE_TREE

    if not REFERENCE_TREE or not os.path.isdir(os.path.join(REFERENCE_TREE, "test")):
        pytest.skip("reference tree not present")
    base = os.path.join(REFERENCE_TREE, "test")
    inp = _refdata("inputs")
    for name in inp.files:
        x = np.loadtxt(os.path.join(base, "SampleInput", name + ".txt"))
        assert np.array_equal(np.isnan(x), np.isnan(inp[name])), name
        assert np.array_equal(x[~np.isnan(x)], inp[name][~np.isnan(x)]), name
    g = _refdata("goldens")
    for key in g.files:
        want = np.loadtxt(os.path.join(base, "SampleOutput", key + "_w100.txt"))
        got = g[key].astype(np.float64)
        assert np.array_equal(np.isnan(want), np.isnan(got)), key
        ok = ~np.isnan(want)
        assert np.max(np.abs(want[ok] - got[ok]) / np.maximum(np.abs(want[ok]), 1.0)) <= 1e-7, key


def _ref_cases():
    rng = np.random.default_rng(99)
    cases = []
    for n, m in [(3000, 100), (2000, 7), (1777, 64)]:
        a = np.cumsum(rng.standard_normal(n))
        cases.append(("self%d" % n, a, None, m, {}))
    a = np.cumsum(rng.standard_normal(2500))
    b = np.cumsum(rng.standard_normal(1800))
    b[rng.choice(1800, 9, replace=False)] = np.nan
    cases.append(("ab_keep", a, b, 50, {"keep_rows": True}))
    cases.append(("ab_cols", a, b, 50, {"computing_rows": False}))
    cases.append(("ab_aligned", a, a.copy(), 50, {"aligned": True, "computing_rows": False}))
    return cases


@pytest.mark.parametrize("case", _ref_cases(), ids=lambda c: c[0])
def test_oracle_vs_compiled_reference(oracle_mod, case):
    if not oracle_mod.ref_available():
        pytest.skip("reference CPU path not built here")
    name, a, b, m, kw = case
    want = oracle_mod.ref_join(a, b, m, threads=4, **kw)
    got = oracle_mod.join(a, b, m, **kw)
    for side in ("a", "b"):
        key = "packed_" + side
        if key not in want:
            continue
        wc, wi = oracle_mod.unpack(want[key])
        gc, gi = oracle_mod.unpack(got[key])
        assert np.array_equal(wc < -1, gc < -1)
        ok = wc >= -1
        # float32 correlations: bit-identical or one ulp apart
        assert np.max(np.abs(wc[ok].astype(np.float64) - gc[ok])) <= 2.5e-7
        # index mismatches only where the float32 correlations tie
        # (test/test_common.py:3-16)
        mism = ok & (wi != gi)
        assert np.all(np.abs(wc[mism].astype(np.float64) - gc[mism]) <= 2.5e-7)


def _random_case(seed):
    """One seeded join configuration: window, lengths, self or AB, NaN and
    flat stretches, profile type, threshold, keep_rows / columns-only /
    aligned."""
    rng = np.random.default_rng(seed)
    m = int(rng.choice([3, 4, 8, 16, 33, 64]))
    na = int(rng.integers(m, 2500))
    ab = rng.random() < 0.6
    nb = int(rng.integers(m, 2500)) if ab else None
    a = np.cumsum(rng.standard_normal(na))
    b = np.cumsum(rng.standard_normal(nb)) if ab else None
    if rng.random() < 0.3:
        a[rng.integers(0, na, 3)] = np.nan
    if rng.random() < 0.2:
        s = int(rng.integers(0, max(1, na - 50)))
        a[s:s + 40] = 1.5
    kw = {"profile": str(rng.choice(["1NN_INDEX", "SUM_THRESH", "1NN"]))}
    if kw["profile"] == "SUM_THRESH":
        kw["threshold"] = float(rng.choice([0.0, 0.3, 0.8]))
    if rng.random() < 0.5:
        kw["keep_rows"] = True
    if ab and rng.random() < 0.3:
        kw["computing_rows"] = False
        kw.pop("keep_rows", None)
    if ab and rng.random() < 0.25:
        kw["aligned"] = True
    return a, b, m, kw


@pytest.mark.parametrize("seed", range(40))
def test_oracle_vs_compiled_reference_randomized(oracle_mod, seed):
    """Seeded random configurations, one reference tile (the tile-free
    engine's semantics): same no-match pattern and values to float32
    resolution for every profile the reference returns."""
    if not oracle_mod.ref_available():
        pytest.skip("reference CPU path not built here")
    a, b, m, kw = _random_case(1000 + seed)
    want = oracle_mod.ref_join(a, b, m, threads=1, **kw)
    got = oracle_mod.join(a, b, m, **kw)
    for side in ("a", "b"):
        if "packed_" + side in want:
            wc, _ = oracle_mod.unpack(want["packed_" + side])
            gc, _ = oracle_mod.unpack(got["packed_" + side])
            assert np.array_equal(wc < -1, gc < -1)
            ok = wc >= -1
            assert np.max(np.abs(wc[ok].astype(np.float64) - gc[ok]), initial=0.0) <= 2.5e-7
        if "max_" + side in want:
            w, g = want["max_" + side].astype(np.float64), got["max_" + side].astype(np.float64)
            assert np.array_equal(w < -1, g < -1)
            assert np.max(np.abs(w[w >= -1] - g[w >= -1]), initial=0.0) <= 2.5e-7
        if "sum_" + side in want:
            np.testing.assert_allclose(got["sum_" + side], want["sum_" + side], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("thr", [0.0, 0.5])
def test_oracle_sum_vs_compiled_reference(oracle_mod, thr):
    if not oracle_mod.ref_available():
        pytest.skip("reference CPU path not built here")
    rng = np.random.default_rng(5)
    a = np.cumsum(rng.standard_normal(2000))
    b = np.cumsum(rng.standard_normal(1500))
    for bb, kw in ((None, {}), (b, {"keep_rows": True})):
        want = oracle_mod.ref_join(a, bb, 64, profile="SUM_THRESH", threshold=thr, threads=2, **kw)
        got = oracle_mod.join(a, bb, 64, profile="SUM_THRESH", threshold=thr, **kw)
        for side in ("sum_a", "sum_b"):
            if side in want:
                np.testing.assert_allclose(got[side], want[side], rtol=1e-6, atol=1e-6)


def test_oracle_vs_committed_golden_fixtures(oracle_mod):
    files = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
    assert files, "no golden fixtures committed"
    for f in files:
        z = np.load(f, allow_pickle=False)
        kw = {k[3:]: (bool(z[k]) if z[k].dtype == bool else z[k].item())
              for k in z.files if k.startswith("kw_")}
        a = z["a"]
        b = z["b"] if "b" in z.files else None
        m = int(z["m"])
        got = oracle_mod.join(a, b, m, **kw)
        for side in ("a", "b"):
            if "packed_" + side in z.files:
                wc, wi = oracle_mod.unpack(z["packed_" + side])
                gc, gi = oracle_mod.unpack(got["packed_" + side])
                ok = wc >= -1
                assert np.array_equal(wc < -1, gc < -1), f
                assert np.max(np.abs(wc[ok].astype(np.float64) - gc[ok])) <= 2.5e-7, f
            if "sum_" + side in z.files:
                np.testing.assert_allclose(got["sum_" + side], z["sum_" + side], rtol=1e-6, atol=1e-6)
            if "max_" + side in z.files:
                w, g = z["max_" + side].astype(np.float64), got["max_" + side].astype(np.float64)
                assert np.array_equal(w < -1, g < -1), f
                assert np.max(np.abs(w[w >= -1] - g[w >= -1])) <= 2.5e-7, f


@pytest.mark.parametrize("m", [4, 10, 33])
def test_oracle_recurrence_vs_brute_force(oracle_mod, m):
    rng = np.random.default_rng(m)
    a = np.cumsum(rng.standard_normal(700))
    a[rng.choice(700, 3, replace=False)] = np.nan
    b = np.cumsum(rng.standard_normal(500))
    for bb, kw in ((None, {}), (b, {"keep_rows": True})):
        fast = oracle_mod.join(a, bb, m, **kw)
        brute = oracle_mod.join(a, bb, m, brute=True, **kw)
        for side in ("a", "b"):
            if "corr_" + side not in fast:
                continue
            assert np.array_equal(fast["idx_" + side] < 0, brute["idx_" + side] < 0)
            ok = brute["idx_" + side] >= 0
            assert np.max(np.abs(fast["corr_" + side][ok] - brute["corr_" + side][ok])) < 1e-10


def test_oracle_vs_numpy_corrcoef(oracle_mod):
    # distance_matrix_np (test/distance_matrix_fast.py): corrcoef over all
    # window pairs, exclusion |i - j| < m/4 masked, column max.
    rng = np.random.default_rng(8)
    a = rng.standard_normal(400)
    m = 20
    W = np.lib.stride_tricks.sliding_window_view(a, m)
    C = np.corrcoef(W)
    ns = len(W)
    ii, jj = np.meshgrid(np.arange(ns), np.arange(ns), indexing="ij")
    C[np.abs(ii - jj) < m // 4] = -2
    got = oracle_mod.join(a, None, m)
    np.testing.assert_allclose(got["corr_a"], C.max(axis=0), atol=1e-12)
    r = pair_corr(a, a, m, got["idx_a"], np.arange(ns))
    np.testing.assert_allclose(r, C.max(axis=0), atol=1e-12)


def test_oracle_stats_restatement(oracle_mod):
    # compute_statistics_cpu semantics (src/cpu_stats.cpp:123-160)
    rng = np.random.default_rng(2)
    T = np.cumsum(rng.standard_normal(500))
    T[100] = np.nan
    T[300:340] = 1.5
    m = 16
    s = oracle_mod.stats(T, m)
    assert s["nanwin"][85:101].all() and not s["nanwin"][84] and not s["nanwin"][101]
    assert np.isnan(s["invnorm"][300:325]).all()  # flat windows
    Tc = s["clean"]
    ns = len(T) - m + 1
    assert s["df"][ns - 1] == 0 and s["dg"][ns - 1] == 0
    i = 50
    assert np.isclose(s["df"][i], (Tc[i + m] - Tc[i]) / 2)
    mu = np.array([Tc[k:k + m].mean() for k in range(ns)])
    np.testing.assert_allclose(s["mean"], mu, rtol=1e-12, atol=1e-12)
