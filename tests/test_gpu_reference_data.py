"""GPU parity on the reference's own test data and at the benchmark sizes.

The engine (through its C ABI) against:
  * the reference's shipped golden profiles (test/SampleOutput: self-joins of
    randomwalk8K..64K_nan and the AB-joins 16K x 32K / 32K x 16K at m = 100,
    test/run_tests.sh:11-13, 80-135), with its own tolerances (distance
    within 0.01, test/difference.py:24; at most 1% of the indices
    different, test/run_tests.sh:36) and, in r, within this path's
    tolerance with the near-tie rule;
  * the reference's compiled CPU path on its static stress inputs
    (test/run_tests.py:12-17) and on the earthquake series its
    documentation names as the one that breaks reduced precision
    (docs/source/cli.rst:127) -- fixtures of tests/golden/reference_data;
  * the CPU oracle at the full size of the self-join benchmark (n = 131072,
    m = 100), on a quarter-size AB benchmark join (2^18 x 2^17, m = 256, both
    directions) and on adversarial series (quantized, monotone stretches,
    exact repeats) long enough for the mixed form's shipped anchor interval
    (32 m rows).

FP64 within 1e-9 in r, mixed within 1e-5; an index either equals the
oracle's or points at a window whose FP64 r is within the tolerance of the
best (parity.check_1nn).
"""
import functools
import os

import numpy as np
import pytest

from parity import TOL_FP64, TOL_MIXED, check_1nn, check_1nn_direct, check_sum, pair_corr

pytestmark = pytest.mark.gpu

PRECISIONS = [("double", TOL_FP64), ("mixed", TOL_MIXED)]
REFDATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_data")
GOLDEN_SELF = ["randomwalk8K", "randomwalk16K", "randomwalk32K", "randomwalk64K",
               "randomwalk64K_nan"]


@functools.lru_cache(maxsize=None)
def _refdata(kind):
    z = np.load(os.path.join(REFDATA, kind + ".npz"), allow_pickle=False)
    return {k: z[k] for k in z.files}


_ORACLE_CACHE = {}


def _oracle_join(oracle, key, a, b, m, **kw):
    """The oracle's join of a named case, computed once per session."""
    if key not in _ORACLE_CACHE:
        _ORACLE_CACHE[key] = oracle.join(a, b, m, exact_flat=True, **kw)
    return _ORACLE_CACHE[key]


def _engine_1nn(engine, oracle, key, a, b, m, precision, tol, **kw):
    """Engine join vs FP64: every reported value against the direct FP64
    correlation of its pair (within tol and within the join's reported
    max_abs_r_err), every partner no worse than the oracle's by more than
    tol, the no-match pattern the oracle's; the mixed form's values also
    within tol of the oracle's.  Returns the engine's result."""
    got = engine.join(a, b, m, "1NN_INDEX", precision, return_corr=True, **kw)
    want = _oracle_join(oracle, key, a, b, m, **kw)
    other = a if b is None else b
    sides = [("A", "a", a, other)]
    if kw.get("keep_rows"):
        sides.append(("B", "b", other, a))
    assert got["max_abs_r_err"] > 0
    for tag, s, t_self, t_other in sides:
        _, gi = engine.unpack_profile(got["profile_" + s])
        check_1nn_direct("%s/%s" % (key, tag), got["corr_" + s], gi, want["idx_" + s], tol,
                         t_self, t_other, m, bound=got["max_abs_r_err"])
        if precision != "double":
            check_1nn("%s/%s" % (key, tag), got["corr_" + s], gi, want["corr_" + s],
                      want["idx_" + s], tol, t_self, t_other, m)
    return got


def _vs_golden(engine, got, gd, gi, tol, T_self, T_other, m, name):
    """The reference's shipped golden (distances from float32 r): its own
    rules (distance within 0.01, <= 1% index differences) and, in r, within
    tol plus the golden's float32 rounding, with differing indices near-ties
    of the golden's r."""
    c32, idx = engine.unpack_profile(got["profile_a"])
    d = np.sqrt(np.maximum(2.0 * m * (1.0 - c32.astype(np.float64)), 0.0))
    d[idx < 0] = np.nan
    assert np.array_equal(np.isnan(d), np.isnan(gd)), name
    ok = ~np.isnan(gd)
    assert np.max(np.abs(d[ok] - gd[ok])) <= 0.01, name
    assert np.sum(idx[ok] != gi[ok]) <= len(gi) // 100, name
    gd64 = gd.astype(np.float64)
    r_gold = 1.0 - gd64 ** 2 / (2.0 * m)
    # the golden r is a float32 (2.5e-7 at most), its distance is stored
    # here as a float32 (relative 6e-8, so r moves by up to 1.2e-7 d^2 / m)
    slack = 3e-7 + 1.2e-7 * np.nan_to_num(gd64) ** 2 / m
    err = np.abs(got["corr_a"][ok] - r_gold[ok])
    assert np.all(err <= tol + slack[ok]), (name, float(err.max()))
    mism = np.nonzero(ok & (idx != gi))[0]
    if mism.size:
        r = pair_corr(T_other, T_self, m, idx[mism], mism)
        assert np.all(np.abs(r - r_gold[mism]) <= tol + slack[mism]), name


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("name", GOLDEN_SELF)
def test_reference_golden_selfjoin(gpu_engine, oracle_mod, precision, tol, name):
    a = _refdata("inputs")[name]
    got = _engine_1nn(gpu_engine, oracle_mod, name, a, None, 100, precision, tol)
    g = _refdata("goldens")
    _vs_golden(gpu_engine, got, g["mp_" + name], g["mpi_" + name].astype(np.int64), tol, a, a,
               100, name)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("na,nb", [("randomwalk16K", "randomwalk32K"),
                                   ("randomwalk32K", "randomwalk16K")])
def test_reference_golden_abjoin(gpu_engine, oracle_mod, precision, tol, na, nb):
    inp = _refdata("inputs")
    a, b = inp[na], inp[nb]
    key = "%s_%s" % (na, nb)
    got = _engine_1nn(gpu_engine, oracle_mod, key, a, b, 100, precision, tol,
                      computing_rows=False)
    g = _refdata("goldens")
    _vs_golden(gpu_engine, got, g["mp_" + key], g["mpi_" + key].astype(np.int64), tol, a, b,
               100, key)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_reference_golden_keep_rows_both_directions(gpu_engine, oracle_mod, precision, tol):
    """test/run_tests.sh:137-206: one AB-join with keep_rows gives both
    directions' goldens."""
    inp = _refdata("inputs")
    a, b = inp["randomwalk32K"], inp["randomwalk16K"]
    got = _engine_1nn(gpu_engine, oracle_mod, "keep32K16K", a, b, 100, precision, tol,
                      keep_rows=True)
    g = _refdata("goldens")
    _vs_golden(gpu_engine, got, g["mp_randomwalk32K_randomwalk16K"],
               g["mpi_randomwalk32K_randomwalk16K"].astype(np.int64), tol, a, b, 100, "A")
    got_b = {"profile_a": got["profile_b"], "corr_a": got["corr_b"]}
    _vs_golden(gpu_engine, got_b, g["mp_randomwalk16K_randomwalk32K"],
               g["mpi_randomwalk16K_randomwalk32K"].astype(np.int64), tol, b, a, 100, "B")


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_reference_golden_aligned_self_as_ab(gpu_engine, oracle_mod, precision, tol):
    """test/run_tests.sh:49-77: the aligned AB-join of a series with itself
    gives its self-join golden."""
    a = _refdata("inputs")["randomwalk8K"]
    got = gpu_engine.join(a, a.copy(), 100, "1NN_INDEX", precision, computing_rows=False,
                          aligned=True, return_corr=True)
    g = _refdata("goldens")
    _vs_golden(gpu_engine, got, g["mp_randomwalk8K"], g["mpi_randomwalk8K"].astype(np.int64),
               tol, a, a, 100, "aligned8K")


def _compiled_vs_engine(engine, got, packed, x, m, tol, name, ref_err=2.5e-7):
    """Engine vs the reference's compiled CPU path (packed float32 profile).
    The reference's sequential SSD can leave an exactly flat window valid
    (with a residue norm, so an arbitrary r) where the engine marks it
    invalid: such windows, and windows whose reference partner is one, are
    left out; every other window agrees within tol + ref_err (the
    reference's float32 rounding, and where its statistics drift, their
    error)."""
    from parity import window_stats

    wc = (packed & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.float32).astype(np.float64)
    wi = (packed >> np.uint64(32)).astype(np.int64)
    valid_win = ~np.isnan(window_stats(x, m)[2])
    valid_ref = wc >= -1
    valid_eng = got["corr_a"] >= -1
    assert np.all(valid_eng <= valid_ref), name  # never a match the reference lacks
    extra = valid_ref & ~valid_eng
    assert not np.any(valid_win[extra]), name     # only windows that are exactly flat
    both = valid_ref & valid_eng
    both[both] &= valid_win[wi[both]]
    err = np.abs(got["corr_a"][both] - wc[both])
    assert np.max(err, initial=0.0) <= tol + ref_err, (name, float(err.max(initial=0.0)))


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("name", ["poorly_conditioned_test", "randomwalk1K_nan"])
def test_reference_static_inputs(gpu_engine, oracle_mod, precision, tol, name):
    """The reference's static stress inputs at every window it tests:
    1NN_INDEX against the oracle and the compiled reference, SUM_THRESH at
    its thresholds against the oracle (whole threshold-edge cells allowed,
    the reference's rule)."""
    x = _refdata("inputs")[name]
    comp = _refdata("compiled")
    for m in (5, 7, 13, 25, 33, 78, 92, 100, 189, 339, 500):
        if m > len(x) // 2:
            continue
        key = "%s_m%d" % (name, m)
        got = _engine_1nn(gpu_engine, oracle_mod, key, x, None, m, precision, tol)
        _compiled_vs_engine(gpu_engine, got, comp[key + "_1nn"], x, m, tol, key)
        for thr in (0.0, 0.125, 0.5):
            g = gpu_engine.join(x, None, m, "SUM_THRESH", precision, threshold=thr)
            w = oracle_mod.join(x, None, m, profile="SUM_THRESH", threshold=thr, exact_flat=True)
            check_sum("%s thr=%g" % (key, thr), g["sum_a"], w["sum_a"], thr,
                      1e-9 if precision == "double" else 2e-5,
                      cell_tol=0.0 if precision == "double" else TOL_MIXED)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("m", [100, 1000])
def test_reference_earthquake(gpu_engine, oracle_mod, precision, tol, m):
    """The series the reference names as breaking its mixed and single
    precision (docs/source/cli.rst:127): both forms here stay within their
    tolerance of the FP64 oracle (brute-force accurate statistics) and agree
    with the compiled reference.  On this series the reference's own DOUBLE
    path carries r errors up to 9.4e-7 at m = 100: its running SSD drifts
    (inverse norms off by up to 1.7e-6 relative against a direct sum), so
    the comparison with it allows that much more."""
    x = _refdata("inputs")["earthquake_precision_test100K"]
    key = "earthquake_m%d" % m
    got = _engine_1nn(gpu_engine, oracle_mod, key, x, None, m, precision, tol)
    _compiled_vs_engine(gpu_engine, got, _refdata("compiled")[
        "earthquake_precision_test100K_m%d_1nn" % m], x, m, tol, key, ref_err=1.2e-6)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_selfjoin_benchmark_size(gpu_engine, oracle_mod, precision, tol):
    """The self-join benchmark at its full size: a seeded random walk of
    131072 points, m = 100."""
    from scamp_gb300 import workloads

    a, m = workloads.walk_selfjoin()
    _engine_1nn(gpu_engine, oracle_mod, "selfjoin131072", a, None, m, precision, tol)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_abjoin_benchmark_quarter_size(gpu_engine, oracle_mod, precision, tol):
    """The AB benchmark's distribution at a quarter of its size: random walks
    of 2^18 and 2^17 points with planted motifs and NaN samples, m = 256,
    both directions."""
    from scamp_gb300 import workloads

    a, b, m = workloads.motif_abjoin(na=1 << 18, nb=1 << 17)
    _engine_1nn(gpu_engine, oracle_mod, "ab2e18", a, b, m, precision, tol, keep_rows=True)


def _adversarial(kind, n):
    rng = np.random.default_rng({"quantized": 21, "monotone": 22, "repeats": 23}[kind])
    if kind == "quantized":
        # integer-valued walk: many exactly equal windows and r ties
        return np.cumsum(rng.integers(-2, 3, n)).astype(np.float64)
    if kind == "monotone":
        # long monotone stretches (ramps of random slope and length) with
        # little noise: correlated increments along every diagonal
        out, x = [], 0.0
        while len(out) < n:
            L = int(rng.integers(500, 5000))
            s = rng.uniform(-1, 1)
            out.extend(x + s * np.arange(L) + 0.01 * rng.standard_normal(L))
            x = out[-1]
        return np.asarray(out[:n])
    # exact repeats: one period-97 pattern of quantized values, repeated
    pat = np.round(rng.standard_normal(97) * 8) / 8
    return np.tile(pat, n // 97 + 1)[:n]


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("kind,n,m", [("quantized", 1 << 18, 64), ("monotone", 1 << 18, 64),
                                      ("repeats", 1 << 18, 64), ("quantized", 1 << 19, 256)])
def test_adversarial_series_shipped_anchor_interval(gpu_engine, oracle_mod, precision, tol,
                                                    kind, n, m):
    """Series that defeat a random-rounding model of the FP32 drift, at
    lengths where the mixed form runs its shipped anchor interval (32 m
    rows): quantized values (exact ties), monotone stretches (correlated
    increments), exact repeats (many cells at r = 1)."""
    x = _adversarial(kind, n)
    _engine_1nn(gpu_engine, oracle_mod, "%s_%d_%d" % (kind, n, m), x, None, m, precision, tol)
