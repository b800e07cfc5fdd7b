"""GPU parity: the engine through its C ABI against the CPU oracle.

Cases mirror the reference's own tests (test/run_tests.sh, test/run_tests.py,
test/test_pyscamp.py): self-joins and AB-joins, with and without NaN
windows, keep_rows (both directions), aligned AB joins, SUM_THRESH with
several thresholds, tiny and ragged sizes.
"""
import numpy as np
import pytest

from parity import TOL_FP64, TOL_MIXED, check_1nn, check_sum

pytestmark = pytest.mark.gpu

PRECISIONS = [("double", TOL_FP64), ("mixed", TOL_MIXED)]


def rw(rng, n):
    return np.cumsum(rng.standard_normal(n))


def run_1nn(engine, oracle, a, b, m, precision, tol, keep_rows=False, rows=True,
            aligned=False, name="", brute=False, oracle_precision=3, filter_mode=0, **kw):
    got = engine.join(a, b, m, "1NN_INDEX", precision, computing_rows=rows,
                      keep_rows=keep_rows, aligned=aligned, return_corr=True,
                      filter_mode=filter_mode, **kw)
    # exact_flat: flatness decided from an exact ssd (the engine's rule); the
    # reference's sequential ssd can leave flat windows "valid".
    want = oracle.join(a, b, m, "1NN_INDEX", computing_rows=rows, keep_rows=keep_rows,
                       aligned=aligned, exact_flat=True, brute=brute,
                       precision=oracle_precision, **kw)
    _, gi = engine.unpack_profile(got["profile_a"])
    T_other = a if b is None else b
    check_1nn(name + "/A", got["corr_a"], gi, want["corr_a"], want["idx_a"], tol, a, T_other, m)
    if keep_rows:
        _, gib = engine.unpack_profile(got["profile_b"])
        Tb = a if b is None else b
        check_1nn(name + "/B", got["corr_b"], gib, want["corr_b"], want["idx_b"], tol, Tb, a, m)
    # packed float32 correlations agree with the oracle's packed profile
    gc, _ = engine.unpack_profile(got["profile_a"])
    wc, _ = oracle.unpack(want["packed_a"])
    ok = wc >= -1
    assert np.all(np.abs(gc[ok].astype(np.float64) - wc[ok]) <= max(tol, 2e-7))
    assert got["comparisons"] > 0 and got["gpu_launches"] >= 3
    return got, want


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("n,m", [(5000, 100), (3000, 8), (2500, 333), (4097, 64)])
def test_selfjoin_random_walk(gpu_engine, oracle_mod, precision, tol, n, m):
    rng = np.random.default_rng(n + m)
    a = rw(rng, n)
    run_1nn(gpu_engine, oracle_mod, a, None, m, precision, tol, name="self%d_%d" % (n, m))


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_selfjoin_randn(gpu_engine, oracle_mod, precision, tol):
    # run_tests.py style: i.i.d. normal inputs
    rng = np.random.default_rng(13)
    for n, m in [(20, 5), (100, 7), (250, 13), (500, 25), (1500, 33), (8000, 100)]:
        a = rng.standard_normal(n)
        run_1nn(gpu_engine, oracle_mod, a, None, m, precision, tol, name="randn%d" % n)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_selfjoin_nan_and_flat(gpu_engine, oracle_mod, precision, tol):
    rng = np.random.default_rng(5)
    a = rw(rng, 6000)
    a[rng.choice(6000, 30, replace=False)] = np.nan
    a[1000:1400] = 3.25  # flat region: ssd <= 1e-13 windows
    a[2000] = np.inf
    run_1nn(gpu_engine, oracle_mod, a, None, 64, precision, tol, name="nanflat")


@pytest.mark.parametrize("precision,tol", PRECISIONS)
@pytest.mark.parametrize("na,nb", [(4000, 3000), (2000, 5000), (1500, 1500)])
def test_abjoin_keep_rows(gpu_engine, oracle_mod, precision, tol, na, nb):
    rng = np.random.default_rng(na * 7 + nb)
    a, b = rw(rng, na), rw(rng, nb)
    b[rng.choice(nb, 10, replace=False)] = np.nan
    run_1nn(gpu_engine, oracle_mod, a, b, 50, precision, tol, keep_rows=True, name="ab")


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_abjoin_columns_only(gpu_engine, oracle_mod, precision, tol):
    # pyscamp.abjoin: computing_rows = False
    rng = np.random.default_rng(11)
    a, b = rng.random(3000), rng.random(2500)
    run_1nn(gpu_engine, oracle_mod, a, b, 128, precision, tol, rows=False, name="abcols")


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_aligned_abjoin_equals_selfjoin(gpu_engine, oracle_mod, precision, tol):
    # run_tests.sh:50-77: an aligned AB-join of a series with itself must give
    # the self-join's profile.
    rng = np.random.default_rng(3)
    a = rw(rng, 3000)
    got_ab, _ = run_1nn(gpu_engine, oracle_mod, a, a.copy(), 100, precision, tol,
                        rows=False, aligned=True, name="aligned")
    got_self = gpu_engine.join(a, None, 100, "1NN_INDEX", precision, return_corr=True)
    assert np.max(np.abs(got_ab["corr_a"] - got_self["corr_a"])) <= tol


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_selfjoin_keep_rows_separate(gpu_engine, oracle_mod, precision, tol):
    rng = np.random.default_rng(9)
    a = rw(rng, 3000)
    run_1nn(gpu_engine, oracle_mod, a, None, 40, precision, tol, keep_rows=True, name="selfkr")


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_profile_type_1nn(gpu_engine, oracle_mod, precision):
    """PROFILE_TYPE_1NN: the best correlation per window (float32, -2 where
    none) -- the 1NN_INDEX search without the index -- merged by max into a
    given best-so-far profile."""
    rng = np.random.default_rng(44)
    a = rw(rng, 3000)
    b = rw(rng, 2200)
    tol = TOL_FP64 if precision == "double" else TOL_MIXED
    for bb, kw in ((None, {}), (b, {"keep_rows": True})):
        got = gpu_engine.join(a, bb, 60, "1NN", precision, **kw)
        want = oracle_mod.join(a, bb, 60, profile="1NN", **kw)
        for side in ("a", "b"):
            if "max_" + side not in want:
                continue
            g = got["profile_" + side]
            assert g.dtype == np.float32
            w = want["max_" + side].astype(np.float64)
            assert np.array_equal(g < -1, w < -1)
            assert np.max(np.abs(g[w >= -1] - w[w >= -1])) <= tol + 2.5e-7
    # merge: a best-so-far above every correlation survives; -2 entries fill
    init = np.full(len(a) - 60 + 1, -2.0, dtype=np.float32)
    init[::7] = 1.0
    got = gpu_engine.join(a, None, 60, "1NN", precision, profile_a=init)
    plain = gpu_engine.join(a, None, 60, "1NN", precision)
    assert np.all(got["profile_a"][::7] == 1.0)
    mask = np.ones(len(init), bool)
    mask[::7] = False
    assert np.array_equal(got["profile_a"][mask], plain["profile_a"][mask])


def test_ultra_against_oracle(gpu_engine, oracle_mod):
    """ULTRA: brute-force window statistics and the reference's combined
    update terms (the oracle's precision=4 restates them; the reference's own
    ULTRA output is pinned by the golden fixtures), FP64 tolerance."""
    rng = np.random.default_rng(41)
    a = rw(rng, 4000)
    b = rw(rng, 2500)
    run_1nn(gpu_engine, oracle_mod, a, None, 64, "ultra", TOL_FP64, name="ultra-self",
            oracle_precision=4)
    run_1nn(gpu_engine, oracle_mod, a, None, 64, "ultra", TOL_FP64, keep_rows=True,
            name="ultra-self-kr", oracle_precision=4)
    run_1nn(gpu_engine, oracle_mod, a, b, 64, "ultra", TOL_FP64, keep_rows=True,
            name="ultra-ab", oracle_precision=4)
    run_1nn(gpu_engine, oracle_mod, 1e4 + a, 1e4 + b, 50, "ultra", TOL_FP64, keep_rows=True,
            name="ultra-ab-offset", oracle_precision=4)


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("thr", [0.0, 0.125, 0.5, 0.9])
def test_sum_thresh(gpu_engine, oracle_mod, precision, thr):
    rng = np.random.default_rng(21)
    a = rw(rng, 3000)
    b = rw(rng, 2000)
    rtol = 1e-9 if precision == "double" else 2e-5
    ctol = 0.0 if precision == "double" else TOL_MIXED
    got = gpu_engine.join(a, None, 64, "SUM_THRESH", precision, threshold=thr)
    want = oracle_mod.join(a, None, 64, "SUM_THRESH", threshold=thr)
    check_sum("selfsum", got["sum_a"], want["sum_a"], thr, rtol, ctol)
    got = gpu_engine.join(a, b, 64, "SUM_THRESH", precision, threshold=thr, keep_rows=True)
    want = oracle_mod.join(a, b, 64, "SUM_THRESH", threshold=thr, keep_rows=True)
    check_sum("absum/A", got["sum_a"], want["sum_a"], thr, rtol, ctol)
    check_sum("absum/B", got["sum_b"], want["sum_b"], thr, rtol, ctol)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_sum_thresh_geometries(gpu_engine, oracle_mod, precision):
    """SUM_THRESH over the other join geometries: AB columns only, aligned
    AB with distributed offsets, NaN gaps and flat stretches, a window of 8."""
    rng = np.random.default_rng(52)
    rtol = 1e-9 if precision == "double" else 2e-5
    ctol = 0.0 if precision == "double" else TOL_MIXED
    a = rw(rng, 3500)
    b = rw(rng, 2600)
    thr = 0.6
    cases = [
        (a, b, 64, dict(computing_rows=False)),
        (a, a[:3000].copy(), 64, dict(aligned=True, keep_rows=True, start_row=100, start_col=130)),
        (a, None, 8, {}),
    ]
    g = a.copy()
    g[rng.choice(len(g), 10, replace=False)] = np.nan
    g[900:1000] = 3.0
    cases.append((g, None, 48, {}))
    for x, y, m, kw in cases:
        got = gpu_engine.join(x, y, m, "SUM_THRESH", precision, threshold=thr, **kw)
        want = oracle_mod.join(x, y, m, "SUM_THRESH", threshold=thr, exact_flat=True, **kw)
        check_sum("geom/A %s" % sorted(kw), got["sum_a"], want["sum_a"], thr, rtol, ctol)
        if "sum_b" in want:
            check_sum("geom/B %s" % sorted(kw), got["sum_b"], want["sum_b"], thr, rtol, ctol)


def test_sum_thresh_many_units(gpu_engine):
    """Mixed SUM_THRESH over thousands of band units of both AB problems
    (their column series differ in length), against the FP64 form, which the
    other tests tie to the oracle."""
    rng = np.random.default_rng(33)
    a = rw(rng, 200_000)
    b = rw(rng, 60_000)
    for thr in (0.5, 0.9):
        want = gpu_engine.join(a, b, 64, "SUM_THRESH", "double", threshold=thr, keep_rows=True)
        for _ in range(2):
            got = gpu_engine.join(a, b, 64, "SUM_THRESH", "mixed", threshold=thr, keep_rows=True)
            check_sum("A", got["sum_a"], want["sum_a"], thr, 2e-5, TOL_MIXED)
            check_sum("B", got["sum_b"], want["sum_b"], thr, 2e-5, TOL_MIXED)


def test_single_precision_is_served_by_the_mixed_form(gpu_engine, oracle_mod):
    """PRECISION_SINGLE (pyscamp precision='single') runs the mixed engine,
    so it meets the mixed tolerance (stricter than the reference's SINGLE)."""
    rng = np.random.default_rng(71)
    a, b = rw(rng, 4000), rw(rng, 2500)
    run_1nn(gpu_engine, oracle_mod, a, None, 64, "single", TOL_MIXED, name="single/self")
    run_1nn(gpu_engine, oracle_mod, a, b, 50, "single", TOL_MIXED, keep_rows=True,
            name="single/ab")
    got = gpu_engine.join(a, b, 64, "SUM_THRESH", "single", threshold=0.7, keep_rows=True)
    want = oracle_mod.join(a, b, 64, "SUM_THRESH", threshold=0.7, keep_rows=True)
    check_sum("single/sumA", got["sum_a"], want["sum_a"], 0.7, 2e-5, TOL_MIXED)
    check_sum("single/sumB", got["sum_b"], want["sum_b"], 0.7, 2e-5, TOL_MIXED)
    prof, idx = gpu_engine.selfjoin(a, 64, precision="single")
    assert prof.dtype == np.float32 and len(idx) == len(a) - 63


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_distributed_offsets_1nn(gpu_engine, oracle_mod, precision, tol):
    """1NN_INDEX with the distributed tile offsets (--global_row/col): the
    aligned AB-joins of a self-join split into tiles of W windows at
    multiples of W (the layout of SCAMP's distributed joins), where the
    trivial-match zone runs along a diagonal tile's main diagonal or touches
    an off-diagonal tile's corner."""
    rng = np.random.default_rng(72)
    W, m = 6000, 64
    x = rw(rng, 3 * W + m)
    tile = lambda k: x[k * W:(k + 1) * W + m - 1].copy()  # noqa: E731
    for r, c in ((1, 0), (0, 1), (1, 1)):
        run_1nn(gpu_engine, oracle_mod, tile(c), tile(r), m, precision, tol, keep_rows=True,
                aligned=True, start_row=r * W, start_col=c * W, name="tile%d%d" % (r, c))


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_tiny_and_edge_sizes(gpu_engine, oracle_mod, precision, tol):
    rng = np.random.default_rng(17)
    # n == m (one window, nothing to compare), m = 3, n just above m
    for n, m in [(3, 3), (10, 3), (7, 5), (40, 30), (600, 3)]:
        a = rng.standard_normal(n)
        run_1nn(gpu_engine, oracle_mod, a, None, m, precision, tol, name="edge%d_%d" % (n, m))
        b = rng.standard_normal(n + 3)
        run_1nn(gpu_engine, oracle_mod, a, b, m, precision, tol, keep_rows=True,
                name="edgeab%d_%d" % (n, m))


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_merge_into_best_so_far(gpu_engine, oracle_mod, precision, tol):
    # do_SCAMP merges into the profile it is given (src/tile.cpp:322-389,
    # src/common.cpp:175-187): entries already better than anything in this
    # join must survive.
    rng = np.random.default_rng(23)
    a = rw(rng, 2000)
    m = 50
    base = gpu_engine.join(a, None, m, "1NN_INDEX", precision)["profile_a"]
    prior = base.copy()
    keep = rng.choice(len(prior), 100, replace=False)
    prior[keep] = (np.uint64(7) << np.uint64(32)) | np.uint64(np.float32(1.0).view(np.uint32))
    got = gpu_engine.join(a, None, m, "1NN_INDEX", precision, profile_a=prior)["profile_a"]
    gc, gi = gpu_engine.unpack_profile(got)
    assert np.all(gc[keep] == 1.0) and np.all(gi[keep] == 7)
    others = np.setdiff1d(np.arange(len(prior)), keep)
    if precision == "double":
        assert np.array_equal(got[others], base[others])
    else:
        # The mixed form's work depends on the starting thresholds (which
        # candidates get verified), so untouched entries agree to tolerance.
        bc, bi = gpu_engine.unpack_profile(base)
        assert np.max(np.abs(gc[others].astype(np.float64) - bc[others])) <= tol


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_extreme_scale_and_offset(gpu_engine, oracle_mod, precision, tol):
    # the batched workload's regime: random walks scaled by 1e-3..1e3 and offset by up to 1e4
    rng = np.random.default_rng(31)
    for s, o in [(1e-3, 1e4), (1e3, -1e4), (1.0, 0.0)]:
        a = rw(rng, 3000) * s + o
        # Offset 1e4 with scale 1e-3 leaves ~9 significant digits of signal
        # per sample: the reference's own recurrence is 1e-8 off the exact
        # answer here, so the check is against per-cell brute force.
        run_1nn(gpu_engine, oracle_mod, a, None, 32, precision, tol, name="scale%g" % s,
                brute=True)


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_motif_abjoin_small(gpu_engine, oracle_mod, precision, tol):
    from scamp_gb300 import workloads

    a, b, m = workloads.motif_abjoin(na=1 << 14, nb=1 << 13, motifs=16)
    run_1nn(gpu_engine, oracle_mod, a, b, m, precision, tol, keep_rows=True, name="motif_ab_small")


@pytest.mark.parametrize("precision,tol", PRECISIONS)
def test_against_reference_golden_fixtures(gpu_engine, precision, tol):
    """tests/golden/*.npz hold outputs of the reference's own CPU path
    (tests/golden/make_golden.py).  The reference stores r as float32, so
    agreement is at float32 resolution plus the form's tolerance; index
    mismatches must be near-ties (checked in FP64)."""
    import glob
    import os

    from parity import pair_corr, window_stats

    files = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
    assert files
    for f in files:
        z = np.load(f, allow_pickle=False)
        kw = {k[3:]: (bool(z[k]) if z[k].dtype == bool else z[k].item())
              for k in z.files if k.startswith("kw_")}
        profile = kw.pop("profile", "1NN_INDEX")
        thr = kw.pop("threshold", 0.0)
        rows = kw.pop("computing_rows", True)
        form = precision
        if kw.pop("precision", 3) == 4:
            # an ULTRA fixture: the reference's ULTRA path against ours
            if precision != "double":
                continue
            form = "ultra"
        a = z["a"]
        b = z["b"] if "b" in z.files else None
        m = int(z["m"])
        got = gpu_engine.join(a, b, m, profile, form, computing_rows=rows,
                              threshold=thr, **kw)
        for side in ("a", "b"):
            if "packed_" + side in z.files:
                wc = (z["packed_" + side] & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.float32)
                wi = (z["packed_" + side] >> np.uint64(32)).astype(np.int64)
                gc, gi = gpu_engine.unpack_profile(got["profile_" + side])
                mine = a if side == "a" else (b if b is not None else a)
                other = (b if b is not None else a) if side == "a" else a
                # Windows the reference treats as valid only through the
                # rounding residue of its sequential ssd (exactly flat
                # windows) are excluded, with every entry pointing at one.
                _, _, inv_mine = window_stats(mine, m)
                _, _, inv_other = window_stats(other, m)
                art = np.isnan(inv_mine)
                art |= (wi >= 0) & (wi < len(inv_other)) & np.isnan(inv_other[np.clip(wi, 0, len(inv_other) - 1)]) & (wc >= -1)
                ok = (wc >= -1) & ~art
                assert np.array_equal((gc < -1)[~art], (wc < -1)[~art]), f
                err = np.abs(gc[ok].astype(np.float64) - wc[ok])
                assert err.max() <= tol + 2.5e-7, (f, err.max())
                mism = np.nonzero(ok & (gi != wi))[0]
                if mism.size:
                    r = pair_corr(other, mine, m, gi[mism], mism)
                    assert np.all(np.abs(r - wc[mism]) <= tol + 2.5e-7), f
            if "max_" + side in z.files:
                w = z["max_" + side].astype(np.float64)
                g = got["profile_" + side].astype(np.float64)
                assert np.array_equal(w < -1, g < -1), f
                assert np.max(np.abs(w[w >= -1] - g[w >= -1])) <= tol + 2.5e-7, f
            if "sum_" + side in z.files:
                rt = 1e-9 if precision == "double" else 2e-5
                check_sum(f, got["sum_" + side], z["sum_" + side], thr, rt,
                          0.0 if precision == "double" else TOL_MIXED)


# Joins of >= 4e9 cells at m >= 64 run the block-averaged seeding pre-pass
# before the mixed band kernel; the result must be the unseeded join's.
@pytest.mark.parametrize("keep_rows", [True, False])
def test_seeded_abjoin(gpu_engine, oracle_mod, keep_rows):
    from scamp_gb300 import workloads

    a, b, m = workloads.motif_abjoin(na=1 << 17, nb=1 << 16, motifs=16)
    assert gpu_engine.count_cells(len(a), m, len_b=len(b)) >= 4 << 30
    got, _ = run_1nn(gpu_engine, oracle_mod, a, b, m, "mixed", TOL_MIXED, keep_rows=keep_rows,
                     rows=keep_rows, name="seeded_ab")
    assert got["gpu_launches"] > 12  # pre-pass launches included


def test_seeded_selfjoin(gpu_engine, oracle_mod):
    rng = np.random.default_rng(123)
    a = rw(rng, 1 << 17)
    got, _ = run_1nn(gpu_engine, oracle_mod, a, None, 128, "mixed", TOL_MIXED, name="seeded_self")
    assert got["gpu_launches"] > 8


@pytest.mark.parametrize("filter_mode", [1, 2])
def test_mixed_filters_both_forms(gpu_engine, oracle_mod, filter_mode):
    """The mixed band kernel's two fast-path filters (per-cell r, and the
    per-step covariance bound chosen for long windows) give the same
    parity, at short and long windows, self and AB, 1NN_INDEX and
    SUM_THRESH."""
    rng = np.random.default_rng(31)
    a = rw(rng, 6000)
    b = rw(rng, 4500)
    a[rng.choice(6000, 8, replace=False)] = np.nan
    for m in (16, 100, 700):
        run_1nn(gpu_engine, oracle_mod, a, None, m, "mixed", TOL_MIXED,
                name="filter%d/self%d" % (filter_mode, m), filter_mode=filter_mode)
        run_1nn(gpu_engine, oracle_mod, a, b, m, "mixed", TOL_MIXED, keep_rows=True,
                name="filter%d/ab%d" % (filter_mode, m), filter_mode=filter_mode)
        got = gpu_engine.join(a, b, m, "SUM_THRESH", "mixed", threshold=0.6, keep_rows=True,
                              filter_mode=filter_mode)
        want = oracle_mod.join(a, b, m, "SUM_THRESH", threshold=0.6, keep_rows=True)
        check_sum("filter%d/sum%d/A" % (filter_mode, m), got["sum_a"], want["sum_a"], 0.6,
                  2e-5, TOL_MIXED)
        check_sum("filter%d/sum%d/B" % (filter_mode, m), got["sum_b"], want["sum_b"], 0.6,
                  2e-5, TOL_MIXED)
