"""The reference's experimental profile types, APPROX_ALL_NEIGHBORS (pyscamp
selfjoin_knn / abjoin_knn) and MATRIX_SUMMARY (selfjoin_matrix /
abjoin_matrix), against brute-force correlation matrices.  The engine
computes them exactly (the reference approximates both), so every reported
value must equal the brute-force one within float32 rounding, and the k best
per window must be the true k best up to near-ties."""
import numpy as np
import pytest

from parity import TOL_MIXED, window_stats

pytestmark = pytest.mark.gpu

TOL = 1e-6  # float32 rounding of an FP64 correlation


def corr_matrix(rows, cols, m):
    """C[i, j]: r of row window i (of `rows`) and column window j."""
    Tr, mur, invr = window_stats(rows, m)
    Tc, muc, invc = window_stats(cols, m)
    Wr = np.lib.stride_tricks.sliding_window_view(Tr, m)[: len(mur)] - mur[:, None]
    Wc = np.lib.stride_tricks.sliding_window_view(Tc, m)[: len(muc)] - muc[:, None]
    return (Wr @ Wc.T) * invr[:, None] * invc[None, :]


def rw(rng, n):
    return np.cumsum(rng.standard_normal(n))


def check_knn(gpu_engine, entries, k, C, thr, name, tol=TOL):
    """entries: k packed entries per column window; C[:, j]: that column's
    candidates (NaN where excluded).  With the mixed form's tolerance the
    lists are the k best up to near-ties within `tol` (candidates chosen by
    FP32 values) and cells within `tol` of the threshold; reported values are
    FP64 either way."""
    corr, idx = gpu_engine.unpack_profile(np.asarray(entries))
    corr = corr.reshape(-1, k).astype(np.float64)
    idx = idx.reshape(-1, k)
    ns = C.shape[1]
    assert corr.shape[0] == ns
    for j in range(ns):
        col = C[:, j]
        cand = np.nonzero(col > thr)[0]
        order = cand[np.lexsort((cand, -col[cand]))][:k]
        want = col[order]
        got_ok = idx[j] >= 0
        if tol == TOL:
            assert got_ok.sum() == len(order), (name, j)
        else:
            edge = int(np.sum(np.abs(col[col == col] - thr) <= tol))
            assert abs(int(got_ok.sum()) - len(order)) <= edge, (name, j)
        g = corr[j][got_ok]
        # best first, values equal to the true k best (ties may swap indices)
        assert np.all(np.diff(g) <= TOL), (name, j)
        nn = min(len(g), len(want))
        assert np.max(np.abs(g[:nn] - want[:nn]), initial=0.0) <= tol, (name, j, g, want)
        # every reported match is the cell it names
        assert np.max(np.abs(col[idx[j][got_ok]] - g), initial=0.0) <= TOL, (name, j)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_knn_selfjoin(gpu_engine, precision):
    rng = np.random.default_rng(61)
    a = rw(rng, 2500)
    m, k = 50, 4
    r = gpu_engine.join(a, None, m, "ALL_NEIGHBORS", precision, threshold=0.3, max_matches=k)
    C = corr_matrix(a, a, m)
    ns = C.shape[0]
    ii, jj = np.indices(C.shape)
    C[np.abs(ii - jj) < m // 4] = np.nan
    check_knn(gpu_engine, r["knn_a"], k, C, 0.3, "self", TOL if precision == "double" else TOL_MIXED)
    assert ns == len(a) - m + 1
    if precision == "mixed":
        # the band kernel's form: FP64 values, the tie margin stated
        assert r["max_abs_r_err"] < 1e-9 and 0 <= r["max_tie_margin"] <= TOL_MIXED


@pytest.mark.parametrize("k", [1, 5, 16])
def test_knn_mixed_vs_fp64(gpu_engine, k):
    """The mixed k-best form (band kernel, lists in the exact path and the
    verification kernel, FP64 re-evaluation) against the FP64 visit kernel on
    a self-join with NaN windows and an AB-join with both profiles."""
    rng = np.random.default_rng(67 + k)
    a, b = rw(rng, 30000), rw(rng, 20000)
    a[7000:7030] = np.nan
    m = 128
    for bb, kw in ((None, {}), (b, {"keep_rows": True})):
        f = gpu_engine.join(a, bb, m, "ALL_NEIGHBORS", "double", threshold=0.6, max_matches=k, **kw)
        x = gpu_engine.join(a, bb, m, "ALL_NEIGHBORS", "mixed", threshold=0.6, max_matches=k, **kw)
        for side in ("knn_a", "knn_b") if bb is not None else ("knn_a",):
            fc, fi = gpu_engine.unpack_profile(f[side])
            xc, xi = gpu_engine.unpack_profile(x[side])
            fc, xc = fc.reshape(-1, k).astype(np.float64), xc.reshape(-1, k).astype(np.float64)
            fi, xi = fi.reshape(-1, k), xi.reshape(-1, k)
            both = (fi >= 0) & (xi >= 0)
            # rank by rank the same values up to near-ties; the same entries
            # present except at the threshold's edge
            assert np.max(np.abs(fc[both] - xc[both]), initial=0.0) <= TOL_MIXED
            only = (fi >= 0) != (xi >= 0)
            assert np.all(np.abs(np.where(fi >= 0, fc, xc)[only] - 0.6) <= 1e-4)
            # indices agree except where values tie within the tolerance
            diff = both & (fi != xi)
            assert diff.sum() <= max(1, 0.01 * both.sum())
        assert 0 <= x["max_tie_margin"] <= TOL_MIXED


def test_knn_abjoin_and_pyscamp_surface(gpu_engine):
    rng = np.random.default_rng(62)
    a, b = rw(rng, 2200), rw(rng, 1700)
    m, k = 40, 3
    r = gpu_engine.join(a, b, m, "ALL_NEIGHBORS", "double", computing_rows=False,
                        max_matches=k)
    C = corr_matrix(b, a, m)  # rows: windows of b, columns: windows of a
    check_knn(gpu_engine, r["knn_a"], k, C, 0.0, "ab")
    # pyscamp.abjoin_knn: (column, row, value) tuples, per column from the
    # lowest correlation up; pearson values are the correlations
    tup = gpu_engine.abjoin_knn(a, b, m, k, pearson=True)
    assert len(tup) == int(np.sum(gpu_engine.unpack_profile(r["knn_a"])[1] >= 0))
    cols = np.array([t[0] for t in tup])
    assert np.all(np.diff(cols) >= 0)
    for c, row, v in tup[:200]:
        assert abs(C[row, c] - v) <= TOL
    dist = gpu_engine.abjoin_knn(a, b, m, k)
    c, row, v = dist[0]
    assert abs(v - np.sqrt(max(2 * m * (1 - C[row, c]), 0))) < 1e-3


def check_matrix(mat, C, h, w, thr, tol=TOL):
    """Grid entries against the brute-force maxima above `thr`; with the
    mixed form's tolerance an entry whose largest cell lies within `tol` of
    the threshold may be either side of it."""
    rpc = -(-C.shape[0] // h)
    cpc = -(-C.shape[1] // w)
    want = np.full((h, w), -2.0)
    top = np.full((h, w), -2.0)
    for y in range(h):
        for x in range(w):
            blk = C[y * rpc:(y + 1) * rpc, x * cpc:(x + 1) * cpc]
            if np.any(blk == blk):
                top[y, x] = np.nanmax(blk)
            v = blk[blk > thr]
            if v.size:
                want[y, x] = v.max()
    edge = np.abs(top - thr) <= tol
    assert np.array_equal((mat < -1)[~edge], (want < -1)[~edge])
    ok = (want >= -1) & (mat >= -1)
    assert np.max(np.abs(mat[ok] - want[ok]), initial=0.0) <= tol
    assert np.all(mat[(mat >= -1) & (want < -1)] <= thr + tol)


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_matrix_summary(gpu_engine, precision):
    rng = np.random.default_rng(63)
    a, b = rw(rng, 3000), rw(rng, 2000)
    m = 64
    # self-join: columns only, so the cells with j - i >= m/4 (upper triangle)
    tol = TOL if precision == "double" else TOL_MIXED
    r = gpu_engine.join(a, None, m, "MATRIX_SUMMARY", precision, threshold=0.2,
                        matrix_height=20, matrix_width=30)
    C = corr_matrix(a, a, m)
    ii, jj = np.indices(C.shape)
    C[jj - ii < m // 4] = np.nan
    check_matrix(r["matrix"].astype(np.float64), C, 20, 30, 0.2, tol)
    if precision == "mixed":
        # the band kernel's form (grid entries of >= 64 windows each) states
        # its bound: the largest drift margin of a published maximum
        assert 0 < r["max_abs_r_err"] < 1e-3
    # AB-join: every (window of b, window of a) cell
    r = gpu_engine.join(a, b, m, "MATRIX_SUMMARY", precision, computing_rows=False,
                        matrix_height=17, matrix_width=23)
    check_matrix(r["matrix"].astype(np.float64), corr_matrix(b, a, m), 17, 23, 0.0, tol)
    # pyscamp surface: distances (NaN where none), shape (mheight, mwidth)
    d = gpu_engine.abjoin_matrix(a, b, m, mheight=17, mwidth=23)
    assert d.shape == (17, 23)
    mat = r["matrix"].astype(np.float64)
    want = np.where(mat < -1, np.nan, np.sqrt(np.maximum(2 * m * (1 - mat), 0)))
    np.testing.assert_allclose(d, want, rtol=1e-5, atol=1e-4)
    p = gpu_engine.selfjoin_matrix(a, m, pearson=True, mheight=5, mwidth=5)
    assert p.shape == (5, 5)


@pytest.mark.parametrize("shape", [(7, 5), (3, 64), (50, 2)])
def test_matrix_summary_mixed_vs_fp64(gpu_engine, shape):
    """The mixed form (band kernel, grid entries crossing its blocks at
    uneven boundaries, NaN windows) against the FP64 visit kernel on a larger
    self-join and an AB-join with both profiles' transposed halves."""
    rng = np.random.default_rng(66)
    a, b = rw(rng, 40000), rw(rng, 30000)
    a[5000:5040] = np.nan
    m = 100
    h, w = shape
    for bb in (None, b):
        kw = dict(threshold=0.5, matrix_height=h, matrix_width=w)
        if bb is not None:
            kw["computing_rows"] = False
        f = gpu_engine.join(a, bb, m, "MATRIX_SUMMARY", "double", **kw)
        x = gpu_engine.join(a, bb, m, "MATRIX_SUMMARY", "mixed", **kw)
        fm, xm = f["matrix"].astype(np.float64), x["matrix"].astype(np.float64)
        both = (fm >= -1) & (xm >= -1)
        assert both.sum() >= 0.9 * max((fm >= -1).sum(), 1)
        assert np.max(np.abs(fm[both] - xm[both]), initial=0.0) <= TOL_MIXED
        # an entry on one side only lies at the threshold's edge
        assert np.all(fm[(fm >= -1) & (xm < -1)] <= 0.5 + TOL_MIXED)
        assert np.all(xm[(xm >= -1) & (fm < -1)] <= 0.5 + TOL_MIXED)
        # the stated bound covers the observed error
        assert np.max(np.abs(fm[both] - xm[both]), initial=0.0) <= x["max_abs_r_err"] < 1e-3


def test_matrix_merges_into_given_matrix(gpu_engine):
    rng = np.random.default_rng(64)
    a = rw(rng, 1500)
    init = np.full((4, 4), -2.0, dtype=np.float32)
    init[0, 3] = 1.0
    r = gpu_engine.join(a, None, 32, "MATRIX_SUMMARY", "double", profile_a=init,
                        matrix_height=4, matrix_width=4)
    plain = gpu_engine.join(a, None, 32, "MATRIX_SUMMARY", "double", matrix_height=4,
                            matrix_width=4)
    assert r["matrix"][0, 3] == 1.0
    mask = np.ones((4, 4), bool)
    mask[0, 3] = False
    assert np.array_equal(r["matrix"][mask], plain["matrix"][mask])


@pytest.mark.parametrize("profile", ["1NN", "ALL_NEIGHBORS", "MATRIX_SUMMARY"])
def test_device_entry_matches_host_entry(gpu_engine, profile):
    """join_device (device buffers, merged in place) gives what join (host
    buffers) gives for the float32, k-best and matrix outputs."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(65)
    a, b = rw(rng, 2600), rw(rng, 1900)
    m, k, h, w = 48, 3, 9, 11
    kw = dict(max_matches=k, matrix_height=h, matrix_width=w)
    host = gpu_engine.join(a, b, m, profile, "double", keep_rows=profile != "MATRIX_SUMMARY",
                           threshold=0.1, **kw)
    dev = torch.device("cuda", 0)
    a_d = torch.from_numpy(a).to(dev)
    b_d = torch.from_numpy(b).to(dev)
    nsa, nsb = len(a) - m + 1, len(b) - m + 1
    no_match = int(np.array([gpu_engine.NO_MATCH], np.uint64).view(np.int64)[0])
    ptrs, outs = {}, {}
    if profile == "1NN":
        for side, ns in (("a", nsa), ("b", nsb)):
            outs["max_" + side] = torch.full((ns,), -2.0, dtype=torch.float32, device=dev)
            ptrs["max_%s_ptr" % side] = outs["max_" + side].data_ptr()
    elif profile == "ALL_NEIGHBORS":
        for side, ns in (("a", nsa), ("b", nsb)):
            outs["knn_" + side] = torch.full((ns * k,), no_match, dtype=torch.int64, device=dev)
            ptrs["knn_%s_ptr" % side] = outs["knn_" + side].data_ptr()
    else:
        outs["matrix"] = torch.full((h, w), -2.0, dtype=torch.float32, device=dev)
        ptrs["matrix_ptr"] = outs["matrix"].data_ptr()
    stream = torch.cuda.current_stream(dev)
    gpu_engine.join_device(a_d.data_ptr(), len(a), m, b_d.data_ptr(), len(b), profile, "double",
                           keep_rows=profile != "MATRIX_SUMMARY", threshold=0.1,
                           stream=stream.cuda_stream, **ptrs, **kw)
    torch.cuda.synchronize(dev)
    for key, t in outs.items():
        got = t.cpu().numpy()
        want = host[key.replace("max_", "profile_")]
        if got.dtype == np.int64:
            got = got.view(np.uint64)
        assert np.array_equal(got.reshape(want.shape), want), key
