"""Parity checks between the engine and the CPU oracle.

Tolerances follow the requirement for this path: FP64 form within 1e-9 in
the Pearson correlation r, mixed form within 1e-5; an index must match the
oracle's exactly or, under a near-tie, point at a window whose correlation
(recomputed here in FP64) is within the same tolerance of the best.  The
reference's own test accepts an index mismatch when the FP32 correlations
agree (test/test_common.py:3-16); this rule is stricter for FP64.
"""
import numpy as np

TOL_FP64 = 1e-9
TOL_MIXED = 1e-5


def window_stats(T, m):
    """Cleaned series, per-window mean and 1/norm (NaN for windows holding a
    non-finite sample or with ssd <= 1e-13), all in FP64 (brute force)."""
    T = np.asarray(T, dtype=np.float64)
    bad = ~np.isfinite(T)
    Tc = np.where(bad, 0.0, T)
    ns = len(T) - m + 1
    W = np.lib.stride_tricks.sliding_window_view(Tc, m)
    mu = W.mean(axis=1)
    ssd = ((W - mu[:, None]) ** 2).sum(axis=1)
    badw = np.lib.stride_tricks.sliding_window_view(bad, m).any(axis=1)
    inv = np.where(badw | (ssd <= 1e-13), np.nan, 1.0 / np.sqrt(np.where(ssd > 0, ssd, 1)))
    return Tc, mu[:ns], inv[:ns]


def pair_corr(Tr, Tc, m, rows, cols):
    """FP64 Pearson correlation of row windows `rows` of Tr with column
    windows `cols` of Tc (element-wise pairs)."""
    Rc, mur, ivr = window_stats(Tr, m)
    Cc, muc, ivc = window_stats(Tc, m)
    out = np.empty(len(rows))
    for k, (i, j) in enumerate(zip(rows, cols)):
        x = Rc[i:i + m] - mur[i]
        y = Cc[j:j + m] - muc[j]
        out[k] = np.dot(x, y) * ivr[i] * ivc[j]
    return out


def check_1nn(name, got_corr, got_idx, want_corr, want_idx, tol, T_self, T_other, m,
              self_side="col"):
    """Assert that a 1NN_INDEX profile matches the oracle.

    got_corr / want_corr: double correlations (-2 = no match); got_idx /
    want_idx: int64 indices (-1 = no match).  T_self is the series the
    profile belongs to, T_other the series its indices point into.
    """
    got_corr = np.asarray(got_corr, dtype=np.float64)
    want_corr = np.asarray(want_corr, dtype=np.float64)
    got_none = got_idx < 0
    want_none = want_idx < 0
    assert np.array_equal(got_none, want_none), (
        "%s: no-match pattern differs at %s" % (name, np.nonzero(got_none != want_none)[0][:10]))
    ok = ~want_none
    err = np.abs(got_corr[ok] - want_corr[ok])
    maxerr = float(err.max()) if err.size else 0.0
    assert maxerr <= tol, "%s: max |r err| %.3g > %.1g" % (name, maxerr, tol)
    mism = np.nonzero(ok & (got_idx != want_idx))[0]
    if mism.size:
        # the index we returned must be a near-tie of the best
        r = pair_corr(T_other, T_self, m, got_idx[mism], mism)
        gap = np.abs(r - want_corr[mism])
        assert np.all(gap <= tol), "%s: %d index mismatches beyond tolerance (worst %.3g)" % (
            name, int(np.sum(gap > tol)), float(gap.max()))
    return maxerr, int(mism.size)


def check_sum(name, got, want, thr, rtol, cell_tol=0.0):
    """SUM_THRESH: relative agreement, allowing whole multiples of the
    threshold where a correlation sits on the threshold edge (the reference's
    compare_vectors_sum, test/test_common.py:27-51).

    That rule accepts a difference slightly above k * thr: a cell just above
    the threshold that one side missed.  A form whose correlations carry
    errors up to cell_tol (the mixed form: TOL_MIXED) may also count a cell
    up to cell_tol below the threshold, a difference up to k * cell_tol below
    k * thr; with cell_tol > 0 a difference within rtol * |sum| + k * cell_tol
    of the nearest multiple k * thr passes."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    diff = np.abs(got - want)
    scale = np.maximum(np.abs(want), 1.0)
    bad = diff > rtol * scale
    if np.any(bad) and thr > 0:
        q = np.round(diff[bad] / thr, 6)
        frac = q - np.floor(q)
        still = frac > 1e-3
        if cell_tol > 0:
            k = np.round(diff[bad] / thr)
            still &= np.abs(diff[bad] - k * thr) > rtol * scale[bad] + k * cell_tol
        n_bad = int(np.sum(still))
    else:
        n_bad = int(np.sum(bad))
    assert n_bad == 0, "%s: %d sums differ (max rel %.3g)" % (name, n_bad, float((diff / scale).max()))
    return float((diff / scale).max()) if diff.size else 0.0


def cell_corr(T_rows, T_cols, m, rows, cols, chunk=4096):
    """FP64 Pearson correlation of row window rows[k] of T_rows with column
    window cols[k] of T_cols, computed directly for each pair (centred dot
    product over centred sums of squares), vectorised in chunks."""
    Rc = np.where(np.isfinite(T_rows), T_rows, 0.0).astype(np.float64)
    Cc = np.where(np.isfinite(T_cols), T_cols, 0.0).astype(np.float64)
    WR = np.lib.stride_tricks.sliding_window_view(Rc, m)
    WC = np.lib.stride_tricks.sliding_window_view(Cc, m)
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    out = np.empty(len(rows))
    for s in range(0, len(rows), chunk):
        X = WR[rows[s:s + chunk]]
        Y = WC[cols[s:s + chunk]]
        X = X - X.mean(axis=1, keepdims=True)
        Y = Y - Y.mean(axis=1, keepdims=True)
        out[s:s + chunk] = np.einsum("ij,ij->i", X, Y) / np.sqrt(
            np.einsum("ij,ij->i", X, X) * np.einsum("ij,ij->i", Y, Y))
    return out


def check_1nn_direct(name, got_corr, got_idx, want_idx, tol, T_self, T_other, m, bound=None):
    """A 1NN_INDEX profile against direct FP64 correlations (for sizes where
    the oracle's own long recurrences drift by more than the FP64 form's
    tolerance; the oracle still gives the no-match pattern and its choice of
    partner):
      * the no-match pattern equals the oracle's;
      * every reported value is within tol (and within the engine's reported
        bound, when given, plus numpy's own rounding) of the direct FP64
        correlation of its (window, partner) pair;
      * the reported partner is no worse than the oracle's by more than tol
        (both evaluated directly).
    Returns (max |value error|, worst shortfall against the oracle's partner)."""
    got_corr = np.asarray(got_corr, dtype=np.float64)
    got_none = got_idx < 0
    want_none = want_idx < 0
    assert np.array_equal(got_none, want_none), (
        "%s: no-match pattern differs at %s" % (name, np.nonzero(got_none != want_none)[0][:10]))
    w = np.nonzero(~want_none)[0]
    if w.size == 0:
        return 0.0, 0.0
    r_got = cell_corr(T_other, T_self, m, got_idx[w], w)
    err = np.abs(got_corr[w] - r_got)
    maxerr = float(err.max())
    assert maxerr <= tol, "%s: max |r - direct r| %.3g > %.1g" % (name, maxerr, tol)
    if bound is not None:
        assert maxerr <= bound + 1e-13, "%s: value error %.3g above the reported bound %.3g" % (
            name, maxerr, bound)
    diff = np.nonzero(got_idx[w] != want_idx[w])[0]
    short = 0.0
    if diff.size:
        r_want = cell_corr(T_other, T_self, m, want_idx[w[diff]], w[diff])
        short = float(np.max(r_want - r_got[diff]))
        assert short <= tol, "%s: a reported partner is %.3g below the oracle's" % (name, short)
    return maxerr, short
