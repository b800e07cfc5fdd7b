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
