"""scamp_gb300 -- GB300-native SCAMP matrix-profile engine, Python front.

Drop-in for pyscamp's join functions (reference: python/SCAMP_python.cpp of
zpzim/GPU-SCRIMP-LARGE): ``selfjoin``, ``abjoin``, ``selfjoin_sum``,
``abjoin_sum`` and ``gpu_supported`` keep their names, arguments, keyword
validation, defaults and output conventions.  Every join runs on the GPU
through the C ABI in include/scamp_gb300.h; there is no CPU fallback.

``join`` is the lower-level entry that exposes the full SCAMPArgs surface
(keep_rows, aligned, distributed offsets, precision, profile buffers to merge
into) and returns the reference's packed 1NN_INDEX entries.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import SCAMPError

__all__ = [
    "selfjoin", "abjoin", "selfjoin_sum", "abjoin_sum", "selfjoin_knn", "abjoin_knn",
    "selfjoin_matrix", "abjoin_matrix", "gpu_supported",
    "join", "join_device", "join_batch", "tune_batch", "SCAMPError", "count_cells", "pipe_peak",
    "unpack_profile", "to_distance", "version",
]

_PRECISION = {
    "single": _lib.PRECISION_SINGLE,
    "mixed": _lib.PRECISION_MIXED,
    "double": _lib.PRECISION_DOUBLE,
    "ultra": _lib.PRECISION_ULTRA,
}
_PROFILE = {"1NN_INDEX": _lib.PROFILE_1NN_INDEX, "SUM_THRESH": _lib.PROFILE_SUM_THRESH,
            "1NN": _lib.PROFILE_1NN, "ALL_NEIGHBORS": _lib.PROFILE_APPROX_ALL_NEIGHBORS,
            "APPROX_ALL_NEIGHBORS": _lib.PROFILE_APPROX_ALL_NEIGHBORS,
            "MATRIX_SUMMARY": _lib.PROFILE_MATRIX_SUMMARY}

# 1NN_INDEX "no match" entry {corr = -2.0f, index = 0xFFFFFFFF}
# (src/common.cpp:294-299).
NO_MATCH = np.uint64((0xFFFFFFFF << 32) | int(np.float32(-2.0).view(np.uint32)))


def version():
    """The engine library's version string."""
    return _lib.load().scamp_gb300_version().decode()


def gpu_supported():
    """True when the engine library loads and a CUDA device is visible
    (pyscamp gpu_supported, python/SCAMP_python.cpp:363-369)."""
    try:
        return bool(_lib.load().scamp_gb300_gpu_supported())
    except OSError:
        return False


def _args(a, b, m, profile, precision, computing_rows, computing_cols,
          keep_rows, aligned, threshold, start_row, start_col, max_tile_size,
          anchor_interval, device, silent, max_matches=5, matrix_height=50, matrix_width=50,
          filter_mode=0, anchor_mode=0):
    ca = _lib.CArgs()
    ca.timeseries_a = a.ctypes.data if a is not None else None
    ca.len_a = len(a) if a is not None else 0
    ca.has_b = 1 if b is not None else 0
    ca.timeseries_b = b.ctypes.data if b is not None else None
    ca.len_b = len(b) if b is not None else 0
    ca.window = int(m)
    ca.max_tile_size = int(max_tile_size)
    ca.distributed_start_row = int(start_row)
    ca.distributed_start_col = int(start_col)
    ca.distance_threshold = float(threshold)
    ca.precision_type = _PRECISION[precision] if isinstance(precision, str) else int(precision)
    ca.profile_type = _PROFILE[profile] if isinstance(profile, str) else int(profile)
    ca.computing_rows = int(bool(computing_rows))
    ca.computing_columns = int(bool(computing_cols))
    ca.keep_rows_separate = int(bool(keep_rows))
    ca.is_aligned = int(bool(aligned))
    ca.silent_mode = int(bool(silent))
    ca.anchor_interval = int(anchor_interval)
    ca.device = int(device)
    ca.max_matches_per_column = int(max_matches)
    ca.matrix_height = int(matrix_height)
    ca.matrix_width = int(matrix_width)
    ca.filter_mode = int(filter_mode)
    ca.anchor_mode = int(anchor_mode)
    return ca


def count_cells(len_a, m, len_b=None, aligned=False, start_row=-1, start_col=-1):
    """Distance-matrix cells a join evaluates (host logic, no GPU needed):
    the comparisons of the comparisons/s metric, with the reference's
    exclusion zones (src/tile.cpp:12-138)."""
    lib = _lib.load()
    a = np.zeros(1)
    ca = _args(None, None, m, "1NN_INDEX", "double", True, True, False, aligned,
               0.0, start_row, start_col, max(128000, 2 * m), 0, 0, True)
    ca.timeseries_a = a.ctypes.data
    ca.len_a = int(len_a)
    if len_b is not None:
        ca.has_b = 1
        ca.timeseries_b = a.ctypes.data
        ca.len_b = int(len_b)
    return int(lib.scamp_gb300_count_cells(ctypes.byref(ca)))


def pipe_peak(kind="fp32", device=0):
    """Measured FMA lane-operations per second of the FP32 or FP64 pipe."""
    out = ctypes.c_double(0)
    rc = _lib.load().scamp_gb300_pipe_peak(int(device), 0 if kind == "fp32" else 1,
                                           ctypes.byref(out))
    if rc:
        raise SCAMPError(rc, "pipe peak probe failed")
    return out.value


def anchor_check(device=0):
    """Self-check of the mixed form's tensor-core anchors (C ABI
    scamp_gb300_anchor_check): (largest |anchor - FP64 cov| * invnorm_r *
    invnorm_c on a seeded random walk, True when joins use them)."""
    err = ctypes.c_double(0)
    avail = ctypes.c_int(0)
    buf = ctypes.create_string_buffer(1024)
    rc = _lib.load().scamp_gb300_anchor_check(int(device), ctypes.byref(err), ctypes.byref(avail),
                                              buf, 1024)
    _check(rc, buf)
    return err.value, bool(avail.value)


def window_stats(series, m, high_precision_norms=False, device=0):
    """Window statistics as the joins compute them on the device (C ABI
    scamp_gb300_window_stats; the reference's compute_statistics_cpu,
    src/cpu_stats.cpp:123-160): (mean, invnorm, df, dg), FP64 arrays of
    len(series) - m + 1 windows."""
    x = np.ascontiguousarray(series, dtype=np.float64)
    ns = len(x) - int(m) + 1
    if int(m) < 3 or ns < 1:
        raise ValueError("window statistics need a window >= 3 and a series at least that long")
    out = [np.empty(ns, dtype=np.float64) for _ in range(4)]
    buf = ctypes.create_string_buffer(1024)
    ptr = lambda a: a.ctypes.data_as(_lib._dp)
    rc = _lib.load().scamp_gb300_window_stats(int(device), ptr(x), len(x), int(m),
                                              1 if high_precision_norms else 0,
                                              *[ptr(o) for o in out], buf, 1024)
    _check(rc, buf)
    return tuple(out)


def _check(rc, err):
    if rc != _lib.SCAMP_OK:
        msg = err.value.decode(errors="replace") or _lib.ERROR_NAMES.get(rc, str(rc))
        if rc == 100:
            raise ValueError(msg)
        raise SCAMPError(rc, msg)


def join(a, b=None, m=None, profile="1NN_INDEX", precision="double",
         computing_rows=True, computing_cols=True, keep_rows=False,
         aligned=False, threshold=0.0, start_row=-1, start_col=-1,
         max_tile_size=128000, anchor_interval=0, device=0, profile_a=None,
         profile_b=None, return_corr=False, silent=True, inplace=False, max_matches=5,
         matrix_height=50, matrix_width=50, filter_mode=0, anchor_mode=0):
    """Run one join (the C ABI's scamp_gb300_join, host buffers; the
    reference's SCAMP::do_SCAMP, src/SCAMP.cpp:261-334, with the arguments
    of SCAMPArgs, src/common.h:164-188).

    For 1NN_INDEX returns ``profile_a`` (and ``profile_b`` with keep_rows) as
    uint64 arrays in the reference's packed layout; ``profile_a`` /
    ``profile_b`` given on input are merged into, like a best-so-far profile
    passed to do_SCAMP.  For 1NN (the reference's PROFILE_TYPE_1NN) they are
    float32 arrays of the best correlation, -2 where there is none.  For
    SUM_THRESH returns ``sum_a`` / ``sum_b``.  For ALL_NEIGHBORS returns
    ``knn_a`` (and ``knn_b``): ``max_matches`` packed entries per window,
    best first, -2 / index 0xFFFFFFFF where unused.  For MATRIX_SUMMARY
    returns ``matrix``, a (matrix_height, matrix_width) float32 array of the
    largest correlation per grid cell (-2 where none); ``profile_a`` given
    on input is the initial matrix.
    ``corr_a`` / ``corr_b`` (double correlations) when return_corr.
    With ``inplace`` the given profile arrays (contiguous uint64 / float64)
    are updated directly instead of copied (e.g. pinned host buffers).
    """
    lib = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    if b is not None:
        b = np.ascontiguousarray(b, dtype=np.float64)
    if m is None:
        raise ValueError("window m is required")
    ca = _args(a, b, m, profile, precision, computing_rows, computing_cols,
               keep_rows, aligned, threshold, start_row, start_col,
               max_tile_size, anchor_interval, device, silent, max_matches,
               matrix_height, matrix_width, filter_mode, anchor_mode)
    err = ctypes.create_string_buffer(1024)
    rc = lib.scamp_gb300_validate(ctypes.byref(ca), err, 1024)
    _check(rc, err)
    nsa = len(a) - m + 1
    nsb = (len(b) if b is not None else len(a)) - m + 1
    res = _lib.CResult()
    out = {}
    is_1nn = ca.profile_type == _lib.PROFILE_1NN_INDEX
    max_only = ca.profile_type == _lib.PROFILE_1NN

    def _buf(given, n, dtype, fill):
        if given is None:
            return np.full(n, fill, dtype=dtype)
        if len(given) != n:
            raise ValueError("profile buffer has %d entries, expected %d" % (len(given), n))
        if inplace and given.dtype == dtype and given.flags["C_CONTIGUOUS"]:
            return given
        return np.array(given, dtype=dtype, copy=True)

    if ca.profile_type == _lib.PROFILE_APPROX_ALL_NEIGHBORS:
        k = int(max_matches)
        ka = _buf(profile_a, nsa * k, np.uint64, NO_MATCH)
        out["knn_a"] = ka
        res.knn_a = ka.ctypes.data
        if keep_rows:
            kb = _buf(profile_b, nsb * k, np.uint64, NO_MATCH)
            out["knn_b"] = kb
            res.knn_b = kb.ctypes.data
    elif ca.profile_type == _lib.PROFILE_MATRIX_SUMMARY:
        mat = _buf(None if profile_a is None else np.asarray(profile_a).ravel(),
                   int(matrix_height) * int(matrix_width), np.float32, np.float32(-2.0))
        out["matrix"] = mat.reshape(int(matrix_height), int(matrix_width))
        res.matrix = mat.ctypes.data
    elif is_1nn or max_only:
        dt, fill = (np.float32, np.float32(-2.0)) if max_only else (np.uint64, NO_MATCH)
        pa = _buf(profile_a, nsa, dt, fill)
        out["profile_a"] = pa
        pb = _buf(profile_b, nsb, dt, fill) if keep_rows else None
        if keep_rows:
            out["profile_b"] = pb
        if max_only:
            res.max_a = pa.ctypes.data
            res.max_b = pb.ctypes.data if keep_rows else None
        else:
            res.profile_a = pa.ctypes.data
            res.profile_b = pb.ctypes.data if keep_rows else None
        if return_corr:
            out["corr_a"] = np.empty(nsa)
            res.corr_a = out["corr_a"].ctypes.data
            if keep_rows:
                out["corr_b"] = np.empty(nsb)
                res.corr_b = out["corr_b"].ctypes.data
    else:
        sa = _buf(profile_a, nsa, np.float64, 0.0)
        out["sum_a"] = sa
        res.sum_a = sa.ctypes.data
        if keep_rows:
            sb = _buf(profile_b, nsb, np.float64, 0.0)
            out["sum_b"] = sb
            res.sum_b = sb.ctypes.data
    rc = lib.scamp_gb300_join(ctypes.byref(ca), ctypes.byref(res), err, 1024)
    _check(rc, err)
    out["elapsed_ms"] = res.elapsed_ms
    out["join_kernel_ms"] = res.join_kernel_ms
    out["comparisons"] = int(res.comparisons)
    out["gpu_launches"] = int(res.gpu_launches)
    out["counters"] = {"steps": int(res.steps), "slow_steps": int(res.slow_steps),
                       "verifications": int(res.verifications),
                       "inplace_verifications": int(res.inplace_verifications),
                       "verify_kernel_ms": float(res.verify_kernel_ms)}
    out["max_abs_r_err"] = float(res.max_abs_r_err)
    out["max_tie_margin"] = float(res.max_tie_margin)
    return out


def join_device(a_ptr, len_a, m, b_ptr=None, len_b=0, profile="1NN_INDEX",
                precision="double", computing_rows=True, computing_cols=True,
                keep_rows=False, aligned=False, threshold=0.0,
                profile_a_ptr=None, profile_b_ptr=None, sum_a_ptr=None,
                sum_b_ptr=None, corr_a_ptr=None, corr_b_ptr=None, stream=0,
                anchor_interval=0, device=0, max_tile_size=128000, max_a_ptr=None,
                max_b_ptr=None, knn_a_ptr=None, knn_b_ptr=None, matrix_ptr=None,
                max_matches=5, matrix_height=50, matrix_width=50, filter_mode=0,
                anchor_mode=0):
    """scamp_gb300_join_dev: every pointer is device memory (integers, e.g.
    ``tensor.data_ptr()``), results merged in place, ordered on ``stream``.
    ``max_a_ptr`` / ``max_b_ptr``: float32 profiles of the 1NN type;
    ``knn_a_ptr`` / ``knn_b_ptr``: ``max_matches`` packed entries per window
    (ALL_NEIGHBORS); ``matrix_ptr``: the float32 grid (MATRIX_SUMMARY)."""
    lib = _lib.load()
    ca = _args(None, None, m, profile, precision, computing_rows, computing_cols,
               keep_rows, aligned, threshold, -1, -1, max_tile_size,
               anchor_interval, device, True, max_matches, matrix_height, matrix_width,
               filter_mode, anchor_mode)
    ca.timeseries_a = a_ptr
    ca.len_a = int(len_a)
    if b_ptr is not None:
        ca.has_b = 1
        ca.timeseries_b = b_ptr
        ca.len_b = int(len_b)
    res = _lib.CResult()
    res.profile_a, res.profile_b = profile_a_ptr, profile_b_ptr
    res.sum_a, res.sum_b = sum_a_ptr, sum_b_ptr
    res.corr_a, res.corr_b = corr_a_ptr, corr_b_ptr
    res.max_a, res.max_b = max_a_ptr, max_b_ptr
    res.knn_a, res.knn_b, res.matrix = knn_a_ptr, knn_b_ptr, matrix_ptr
    err = ctypes.create_string_buffer(1024)
    rc = lib.scamp_gb300_join_dev(ctypes.byref(ca), ctypes.byref(res),
                                  ctypes.c_void_p(stream), err, 1024)
    _check(rc, err)
    return {"elapsed_ms": res.elapsed_ms, "join_kernel_ms": res.join_kernel_ms,
            "counters": {"steps": int(res.steps), "slow_steps": int(res.slow_steps),
                         "verifications": int(res.verifications),
                       "inplace_verifications": int(res.inplace_verifications),
                         "verify_kernel_ms": float(res.verify_kernel_ms)},
            "comparisons": int(res.comparisons),
            "gpu_launches": int(res.gpu_launches),
            "max_abs_r_err": float(res.max_abs_r_err),
            "max_tie_margin": float(res.max_tie_margin)}


def _batch_args(series, windows, precision, device):
    """(float64 arrays, windows, CArgs array) of a batch of self-joins."""
    n = len(series)
    if isinstance(windows, (int, np.integer)):
        windows = [int(windows)] * n
    if len(windows) != n:
        raise ValueError("one window per series")
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in series]
    cargs = (_lib.CArgs * n)()
    for k, (x, m) in enumerate(zip(arrs, windows)):
        ca = _args(x, None, m, "1NN_INDEX", precision, True, True, False, False, 0.0,
                   -1, -1, max(128000, 2 * int(m)), 0, device, True)
        ctypes.memmove(ctypes.byref(cargs[k]), ctypes.byref(ca), ctypes.sizeof(ca))
    return arrs, windows, cargs


def tune_batch(series, windows, precision="mixed", retune=False, device=0):
    """scamp_gb300_tune_batch: picks, per window length, the batched join's
    segment length (tile height, also the anchor interval) by timing the
    band kernel on a sample of these series; later join_batch calls on the
    device use it.  Windows tuned before are kept unless ``retune``.
    Returns the segment length each series will use."""
    lib = _lib.load()
    arrs, windows, cargs = _batch_args(series, windows, precision, device)
    n = len(arrs)
    seg = np.zeros(n, dtype=np.int64)
    err = ctypes.create_string_buffer(1024)
    rc = lib.scamp_gb300_tune_batch(cargs, n, 1 if retune else 0,
                                    seg.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), err, 1024)
    _check(rc, err)
    return seg


def join_batch(series, windows, precision="mixed", return_corr=False, device=0,
               autotune=False):
    """scamp_gb300_join_batch: independent 1NN_INDEX self-joins of every
    series in ``series`` (window ``windows[k]``, or one int for all) in one
    batched call.  Returns a list of dicts with ``profile_a`` (packed
    entries), ``corr_a`` (with ``return_corr``) and the batch's timings.
    ``autotune``: first run tune_batch for windows not tuned yet."""
    lib = _lib.load()
    if autotune:
        tune_batch(series, windows, precision, False, device)
    arrs, windows, cargs = _batch_args(series, windows, precision, device)
    n = len(arrs)
    cres = (_lib.CResult * n)()
    profs, corrs = [], []
    for k, (x, m) in enumerate(zip(arrs, windows)):
        ns = len(x) - int(m) + 1
        p = np.full(max(ns, 0), NO_MATCH, dtype=np.uint64)
        profs.append(p)
        cres[k].profile_a = p.ctypes.data if ns > 0 else None
        if return_corr:
            c = np.empty(max(ns, 0), dtype=np.float64)
            corrs.append(c)
            cres[k].corr_a = c.ctypes.data if ns > 0 else None
    err = ctypes.create_string_buffer(1024)
    rc = lib.scamp_gb300_join_batch(cargs, cres, n, err, 1024)
    _check(rc, err)
    out = []
    for k in range(n):
        d = {"profile_a": profs[k], "comparisons": int(cres[k].comparisons),
             "elapsed_ms": cres[k].elapsed_ms, "join_kernel_ms": cres[k].join_kernel_ms,
             "gpu_launches": int(cres[k].gpu_launches),
             "counters": {"steps": int(cres[k].steps), "slow_steps": int(cres[k].slow_steps),
                          "verifications": int(cres[k].verifications),
                          "inplace_verifications": int(cres[k].inplace_verifications),
                          "verify_kernel_ms": float(cres[k].verify_kernel_ms)},
             "max_abs_r_err": float(cres[k].max_abs_r_err),
             "max_tie_margin": float(cres[k].max_tie_margin)}
        if return_corr:
            d["corr_a"] = corrs[k]
        out.append(d)
    return out


def unpack_profile(packed):
    """(float32 correlation, int64 index) from packed 1NN_INDEX entries
    (mp_entry, src/common.h:70-74); index -1 where there was no match."""
    packed = np.asarray(packed, dtype=np.uint64)
    corr = (packed & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.float32)
    idx = (packed >> np.uint64(32)).astype(np.int64)
    idx[corr < -1] = -1
    return corr, idx


def to_distance(corr, m):
    """ConvertToEuclidean (src/scamp_utils.cpp:127-133): sqrt(max(2m(1-r), 0)),
    NaN where there was no match (r < -1)."""
    corr = np.asarray(corr, dtype=np.float64)
    with np.errstate(invalid="ignore"):
        d = np.sqrt(np.maximum(2.0 * m * (1.0 - corr), 0.0))
    d[corr < -1] = np.nan
    return d


# ---------------------------------------------------------------------------
# pyscamp-compatible surface (python/SCAMP_python.cpp).
# ---------------------------------------------------------------------------
_NN_KEYS = {"verbose", "precision", "pearson", "gpus", "threads"}
_SUM_KEYS = _NN_KEYS | {"threshold"}


def _parse_kwargs(kwargs, allowed):
    """Keyword handling of get_args_based_on_kwargs
    (python/SCAMP_python.cpp:91-177); errors are ValueError like pybind11's
    mapping of std::invalid_argument."""
    opts = {"precision": "double", "pearson": False, "silent": True,
            "threshold": 0.0, "device": 0}
    for key, val in kwargs.items():
        if key not in allowed:
            raise ValueError("Invalid keyword argument specified unknown argument: " + key)
        if key == "threshold":
            thr = float(val)
            if thr > 1 or thr < -1:
                raise ValueError("Invalid threshold specified: value must be between -1 and 1")
            opts["threshold"] = thr
        elif key == "verbose":
            opts["silent"] = not bool(val)
        elif key == "precision":
            if val not in _PRECISION:
                raise ValueError("Invalid precision type specified: valid options are single, "
                                 "mixed, double, ultra")
            opts["precision"] = val
        elif key == "pearson":
            opts["pearson"] = bool(val)
        elif key == "gpus":
            gpus = [int(x) for x in val]
            # One GPU per engine instance: the first listed device is used.
            if gpus:
                opts["device"] = gpus[0]
        elif key == "threads":
            if int(val) < 0:
                raise ValueError("Invalid number of cpu worker threads specified, must be "
                                 "greater than or equal to 0.")
            # Accepted for compatibility; this engine has no CPU workers.
    return opts


_KNN_KEYS = _SUM_KEYS
_MATRIX_KEYS = _SUM_KEYS | {"mheight", "mwidth"}


def _convert(corr, pearson, m):
    """CleanupPearson / ConvertToEuclidean (src/scamp_utils.cpp:127-141):
    NaN where there is no match."""
    corr = np.asarray(corr, dtype=np.float64)
    if pearson:
        v = corr.copy()
    else:
        with np.errstate(invalid="ignore"):
            v = np.sqrt(np.maximum(2.0 * m * (1.0 - corr), 0.0))
    v[corr < -1] = np.nan
    return v


def _split_knn(entries, k, pearson, m):
    """SplitProfileKNN (python/SCAMP_python.cpp:31-49): one (column, row,
    value) tuple per match, columns in order, each column's matches from
    the lowest correlation up."""
    e = np.asarray(entries, dtype=np.uint64).reshape(-1, k)[:, ::-1]
    corr, idx = unpack_profile(e.ravel())
    cols = np.repeat(np.arange(e.shape[0], dtype=np.int64), k)
    ok = idx >= 0
    vals = _convert(corr[ok], pearson, m).astype(np.float32)
    return list(zip(cols[ok].tolist(), idx[ok].tolist(), vals.tolist()))


def _parse_matrix_kwargs(kwargs):
    o = _parse_kwargs({k: v for k, v in kwargs.items() if k not in ("mheight", "mwidth")},
                      _MATRIX_KEYS)
    for k, name in (("mheight", "height"), ("mwidth", "width")):
        v = int(kwargs.get(k, 50))
        if v <= 0:
            raise ValueError("Invalid matrix %s specified: value must be greater than 0" % name)
        o[k] = v
    return o


def selfjoin_knn(a, m, k, **kwargs):
    """The ``k`` best matches above ``threshold`` (default 0) of every window
    of ``a``: a list of (column, row, value) tuples (pyscamp.selfjoin_knn,
    python/SCAMP_python.cpp:239-259, 475-490).  These are the exact k best;
    the reference's lists are approximate."""
    o = _parse_kwargs(kwargs, _KNN_KEYS)
    r = join(np.asarray(a, dtype=np.float64), None, int(m), "ALL_NEIGHBORS", o["precision"],
             computing_rows=True, computing_cols=True, threshold=o["threshold"],
             silent=o["silent"], device=o["device"], max_matches=int(k))
    return _split_knn(r["knn_a"], int(k), o["pearson"], int(m))


def abjoin_knn(a, b, m, k, **kwargs):
    """For every window of ``a``, its ``k`` best matches in ``b`` above
    ``threshold`` (pyscamp.abjoin_knn, python/SCAMP_python.cpp:261-280,
    491-508)."""
    o = _parse_kwargs(kwargs, _KNN_KEYS)
    r = join(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), int(m),
             "ALL_NEIGHBORS", o["precision"], computing_rows=False, computing_cols=True,
             threshold=o["threshold"], silent=o["silent"], device=o["device"],
             max_matches=int(k))
    return _split_knn(r["knn_a"], int(k), o["pearson"], int(m))


def selfjoin_matrix(a, m, **kwargs):
    """An (mheight, mwidth) summary of the self-join's distance matrix, each
    entry the best match above ``threshold`` in its block (pyscamp
    .selfjoin_matrix, python/SCAMP_python.cpp:320-339, 509-526); distances,
    or correlations with pearson=True."""
    o = _parse_matrix_kwargs(kwargs)
    r = join(np.asarray(a, dtype=np.float64), None, int(m), "MATRIX_SUMMARY", o["precision"],
             threshold=o["threshold"], silent=o["silent"], device=o["device"],
             matrix_height=o["mheight"], matrix_width=o["mwidth"])
    return _convert(r["matrix"], o["pearson"], int(m)).astype(np.float32)


def abjoin_matrix(a, b, m, **kwargs):
    """An (mheight, mwidth) summary of the AB-join's distance matrix (rows:
    windows of b, columns: windows of a) (pyscamp.abjoin_matrix,
    python/SCAMP_python.cpp:341-361, 527-548)."""
    o = _parse_matrix_kwargs(kwargs)
    r = join(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), int(m),
             "MATRIX_SUMMARY", o["precision"], computing_rows=False, computing_cols=True,
             threshold=o["threshold"], silent=o["silent"], device=o["device"],
             matrix_height=o["mheight"], matrix_width=o["mwidth"])
    return _convert(r["matrix"], o["pearson"], int(m)).astype(np.float32)


def _split_1nn(packed, pearson, m):
    """SplitProfile1NNINDEX (python/SCAMP_python.cpp:12-29)."""
    corr, _ = unpack_profile(packed)
    idx = (np.asarray(packed, dtype=np.uint64) >> np.uint64(32)).astype(np.uint32).view(np.int32)
    if pearson:
        nn = corr.astype(np.float64)
        nn[nn < -1] = np.nan
    else:
        nn = to_distance(corr, m)
    return nn.astype(np.float32), idx.copy()


def selfjoin(a, m, **kwargs):
    """Matrix profile of series ``a`` with window ``m``: (distances float32,
    indices int32).  Same contract as pyscamp.selfjoin
    (python/SCAMP_python.cpp:196-217, 420-430)."""
    o = _parse_kwargs(kwargs, _NN_KEYS)
    r = join(np.asarray(a, dtype=np.float64), None, int(m), "1NN_INDEX", o["precision"],
             computing_rows=True, computing_cols=True, silent=o["silent"], device=o["device"])
    return _split_1nn(r["profile_a"], o["pearson"], int(m))


def abjoin(a, b, m, **kwargs):
    """For each window of ``a``, its nearest neighbour in ``b``: (distances
    float32, indices into b int32).  Same contract as pyscamp.abjoin
    (python/SCAMP_python.cpp:219-237, 431-444)."""
    o = _parse_kwargs(kwargs, _NN_KEYS)
    r = join(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), int(m),
             "1NN_INDEX", o["precision"], computing_rows=False, computing_cols=True,
             silent=o["silent"], device=o["device"])
    return _split_1nn(r["profile_a"], o["pearson"], int(m))


def _sum_out(v):
    # vec2pyarr with its default pearson=true (python/SCAMP_python.cpp:52-65,
    # 297): values below -1 come back as NaN.
    v = np.array(v, dtype=np.float64)
    v[v < -1] = np.nan
    return v


def selfjoin_sum(a, m, **kwargs):
    """Per window of ``a``, the sum of correlations above ``threshold``
    (default 0) to the other windows of ``a`` (pyscamp.selfjoin_sum,
    python/SCAMP_python.cpp:282-299, 445-458)."""
    o = _parse_kwargs(kwargs, _SUM_KEYS)
    r = join(np.asarray(a, dtype=np.float64), None, int(m), "SUM_THRESH", o["precision"],
             computing_rows=True, computing_cols=True, threshold=o["threshold"],
             silent=o["silent"], device=o["device"])
    return _sum_out(r["sum_a"])


def abjoin_sum(a, b, m, **kwargs):
    """Per window of ``a``, the sum of correlations above ``threshold`` to the
    windows of ``b`` (pyscamp.abjoin_sum, python/SCAMP_python.cpp:301-318,
    459-474)."""
    o = _parse_kwargs(kwargs, _SUM_KEYS)
    r = join(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), int(m),
             "SUM_THRESH", o["precision"], computing_rows=False, computing_cols=True,
             threshold=o["threshold"], silent=o["silent"], device=o["device"])
    return _sum_out(r["sum_a"])
