"""ctypes front of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference legs import this module.  The engine never does.

``join`` runs oracle/scamp_oracle.c (a C restatement of the reference CPU
path that keeps correlations in double); ``ref_join`` runs the reference's own
CPU path compiled from its sources (oracle/_ref/libscampref.so), which exists
only where the reference tree was present at build time.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libscampref.so")

PROFILE_1NN_INDEX = 1
PROFILE_SUM_THRESH = 2
PROFILE_1NN = 6
_PROFILE = {"1NN_INDEX": PROFILE_1NN_INDEX, "SUM_THRESH": PROFILE_SUM_THRESH,
            "1NN": PROFILE_1NN}

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class _Args(ctypes.Structure):
    _fields_ = [
        ("a", _dp), ("na", ctypes.c_int64),
        ("b", _dp), ("nb", ctypes.c_int64),
        ("m", ctypes.c_int64),
        ("profile_type", ctypes.c_int),
        ("computing_rows", ctypes.c_int),
        ("computing_cols", ctypes.c_int),
        ("keep_rows_separate", ctypes.c_int),
        ("is_aligned", ctypes.c_int),
        ("start_row", ctypes.c_int64),
        ("start_col", ctypes.c_int64),
        ("threshold", ctypes.c_double),
        ("threads", ctypes.c_int),
        ("brute_force", ctypes.c_int),
        ("high_precision_stats", ctypes.c_int),
        ("exact_flat", ctypes.c_int),
        ("combined_terms", ctypes.c_int),
    ]


class _Out(ctypes.Structure):
    _fields_ = [
        ("corr_a", _dp), ("idx_a", _i64p), ("sum_a", _dp),
        ("corr_b", _dp), ("idx_b", _i64p), ("sum_b", _dp),
    ]


_lib = None
_ref = None


def build():
    """Compile liboracle.so with the committed Makefile (portable C, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        lib.oracle_join.argtypes = [ctypes.POINTER(_Args), ctypes.POINTER(_Out)]
        lib.oracle_join.restype = ctypes.c_int
        lib.oracle_pack.argtypes = [_dp, _i64p, ctypes.c_int64, _u64p]
        lib.oracle_clean.argtypes = [_dp, ctypes.c_int64, ctypes.c_int64, _dp, _u8p]
        lib.oracle_stats.argtypes = [_dp, _u8p, ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_int, _dp, _dp, _dp, _dp]
        lib.oracle_qt_row.argtypes = [_dp, _dp, ctypes.c_int64, ctypes.c_int64, _dp]
        lib.oracle_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _ptr(arr, typ):
    return arr.ctypes.data_as(typ) if arr is not None else None


def max_threads():
    return load().oracle_max_threads()


def stats(T, m, high_precision=False):
    """Cleaned series, NaN-window flags, means, inverse norms, df, dg."""
    lib = load()
    T = np.ascontiguousarray(T, dtype=np.float64)
    n = len(T)
    ns = n - m + 1
    Tc = np.empty(n)
    nanwin = np.empty(ns, dtype=np.uint8)
    lib.oracle_clean(_ptr(T, _dp), n, m, _ptr(Tc, _dp), _ptr(nanwin, _u8p))
    mu, inv, df, dg = (np.empty(ns) for _ in range(4))
    lib.oracle_stats(_ptr(Tc, _dp), _ptr(nanwin, _u8p), n, m, int(high_precision),
                     _ptr(mu, _dp), _ptr(inv, _dp), _ptr(df, _dp), _ptr(dg, _dp))
    return dict(clean=Tc, nanwin=nanwin.astype(bool), mean=mu, invnorm=inv, df=df, dg=dg)


def qt_row(T, Q, count, m):
    lib = load()
    T = np.ascontiguousarray(T, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    out = np.empty(count)
    lib.oracle_qt_row(_ptr(T, _dp), _ptr(Q, _dp), count, m, _ptr(out, _dp))
    return out


def pack(corr, idx):
    """Reference 1NN_INDEX layout: float32 corr low word, uint32 index high."""
    corr = np.ascontiguousarray(corr, dtype=np.float64)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(len(corr), dtype=np.uint64)
    load().oracle_pack(_ptr(corr, _dp), _ptr(idx, _i64p), len(corr), _ptr(out, _u64p))
    return out


def join(a, b=None, m=None, profile="1NN_INDEX", computing_rows=True,
         computing_cols=True, keep_rows=False, aligned=False, start_row=-1,
         start_col=-1, threshold=0.0, threads=0, brute=False,
         high_precision_stats=False, exact_flat=False, precision=3):
    """Matrix-profile join on the CPU oracle.

    ``precision`` takes the reference's SCAMPPrecisionType values; 4 (ULTRA)
    selects its brute-force statistics and combined update terms
    (src/SCAMP.cpp:200-212), any other value the DOUBLE path.

    Returns a dict with, per profile side that is produced, ``corr_*``
    (double, -2 where no match), ``idx_*`` (int64, -1 where no match),
    ``packed_*`` (reference uint64 layout) for 1NN_INDEX, or ``sum_*``.
    """
    if profile == "1NN":
        # the reference's PROFILE_TYPE_1NN: each window's best correlation as
        # float32, -2 where none (the 1NN_INDEX search without the index)
        r = join(a, b, m, "1NN_INDEX", computing_rows, computing_cols, keep_rows, aligned,
                 start_row, start_col, threshold, threads, brute, high_precision_stats,
                 exact_flat, precision)
        r["max_a"] = r["corr_a"].astype(np.float32)
        if keep_rows:
            r["max_b"] = r["corr_b"].astype(np.float32)
        return r
    lib = load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    has_b = b is not None
    if has_b:
        b = np.ascontiguousarray(b, dtype=np.float64)
    ptype = _PROFILE[profile]
    nsa = len(a) - m + 1
    nsb = (len(b) if has_b else len(a)) - m + 1
    args = _Args(_ptr(a, _dp), len(a), _ptr(b, _dp) if has_b else None,
                 len(b) if has_b else 0, m, ptype, int(computing_rows),
                 int(computing_cols), int(keep_rows), int(aligned), start_row,
                 start_col, float(threshold), int(threads), int(brute),
                 int(high_precision_stats or precision == 4), int(exact_flat),
                 int(precision == 4))
    res = {}
    out = _Out()
    if ptype == PROFILE_1NN_INDEX:
        res["corr_a"], res["idx_a"] = np.empty(nsa), np.empty(nsa, dtype=np.int64)
        out.corr_a, out.idx_a = _ptr(res["corr_a"], _dp), _ptr(res["idx_a"], _i64p)
        if keep_rows:
            res["corr_b"], res["idx_b"] = np.empty(nsb), np.empty(nsb, dtype=np.int64)
            out.corr_b, out.idx_b = _ptr(res["corr_b"], _dp), _ptr(res["idx_b"], _i64p)
    else:
        res["sum_a"] = np.empty(nsa)
        out.sum_a = _ptr(res["sum_a"], _dp)
        if keep_rows:
            res["sum_b"] = np.empty(nsb)
            out.sum_b = _ptr(res["sum_b"], _dp)
    rc = lib.oracle_join(ctypes.byref(args), ctypes.byref(out))
    if rc != 0:
        raise RuntimeError("oracle_join failed with code %d" % rc)
    if ptype == PROFILE_1NN_INDEX:
        res["packed_a"] = pack(res["corr_a"], res["idx_a"])
        if keep_rows:
            res["packed_b"] = pack(res["corr_b"], res["idx_b"])
    return res


def ref_available():
    return os.path.exists(REF_PATH)


def _load_ref():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_PATH)
        lib.ref_scamp_join.argtypes = [
            _dp, ctypes.c_uint64, _dp, ctypes.c_uint64, ctypes.c_int,
            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_int,
            _u64p, _u64p, _dp, _dp, ctypes.c_char_p, ctypes.c_uint64]
        lib.ref_scamp_join.restype = ctypes.c_int
        _ref = lib
    return _ref


def ref_join(a, b=None, m=None, profile="1NN_INDEX", computing_rows=True,
             computing_cols=True, keep_rows=False, aligned=False, start_row=-1,
             start_col=-1, threshold=0.0, threads=1, max_tile_size=128000,
             precision=3):
    """Run the reference's own CPU path (DOUBLE precision by default)."""
    lib = _load_ref()
    a = np.ascontiguousarray(a, dtype=np.float64)
    has_b = b is not None
    bb = np.ascontiguousarray(b, dtype=np.float64) if has_b else a
    nsa = len(a) - m + 1
    nsb = len(bb) - m + 1
    ptype = _PROFILE[profile]
    pa = np.empty(nsa, dtype=np.uint64)
    pb = np.empty(nsb, dtype=np.uint64)
    sa = np.empty(nsa)
    sb = np.empty(nsb)
    err = ctypes.create_string_buffer(512)
    rc = lib.ref_scamp_join(_ptr(a, _dp), len(a), _ptr(bb, _dp), len(bb),
                            int(has_b), m, max_tile_size, ptype, precision,
                            int(computing_rows), int(computing_cols),
                            int(keep_rows), int(aligned), start_row, start_col,
                            float(threshold), int(threads), _ptr(pa, _u64p),
                            _ptr(pb, _u64p), _ptr(sa, _dp), _ptr(sb, _dp), err, 512)
    if rc != 0:
        raise RuntimeError("reference join failed: " + err.value.decode())
    if ptype == PROFILE_1NN_INDEX:
        res = {"packed_a": pa}
        if keep_rows:
            res["packed_b"] = pb
    elif ptype == PROFILE_1NN:
        res = {"max_a": sa.astype(np.float32)}
        if keep_rows:
            res["max_b"] = sb.astype(np.float32)
    else:
        res = {"sum_a": sa}
        if keep_rows:
            res["sum_b"] = sb
    return res


def unpack(packed):
    """Split reference-layout uint64 entries into (float32 corr, int64 index),
    index -1 / corr -2 where no match (src/scamp_utils.cpp:160-167)."""
    packed = np.asarray(packed, dtype=np.uint64)
    corr = (packed & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.float32)
    idx = (packed >> np.uint64(32)).astype(np.int64)
    idx[corr < -1] = -1
    return corr, idx


def to_distance(corr, m):
    """ConvertToEuclidean, src/scamp_utils.cpp:127-133."""
    corr = np.asarray(corr, dtype=np.float64)
    out = np.sqrt(np.maximum(2.0 * m * (1.0 - corr), 0.0))
    out[corr < -1] = np.nan
    return out
