"""scamp_gb300_join_dev_noalloc through the C ABI: the FP64 join on the
library's static device scratch must give what scamp_gb300_join_dev gives,
call after call, and refuse requests beyond its limits.  Collected last on
purpose (file name): it must pass after the other GPU tests as well as alone
in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _walk(seed, n):
    return np.cumsum(np.random.default_rng(seed).standard_normal(n))


def _call(entry, torch, a, b, m, profile, keep_rows=False, threshold=0.0, precision="double",
          rows=True):
    """Runs one join through `entry` (a C-ABI function taking device
    pointers) on fresh best-so-far buffers; returns host copies."""
    import scamp_gb300
    from scamp_gb300 import _lib

    dev = torch.device("cuda", 0)
    a_d = torch.from_numpy(a).to(dev)
    b_d = torch.from_numpy(b).to(dev) if b is not None else None
    nsa = len(a) - m + 1
    nsb = (len(b) - m + 1) if b is not None else nsa
    nn = profile == "1NN_INDEX"
    no_match = np.array([scamp_gb300.NO_MATCH], dtype=np.uint64).view(np.int64)[0]
    outs = {}
    ca = scamp_gb300._args(None, None, m, profile, precision, rows, True, keep_rows, False,
                           threshold, -1, -1, 128000, 0, 0, True)
    ca.timeseries_a = a_d.data_ptr()
    ca.len_a = len(a)
    if b_d is not None:
        ca.has_b, ca.timeseries_b, ca.len_b = 1, b_d.data_ptr(), len(b)
    res = _lib.CResult()
    for side, ns in (("a", nsa), ("b", nsb)):
        if side == "b" and not keep_rows:
            continue
        if nn:
            t = torch.full((ns,), int(no_match), dtype=torch.int64, device=dev)
            setattr(res, "profile_" + side, t.data_ptr())
        else:
            t = torch.zeros(ns, dtype=torch.float64, device=dev)
            setattr(res, "sum_" + side, t.data_ptr())
        outs[side] = t
    stream = torch.cuda.current_stream(dev)
    err = ctypes.create_string_buffer(512)
    rc = entry(ctypes.byref(ca), ctypes.byref(res), ctypes.c_void_p(stream.cuda_stream), err, 512)
    torch.cuda.synchronize(dev)
    return rc, err.value.decode(), {k: v.cpu().numpy() for k, v in outs.items()}


def _compare(got, ref, nn):
    import scamp_gb300

    for side in ref:
        if nn:
            cg, ig = scamp_gb300.unpack_profile(got[side].view(np.uint64))
            cr, ir = scamp_gb300.unpack_profile(ref[side].view(np.uint64))
            assert np.array_equal(ig >= 0, ir >= 0)
            ok = ir >= 0
            assert np.max(np.abs(cg[ok].astype(np.float64) - cr[ok]), initial=0.0) <= TOL
            assert np.array_equal(ig[ok], ir[ok])
        else:
            assert np.allclose(got[side], ref[side], rtol=TOL, atol=TOL)


CASES = [
    # (seed, len_a, len_b, m, profile, keep_rows, threshold, precision, computing_rows)
    (1, 20000, None, 100, "1NN_INDEX", False, 0.0, "double", True),
    (2, 30000, 20000, 64, "1NN_INDEX", True, 0.0, "double", True),
    (3, 65536, None, 256, "1NN_INDEX", False, 0.0, "double", True),
    (4, 12000, None, 50, "SUM_THRESH", False, 0.5, "double", True),
    (5, 20000, None, 64, "1NN_INDEX", False, 0.0, "ultra", True),
    (6, 15000, 10000, 50, "1NN_INDEX", True, 0.0, "ultra", True),
    # self-joins whose rows go to profile B (keep_rows_separate)
    (7, 18000, None, 80, "1NN_INDEX", True, 0.0, "double", True),
    (8, 16000, None, 40, "1NN_INDEX", True, 0.0, "ultra", True),
    # AB-join sums in both directions
    (9, 14000, 11000, 60, "SUM_THRESH", True, 0.3, "double", True),
    # columns only (pyscamp's abjoin) and a self-join without rows
    (10, 25000, 9000, 70, "1NN_INDEX", False, 0.0, "double", False),
    (11, 12000, None, 32, "1NN_INDEX", False, 0.0, "double", False),
]


def test_noalloc_equals_join_dev_twice(gpu_engine):
    torch = pytest.importorskip("torch")
    from scamp_gb300 import _lib

    lib = _lib.load()
    for seed, la, lb, m, profile, keep, thr, prec, rows in CASES:
        a = _walk(seed, la)
        b = _walk(seed + 100, lb) if lb else None
        rc, msg, ref = _call(lib.scamp_gb300_join_dev, torch, a, b, m, profile, keep, thr, prec,
                             rows)
        assert rc == 0, msg
        for _ in range(2):  # two calls in a row on the same static scratch
            rc, msg, got = _call(lib.scamp_gb300_join_dev_noalloc, torch, a, b, m, profile,
                                 keep, thr, prec, rows)
            assert rc == 0, msg
            _compare(got, ref, profile == "1NN_INDEX")


def test_noalloc_rejects_beyond_limits(gpu_engine):
    torch = pytest.importorskip("torch")
    from scamp_gb300 import _lib

    lib = _lib.load()
    a = _walk(5, 65537)
    rc, msg, _ = _call(lib.scamp_gb300_join_dev_noalloc, torch, a, None, 100, "1NN_INDEX")
    assert rc == 100 and "65536" in msg  # SCAMP_ERR_INVALID_ARGS
