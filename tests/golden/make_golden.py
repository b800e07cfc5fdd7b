"""Generates tests/golden/*.npz from the reference's own CPU path.

Run where the reference tree exists (it builds oracle/_ref/libscampref.so
from the reference's sources with oracle/Makefile):
    make -C oracle ref && python tests/golden/make_golden.py [fixture names]
Each fixture holds seeded inputs, the join options and the reference's
output (packed 1NN_INDEX entries, SUM_THRESH sums or 1NN float profiles;
DOUBLE precision, one thread, the pyscamp default max_tile_size of 128000
unless stated).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle  # noqa: E402


def cases():
    rng = np.random.default_rng(20261203)
    rw = lambda n: np.cumsum(rng.standard_normal(n))  # noqa: E731
    out = []
    out.append(("self_rw4000_m100", rw(4000), None, 100, {}))
    a = rw(3000)
    a[rng.choice(3000, 12, replace=False)] = np.nan
    a[1200:1300] = 2.0
    out.append(("self_nanflat3000_m64", a, None, 64, {}))
    out.append(("self_randn20_m5", rng.standard_normal(20), None, 5, {}))
    a, b = rw(3000), rw(2000)
    b[rng.choice(2000, 6, replace=False)] = np.nan
    out.append(("ab_keep_rows_m50", a, b, 50, {"keep_rows": True}))
    out.append(("ab_cols_m50", a, b, 50, {"computing_rows": False}))
    c = rw(2500)
    out.append(("ab_aligned_m100", c, c.copy(), 100, {"aligned": True, "computing_rows": False}))
    out.append(("self_tiles1024_m64", rw(5000), None, 64, {"max_tile_size": 1024}))
    out.append(("sum_self_t05_m64", rw(2500), None, 64, {"profile": "SUM_THRESH", "threshold": 0.5}))
    out.append(("sum_ab_keep_t025_m32", rw(2000), rw(1500), 32,
                {"profile": "SUM_THRESH", "threshold": 0.25, "keep_rows": True}))
    # ULTRA precision (the reference's SCAMPPrecisionType 4): brute-force
    # statistics and combined update terms
    out.append(("ultra_self_rw3000_m64", rw(3000), None, 64, {"precision": 4}))
    out.append(("ultra_ab_keep_offset_m50", 1e4 + rw(2500), 1e4 + rw(1800), 50,
                {"precision": 4, "keep_rows": True}))
    # PROFILE_TYPE_1NN: the best correlation per window, float32, no index
    out.append(("nn_self_rw3000_m64", rw(3000), None, 64, {"profile": "1NN"}))
    out.append(("nn_ab_keep_m40", rw(2000), rw(1500), 40, {"profile": "1NN", "keep_rows": True}))
    # distributed self-join pieces (--global_row / --global_col): aligned
    # AB-joins of tiles of one series, W = 1500 windows each, placed at
    # multiples of W; the trivial-match zone touches a corner of the
    # off-diagonal tiles and runs along the main diagonal of the diagonal ones
    x = rw(4600)
    W, mm = 1500, 64
    tile = lambda k: x[k * W:(k + 1) * W + mm - 1].copy()  # noqa: E731
    out.append(("ab_dist_tile10_m64", tile(0), tile(1), mm,
                {"aligned": True, "keep_rows": True, "start_row": W, "start_col": 0}))
    out.append(("ab_dist_tile01_m64", tile(1), tile(0), mm,
                {"aligned": True, "keep_rows": True, "start_row": 0, "start_col": W}))
    out.append(("ab_dist_tile22_m64", tile(2)[:W], tile(2)[:W], mm,
                {"aligned": True, "keep_rows": True, "start_row": 2 * W, "start_col": 2 * W}))
    out.append(("sum_ab_dist_tile10_t06_m64", tile(0), tile(1), mm,
                {"profile": "SUM_THRESH", "threshold": 0.6, "aligned": True, "keep_rows": True,
                 "start_row": W, "start_col": 0}))
    return out


def main(only=()):
    if not oracle.ref_available():
        raise SystemExit("build the reference first: make -C oracle ref")
    for name, a, b, m, kw in cases():
        if only and name not in only:
            continue
        res = oracle.ref_join(a, b, m, threads=1, **kw)
        data = {"a": a, "m": np.int64(m)}
        if b is not None:
            data["b"] = b
        for k, v in kw.items():
            if k == "max_tile_size":
                continue  # the oracle is tile-free; the fixture still pins it
            data["kw_" + k] = np.array(v)
        data.update(res)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1:])
