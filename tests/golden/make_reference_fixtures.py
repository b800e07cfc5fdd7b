"""Builds the fixtures of the reference's own test data (test infrastructure).

Reads, from the reference tree named by SCAMP_REFERENCE_TREE:
  * its sample inputs (test/SampleInput): the random walks of its golden
    tests (randomwalk8K/16K/32K/64K/64K_nan, test/run_tests.sh:11-13), its
    static stress inputs (randomwalk1K_nan, poorly_conditioned_test,
    test/run_tests.py:12) and the series its documentation names as the one
    that breaks reduced precision (earthquake_precision_test100K,
    docs/source/cli.rst:127);
  * its golden outputs (test/SampleOutput/mp_*_w100.txt, mpi_*_w100.txt):
    distance and index profiles of the self-joins and of the AB-joins
    16K x 32K and 32K x 16K;
and writes them to tests/golden/reference_data/{inputs,goldens}.npz.

It also runs the reference's own CPU path, compiled from its sources
(oracle/_ref/libscampref.so, `make -C oracle ref REF_DIR=...`), on the
stress inputs and the earthquake series and stores those outputs in
tests/golden/reference_data/compiled.npz: packed 1NN_INDEX profiles (the
reference's mp_entry layout) at every window test/run_tests.py:13 tests,
SUM_THRESH at its thresholds (:16), and the earthquake series at windows
100 and 1000.

Run:  SCAMP_REFERENCE_TREE=<tree> python tests/golden/make_reference_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "reference_data")

GOLDEN_SELF = ["randomwalk8K", "randomwalk16K", "randomwalk32K", "randomwalk64K",
               "randomwalk64K_nan"]
GOLDEN_AB = [("randomwalk16K", "randomwalk32K"), ("randomwalk32K", "randomwalk16K")]
STATIC = ["randomwalk1K_nan", "poorly_conditioned_test"]
EARTHQUAKE = "earthquake_precision_test100K"
STATIC_WINDOWS = [5, 7, 13, 25, 33, 78, 92, 100, 189, 339, 500]   # test/run_tests.py:13
STATIC_THRESHOLDS = [0.0, 0.125, 0.5]                            # test/run_tests.py:16
EARTHQUAKE_WINDOWS = [100, 1000]


def main():
    tree = os.environ.get("SCAMP_REFERENCE_TREE", "")
    if not tree or not os.path.isdir(os.path.join(tree, "test")):
        sys.exit("set SCAMP_REFERENCE_TREE to the reference tree")
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    oracle.load()
    if not oracle.ref_available():
        sys.exit("build the compiled reference first: make -C oracle ref REF_DIR=<tree>")
    inp = os.path.join(tree, "test", "SampleInput")
    outp = os.path.join(tree, "test", "SampleOutput")
    os.makedirs(OUT, exist_ok=True)

    inputs = {}
    for name in GOLDEN_SELF + STATIC + [EARTHQUAKE]:
        inputs[name] = np.loadtxt(os.path.join(inp, name + ".txt"), dtype=np.float64)
    np.savez_compressed(os.path.join(OUT, "inputs.npz"), **inputs)

    goldens = {}
    for name in GOLDEN_SELF + ["%s_%s" % ab for ab in GOLDEN_AB]:
        # distances as float32: the reference computes them from float32
        # correlations, and its tests compare them to 0.01
        goldens["mp_" + name] = np.loadtxt(os.path.join(outp, "mp_%s_w100.txt" % name)).astype(np.float32)
        goldens["mpi_" + name] = np.loadtxt(os.path.join(outp, "mpi_%s_w100.txt" % name)).astype(np.int32)
    np.savez_compressed(os.path.join(OUT, "goldens.npz"), **goldens)

    compiled = {}
    threads = max(1, os.cpu_count() or 1)
    for name in STATIC:
        x = inputs[name]
        for m in STATIC_WINDOWS:
            if m > len(x) // 2:
                continue
            r = oracle.ref_join(x, None, m, threads=threads)
            compiled["%s_m%d_1nn" % (name, m)] = r["packed_a"]
            for thr in STATIC_THRESHOLDS:
                s = oracle.ref_join(x, None, m, profile="SUM_THRESH", threshold=thr, threads=threads)
                compiled["%s_m%d_sum%g" % (name, m, thr)] = s["sum_a"]
    for m in EARTHQUAKE_WINDOWS:
        r = oracle.ref_join(inputs[EARTHQUAKE], None, m, threads=threads)
        compiled["%s_m%d_1nn" % (EARTHQUAKE, m)] = r["packed_a"]
    np.savez_compressed(os.path.join(OUT, "compiled.npz"), **compiled)
    for f in sorted(os.listdir(OUT)):
        print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
