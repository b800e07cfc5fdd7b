"""The C++ do_SCAMP drop-in (include/scamp/SCAMP.h) built and run the way a
reference user would: argument errors and the no-device case throw
SCAMPException (CPU), and a DOUBLE self-join through it equals the Python
front's result bit for bit (GPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, PKG_DIR

SRC = os.path.join(REPO, "tests", "cpp", "shim_demo.cpp")


def _build(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = os.path.join(PKG_DIR, "libscamp_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("engine library not built")
    exe = str(tmp_path / "shim_demo")
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), SRC,
                           "-o", exe, "-L", PKG_DIR, "-lscamp_gb300",
                           "-Wl,-rpath," + PKG_DIR])
    return exe


def test_shim_errors(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe, "errors"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK")


def test_shim_utils_match_the_cli_writers(tmp_path):
    """scamp/scamp_utils.h (the reference's utility functions for callers
    of do_SCAMP) reads series and writes every profile type exactly as the
    Python command line does, with and without output_pearson."""
    import scamp_gb300
    from scamp_gb300 import cli

    exe = _build(tmp_path)
    rng = np.random.default_rng(4)
    m, k, h, w = 16, 3, 4, 5
    corr = rng.uniform(-1, 1, 40).astype(np.float32)
    corr[[3, 17]] = -2.0
    idx = rng.integers(0, 1000, 40).astype(np.uint64)
    idx[[3, 17]] = 0xFFFFFFFF
    packed = (idx << np.uint64(32)) | corr.view(np.uint32).astype(np.uint64)
    packed.tofile(tmp_path / "nn_index.bin")
    corr.tofile(tmp_path / "nn.bin")
    sums = rng.uniform(0, 50, 40)
    sums.tofile(tmp_path / "sum.bin")
    knn = packed[:36].copy()  # 12 windows x 3 entries
    knn.tofile(tmp_path / "knn.bin")
    mat = rng.uniform(-1, 1, h * w).astype(np.float32)
    mat[7] = -2.0
    mat.tofile(tmp_path / "matrix.bin")
    series = "1.5\n-2e3\n0.25\n  7\n\n3.125\n9"  # last value: no newline after it
    (tmp_path / "in.txt").write_text(series)
    out = subprocess.run([exe, "utils", str(tmp_path)], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().startswith("OK")
    got = np.fromfile(tmp_path / "read.bin", dtype=np.float64)
    assert np.array_equal(got, np.array(cli.read_series(str(tmp_path / "in.txt"))))
    assert len(got) == 5
    py = tmp_path / "py"
    py.mkdir()
    for pearson in (False, True):
        s = "_pearson" if pearson else ""
        cli.write_profile(str(py / "a.txt"), str(py / "ai.txt"), packed, pearson, m)
        cli.write_max_profile(str(py / "b.txt"), corr, pearson, m)
        cli.write_knn(str(py / "c.txt"), knn, k, pearson, m)
        cli.write_matrix(str(py / "d.txt"), mat.reshape(h, w), pearson, m)
        for mine, theirs in (("a", "out_nn_index"), ("ai", "out_nn_index_i"), ("b", "out_nn"),
                             ("c", "out_knn"), ("d", "out_matrix")):
            assert (py / (mine + ".txt")).read_text() == \
                (tmp_path / (theirs + s + ".txt")).read_text(), (mine, pearson)
    cli.write_sums(str(py / "e.txt"), sums)
    assert (py / "e.txt").read_text() == (tmp_path / "out_sum.txt").read_text()
    assert scamp_gb300.NO_MATCH  # the package imported (engine library present)


@pytest.mark.gpu
def test_shim_selfjoin_matches_python(tmp_path, gpu_engine):
    import scamp_gb300

    exe = _build(tmp_path)
    rng = np.random.default_rng(11)
    x = np.cumsum(rng.standard_normal(3000))
    src = tmp_path / "x.bin"
    dst = tmp_path / "p.bin"
    x.astype(np.float64).tofile(src)
    out = subprocess.run([exe, "join", str(src), str(dst), "64"], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    got = np.fromfile(dst, dtype=np.uint64)
    ref = scamp_gb300.join(x, None, 64, "1NN_INDEX", "double")["profile_a"]
    assert np.array_equal(got, ref)
