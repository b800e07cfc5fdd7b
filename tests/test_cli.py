"""The command line (scamp_gb300.cli) against the reference CLI's behaviour
(src/main.cpp, src/scamp_utils.cpp): flags, input parsing quirks, output
files, error exits; and on the GPU, the files it writes for a golden input."""
import os

import numpy as np
import pytest

from scamp_gb300 import cli


def test_flags_gflags_style():
    f = cli.parse_flags(["--window=100", "--input_a_file_name", "a.txt", "--keep_rows",
                         "--nooutput_pearson", "--threshold=0.5", "--mixed_precision=true"])
    assert f["window"] == 100 and f["input_a_file_name"] == "a.txt"
    assert f["keep_rows"] is True and f["output_pearson"] is False
    assert f["threshold"] == 0.5 and f["mixed_precision"] is True
    with pytest.raises(cli.UsageError):
        cli.parse_flags(["--no_such_flag=1"])
    with pytest.raises(cli.UsageError):
        cli.parse_flags(["--window=abc"])


def test_read_series_quirks(tmp_path):
    p = tmp_path / "x.txt"
    p.write_text("1\n2.5\nnan\n-4e-3\n")
    x = cli.read_series(str(p))
    assert x.shape == (4,) and np.isnan(x[2]) and x[3] == -4e-3
    p.write_text("1\n2\n3")  # no trailing newline: the last value is dropped
    assert cli.read_series(str(p)).tolist() == [1.0, 2.0]
    p.write_text("1\nabc\n")
    with pytest.raises(cli.UsageError):
        cli.read_series(str(p))


def test_write_profile_format(tmp_path):
    import scamp_gb300

    r = np.array([0.5, -2.0, 1.0], dtype=np.float32)
    idx = np.array([7, 0xFFFFFFFF, 3], dtype=np.uint64)
    packed = (idx << np.uint64(32)) | r.view(np.uint32).astype(np.uint64)
    mp, mpi = tmp_path / "mp", tmp_path / "mpi"
    cli.write_profile(str(mp), str(mpi), packed, False, 10)
    assert mp.read_text().split() == [format(np.sqrt(10.0), ".10g"), "nan", "0"]
    assert mpi.read_text().split() == ["7", "-1", "3"]
    cli.write_profile(str(mp), str(mpi), packed, True, 10)
    assert mp.read_text().split() == ["0.5", "nan", "1"]
    assert scamp_gb300.NO_MATCH  # the package imports without a GPU


def test_write_max_profile_format(tmp_path):
    mp = tmp_path / "mp"
    cli.write_max_profile(str(mp), np.array([0.5, -2.0, 1.0], dtype=np.float32), False, 10)
    assert mp.read_text().split() == [format(np.sqrt(10.0), ".10g"), "nan", "0"]
    cli.write_max_profile(str(mp), np.array([0.5, -2.0, 1.0], dtype=np.float32), True, 10)
    assert mp.read_text().split() == ["0.5", "nan", "1"]


@pytest.mark.parametrize("argv,msg", [
    (["--window=2", "--input_a_file_name=x"], "Subsequence length must be at least 3"),
    (["--window=10"], "primary input filename"),
    (["--window=10", "--input_a_file_name=x", "--mixed_precision", "--double_precision"],
     "only one precision flag"),
    (["--window=10", "--max_tile_size=100", "--input_a_file_name=x"], "at least 1024"),
])
def test_cli_errors(capsys, argv, msg):
    assert cli.main(argv) == 1
    assert msg in capsys.readouterr().out


@pytest.mark.gpu
def test_cli_golden_selfjoin(gpu_engine, tmp_path):
    here = os.path.dirname(os.path.abspath(__file__))
    g = np.load(os.path.join(here, "golden", "self_rw4000_m100.npz"))
    a, m = g["a"], int(g["m"])
    src = tmp_path / "a.txt"
    src.write_text("".join(repr(float(v)) + "\n" for v in a))
    mp, mpi = tmp_path / "mp", tmp_path / "mpi"
    assert cli.main(["--window=%d" % m, "--input_a_file_name=%s" % src,
                     "--output_a_file_name=%s" % mp, "--output_a_index_file_name=%s" % mpi]) == 0
    got_d = np.array([float(v) for v in mp.read_text().split()])
    got_i = np.array([int(v) for v in mpi.read_text().split()])
    corr, idx = gpu_engine.unpack_profile(g["packed_a"])
    want_d = gpu_engine.to_distance(corr, m)
    ok = ~np.isnan(want_d)
    assert np.array_equal(ok, ~np.isnan(got_d))
    # the reference's own regression tolerance (test/difference.py: 0.01)
    assert np.max(np.abs(got_d[ok] - want_d[ok])) < 1e-3
    assert np.mean(got_i[ok] != idx[ok]) <= 0.01


@pytest.mark.gpu
def test_cli_abjoin_keep_rows(gpu_engine, tmp_path):
    rng = np.random.default_rng(5)
    a, b = np.cumsum(rng.standard_normal(3000)), np.cumsum(rng.standard_normal(2000))
    fa, fb = tmp_path / "a.txt", tmp_path / "b.txt"
    fa.write_text("".join(repr(float(v)) + "\n" for v in a))
    fb.write_text("".join(repr(float(v)) + "\n" for v in b))
    out = {k: tmp_path / k for k in ("ma", "ia", "mb", "ib")}
    assert cli.main(["--window=64", "--input_a_file_name=%s" % fa, "--input_b_file_name=%s" % fb,
                     "--keep_rows", "--output_pearson", "--mixed_precision",
                     "--output_a_file_name=%s" % out["ma"], "--output_a_index_file_name=%s" % out["ia"],
                     "--output_b_file_name=%s" % out["mb"], "--output_b_index_file_name=%s" % out["ib"]]) == 0
    r = gpu_engine.join(a, b, 64, "1NN_INDEX", "mixed", keep_rows=True)
    for side, mk, ik in (("a", "ma", "ia"), ("b", "mb", "ib")):
        c, i = gpu_engine.unpack_profile(r["profile_" + side])
        got_c = np.array([float(v) for v in out[mk].read_text().split()])
        got_i = np.array([int(v) for v in out[ik].read_text().split()])
        assert np.array_equal(got_i, i)
        ok = c >= -1
        assert np.allclose(got_c[ok], c[ok], rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_cli_profile_type_1nn(gpu_engine, tmp_path):
    rng = np.random.default_rng(6)
    a = np.cumsum(rng.standard_normal(3000))
    fa = tmp_path / "a.txt"
    fa.write_text("".join(repr(float(v)) + "\n" for v in a) + "\n")
    mp = tmp_path / "mp"
    assert cli.main(["--window=50", "--input_a_file_name=%s" % fa, "--profile_type=1NN",
                     "--output_pearson", "--output_a_file_name=%s" % mp]) == 0
    got = np.array([float(v) for v in mp.read_text().split()])
    r = gpu_engine.join(a, None, 50, "1NN_INDEX", "double")
    c, _ = gpu_engine.unpack_profile(r["profile_a"])
    assert np.max(np.abs(got - c.astype(np.float64))) < 1e-8


@pytest.mark.gpu
def test_cli_all_neighbors_and_matrix(gpu_engine, tmp_path):
    rng = np.random.default_rng(7)
    a = np.cumsum(rng.standard_normal(2000))
    fa = tmp_path / "a.txt"
    fa.write_text("".join(repr(float(v)) + "\n" for v in a))
    kf, mf = tmp_path / "knn", tmp_path / "mat"
    assert cli.main(["--window=32", "--input_a_file_name=%s" % fa,
                     "--profile_type=ALL_NEIGHBORS", "--max_matches_per_column=3",
                     "--output_pearson", "--output_a_file_name=%s" % kf]) == 0
    r = gpu_engine.join(a, None, 32, "ALL_NEIGHBORS", "double", max_matches=3)
    corr, idx = gpu_engine.unpack_profile(r["knn_a"])
    lines = [l.split() for l in kf.read_text().splitlines()]
    assert len(lines) == int(np.sum(idx >= 0))
    ok = np.nonzero(idx >= 0)[0]
    for (c, i, v), e in zip(lines[:50], ok[:50]):
        assert int(c) == e // 3 and int(i) == idx[e] and abs(float(v) - corr[e]) < 1e-6
    assert cli.main(["--window=32", "--input_a_file_name=%s" % fa,
                     "--profile_type=MATRIX_SUMMARY", "--reduced_height=4", "--reduced_width=6",
                     "--output_pearson", "--output_a_file_name=%s" % mf]) == 0
    r = gpu_engine.join(a, None, 32, "MATRIX_SUMMARY", "double", matrix_height=4,
                        matrix_width=6)
    rows = [[float(v) for v in l.split()] for l in mf.read_text().splitlines()]
    got = np.array(rows)
    assert got.shape == (4, 6)
    want = np.where(r["matrix"] < -1, np.nan, r["matrix"])
    np.testing.assert_allclose(got, want, atol=1e-6)
