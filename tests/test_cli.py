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


# ---------------------------------------------------------------------------
# The native command-line program (scamp_gb300/scamp, built from
# gpu-scrimp-large_gb300/cli/scamp_main.cpp) behaves as the Python one.
# ---------------------------------------------------------------------------
def _native():
    from conftest import PKG_DIR

    exe = os.path.join(PKG_DIR, "scamp")
    if not os.path.exists(exe):
        pytest.skip("native command line not built")
    return exe


def _both(argv, capsys):
    import subprocess

    rc_py = cli.main(list(argv))
    out_py = capsys.readouterr().out
    p = subprocess.run([_native()] + list(argv), capture_output=True, text=True, timeout=120)
    return (rc_py, out_py), (p.returncode, p.stdout)


def test_read_series_tokens_as_the_reference(tmp_path):
    """Tokens parse as std::stod does: the longest numeric prefix, hex and
    inf/nan forms; no number, or one out of range, is fatal."""
    p = tmp_path / "x.txt"
    p.write_text("1.5\n2x\n0x10\ninf\n-nan\n3e2\n7\n")
    x = cli.read_series(str(p))
    assert x[:4].tolist() == [1.5, 2.0, 16.0, float("inf")] and np.isnan(x[4])
    assert x[5:].tolist() == [300.0, 7.0]
    for text, what in (("1\nabc\n2\n", "a\nFATAL ERROR: invalid argument: Could not parse "
                        "line number 2"),
                       ("1\n1e400\n2\n", "1\nFATAL ERROR: out of range: Could not parse "
                        "line number 2")):
        p.write_text(text)
        with pytest.raises(cli.UsageError, match=what):
            cli.read_series(str(p))


@pytest.mark.parametrize("argv", [
    ["--window=2", "--input_a_file_name=x"],
    ["--window=10"],
    ["--window=10", "--input_a_file_name=x", "--mixed_precision", "--double_precision"],
    ["--window=10", "--max_tile_size=100", "--input_a_file_name=x"],
    ["--window=10", "--max_tile_size=1024", "--input_a_file_name=x", "--window=600"],
    ["--window=abc"],
    ["--threshold=0.5x"],
    ["--no_such_flag=1"],
    ["--window"],
    ["stray"],
    ["--window=10", "--input_a_file_name=x", "--no_gpu"],
    ["--window=10", "--input_a_file_name=x", "--profile_type=FREQUENCY_THRESH"],
    ["--window=10", "--input_a_file_name=/nonexistent/a.txt"],
])
def test_native_cli_errors_match_python(capsys, argv):
    (rc_py, out_py), (rc_c, out_c) = _both(argv, capsys)
    assert rc_py == rc_c == 1
    assert out_py == out_c


def test_native_cli_input_errors_match_python(capsys, tmp_path):
    f = tmp_path / "a.txt"
    for text in ("1\n2\nabc\n3\n", "1\n1e999\n2\n", "1\n2\n3"):
        f.write_text(text)
        (rc_py, out_py), (rc_c, out_c) = _both(["--window=3", "--input_a_file_name=%s" % f],
                                                capsys)
        assert rc_py == rc_c == 1
        assert out_py == out_c


@pytest.mark.gpu
@pytest.mark.parametrize("extra", [
    [],
    ["--keep_rows", "--output_pearson"],
    ["--profile_type=SUM_THRESH", "--threshold=0.6", "--keep_rows"],
    ["--profile_type=1NN", "--keep_rows"],
    ["--profile_type=ALL_NEIGHBORS", "--max_matches_per_column=3", "--keep_rows"],
    ["--profile_type=MATRIX_SUMMARY", "--reduced_height=5", "--reduced_width=7"],
])
def test_native_cli_files_match_python(gpu_engine, capsys, tmp_path, extra):
    """Same flags, same FP64 join: byte-identical output files (sums, whose
    FP64 atomic additions run in any order, to 1e-12)."""
    import subprocess

    rng = np.random.default_rng(8)
    fa, fb = tmp_path / "a.txt", tmp_path / "b.txt"
    fa.write_text("".join(repr(float(v)) + "\n" for v in np.cumsum(rng.standard_normal(2500))))
    fb.write_text("".join(repr(float(v)) + "\n" for v in np.cumsum(rng.standard_normal(1800))))
    outs = {}
    for who in ("py", "c"):
        d = tmp_path / who
        d.mkdir()
        argv = ["--window=48", "--input_a_file_name=%s" % fa, "--input_b_file_name=%s" % fb,
                "--double_precision"] + extra + [
            "--output_a_file_name=%s" % (d / "ma"), "--output_a_index_file_name=%s" % (d / "ia"),
            "--output_b_file_name=%s" % (d / "mb"), "--output_b_index_file_name=%s" % (d / "ib")]
        if who == "py":
            assert cli.main(argv) == 0
        else:
            p = subprocess.run([_native()] + argv, capture_output=True, text=True, timeout=300)
            assert p.returncode == 0, p.stdout + p.stderr
        outs[who] = {f: (d / f).read_bytes() for f in sorted(os.listdir(d))}
    assert outs["py"].keys() == outs["c"].keys() and outs["py"]
    for f in outs["py"]:
        if "SUM_THRESH" in " ".join(extra):
            a = np.array(outs["py"][f].split(), dtype=np.float64)
            b = np.array(outs["c"][f].split(), dtype=np.float64)
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12)
        else:
            assert outs["py"][f] == outs["c"][f], f


@pytest.mark.parametrize("seed", range(60))
def test_native_cli_matches_python_randomized(capsys, tmp_path, seed):
    """Seeded random command lines (valid and invalid flags and values,
    gflags spellings, inputs good and bad): without a GPU every run ends in
    a message, and the two programs print the same one with the same exit
    status."""
    from scamp_gb300 import gpu_supported

    if gpu_supported():
        pytest.skip("compares the paths that end before the join")
    rng = np.random.default_rng(seed)
    good = tmp_path / "good.txt"
    good.write_text("".join("%r\n" % float(v) for v in np.cumsum(rng.standard_normal(300))))
    short = tmp_path / "short.txt"
    short.write_text("1\n2\n3\n")
    bad = tmp_path / "bad.txt"
    bad.write_text("1\n2\nzz\n")
    values = {
        "window": ["10", "2", "abc", "600", "-5", " 12"],
        "max_tile_size": ["1024", "100", "131072", "1e3"],
        "threshold": ["0.5", "x", "-0.25", "1e-3"],
        "profile_type": ["1NN_INDEX", "SUM_THRESH", "1NN", "ALL_NEIGHBORS", "MATRIX_SUMMARY",
                         "KNN"],
        "input_a_file_name": [str(good), str(short), str(bad), str(tmp_path / "missing.txt")],
        "input_b_file_name": [str(good), str(bad)],
        "global_row": ["5", "q"],
        "reduced_height": ["4", "0"],
        "gpus": ["0", ""],
    }
    bools = ["keep_rows", "aligned", "output_pearson", "mixed_precision", "double_precision",
             "ultra_precision", "no_gpu"]
    argv = []
    if rng.random() < 0.8:
        argv.append("--window=%d" % rng.choice([10, 24]))
    if rng.random() < 0.7:
        argv.append("--input_a_file_name=%s" % good)
    for _ in range(int(rng.integers(0, 6))):
        r = rng.random()
        if r < 0.6:
            name = str(rng.choice(list(values)))
            val = str(rng.choice(values[name]))
            argv += (["--%s=%s" % (name, val)] if rng.random() < 0.7 else ["--" + name, val])
        elif r < 0.9:
            name = str(rng.choice(bools))
            argv.append(str(rng.choice(["--%s", "--no%s", "--%s=false", "-%s"])) % name)
        else:
            argv.append(str(rng.choice(["--bogus=1", "stray"])))
    (rc_py, out_py), (rc_c, out_c) = _both(argv, capsys)
    assert (rc_py, out_py) == (rc_c, out_c), argv
