"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU
only): the C oracle over every profile type, geometry and precision it
serves, and the C++ do_SCAMP shim's error and utility paths.  Each is built
with -fsanitize=address,undefined into a temporary directory and run in a
child process; any sanitizer report fails the test."""
import os
import shutil
import subprocess
import sys
import textwrap

import pytest

from conftest import PKG_DIR, REPO

SAN = ["-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
       "-fno-sanitize-recover=undefined"]


def _runtime(lib):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    path = subprocess.run([gcc, "-print-file-name=" + lib], capture_output=True,
                          text=True).stdout.strip()
    if not os.path.isabs(path) or not os.path.exists(path):
        pytest.skip("%s not available" % lib)
    return path


def test_oracle_under_sanitizers(tmp_path):
    preload = " ".join(_runtime(x) for x in ("libasan.so", "libubsan.so"))
    lib = str(tmp_path / "liboracle_san.so")
    subprocess.check_call(["cc"] + SAN + ["-fopenmp", "-fPIC", "-shared", "-std=c11",
                                          os.path.join(REPO, "oracle", "scamp_oracle.c"),
                                          "-o", lib, "-lm"])
    script = textwrap.dedent("""
        import sys
        import numpy as np
        sys.path.insert(0, %r)
        import oracle
        oracle.LIB_PATH = %r
        for seed in range(12):
            r = np.random.default_rng(seed)
            m = int(r.choice([3, 8, 33, 64]))
            a = np.cumsum(r.standard_normal(int(r.integers(m, 900))))
            b = np.cumsum(r.standard_normal(int(r.integers(m, 900))))
            a[r.integers(0, len(a), 3)] = np.nan
            for prof in ("1NN_INDEX", "SUM_THRESH", "1NN"):
                for bb, kw in ((None, {}), (b, {"keep_rows": True}),
                               (b, {"computing_rows": False}),
                               (b, {"aligned": True, "keep_rows": True,
                                    "start_row": 5, "start_col": 40})):
                    kw = dict(kw, profile=prof, threshold=0.3)
                    oracle.join(a, bb, m, **kw)
                    oracle.join(a, bb, m, brute=True, **kw)
                    oracle.join(a, bb, m, precision=4, **kw)
        print("clean")
    """) % (os.path.join(REPO, "oracle"), lib)
    env = dict(os.environ, LD_PRELOAD=preload, ASAN_OPTIONS="detect_leaks=0")
    p = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True,
                       env=env, timeout=600)
    assert p.returncode == 0 and "clean" in p.stdout, p.stdout[-2000:] + p.stderr[-4000:]
    assert "runtime error" not in p.stderr and "AddressSanitizer" not in p.stderr


def test_cpp_shim_under_sanitizers(tmp_path):
    _runtime("libasan.so")
    if not os.path.exists(os.path.join(PKG_DIR, "libscamp_gb300.so")):
        pytest.skip("engine library not built")
    exe = str(tmp_path / "shim_demo_san")
    subprocess.check_call(["g++", "-std=c++17"] + SAN + [
        "-I", os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "shim_demo.cpp"),
        "-o", exe, "-L", PKG_DIR, "-lscamp_gb300", "-Wl,-rpath," + PKG_DIR])
    d = tmp_path / "u"
    d.mkdir()
    import numpy as np

    rng = np.random.default_rng(4)
    corr = rng.uniform(-1, 1, 40).astype(np.float32)
    corr[[3, 17]] = -2.0
    idx = rng.integers(0, 1000, 40).astype(np.uint64)
    packed = (idx << np.uint64(32)) | corr.view(np.uint32).astype(np.uint64)
    packed.tofile(d / "nn_index.bin")
    corr.tofile(d / "nn.bin")
    rng.uniform(0, 50, 40).tofile(d / "sum.bin")
    packed[:36].tofile(d / "knn.bin")
    rng.uniform(-1, 1, 20).astype(np.float32).tofile(d / "matrix.bin")
    (d / "in.txt").write_text("1.5\n-2e3\n0.25\n7\n")
    # protect_shadow_gap=0: the CUDA runtime maps memory where ASan keeps its
    # shadow gap when a GPU driver is present
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:protect_shadow_gap=0")
    for args in (["errors"], ["utils", str(d)]):
        p = subprocess.run([exe] + args, capture_output=True, text=True, env=env, timeout=300)
        assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-4000:]
        assert "runtime error" not in p.stderr and "Sanitizer" not in p.stderr
