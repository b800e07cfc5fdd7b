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
