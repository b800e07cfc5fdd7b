"""Host-side logic that needs no GPU: the C ABI loads and exports every
declared symbol, argument validation mirrors SCAMPArgs::validate
(src/common.cpp:417-436), the comparison count matches its closed form, and
pyscamp-style keyword handling (python/SCAMP_python.cpp:91-177) raises the
same errors."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(REPO, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(REPO, "include", h)).read()
            names |= set(re.findall(r"\b(scamp_gb300_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(engine):
    lib = engine._lib.load()
    decl = declared_symbols()
    assert decl, "no declarations found"
    assert decl == set(engine._lib.EXPORTED_SYMBOLS)
    for name in decl:
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.scamp_gb300_version()


def _args(engine, n=1000, m=10, **kw):
    a = np.zeros(n)
    ca = engine._args(a, None, m, "1NN_INDEX", "double", True, True, False, False,
                      0.0, -1, -1, kw.pop("max_tile_size", 128000), 0, 0, True)
    for k, v in kw.items():
        setattr(ca, k, v)
    return ca, a


@pytest.mark.parametrize("field,value,msg", [
    ("window", 2, "at least 3"),
    ("max_tile_size", 1000, "at least 1024"),
    ("max_tile_size", 1500, "2x larger"),
    ("len_a", 5, "subesequence window size"),
    ("profile_type", 4, "not supported"),
    ("profile_type", 5, "not supported"),
    ("precision_type", 9, "precision"),
])
def test_validate_rejects(engine, field, value, msg):
    m = 800 if (field == "max_tile_size" and value == 1500) else 10
    ca, _keep = _args(engine, m=m)
    setattr(ca, field, value)
    err = ctypes.create_string_buffer(256)
    rc = engine._lib.load().scamp_gb300_validate(ctypes.byref(ca), err, 256)
    assert rc != 0 and msg in err.value.decode()


def test_validate_accepts(engine):
    ca, _keep = _args(engine)
    assert engine._lib.load().scamp_gb300_validate(ctypes.byref(ca), None, 0) == 0
    for ptype in (1, 2, 6, 7, 8):  # 1NN_INDEX, SUM_THRESH, 1NN, ALL_NEIGHBORS, MATRIX
        ca.profile_type = ptype
        ca.max_matches_per_column, ca.matrix_height, ca.matrix_width = 5, 50, 50
        assert engine._lib.load().scamp_gb300_validate(ctypes.byref(ca), None, 0) == 0
    ca.profile_type = 7
    ca.max_matches_per_column = 0
    assert engine._lib.load().scamp_gb300_validate(ctypes.byref(ca), None, 0) != 0
    ca.profile_type = 8
    ca.matrix_height = 0
    assert engine._lib.load().scamp_gb300_validate(ctypes.byref(ca), None, 0) != 0


@pytest.mark.parametrize("n,m", [(131072, 100), (1000, 3), (5000, 1024), (64, 64)])
def test_count_cells_selfjoin(engine, n, m):
    ns, e = n - m + 1, m // 4
    want = (ns - e) * (ns - e + 1) // 2 if ns > e else 0
    assert engine.count_cells(n, m) == want


def test_count_cells_config_sizes(engine):
    # the comparison counts of the benchmark configurations
    assert engine.count_cells(131072, 100) == 8573754826
    assert engine.count_cells(1 << 24, 1024) == 140716039501953
    na, nb, m = 1 << 20, 1 << 19, 256
    assert engine.count_cells(na, m, nb) == (na - m + 1) * (nb - m + 1)


def test_count_cells_aligned(engine):
    n, m = 3000, 100
    ns, e = n - m + 1, m // 4
    # aligned AB of a series with itself: all pairs except |i - j| < m/4
    want = ns * ns - sum(ns - abs(d) for d in range(-e + 1, e))
    assert engine.count_cells(n, m, n, aligned=True) == want


def test_gpu_supported_is_false_without_gpu(engine):
    try:
        import torch

        has = torch.cuda.is_available()
    except Exception:
        has = None
    if has is False:
        assert engine.gpu_supported() is False


def test_pyscamp_kwargs_validation(engine):
    a = np.random.default_rng(0).standard_normal(200)
    with pytest.raises(ValueError, match="unknown argument: threshold"):
        engine.selfjoin(a, 10, threshold=0.5)
    with pytest.raises(ValueError, match="unknown argument: foo"):
        engine.selfjoin_sum(a, 10, foo=1)
    with pytest.raises(ValueError, match="between -1 and 1"):
        engine.selfjoin_sum(a, 10, threshold=1.5)
    with pytest.raises(ValueError, match="valid options"):
        engine.abjoin(a, a, 10, precision="quad")
    with pytest.raises(ValueError, match="greater than or equal to 0"):
        engine.selfjoin(a, 10, threads=-1)
    # knn takes the sum keys; matrix adds mheight / mwidth
    with pytest.raises(ValueError, match="unknown argument: mheight"):
        engine.selfjoin_knn(a, 10, 3, mheight=5)
    with pytest.raises(ValueError, match="matrix height"):
        engine.selfjoin_matrix(a, 10, mheight=0)
    with pytest.raises(ValueError, match="matrix width"):
        engine.abjoin_matrix(a, a, 10, mwidth=-1)
    with pytest.raises(ValueError, match="between -1 and 1"):
        engine.abjoin_knn(a, a, 10, 2, threshold=-2)


def test_join_without_gpu_fails_loudly(engine):
    if engine.gpu_supported():
        pytest.skip("GPU present")
    a = np.random.default_rng(0).standard_normal(500)
    with pytest.raises(engine.SCAMPError, match="no CUDA device"):
        engine.join(a, None, 20)


def test_batch_entries_validate_before_the_device(engine):
    """Batched joins and their autotuner reject what they do not run
    (checked on the host, so without a GPU too)."""
    x = np.cumsum(np.random.default_rng(1).standard_normal(600))
    for call in (engine.join_batch, engine.tune_batch):
        with pytest.raises(ValueError, match="mixed form"):
            call([x, x], [32, 64], precision="double")
        with pytest.raises(ValueError, match="series 1"):
            call([x, x[:20]], [32, 32])
        with pytest.raises(ValueError, match="one window per series"):
            call([x, x], [32])
    if not engine.gpu_supported():
        with pytest.raises(engine.SCAMPError, match="no CUDA device"):
            engine.tune_batch([x], 32)


def test_key_layout_roundtrip_host():
    # The fixed-point key (engine.cuh): q = floor((r + 2) * 2^F); decoding
    # recovers r within 2^-F and preserves order.
    F = 62 - 27
    r = np.array([-1.0, -0.5, -1e-9, 0.0, 1e-9, 0.3, 0.999999, 1.0])
    q = np.floor((r + 2.0) * 2.0 ** F)
    assert np.all(np.diff(q) >= 0)
    back = q / 2.0 ** F - 2.0
    assert np.max(np.abs(back - r)) <= 2.0 ** -F
