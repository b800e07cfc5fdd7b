"""The mixed form's tensor-core anchors (split-BF16x3 tcgen05 contraction,
anchor_tc.cu) through the C ABI: the self-check against FP64 direct dot
products, and mixed joins whose anchors come from the tensor cores against
the oracle and against the same joins anchored on the CUDA cores.

Anchor tolerance: max |anchor - cov_FP64| * invnorm_r * invnorm_c <= 1e-6
(the FP32 data both anchor forms start from carry ~1e-7 of it); joins: the
mixed form's 1e-5 in r with the near-tie rule."""
import numpy as np
import pytest

from parity import TOL_MIXED, check_1nn, check_1nn_direct, check_sum

pytestmark = pytest.mark.gpu


def test_anchor_self_check(gpu_engine):
    err, available = gpu_engine.anchor_check()
    assert available, "tensor-core anchors failed their FP64 self-check (max err %.3g)" % err
    assert err <= 1e-6, err


def _walk(seed, n):
    return np.cumsum(np.random.default_rng(seed).standard_normal(n))


def _join_pair(engine, oracle, a, b, m, name, **kw):
    """The same mixed join with tensor-core and CUDA-core anchors, both
    checked against the oracle; the tensor-core one must have launched the
    contraction (more kernels)."""
    want = oracle.join(a, b, m, exact_flat=True, **kw)
    other = a if b is None else b
    launches = {}
    for mode in (2, 1):
        got = engine.join(a, b, m, "1NN_INDEX", "mixed", return_corr=True, anchor_mode=mode,
                          anchor_interval=2048, **kw)
        launches[mode] = got["gpu_launches"]
        _, gi = engine.unpack_profile(got["profile_a"])
        check_1nn("%s/anchors%d/A" % (name, mode), got["corr_a"], gi, want["corr_a"],
                  want["idx_a"], TOL_MIXED, a, other, m)
        check_1nn_direct("%s/anchors%d/A" % (name, mode), got["corr_a"], gi, want["idx_a"],
                         TOL_MIXED, a, other, m, bound=got["max_abs_r_err"])
        if kw.get("keep_rows"):
            _, gib = engine.unpack_profile(got["profile_b"])
            check_1nn("%s/anchors%d/B" % (name, mode), got["corr_b"], gib, want["corr_b"],
                      want["idx_b"], TOL_MIXED, other, a, m)
    assert launches[2] > launches[1], launches


def test_tc_anchors_selfjoin(gpu_engine, oracle_mod):
    _join_pair(gpu_engine, oracle_mod, _walk(1, 1 << 18), None, 512, "self512")


def test_tc_anchors_abjoin_keep_rows_odd_window(gpu_engine, oracle_mod):
    a, b = _walk(2, 1 << 18), _walk(3, 1 << 17)
    b[np.random.default_rng(4).choice(len(b), 50, replace=False)] = np.nan
    _join_pair(gpu_engine, oracle_mod, a, b, 600, "ab600", keep_rows=True)


def test_tc_anchors_nan_gaps_long_window(gpu_engine, oracle_mod):
    from scamp_gb300 import workloads

    x, _ = workloads.gapped_walk_selfjoin(n=1 << 18, m=1024)
    want = oracle_mod.join(x, None, 1024, exact_flat=True)
    got = gpu_engine.join(x, None, 1024, "1NN_INDEX", "mixed", return_corr=True, anchor_mode=2)
    _, gi = gpu_engine.unpack_profile(got["profile_a"])
    check_1nn("gaps1024", got["corr_a"], gi, want["corr_a"], want["idx_a"], TOL_MIXED, x, x, 1024)


@pytest.mark.parametrize("thr", [0.5, 0.9])
def test_tc_anchors_sum_thresh(gpu_engine, oracle_mod, thr):
    a = _walk(5, 1 << 18)
    want = oracle_mod.join(a, None, 512, "SUM_THRESH", threshold=thr)
    got = gpu_engine.join(a, None, 512, "SUM_THRESH", "mixed", threshold=thr, anchor_mode=2,
                          anchor_interval=2048)
    check_sum("tc-sum", got["sum_a"], want["sum_a"], thr, 2e-5, TOL_MIXED)


def test_device_wait_limit_returns_timeout(gpu_engine):
    """The tensor-core kernel's bounded wait on its MMA barrier, made to run
    out (no MMA issued): the host gets SCAMP_ERR_DEVICE_TIMEOUT and the
    context stays usable for the next join."""
    import ctypes

    from scamp_gb300 import _lib

    lib = _lib.load()
    err = ctypes.create_string_buffer(512)
    rc = lib.scamp_gb300_wait_limit_check(0, err, 512)
    assert rc == 103, (rc, err.value)  # SCAMP_ERR_DEVICE_TIMEOUT
    assert b"timed out" in err.value
    a = _walk(9, 5000)
    r = gpu_engine.join(a, None, 100, "1NN_INDEX", "mixed", return_corr=True)
    assert r["comparisons"] > 0 and np.all(r["corr_a"] >= -1)
