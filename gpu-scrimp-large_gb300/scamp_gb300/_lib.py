"""ctypes binding of libscamp_gb300.so (declarations in include/scamp_gb300.h).

The library is built in-tree by ``scamp_gb300.build`` (nvcc, sm_103a).  There is
no CPU fallback: if the shared library is missing or no GPU is visible, calls
raise instead of computing anything on the host.
"""
import ctypes
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libscamp_gb300.so")

PROFILE_1NN_INDEX = 1
PROFILE_SUM_THRESH = 2
PROFILE_1NN = 6
PROFILE_APPROX_ALL_NEIGHBORS = 7
PROFILE_MATRIX_SUMMARY = 8
PRECISION_SINGLE = 1
PRECISION_MIXED = 2
PRECISION_DOUBLE = 3
PRECISION_ULTRA = 4

SCAMP_OK = 0
ERROR_NAMES = {
    1: "SCAMP_ERR_UNIMPLEMENTED",
    3: "SCAMP_ERR_CUDA",
    6: "SCAMP_ERR_DIM_INCOMPATIBLE",
    100: "SCAMP_ERR_INVALID_ARGS",
    101: "SCAMP_ERR_NO_DEVICE",
    102: "SCAMP_ERR_OUT_OF_MEMORY",
    103: "SCAMP_ERR_DEVICE_TIMEOUT",
}

# Every symbol include/scamp_gb300.h declares.
EXPORTED_SYMBOLS = (
    "scamp_gb300_join",
    "scamp_gb300_join_dev",
    "scamp_gb300_join_dev_noalloc",
    "scamp_gb300_join_batch",
    "scamp_gb300_tune_batch",
    "scamp_gb300_validate",
    "scamp_gb300_count_cells",
    "scamp_gb300_gpu_supported",
    "scamp_gb300_pipe_peak",
    "scamp_gb300_anchor_check",
    "scamp_gb300_wait_limit_check",
    "scamp_gb300_window_stats",
    "scamp_gb300_version",
)

_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class CArgs(ctypes.Structure):
    """Mirror of scamp_c_args."""
    _fields_ = [
        ("timeseries_a", ctypes.c_void_p),
        ("len_a", ctypes.c_uint64),
        ("timeseries_b", ctypes.c_void_p),
        ("len_b", ctypes.c_uint64),
        ("has_b", ctypes.c_int32),
        ("window", ctypes.c_uint64),
        ("max_tile_size", ctypes.c_uint64),
        ("distributed_start_row", ctypes.c_int64),
        ("distributed_start_col", ctypes.c_int64),
        ("distance_threshold", ctypes.c_double),
        ("precision_type", ctypes.c_int32),
        ("profile_type", ctypes.c_int32),
        ("computing_rows", ctypes.c_int32),
        ("computing_columns", ctypes.c_int32),
        ("keep_rows_separate", ctypes.c_int32),
        ("is_aligned", ctypes.c_int32),
        ("silent_mode", ctypes.c_int32),
        ("anchor_interval", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("max_matches_per_column", ctypes.c_int32),
        ("matrix_height", ctypes.c_int32),
        ("matrix_width", ctypes.c_int32),
        ("filter_mode", ctypes.c_int32),
        ("anchor_mode", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 1),
    ]


class CResult(ctypes.Structure):
    """Mirror of scamp_c_result."""
    _fields_ = [
        ("profile_a", ctypes.c_void_p),
        ("profile_b", ctypes.c_void_p),
        ("sum_a", ctypes.c_void_p),
        ("sum_b", ctypes.c_void_p),
        ("corr_a", ctypes.c_void_p),
        ("corr_b", ctypes.c_void_p),
        ("elapsed_ms", ctypes.c_double),
        ("join_kernel_ms", ctypes.c_double),
        ("comparisons", ctypes.c_uint64),
        ("gpu_launches", ctypes.c_uint32),
        ("inplace_verifications", ctypes.c_uint32),
        ("steps", ctypes.c_uint64),
        ("slow_steps", ctypes.c_uint64),
        ("verifications", ctypes.c_uint64),
        ("verify_kernel_ms", ctypes.c_double),
        ("max_a", ctypes.c_void_p),
        ("max_b", ctypes.c_void_p),
        ("knn_a", ctypes.c_void_p),
        ("knn_b", ctypes.c_void_p),
        ("matrix", ctypes.c_void_p),
        ("max_abs_r_err", ctypes.c_double),
        ("max_tie_margin", ctypes.c_double),
    ]


class SCAMPError(RuntimeError):
    """Raised for a non-zero engine status (the reference throws
    SCAMPException, src/scamp_exception.h:7-22)."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


_lib = None


def load():
    """Load the in-tree engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libscamp_gb300.so not found at %s: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    lib.scamp_gb300_join.argtypes = [ctypes.POINTER(CArgs), ctypes.POINTER(CResult),
                                     ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_join.restype = ctypes.c_int
    lib.scamp_gb300_join_dev.argtypes = [ctypes.POINTER(CArgs), ctypes.POINTER(CResult),
                                         ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_join_dev.restype = ctypes.c_int
    lib.scamp_gb300_join_dev_noalloc.argtypes = [ctypes.POINTER(CArgs), ctypes.POINTER(CResult),
                                                 ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_join_dev_noalloc.restype = ctypes.c_int
    lib.scamp_gb300_join_batch.argtypes = [ctypes.POINTER(CArgs), ctypes.POINTER(CResult),
                                           ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_join_batch.restype = ctypes.c_int
    lib.scamp_gb300_tune_batch.argtypes = [ctypes.POINTER(CArgs), ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int64), ctypes.c_char_p,
                                           ctypes.c_size_t]
    lib.scamp_gb300_tune_batch.restype = ctypes.c_int
    lib.scamp_gb300_validate.argtypes = [ctypes.POINTER(CArgs), ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_validate.restype = ctypes.c_int
    lib.scamp_gb300_count_cells.argtypes = [ctypes.POINTER(CArgs)]
    lib.scamp_gb300_count_cells.restype = ctypes.c_uint64
    lib.scamp_gb300_gpu_supported.argtypes = []
    lib.scamp_gb300_gpu_supported.restype = ctypes.c_int
    lib.scamp_gb300_pipe_peak.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
    lib.scamp_gb300_pipe_peak.restype = ctypes.c_int
    lib.scamp_gb300_anchor_check.argtypes = [ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_int),
                                             ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_anchor_check.restype = ctypes.c_int
    lib.scamp_gb300_wait_limit_check.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_wait_limit_check.restype = ctypes.c_int
    lib.scamp_gb300_window_stats.argtypes = [ctypes.c_int, _dp, ctypes.c_int64, ctypes.c_int64,
                                             ctypes.c_int, _dp, _dp, _dp, _dp,
                                             ctypes.c_char_p, ctypes.c_size_t]
    lib.scamp_gb300_window_stats.restype = ctypes.c_int
    lib.scamp_gb300_version.argtypes = []
    lib.scamp_gb300_version.restype = ctypes.c_char_p
    _lib = lib
    return lib
