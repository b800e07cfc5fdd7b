"""Command-line front of the engine, with the reference CLI's flags, input
parsing and output files (zpzim/GPU-SCRIMP-LARGE src/main.cpp:22-243,
src/scamp_utils.cpp:30-74 and 127-225):

    python -m scamp_gb300 --window=100 --input_a_file_name=a.txt \\
        [--input_b_file_name=b.txt --keep_rows] [--mixed_precision] ...

writes the profile to --output_a_file_name (default mp_columns_out) and the
index to --output_a_index_file_name (mp_columns_out_index); with --keep_rows
the row profile goes to --output_b_file_name / --output_b_index_file_name.
Values are z-normalised Euclidean distances (or Pearson correlations with
--output_pearson), 10 significant digits; unmatched entries are "nan" with
index -1.  --profile_type=1NN writes the distances only (no index file),
SUM_THRESH the per-window sums, ALL_NEIGHBORS "column row value" lines
(--max_matches_per_column per window), MATRIX_SUMMARY the
--reduced_height x --reduced_width summary.  Exit status 1 with the
reference's message for invalid arguments.

Flags of the reference that select other machinery (distributed execution,
CPU workers) are accepted and ignored, except --no_gpu, which this engine
cannot honour (it has no CPU path).
"""
import ctypes
import errno
import math
import sys

import numpy as np

# name -> (kind, default)
_FLAGS = {
    "window": ("int", -1),
    "max_tile_size": ("int", 1 << 17),
    "threshold": ("float", 0.0),
    "profile_type": ("str", "1NN_INDEX"),
    "ultra_precision": ("bool", False),
    "double_precision": ("bool", False),
    "mixed_precision": ("bool", False),
    "single_precision": ("bool", False),
    "keep_rows": ("bool", False),
    "aligned": ("bool", False),
    "global_row": ("int", -1),
    "global_col": ("int", -1),
    "input_a_file_name": ("str", ""),
    "input_b_file_name": ("str", ""),
    "output_a_file_name": ("str", "mp_columns_out"),
    "output_a_index_file_name": ("str", "mp_columns_out_index"),
    "output_b_file_name": ("str", "mp_rows_out"),
    "output_b_index_file_name": ("str", "mp_rows_out_index"),
    "output_pearson": ("bool", False),
    "gpus": ("str", ""),
    "print_debug_info": ("bool", False),
    "no_gpu": ("bool", False),
    "max_matches_per_column": ("int", 5),
    "reduced_height": ("int", 50),
    "reduced_width": ("int", 50),
    # accepted, no effect here
    "num_cpu_workers": ("int", 0),
    "distributed_tile_size": ("int", 4000000),
    "hostname_port": ("str", "localhost:30078"),
}


class UsageError(Exception):
    pass


def parse_flags(argv):
    """gflags-style flags: --name=value, --name value, --bool, --nobool."""
    vals = {k: d for k, (_, d) in _FLAGS.items()}
    i = 0
    while i < len(argv):
        tok = argv[i]
        if not tok.startswith("-"):
            raise UsageError("Error: unexpected argument %s" % tok)
        tok = tok.lstrip("-")
        name, eq, value = tok.partition("=")
        kind = _FLAGS.get(name, (None,))[0]
        if kind is None and name.startswith("no") and _FLAGS.get(name[2:], (None,))[0] == "bool":
            vals[name[2:]] = False
            i += 1
            continue
        if kind is None:
            raise UsageError("ERROR: unknown command line flag '%s'" % name)
        if kind == "bool":
            vals[name] = (value.lower() not in ("false", "0", "no")) if eq else True
            i += 1
            continue
        if not eq:
            if i + 1 >= len(argv):
                raise UsageError("ERROR: flag '--%s' is missing its argument" % name)
            value = argv[i + 1]
            i += 1
        try:
            vals[name] = int(value) if kind == "int" else float(value) if kind == "float" else value
        except ValueError:
            raise UsageError("ERROR: illegal value '%s' specified for %s flag '%s'"
                             % (value, kind, name))
        i += 1
    return vals


_STRTOD = None


def _strtod(tok):
    """C strtod on one token, as the reference's std::stod parses it:
    (value, characters used, out of range)."""
    global _STRTOD
    if _STRTOD is None:
        libc = ctypes.CDLL(None, use_errno=True)
        fn = libc.strtod
        fn.restype = ctypes.c_double
        fn.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
        _STRTOD = fn
    buf = ctypes.create_string_buffer(tok)
    endp = ctypes.c_char_p()
    ctypes.set_errno(0)
    val = _STRTOD(buf, ctypes.byref(endp))
    err = ctypes.get_errno()
    used = ctypes.cast(endp, ctypes.c_void_p).value - ctypes.addressof(buf)
    return val, used, err == errno.ERANGE


def read_series(path):
    """The reference's readFile (src/scamp_utils.cpp:30-72): whitespace-
    separated numbers, each parsed as std::stod does (the longest numeric
    prefix of the token); a token with no number, or one out of range, is a
    fatal error that names its first character and its line.  Like the
    reference, a value is kept only when more input follows it, so the last
    value of a file without a trailing newline is dropped."""
    try:
        with open(path, "rb") as f:
            text = f.read()
    except OSError:
        raise UsageError("Unable to open%sfor reading, please make sure it exists" % path)
    out = []
    pos, n = 0, len(text)
    while True:
        while pos < n and text[pos:pos + 1].isspace():
            pos += 1
        if pos >= n:
            break
        end = pos
        while end < n and not text[end:end + 1].isspace():
            end += 1
        tok = text[pos:end]
        val, used, out_of_range = _strtod(tok)
        if used == 0 or out_of_range:
            raise UsageError("%s\nFATAL ERROR: %s: Could not parse line number %d from input file."
                             % (tok[:1].decode("latin-1"),
                                "out of range" if used else "invalid argument", len(out) + 1))
        pos = end
        if pos >= n:  # nothing follows the value
            break
        out.append(val)
    return np.asarray(out, dtype=np.float64)


def _fmt(v):
    if math.isnan(v):
        return "nan"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return format(v, ".10g")


def write_profile(path_mp, path_mpi, packed, pearson, window):
    """WriteProfileToFile for 1NN_INDEX entries (src/scamp_utils.cpp:143-170)."""
    from . import unpack_profile

    corr, idx = unpack_profile(packed)
    corr = corr.astype(np.float64)
    if pearson:
        vals = np.where(corr < -1, np.nan, corr)
    else:
        with np.errstate(invalid="ignore"):
            vals = np.sqrt(np.maximum(2.0 * window * (1.0 - corr), 0.0))
        vals[corr < -1] = np.nan
    with open(path_mp, "w") as f:
        f.write("".join(_fmt(v) + "\n" for v in vals.tolist()))
    with open(path_mpi, "w") as f:
        f.write("".join("%d\n" % i for i in idx.tolist()))


def write_max_profile(path_mp, corr, pearson, window):
    """WriteProfileToFile for 1NN profiles (src/scamp_utils.cpp:172-183):
    distances (or correlations), no index file."""
    corr = np.asarray(corr).astype(np.float64)
    if pearson:
        vals = np.where(corr < -1, np.nan, corr)
    else:
        with np.errstate(invalid="ignore"):
            vals = np.sqrt(np.maximum(2.0 * window * (1.0 - corr), 0.0))
        vals[corr < -1] = np.nan
    with open(path_mp, "w") as f:
        f.write("".join(_fmt(v) + "\n" for v in vals.tolist()))


def _values(corr, pearson, window):
    corr = np.asarray(corr).astype(np.float64)
    if pearson:
        vals = corr.copy()
    else:
        with np.errstate(invalid="ignore"):
            vals = np.sqrt(np.maximum(2.0 * window * (1.0 - corr), 0.0))
    vals[corr < -1] = np.nan
    return vals


def write_knn(path, entries, k, pearson, window):
    """WriteProfileToFile for ALL_NEIGHBORS (src/scamp_utils.cpp:193-212): one
    "column row value" line per match, columns in order, best match first."""
    from . import unpack_profile

    corr, idx = unpack_profile(np.asarray(entries))
    vals = _values(corr, pearson, window)
    cols = np.repeat(np.arange(len(idx) // k), k)
    ok = idx >= 0
    with open(path, "w") as f:
        f.write("".join("%d %d %s\n" % (c, i, _fmt(v))
                        for c, i, v in zip(cols[ok].tolist(), idx[ok].tolist(),
                                           vals[ok].tolist())))


def write_matrix(path, matrix, pearson, window):
    """write_matrix (src/scamp_utils.cpp:9-28): the summary row by row, each
    value followed by a space."""
    vals = _values(np.asarray(matrix), pearson, window)
    with open(path, "w") as f:
        f.write("".join("".join(_fmt(v) + " " for v in row) + "\n" for row in vals.tolist()))


def write_sums(path, sums):
    with open(path, "w") as f:
        f.write("".join(_fmt(v) + "\n" for v in np.asarray(sums, dtype=np.float64).tolist()))


def run(argv):
    import scamp_gb300

    fl = parse_flags(argv)
    prec = [p for p in ("ultra", "double", "mixed", "single") if fl[p + "_precision"]]
    if not prec:
        prec = ["double"]
    if len(prec) != 1:
        raise UsageError("Error: only one precision flag can be enabled at a time")
    if fl["window"] < 3:
        raise UsageError("Error: Subsequence length must be at least 3, please use "
                         "--window=<window_size> to specify your subsequence length.")
    if fl["max_tile_size"] < 1024:
        raise UsageError("Error: max tile size must be at least 1024")
    if fl["max_tile_size"] // 2 < fl["window"]:
        raise UsageError("Error: Tile length and width must be at least 2x larger than the "
                         "window size. Please set a larger --max_tile_size=<max_tile_size>")
    if not fl["input_a_file_name"]:
        raise UsageError("Error: primary input filename must be specified using "
                         "--input_a_file_name")
    if fl["no_gpu"]:
        raise UsageError("Error: this engine runs on the GPU only (--no_gpu is not supported)")
    if fl["profile_type"] not in ("1NN_INDEX", "SUM_THRESH", "1NN", "ALL_NEIGHBORS",
                                  "MATRIX_SUMMARY"):
        raise UsageError("Error: profile type %s is not supported by this engine"
                         % fl["profile_type"])
    self_join = not fl["input_b_file_name"]
    a = read_series(fl["input_a_file_name"])
    b = None if self_join else read_series(fl["input_b_file_name"])
    m = fl["window"]
    if len(a) - m + 1 < 1 or (b is not None and len(b) - m + 1 < 1):
        raise UsageError("Error: window size must be smaller than the timeseries length")
    devices = [int(x) for x in fl["gpus"].split(",") if x.strip()] if fl["gpus"] else [0]
    keep = bool(fl["keep_rows"])
    r = scamp_gb300.join(
        a, b, m, fl["profile_type"], prec[0],
        computing_rows=True if self_join else keep, keep_rows=keep, aligned=fl["aligned"],
        threshold=fl["threshold"], start_row=fl["global_row"], start_col=fl["global_col"],
        max_tile_size=fl["max_tile_size"], device=devices[0],
        silent=not fl["print_debug_info"], max_matches=fl["max_matches_per_column"],
        matrix_height=fl["reduced_height"], matrix_width=fl["reduced_width"])
    if fl["profile_type"] == "1NN_INDEX":
        write_profile(fl["output_a_file_name"], fl["output_a_index_file_name"], r["profile_a"],
                      fl["output_pearson"], m)
        if keep:
            write_profile(fl["output_b_file_name"], fl["output_b_index_file_name"],
                          r["profile_b"], fl["output_pearson"], m)
    elif fl["profile_type"] == "ALL_NEIGHBORS":
        k = fl["max_matches_per_column"]
        write_knn(fl["output_a_file_name"], r["knn_a"], k, fl["output_pearson"], m)
        if keep:
            write_knn(fl["output_b_file_name"], r["knn_b"], k, fl["output_pearson"], m)
    elif fl["profile_type"] == "MATRIX_SUMMARY":
        write_matrix(fl["output_a_file_name"], r["matrix"], fl["output_pearson"], m)
    elif fl["profile_type"] == "1NN":
        write_max_profile(fl["output_a_file_name"], r["profile_a"], fl["output_pearson"], m)
        if keep:
            write_max_profile(fl["output_b_file_name"], r["profile_b"], fl["output_pearson"], m)
    else:
        write_sums(fl["output_a_file_name"], r["sum_a"])
        if keep:
            write_sums(fl["output_b_file_name"], r["sum_b"])
    return 0


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    try:
        return run(argv)
    except UsageError as e:
        print(str(e))
        return 1
    except (ValueError, RuntimeError) as e:  # engine errors (SCAMPException)
        print(str(e))
        return 1
