/*
 * scamp_gb300.h -- C ABI of the GB300 SCAMP matrix-profile engine.
 *
 * The reference (zpzim/GPU-SCRIMP-LARGE) exposes this path through the C++
 * entry SCAMP::do_SCAMP(SCAMPArgs*) (src/SCAMP.h:15-18, src/SCAMP.cpp:261-334)
 * and pyscamp's selfjoin/abjoin (python/SCAMP_python.cpp:196-236).  Both sit on
 * top of the functions below: the C++ shim (include/scamp/SCAMP.h) and the
 * Python package (scamp_gb300) call scamp_gb300_join().  Plain C types only:
 * no exceptions or C++ objects cross this boundary.
 *
 * Precision: SCAMP_PRECISION_DOUBLE runs every step in FP64.
 * SCAMP_PRECISION_MIXED runs the diagonal recurrence and the compare in FP32,
 * re-anchored from FP64-centred data every anchor_interval rows.
 * SCAMP_PRECISION_SINGLE is served by the mixed engine; SCAMP_PRECISION_ULTRA
 * is served by the FP64 engine with brute-force O(nm) window statistics.
 */
#ifndef SCAMP_GB300_H
#define SCAMP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Values of the reference enums SCAMPProfileType / SCAMPPrecisionType
 * (src/common.h:34-58). */
enum {
  SCAMP_PROFILE_1NN_INDEX = 1,
  SCAMP_PROFILE_SUM_THRESH = 2,
  SCAMP_PROFILE_1NN = 6, /* best correlation only, float32 (no index) */
  SCAMP_PROFILE_APPROX_ALL_NEIGHBORS = 7, /* k best matches per window */
  SCAMP_PROFILE_MATRIX_SUMMARY = 8,       /* max correlation per grid cell */
};
enum {
  SCAMP_PRECISION_SINGLE = 1,
  SCAMP_PRECISION_MIXED = 2,
  SCAMP_PRECISION_DOUBLE = 3,
  SCAMP_PRECISION_ULTRA = 4,
};

/* Status codes (0 = success).  The first six mirror SCAMPError_t
 * (src/common.h:359-367); the rest are boundary errors. */
enum {
  SCAMP_OK = 0,
  SCAMP_ERR_UNIMPLEMENTED = 1,
  SCAMP_ERR_CUDA = 3,
  SCAMP_ERR_DIM_INCOMPATIBLE = 6,
  SCAMP_ERR_INVALID_ARGS = 100,
  SCAMP_ERR_NO_DEVICE = 101,
  SCAMP_ERR_OUT_OF_MEMORY = 102,
  SCAMP_ERR_DEVICE_TIMEOUT = 103,
};

/* Join arguments: the plain-C image of SCAMPArgs (src/common.h:164-188). */
typedef struct scamp_c_args {
  const double *timeseries_a; /* host or device memory, see *_dev entry */
  uint64_t len_a;
  const double *timeseries_b; /* ignored unless has_b */
  uint64_t len_b;
  int32_t has_b;              /* 0: self-join of A */
  uint64_t window;            /* subsequence length m (>= 3) */
  uint64_t max_tile_size;     /* validated as the reference does; work is
                                 scheduled on device independently of it */
  int64_t distributed_start_row; /* -1 when unused */
  int64_t distributed_start_col; /* -1 when unused */
  double distance_threshold;  /* SUM_THRESH: sum correlations > threshold */
  int32_t precision_type;     /* SCAMP_PRECISION_* */
  int32_t profile_type;       /* SCAMP_PROFILE_* */
  int32_t computing_rows;
  int32_t computing_columns;
  int32_t keep_rows_separate;
  int32_t is_aligned;
  int32_t silent_mode;
  /* Tuning overrides, 0 = automatic. */
  int32_t anchor_interval;    /* mixed: rows between FP64-centred re-anchors */
  int32_t device;             /* CUDA device ordinal */
  /* APPROX_ALL_NEIGHBORS: matches kept per window (the reference's
   * max_matches_per_column); MATRIX_SUMMARY: grid height (windows of B) and
   * width (windows of A), the reference's matrix_height / matrix_width. */
  int32_t max_matches_per_column;
  int32_t matrix_height;
  int32_t matrix_width;
  /* Mixed form's fast-path filter (tuning override, 0 = automatic): 1 = the
   * largest per-cell correlation of each 8 x 8 block, 2 = a per-block bound
   * (largest covariance times the largest inverse norms), cheaper where
   * neighbouring windows' norms are close (long windows). */
  int32_t filter_mode;
  /* Mixed form's anchors (tuning override, 0 = automatic): 1 = FP32 dot
   * products on the CUDA cores inside the band kernel, 2 = split-BF16x3
   * contraction on the tensor cores into an anchor table. */
  int32_t anchor_mode;
  int32_t reserved[1];
} scamp_c_args;

/* Results.  Profiles are in/out: on entry they hold the best-so-far values
 * (InitProfileMemory semantics, src/scamp_utils.cpp:226-245: 1NN_INDEX
 * entries {corr=-2.0f, index=0xFFFFFFFF}, SUM_THRESH zeros); the join merges
 * into them exactly as the reference merges tiles (src/common.cpp:167-197).
 * 1NN_INDEX entries use the reference layout (src/common.h:70-74): low 32
 * bits = float32 Pearson correlation, high 32 bits = uint32 index. */
typedef struct scamp_c_result {
  uint64_t *profile_a;  /* 1NN_INDEX, len_a - window + 1 entries */
  uint64_t *profile_b;  /* 1NN_INDEX rows when keep_rows_separate */
  double *sum_a;        /* SUM_THRESH, len_a - window + 1 entries */
  double *sum_b;        /* SUM_THRESH rows when keep_rows_separate */
  double *corr_a;       /* optional: best correlation in double, -2 = none */
  double *corr_b;       /* optional */
  /* Filled by the engine. */
  double elapsed_ms;    /* device time of the join (stats .. final profile) */
  double join_kernel_ms;/* device time of the join kernels (the tensor-core
                         * anchors where the mixed form uses them, the band
                         * kernel, then, in the mixed forms, the
                         * verification of deferred candidates) */
  uint64_t comparisons; /* distance-matrix cells evaluated */
  uint32_t gpu_launches;/* kernels launched by this call */
  uint32_t inplace_verifications; /* mixed forms: candidate cells verified by
                         * a direct dot product inside the band kernel because
                         * the request buffer was full (slow; the next join on
                         * the device sizes the buffer for them); saturates */
  /* Work counters of the mixed 1NN_INDEX form (0 otherwise): 8-row steps
   * of one thread, steps recomputed on the exact path, and candidate cells
   * sent to verification by a direct dot product. */
  uint64_t steps;
  uint64_t slow_steps;
  uint64_t verifications;
  double verify_kernel_ms; /* part of join_kernel_ms: the last deferred
                            * verification pass (joins anchored on the tensor
                            * cores verify each chunk's requests after it) */
  /* 1NN (SCAMP_PROFILE_1NN): the best correlation per window as float32,
   * -2.0f = none (the reference's float profile, src/common.cpp:290-292);
   * in/out like profile_a / profile_b. */
  float *max_a;
  float *max_b;
  /* APPROX_ALL_NEIGHBORS: max_matches_per_column entries per window in the
   * 1NN_INDEX layout (correlation, index of the match), best first, unused
   * entries {-2.0f, 0xFFFFFFFF}; in/out, entries given on input must be in
   * that order.  Every match has r > distance_threshold, and these are the
   * exact best matches (the reference's approximate lists may miss some). */
  uint64_t *knn_a;
  uint64_t *knn_b;
  /* MATRIX_SUMMARY: matrix_height x matrix_width floats, row-major; entry
   * (y, x) is the largest r > distance_threshold over the cells whose B window
   * (A window in a self-join) falls in row block y and A window in column
   * block x (blocks of ceil(windows / height or width)), -2.0f where none;
   * in/out (merged by max).  Columns only, as in the reference. */
  float *matrix;
  /* Accuracy of the reported correlations (filled by the engine).
   * max_abs_r_err: bound on |reported r - FP64 r| for every reported value.
   *   1NN_INDEX / 1NN (both forms): after the join the correlation of every
   *   reported (window, partner) pair is recomputed in FP64 from the two
   *   windows (centred dot product over centred sums of squares); the bound
   *   is that computation's rounding plus the profile key's resolution,
   *   deterministic, for corr_a / corr_b (packed float32 entries add their
   *   own rounding, 2^-24 |r|).  Entries given on input and left unchanged
   *   keep their value.
   *   APPROX_ALL_NEIGHBORS, mixed form: the same FP64 recomputation of
   *   every list entry (each list re-sorted by it).
   *   SUM_THRESH and MATRIX_SUMMARY, mixed forms: the largest drift margin of
   *   an FP32 correlation added (or published as a grid maximum) without a
   *   direct dot product (a bound under the filter's rounding model, see
   *   max_tie_margin).
   *   -1 where no bound is tracked (the FP64 forms of SUM_THRESH,
   *   APPROX_ALL_NEIGHBORS and MATRIX_SUMMARY).
   * max_tie_margin: mixed 1NN and k-best forms: the largest drift margin of
   *   an FP32 recurrence value that chose a partner without a direct dot
   *   product.
   *   The reported partner's FP64 correlation is within twice this of the
   *   window's best as long as the FP32 drift stays within its margin (the
   *   filter's model: an Azuma-Hoeffding bound over independent roundings),
   *   plus the rounding of the FP32 direct dot products that chose the
   *   other partners (verified candidates and seeds; not tracked).
   *   -1 for the FP64 form, whose partners are chosen from FP64 recurrence
   *   values (not tracked). */
  double max_abs_r_err;
  double max_tie_margin;
} scamp_c_result;

/* Runs one join.  Inputs and results are HOST memory; the engine copies them
 * to the device, runs every step there and copies the profiles back.
 * Returns SCAMP_OK or an error code; a message goes to errbuf (may be NULL).
 * Replaces SCAMP::do_SCAMP (src/SCAMP.cpp:279-334), whose errors are thrown
 * as SCAMPException (src/common.cpp:417-436, 539-547). */
int scamp_gb300_join(const scamp_c_args *args, scamp_c_result *res,
                     char *errbuf, size_t errlen);

/* Same join with every pointer in args/res being DEVICE memory of
 * args->device, ordered on `stream` (a cudaStream_t, NULL = default stream).
 * Used when the inputs are already resident in HBM.  The call returns once
 * the join has finished on the device: it waits for the join's last event on
 * `stream` to read the timing fields and work counters of `res`. */
int scamp_gb300_join_dev(const scamp_c_args *args, scamp_c_result *res,
                         void *stream, char *errbuf, size_t errlen);

/* Many independent self-joins in one call: count series (args[k], host
 * buffers, has_b = 0, computing rows and columns, no keep_rows, 1NN_INDEX,
 * precision SINGLE or MIXED, one device), each merged into res[k].profile_a
 * (and res[k].corr_a when set).  All series run in one persistent launch of
 * the mixed band kernel, with one statistics, key-conversion and
 * verification launch for the whole batch.  Timing fields and work counters
 * of every res[k] describe the whole batch; comparisons are per series.
 * Extends do_SCAMP (src/SCAMP.cpp:261-334), which takes one join per call. */
int scamp_gb300_join_batch(const scamp_c_args *args, scamp_c_result *res, int count,
                           char *errbuf, size_t errlen);

/* Autotuner of scamp_gb300_join_batch's tile height: for each window length
 * among the count series (same rules as scamp_gb300_join_batch; no result
 * buffers), times the band kernel on a sample of those series at the
 * segment lengths K (rows per half-unit, also the anchor interval) of the
 * cold-start rule (8 m within [1024, 4096]), half and a quarter of it, and
 * keeps the fastest for every later batch on args[0].device.  retune = 0
 * skips windows already tuned.
 * segment (optional, count entries) receives the K each series will use.
 * No counterpart in the reference, which has no batched joins. */
int scamp_gb300_tune_batch(const scamp_c_args *args, int count, int retune, int64_t *segment,
                           char *errbuf, size_t errlen);

/* The FP64 form of scamp_gb300_join_dev without any allocation: every
 * intermediate buffer lives in one static device array of the library
 * (about 8.6 MB per device), so the join calls no allocator.  For callers
 * that must not allocate device memory at join time (a host that gives all
 * device memory to its own pool up front, or a loop that cannot wait on the
 * allocator).  Has no counterpart in the reference.
 *   - series of at most 65536 samples each; precision DOUBLE or ULTRA;
 *     1NN_INDEX or SUM_THRESH; larger or other requests return
 *     SCAMP_ERR_INVALID_ARGS with a message.
 *   - all pointers are device memory of args->device; the work is ordered on
 *     `stream` and not synchronised: results are ready when the stream
 *     reaches the end of this call.  Timing fields and work counters of
 *     `res` are left 0.
 *   - the first call on a device looks up the static array and the SM
 *     count; make it before starting any stream capture.
 *   - calls that overlap on one device (other streams, other threads) race
 *     on the shared array: serialise them on one stream.
 *   - the entry zeroes the array's work counters itself on `stream`; every
 *     other part of the array is written before it is read. */
int scamp_gb300_join_dev_noalloc(const scamp_c_args *args, scamp_c_result *res,
                                 void *stream, char *errbuf, size_t errlen);

/* Checks arguments the way SCAMPArgs::validate does (src/common.cpp:417-436).
 * Pure host logic, needs no GPU. */
int scamp_gb300_validate(const scamp_c_args *args, char *errbuf, size_t errlen);

/* Number of distance-matrix cells a join evaluates (the comparisons of the
 * comparisons/s metric).  Pure host logic. */
uint64_t scamp_gb300_count_cells(const scamp_c_args *args);

/* 1 if a CUDA device is usable (pyscamp gpu_supported,
 * python/SCAMP_python.cpp:363-369). */
int scamp_gb300_gpu_supported(void);

/* Measured throughput of one GPU pipe, for roofline denominators:
 * kind 0 = FP32 FMA lane-ops/s (packed f32x2), 1 = FP64 FMA lane-ops/s.
 * Has no counterpart in the reference. */
int scamp_gb300_pipe_peak(int device, int kind, double *ops_per_s);

/* Window statistics of one series, as every join computes them on the
 * device (compensated FP64): for each of the n - window + 1 windows its mean,
 * inverse norm 1/sqrt(sum of squared differences from the mean), NaN when
 * the window holds a non-finite sample or is flat, and the update terms
 * df[i] = (T[i+m] - T[i]) / 2, dg[i] = (T[i+m] - mean[i+1]) + (T[i] - mean[i])
 * (0 at the last window), non-finite samples counted as 0.
 * high_precision_norms = 1 sums every window directly (ULTRA).  Replaces
 * compute_statistics_cpu (src/cpu_stats.cpp:123-160); host arrays. */
int scamp_gb300_window_stats(int device, const double *series, int64_t n,
                             int64_t window, int high_precision_norms,
                             double *mean, double *invnorm, double *df, double *dg,
                             char *errbuf, size_t errlen);

/* Self-check of the mixed form's tensor-core anchors on `device` (the
 * check every process runs once before its first mixed join of long
 * windows): anchors of a seeded random walk (32768 samples, m = 512) from the
 * split-BF16x3 tcgen05 contraction against FP64 direct dot products.
 * *max_err: the largest |anchor - cov| * invnorm_r * invnorm_c; *available:
 * 1 when the joins use the tensor-core anchors (error within 1e-5), else 0
 * (they use the band kernel's CUDA-core anchors).  Has no counterpart in
 * the reference, whose seeds come from cuFFT (src/qt_helper.cpp:75-121). */
int scamp_gb300_anchor_check(int device, double *max_err, int *available,
                             char *errbuf, size_t errlen);

/* Self-test of the device wait limits on `device`: runs the tensor-core
 * anchor kernel with no MMA issued, so that its bounded wait on the MMA
 * completion barrier (about two seconds) runs out; the kernel sets the
 * error word, waits once more (bounded), frees its tensor memory and
 * returns.  Returns SCAMP_ERR_DEVICE_TIMEOUT when the limit worked (the
 * context stays usable); any other code is a failure.  No counterpart in
 * the reference. */
int scamp_gb300_wait_limit_check(int device, char *errbuf, size_t errlen);

/* Library version string. */
const char *scamp_gb300_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SCAMP_GB300_H */
