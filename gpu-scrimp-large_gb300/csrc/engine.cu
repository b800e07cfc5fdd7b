// engine.cu -- host orchestration of a join and the C ABI (scamp_gb300.h).
//
// Replaces the reference's SCAMP_Operation (src/SCAMP.cpp:25-259) and Tile
// (src/tile.cpp) host machinery.  Where the reference moves every tile's
// series, statistics and best-so-far profile over PCIe and merges on the host
// under a mutex (src/tile.cpp:312-544, src/common.cpp:364-415), this engine
// keeps the whole problem resident in HBM:
//   H2D(series, initial profile) -> stats kernel -> join kernel (persistent,
//   device work queue over every band x segment unit) -> key->profile kernel
//   -> D2H(profile)
// with no host synchronisation in between.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "engine.cuh"
#include "scamp_gb300.h"

namespace scamp_gb300 {

// NVTX range over a phase of a join's host-side enqueueing (header-only
// NVTX3: free unless a profiler is attached), so that a timeline shows the
// statistics, seeding, anchors and band kernel, verification, re-evaluation
// and the copies of every join.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

int fp64_band_width();
int fp64_slab_rows();
int fp64_threads();
int visit_band_width();
int visit_threads();
int mixed_1nn_band_width();
int mixed_1nn_slab_rows();
int mixed_1nn_threads();
size_t mixed_1nn_smem_bytes();
size_t anchor_gemm_smem_bytes(int64_t m_pad);
int64_t anchor_max_window();
int anchor_tile_cols();
int anchor_rows_per_tile();
int measure_pipe_peak(int device, int kind, double* ops_per_s);

namespace {

// Rows between re-anchors of the mixed form: 32 m within [1024, 16384], and
// at least 2 m.  Longer intervals trade anchor dots (m FP32 FMAs per diagonal
// per interval) for exact verifications of the cells whose drift bound
// passes the trust threshold, so the error of the reported values does not
// grow with K.  Measured (time per join, max |r| error vs FP64):
//   AB-join 2^20 x 2^19 random walks, m = 256: K = 2048 107.6 ms, 4096
//     104.9, 8192 104.4, 12288 105.7 (6.6e-6 at every K);
//   self-join of a 2^21 noisy random walk, m = 1024: K = 4096 423 ms, 8192
//     404, 16384 396 (3.0e-6, 3.0e-6, 2.9e-6);
//   2^21 random walk with NaN gaps, m = 4096: K = 8192 533 ms, 16384 509,
//     32768 512 (2.6e-6, 2.5e-6, 2.5e-6);
//   2^21 random walk, m = 128: K = 1024 447 ms, 2048 426, 4096 416; m = 64:
//     K = 1024 601 ms, 2048 583 (3.0e-6 and 2.9e-6 at every K).
int64_t default_anchor_interval(int64_t m) {
  return std::min<int64_t>(std::max<int64_t>(1024, 32 * m), std::max<int64_t>(16384, 2 * m));
}

// Anchor interval of the mixed SUM_THRESH, k-best and matrix-summary joins:
// much shorter, since every cell within its drift margin of the threshold
// (or of a window's k-th best) must be settled one by one, where a 1NN join
// only settles the cells near a window's best.  AB-join of 2^19 x 2^18
// random walks, m = 256, sums above 0.5: K = 8192 (the 1NN rule) 254 ms
// (2.2e7 verifications), 4096 205, 2048 171, 1024 149, 512 139 (1.0e6); above
// 0.9: 119, 110, 105, 104, 109 ms.  k = 5 best above 0.5, 2^18-sample walks:
// self-join K = 8192 / 2048 / 1024 / 512 47.3 / 35.5 / 28.4 / 26.1 ms, AB
// (2^18 x 2^17, both profiles) 192.8 / 102.1 / 48.6 / 36.3 ms; the matrix
// summary's time does not change (29.5-30.1 ms), its stated bound falls.
int64_t short_anchor_interval(int64_t m) { return std::max<int64_t>(512, 2 * m); }

// Windows from which the mixed band kernel filters blocks by the per-step
// covariance bound (join_mixed_1nn.cu, kCoarse) instead of per-cell r: the
// inverse norms of windows that overlap in all but a few samples are close,
// so the bound stays tight.  Band kernel time, per-step bound against
// per-cell filter (flagged 8-row steps in brackets): random walks of 2^21
// samples, m = 64: 3260 / 474 ms (5.5e9 / 1.6e8), m = 256: 990 / 365
// (7.3e8 / 6.5e6), m = 512: 541 / 364 (1.9e8 / 4.0e6); the 2^22-sample
// noisy walk, m = 1024: 1430 / 1458 (1.5e8 / 9.0e6); a 2^21-sample walk
// with NaN gaps, m = 4096: 368 / 412.
constexpr int64_t kCoarseFilterMinWindow = 1024;

// Windows from which the mixed form takes its anchors from the tensor-core
// contraction (anchor_tc.cu) when the anchor interval allows it (a multiple
// of 1024 rows): the CUDA-core anchors cost m FMAs per diagonal per K rows,
// m / (2K) of the recurrence's work, 1/64 at K = 32 m but up to 1/8 where K
// stops growing (m = 4096 at 16384 rows).
constexpr int64_t kTcMinWindow = 512;
// Budget of one chunk's anchor table (bytes); a chunk covers at least 16
// unit rows (32 anchor rows, one tile of the contraction).
constexpr double kTcTableBudget = 4.0 * (1 << 30);
// Unit rows of a chunk of the anchor table: at least this many (a chunk's
// anchor rows fill whole 16-row tiles), down to half of it when a chunk's
// verification requests approach the buffer's capacity.
constexpr int64_t kTcMinChunkRows = 16;
// Mixed MATRIX_SUMMARY: the least windows per grid row and column (a band
// kernel block spans 8 rows and 15 columns).
constexpr int64_t kMatMixedMinSpan = 64;
// Largest |anchor - FP64| inv_r inv_c the self-check accepts.
constexpr double kTcCheckTol = 1e-5;

// Anchor interval of joins that start cold (batched joins: diagonal seeds
// only, the bests still rising through the first slabs): 8 m within [1024,
// 4096].  A longer interval widens the filter margin while many cells are
// still near their rows' and columns' bests.  4096-series batch (lengths
// 2^10-2^16, m in {32, 64, 128}): 1157 ms with 1024 rows for every window,
// 1224 ms with 2048 rows for m = 64 and 128.
int64_t cold_anchor_interval(int64_t m) {
  return std::min<int64_t>(std::max<int64_t>(4096, 2 * m), std::max<int64_t>(1024, 8 * m));
}

// Rows between seeds of the FP64 form.  The FP64 recurrence drifts by
// ~2^-53 per row, so seeds only bound the work lost to them: 32 m rows keep
// the direct-dot seeds at 1/32 of the FP64 pipe's work.
int64_t fp64_segment(int64_t m) { return std::max<int64_t>(32 * m, 8192); }

// Bound on |reported r - FP64 r| after final_eval_kernel: twice
// gamma_{ceil(m/16) + 10} (u = 2^-53) for the direct FP64 evaluation, plus
// the key's resolution 2^-F (final_eval.cu derives it).
double final_eval_bound(int64_t m, int frac_bits) {
  const double u = std::ldexp(1.0, -53);
  const double k = static_cast<double>((m + 15) / 16 + 10);
  return 2.0 * k * u / (1.0 - k * u) + std::ldexp(1.0, -frac_bits);
}

struct Error {
  int code;
  std::string msg;
};

void set_err(char* buf, size_t len, const std::string& msg) {
  if (buf && len) {
    std::snprintf(buf, len, "%s", msg.c_str());
  }
}

// ---------------------------------------------------------------------------
// Host-side planning (no GPU needed).
// ---------------------------------------------------------------------------
struct ProblemPlan {
  int rows_series;  // 0 = A, 1 = B
  int cols_series;
  int64_t n_r, n_c;
  int64_t d_lo, d_hi, x_lo, x_hi;
  int col_target;   // 0 = profile A, 1 = profile B, -1 none
  int row_target;
};

struct Plan {
  bool self_join;
  int64_t m, ns_a, ns_b;
  std::vector<ProblemPlan> probs;
  uint64_t cells;
};

// Mirrors SCAMPArgs::validate (src/common.cpp:417-436) plus the profile and
// precision types this engine serves.
int validate(const scamp_c_args* a, std::string* msg) {
  if (!a) { *msg = "Error: Invalid arguments provided to SCAMP"; return SCAMP_ERR_INVALID_ARGS; }
  if (a->window < 3) { *msg = "Error: Subsequence length must be at least 3"; return SCAMP_ERR_INVALID_ARGS; }
  if (a->max_tile_size < 1024) { *msg = "Error: max tile size must be at least 1024"; return SCAMP_ERR_INVALID_ARGS; }
  if (a->max_tile_size / 2 < a->window) {
    *msg = "Error: Tile length and width must be at least 2x larger than the window size";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (!a->timeseries_a || a->len_a < a->window || (a->has_b && (!a->timeseries_b || a->len_b < a->window))) {
    *msg = "Error: Input time series must be at least 'subesequence window size' in length";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (a->profile_type != SCAMP_PROFILE_1NN_INDEX && a->profile_type != SCAMP_PROFILE_SUM_THRESH &&
      a->profile_type != SCAMP_PROFILE_1NN &&
      a->profile_type != SCAMP_PROFILE_APPROX_ALL_NEIGHBORS &&
      a->profile_type != SCAMP_PROFILE_MATRIX_SUMMARY) {
    *msg = "Error: profile type not supported by this engine";
    return SCAMP_ERR_UNIMPLEMENTED;
  }
  if (a->profile_type == SCAMP_PROFILE_APPROX_ALL_NEIGHBORS &&
      (a->max_matches_per_column < 1 || a->max_matches_per_column > 1024)) {
    *msg = "Error: max_matches_per_column must be between 1 and 1024";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (a->profile_type == SCAMP_PROFILE_MATRIX_SUMMARY &&
      (a->matrix_height <= 0 || a->matrix_width <= 0)) {
    *msg = "Error: matrix height and width must be greater than 0";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (a->precision_type < SCAMP_PRECISION_SINGLE || a->precision_type > SCAMP_PRECISION_ULTRA) {
    *msg = "Error: invalid precision type";
    return SCAMP_ERR_INVALID_ARGS;
  }
  const uint64_t nsa = a->len_a - a->window + 1;
  const uint64_t nsb = a->has_b ? a->len_b - a->window + 1 : nsa;
  if (nsa >= (1ull << 32) || nsb >= (1ull << 32)) {
    *msg = "Error: series longer than 2^32 windows are not supported";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (a->anchor_interval < 0) { *msg = "Error: anchor_interval must be >= 0"; return SCAMP_ERR_INVALID_ARGS; }
  if (a->filter_mode < 0 || a->filter_mode > 2) {
    *msg = "Error: filter_mode must be 0, 1 or 2";
    return SCAMP_ERR_INVALID_ARGS;
  }
  return SCAMP_OK;
}

uint64_t diag_cells(int64_t n_r, int64_t n_c, int64_t d_lo, int64_t d_hi) {
  // sum over d in [d_lo, d_hi) of min(n_r, n_c - d), d_hi <= n_c
  if (d_hi <= d_lo) return 0;
  uint64_t total = 0;
  // part with n_c - d >= n_r  <=> d <= n_c - n_r
  const int64_t split = n_c - n_r;  // d <= split -> n_r rows
  const int64_t a_hi = std::min(d_hi - 1, split);
  if (a_hi >= d_lo) total += static_cast<uint64_t>(a_hi - d_lo + 1) * n_r;
  const int64_t b_lo = std::max(d_lo, split + 1);
  if (b_lo < d_hi) {
    // sum_{d=b_lo}^{d_hi-1} (n_c - d)
    const uint64_t first = n_c - b_lo, last = n_c - (d_hi - 1);
    total += (first + last) * static_cast<uint64_t>(d_hi - b_lo) / 2;
  }
  return total;
}

Plan make_plan(const scamp_c_args* a) {
  Plan p;
  p.self_join = !a->has_b;
  p.m = static_cast<int64_t>(a->window);
  p.ns_a = static_cast<int64_t>(a->len_a - a->window + 1);
  p.ns_b = a->has_b ? static_cast<int64_t>(a->len_b - a->window + 1) : p.ns_a;
  const int64_t excl = p.m / 4;  // src/tile.cpp:14
  p.cells = 0;
  if (p.self_join) {
    // Upper triangle, diagonals >= m/4 (src/tile.cpp:12-38).  Row results go to
    // profile A unless keep_rows_separate (src/tile.cpp:532-541).
    ProblemPlan q{0, 0, p.ns_a, p.ns_a, excl, p.ns_a, 0, 0,
                  a->computing_columns ? 0 : -1,
                  a->computing_rows ? (a->keep_rows_separate ? 1 : 0) : -1};
    if (q.d_hi > q.d_lo) p.probs.push_back(q);
  } else {
    const int col_t = a->computing_columns ? 0 : -1;
    const int row_t = (a->computing_rows && a->keep_rows_separate) ? 1 : -1;
    // Above the main diagonal: rows = B, cols = A.  Below it, transposed:
    // rows = A, cols = B, diagonals >= 1 (src/tile.cpp:645-707).
    ProblemPlan up{1, 0, p.ns_b, p.ns_a, 0, p.ns_a, 0, 0, col_t, row_t};
    ProblemPlan lo{0, 1, p.ns_a, p.ns_b, 1, p.ns_b, 0, 0, row_t, col_t};
    if (a->is_aligned) {
      // Trivial-match exclusion |global_col - global_row| < m/4.  The
      // reference decides it per tile from the tile's corners
      // (src/tile.cpp:12-19, 44-138): the same cells when the global
      // offsets differ by a multiple of its tile width (the tiles of its
      // distributed joins); for other offsets its zone is shifted or
      // missing, depending on its tile width.
      int64_t off = 0;
      if (a->distributed_start_row >= 0 && a->distributed_start_col >= 0)
        off = a->distributed_start_col - a->distributed_start_row;
      up.x_lo = -off - excl + 1;
      up.x_hi = -off + excl;
      lo.x_lo = off - excl + 1;
      lo.x_hi = off + excl;
    }
    if (up.d_hi > up.d_lo && (up.col_target >= 0 || up.row_target >= 0)) p.probs.push_back(up);
    if (lo.d_hi > lo.d_lo && (lo.col_target >= 0 || lo.row_target >= 0)) p.probs.push_back(lo);
  }
  for (const auto& q : p.probs) {
    uint64_t c = diag_cells(q.n_r, q.n_c, q.d_lo, q.d_hi);
    // excluded diagonals inside the range
    const int64_t xl = std::max(q.x_lo, q.d_lo), xh = std::min(q.x_hi, q.d_hi);
    if (xh > xl) c -= diag_cells(q.n_r, q.n_c, xl, xh);
    p.cells += c;
  }
  return p;
}

KeyLayout make_key_layout(int64_t ns_max) {
  KeyLayout kl;
  int bits = 1;
  while ((1ll << bits) < ns_max + 1) ++bits;
  bits = std::max(bits, 20);
  kl.idx_bits = bits;
  kl.frac_bits = 62 - bits;
  kl.idx_mask = (1ull << bits) - 1;
  return kl;
}

// ---------------------------------------------------------------------------
// Device workspace (grow-only, one per device, one join at a time).
// ---------------------------------------------------------------------------
struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct Workspace {
  std::mutex mu;
  int device = -1;
  int sms = 0;
  std::vector<Buf> bufs;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t evk0 = nullptr, evk1 = nullptr;  // around the join kernels
  cudaEvent_t evkv = nullptr;                   // before the verification kernel
  bool timed_kernel = false;
  bool timed_verify = false;
  // the mixed form's largest trusted drift margin (work counter 4) is the
  // join's max_tie_margin (1NN) or max_abs_r_err (SUM_THRESH)
  bool tracked_tie_margin = false;
  bool tracked_sum_margin = false;
  // Tensor-core anchors: 0 = not checked yet, 1 = checked (tc_desc_mode
  // holds the descriptor orientation that matched FP64), 2 = unavailable;
  // tc_check_err: the self-check's max |anchor - FP64| inv_r inv_c.
  int tc_state = 0;
  int tc_desc_mode = 0;
  double tc_check_err = 0.0;
  // Verification requests of the mixed 1NN join: capacity of the buffer, and
  // the largest count a join asked for (the buffer grows to it on the next
  // join; requests beyond the capacity are verified inline, more slowly).
  int64_t vreq_cap = 0;
  int64_t vreq_seen = 0;
  // Batched joins: the executable graph of the last batch layout (replayed
  // while the layout repeats) and the autotuned segment length per window.
  cudaGraphExec_t batch_exec = nullptr;
  std::vector<int64_t> batch_key;
  std::map<int64_t, int64_t> batch_seg;
  // Pinned host staging of the batched joins' copies (grow-only): the
  // gathered series in, the profiles in and out, the correlations out.
  std::vector<Buf> pinned;
};

constexpr int64_t kMinVerifyReqs = int64_t{1} << 22;
constexpr int64_t kMaxVerifyReqs = int64_t{1} << 30;  // 16 GiB of requests

Workspace g_ws[64];

// Pinned host buffer `slot` of at least `bytes` (grow-only; no copy may be in
// flight on the old one: the batched join ends with a stream sync).
int ensure_pinned(Workspace& ws, size_t slot, size_t bytes, void** out, std::string* msg) {
  if (ws.pinned.size() <= slot) ws.pinned.resize(slot + 1);
  Buf& b = ws.pinned[slot];
  if (b.bytes < bytes) {
    if (b.p) cudaFreeHost(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (cudaHostAlloc(&b.p, bytes, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      *msg = "Error: out of pinned host memory";
      return SCAMP_ERR_OUT_OF_MEMORY;
    }
    b.bytes = bytes;
  }
  *out = b.p;
  return SCAMP_OK;
}

int ensure(Workspace& ws, size_t slot, size_t bytes, void** out, std::string* msg) {
  if (ws.bufs.size() <= slot) ws.bufs.resize(slot + 1);
  Buf& b = ws.bufs[slot];
  if (b.bytes < bytes) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    const size_t want = std::max<size_t>(bytes, 256);
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
      cudaGetLastError();
      *msg = "Error: out of device memory allocating " + std::to_string(want) + " bytes";
      return SCAMP_ERR_OUT_OF_MEMORY;
    }
    b.bytes = want;
  }
  *out = b.p;
  return SCAMP_OK;
}

enum Slot {
  S_RAW_A, S_RAW_B,
  S_T_A, S_MEAN_A, S_INV_A, S_DF_A, S_DG_A, S_INV32_A, S_DF32_A, S_DG32_A,
  S_T_B, S_MEAN_B, S_INV_B, S_DF_B, S_DG_B, S_INV32_B, S_DF32_B, S_DG32_B,
  S_KEY_A, S_KEY_B, S_SUM_A, S_SUM_B, S_PROF_A, S_PROF_B, S_CORR_A, S_CORR_B,
  S_PREFIX, S_COUNTER, S_T32_A, S_T32_B, S_BHI_A, S_BLO_A, S_MUREL_A,
  S_BHI_B, S_BLO_B, S_MUREL_B, S_VREQ, S_PAA_A, S_PAA_B, S_SEED_A, S_SEED_B,
  S_BATCH, S_MAX_A, S_MAX_B, S_KNN_A, S_KNN_B, S_MAT,
  S_TC_TAB, S_TC_W, S_TC_XS, S_TC_RAW, S_TC_OUT, S_TC_XI,
};

#define CUDA_TRY(expr)                                                     \
  do {                                                                     \
    cudaError_t e_ = (expr);                                               \
    if (e_ != cudaSuccess) {                                               \
      *msg = std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " \
             + #expr;                                                      \
      return SCAMP_ERR_CUDA;                                               \
    }                                                                      \
  } while (0)

// Device outputs of the profile types beyond 1NN_INDEX and SUM_THRESH.
struct ExtraOut {
  float* max[2] = {nullptr, nullptr};     // 1NN: best correlation per window
  uint64_t* knn[2] = {nullptr, nullptr};  // APPROX_ALL_NEIGHBORS: k entries per window
  float* matrix = nullptr;                // MATRIX_SUMMARY: height x width
};

struct SeriesBufs {
  double *T, *mean, *inv, *df, *dg;
  float *inv32, *df32, *dg32, *T32, *bhi, *blo, *mu_rel;
  int bshift;
};

// Block size of the locally offset FP32 copy: 32 samples, or m/16 for long
// windows (a window then spans at most 17 blocks).
int block_shift(int64_t m) {
  int s = 5;
  while ((1ll << s) * 16 < m) ++s;
  return s;
}

int alloc_series(Workspace& ws, int which, int64_t n, int64_t ns, SeriesBufs* s,
                 std::string* msg) {
  const int base = which == 0 ? S_T_A : S_T_B;
  void* p;
  int rc;
  if ((rc = ensure(ws, base + 0, n * 8, &p, msg))) return rc; s->T = (double*)p;
  if ((rc = ensure(ws, base + 1, ns * 8, &p, msg))) return rc; s->mean = (double*)p;
  if ((rc = ensure(ws, base + 2, ns * 8, &p, msg))) return rc; s->inv = (double*)p;
  if ((rc = ensure(ws, base + 3, ns * 8, &p, msg))) return rc; s->df = (double*)p;
  if ((rc = ensure(ws, base + 4, ns * 8, &p, msg))) return rc; s->dg = (double*)p;
  if ((rc = ensure(ws, base + 5, ns * 4, &p, msg))) return rc; s->inv32 = (float*)p;
  if ((rc = ensure(ws, base + 6, ns * 4, &p, msg))) return rc; s->df32 = (float*)p;
  if ((rc = ensure(ws, base + 7, ns * 4, &p, msg))) return rc; s->dg32 = (float*)p;
  if ((rc = ensure(ws, which == 0 ? S_T32_A : S_T32_B, n * 4, &p, msg))) return rc; s->T32 = (float*)p;
  const int64_t nblk = (n >> s->bshift) + 1;
  if ((rc = ensure(ws, which == 0 ? S_BHI_A : S_BHI_B, nblk * 4, &p, msg))) return rc; s->bhi = (float*)p;
  if ((rc = ensure(ws, which == 0 ? S_BLO_A : S_BLO_B, nblk * 4, &p, msg))) return rc; s->blo = (float*)p;
  if ((rc = ensure(ws, which == 0 ? S_MUREL_A : S_MUREL_B, ns * 4, &p, msg))) return rc; s->mu_rel = (float*)p;
  return SCAMP_OK;
}

SeriesDev to_dev(const SeriesBufs& s, int64_t n, int64_t ns) {
  SeriesDev d;
  d.T = s.T; d.mean = s.mean; d.inv = s.inv; d.df = s.df; d.dg = s.dg;
  d.inv32 = s.inv32; d.df32 = s.df32; d.dg32 = s.dg32;
  d.T32 = s.T32; d.bhi = s.bhi; d.blo = s.blo; d.mu_rel = s.mu_rel; d.bshift = s.bshift;
  d.n = n; d.ns = ns;
  return d;
}

// One problem's chunk of tensor-core anchors: anchor rows s0 .. s0 + nrows
// - 1 of the row series against every diagonal of the problem, into `table`
// (nrows x wp_pad floats, the layout of anchor_tc.cu).
int tc_anchor_chunk(Workspace& ws, const Problem& pr, int64_t K, int64_t s0, int64_t nrows,
                    int64_t wp_pad, float* table, int* error_flag, int desc_mode,
                    cudaStream_t st, std::string* msg, AnchorArgs* out_args = nullptr,
                    int wait_test = 0) {
  AnchorArgs A{};
  A.wait_test = wait_test;
  A.R = pr.R;
  A.C = pr.C;
  A.m = pr.m;
  A.m_pad = (pr.m + 15) / 16 * 16;
  A.K = K;
  A.d_lo = pr.d_lo;
  A.s0 = s0;
  A.nrows = nrows;
  const int64_t rpt = anchor_rows_per_tile();
  A.rows_pad = (nrows + rpt - 1) / rpt * rpt;
  A.wp_pad = wp_pad;
  A.col_tiles = ((rpt - 1) * K + wp_pad) / anchor_tile_cols();
  A.table = table;
  A.error_flag = error_flag;
  A.desc_mode = desc_mode;
  A.nsub = (A.m_pad + 63) / 64;
  void* p;
  int rc;
  if ((rc = ensure(ws, S_TC_XI, static_cast<size_t>(A.rows_pad * A.nsub) * 4, &p, msg))) return rc;
  A.xi = static_cast<float*>(p);
  if ((rc = ensure(ws, S_TC_W, static_cast<size_t>(3 * A.rows_pad * A.m_pad) * 2, &p, msg))) return rc;
  A.wsplit = static_cast<__nv_bfloat16*>(p);
  if ((rc = ensure(ws, S_TC_XS, static_cast<size_t>(A.rows_pad) * 4, &p, msg))) return rc;
  A.xsum = static_cast<float*>(p);
  anchor_split_kernel<<<static_cast<unsigned>(A.rows_pad), 256, 0, st>>>(A);
  const size_t smem = anchor_gemm_smem_bytes(A.m_pad);
  CUDA_TRY(cudaFuncSetAttribute(reinterpret_cast<const void*>(anchor_gemm_kernel),
                                cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int64_t tiles = (A.rows_pad / rpt) * A.col_tiles;
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(ws.sms, tiles));
  anchor_gemm_kernel<<<static_cast<unsigned>(grid), 128, smem, st>>>(A);
  CUDA_TRY(cudaGetLastError());
  if (out_args) *out_args = A;
  return SCAMP_OK;
}

// Self-check of the tensor-core anchors, once per device: a seeded random
// walk (32768 samples, m = 512, anchor interval 1024) is joined's anchors
// computed both ways; the descriptor orientation whose table matches FP64
// direct dots to kTcCheckTol is kept, else the tensor-core path stays off
// (the band kernel's own anchors serve every join).  Uses the series-A
// slots (the join computes its statistics afterwards) and synchronises.
int tc_self_check(Workspace& ws, cudaStream_t st, std::string* msg, bool wait_test = false) {
  constexpr int64_t n = 32768, m = 512, K = 1024;
  std::vector<double> x(n);
  uint64_t z = 0x9E3779B97F4A7C15ull;
  double v = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    // xorshift increments, uniform in [-0.5, 0.5): a random walk
    z ^= z << 13;
    z ^= z >> 7;
    z ^= z << 17;
    v += static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    x[static_cast<size_t>(i)] = v;
  }
  void* p;
  int rc;
  if ((rc = ensure(ws, S_TC_RAW, n * 8, &p, msg))) return rc;
  double* raw = static_cast<double*>(p);
  CUDA_TRY(cudaMemcpyAsync(raw, x.data(), n * 8, cudaMemcpyHostToDevice, st));
  const int64_t ns = n - m + 1;
  SeriesBufs sb{};
  sb.bshift = block_shift(m);
  if ((rc = alloc_series(ws, 0, n, ns, &sb, msg))) return rc;
  const int chunk = 64;
  stats_kernel<<<static_cast<unsigned>(((ns + chunk - 1) / chunk + 127) / 128), 128, 0, st>>>(
      raw, n, m, 0, chunk, sb.bshift, sb.T, sb.T32, sb.bhi, sb.blo, sb.mu_rel, sb.mean, sb.inv,
      sb.df, sb.dg, sb.inv32, sb.df32, sb.dg32);
  CUDA_TRY(cudaGetLastError());
  Problem pr{};
  pr.R = pr.C = to_dev(sb, n, ns);
  pr.d_lo = m / 4;
  pr.d_hi = ns;
  pr.m = m;
  const int64_t nrows = 32;
  const int64_t wp_pad = (ns - pr.d_lo + 1023) / 1024 * 1024;
  if ((rc = ensure(ws, S_TC_TAB, static_cast<size_t>(nrows * wp_pad) * 4, &p, msg))) return rc;
  float* table = static_cast<float*>(p);
  if ((rc = ensure(ws, S_TC_OUT, 64, &p, msg))) return rc;
  unsigned long long* out = static_cast<unsigned long long*>(p);
  int* flag = reinterpret_cast<int*>(out + 4);
  if (wait_test) {
    // the contraction with no MMA issued: its first bounded wait must give
    // up, set the error word and return
    CUDA_TRY(cudaMemsetAsync(out, 0, 64, st));
    if ((rc = tc_anchor_chunk(ws, pr, K, 0, nrows, wp_pad, table, flag, ws.tc_desc_mode, st, msg,
                              nullptr, 1)))
      return rc;
    int h = 0;
    CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (h != 0) {
      *msg = "Error: a wait on the tensor cores timed out on the device (wait-limit self-test)";
      return SCAMP_ERR_DEVICE_TIMEOUT;
    }
    *msg = "Error: the wait-limit self-test finished without its wait running out";
    return SCAMP_ERR_CUDA;
  }
  ws.tc_state = 2;
  for (int mode = 0; mode < 2; ++mode) {
    CUDA_TRY(cudaMemsetAsync(out, 0, 64, st));
    CUDA_TRY(cudaMemsetAsync(table, 0, static_cast<size_t>(nrows * wp_pad) * 4, st));
    AnchorArgs A{};
    if ((rc = tc_anchor_chunk(ws, pr, K, 0, nrows, wp_pad, table, flag, mode, st, msg, &A))) return rc;
    anchor_check_kernel<<<static_cast<unsigned>(ws.sms * 4), 256, 0, st>>>(A, 7, out);
    CUDA_TRY(cudaGetLastError());
    unsigned long long h[5] = {0, 0, 0, 0, 0};
    CUDA_TRY(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    double err;
    std::memcpy(&err, &h[0], 8);
    if (static_cast<int>(h[4] & 0xFFFFFFFFull) != 0) {
      *msg = "Error: tensor-core anchor self-check timed out on the device";
      return SCAMP_ERR_DEVICE_TIMEOUT;
    }
    if (mode == 0 || err < ws.tc_check_err) ws.tc_check_err = h[1] > 1000 ? err : 1.0;
    if (h[1] > 1000 && err <= kTcCheckTol) {
      ws.tc_state = 1;
      ws.tc_desc_mode = mode;
      ws.tc_check_err = err;
      break;
    }
  }
  return SCAMP_OK;
}

// Runs a join whose inputs are device pointers; profile_a/b (packed entries)
// and sum_a/b are device pointers too and are merged in place.
// Seeding pre-pass of the mixed 1NN join: when and how.  The block-averaged
// join costs ~1/64 of the join's cells; below a few 1e9 cells it does not pay.
constexpr float kSeedFloor = 0.8f;  // partners below it are not worth a seed
// Shortest window seeded by the pre-pass (single joins and batches): below
// it the averaged windows (< 16 samples) pair blocks almost at random.
constexpr int64_t kSeedMinWindow = 64;

// Block size of the pre-pass: the largest power of two <= m / 16 within
// [4, 64] (window m / f of about 16 samples).  On the AB-join of 2^20 x 2^19
// random walks at m = 256: no seeds 138.6 ms, f = 8: 127.1, f = 16: 126.2.
int seed_factor(int64_t m) {
  int f = 4;
  while (f < 64 && 2 * f * 16 <= m) f *= 2;
  return f;
}
constexpr uint64_t kSeedMinCells = uint64_t{4} << 30;

// Seedable configurations: a self-join into one profile, or an AB join
// (columns, and rows when kept separately), without alignment offsets.
bool seedable(const scamp_c_args* a, const Plan& plan) {
  if (a->is_aligned || a->distributed_start_row >= 0 || a->distributed_start_col >= 0) return false;
  if (plan.m < kSeedMinWindow || plan.cells < kSeedMinCells) return false;
  if (!a->computing_columns) return false;
  if (plan.self_join) return a->computing_rows && !a->keep_rows_separate;
  return !a->computing_rows || a->keep_rows_separate;
}

int run_device(Workspace& ws, const scamp_c_args* a, scamp_c_result* res,
               const double* dA, const double* dB, uint64_t* dprof_a,
               uint64_t* dprof_b, double* dsum_a, double* dsum_b,
               double* dcorr_a, double* dcorr_b, cudaStream_t st,
               std::string* msg, bool nested = false, const ExtraOut* ex = nullptr);

// Block-averaged join of the inputs (window m / 8) into the seed profiles
// S_SEED_A/B; returns their device pointers (seed_b null when not kept).
int seed_prepass(Workspace& ws, const scamp_c_args* a, const Plan& plan, const double* dA,
                 const double* dB, cudaStream_t st, uint64_t** seed_a, uint64_t** seed_b,
                 int64_t* ns_a, int64_t* ns_b, uint32_t* launches, std::string* msg) {
  const int f = seed_factor(plan.m);
  const int64_t na = static_cast<int64_t>(a->len_a) / f;
  const int64_t nb = a->has_b ? static_cast<int64_t>(a->len_b) / f : 0;
  const int64_t m2 = plan.m / f;
  const bool want_b = a->has_b && a->keep_rows_separate && a->computing_rows;
  void *pa, *pb = nullptr, *qa, *qb = nullptr;
  int rc;
  if ((rc = ensure(ws, S_PAA_A, na * 8, &pa, msg))) return rc;
  paa_kernel<<<static_cast<unsigned>((na + 255) / 256), 256, 0, st>>>(dA, na, f, static_cast<double*>(pa));
  ++*launches;
  if (a->has_b) {
    if ((rc = ensure(ws, S_PAA_B, nb * 8, &pb, msg))) return rc;
    paa_kernel<<<static_cast<unsigned>((nb + 255) / 256), 256, 0, st>>>(dB, nb, f, static_cast<double*>(pb));
    ++*launches;
  }
  *ns_a = na - m2 + 1;
  *ns_b = a->has_b ? nb - m2 + 1 : *ns_a;
  if ((rc = ensure(ws, S_SEED_A, *ns_a * 8, &qa, msg))) return rc;
  fill_floor_kernel<<<static_cast<unsigned>((*ns_a + 255) / 256), 256, 0, st>>>(
      static_cast<uint64_t*>(qa), *ns_a, kSeedFloor);
  ++*launches;
  if (want_b) {
    if ((rc = ensure(ws, S_SEED_B, *ns_b * 8, &qb, msg))) return rc;
    fill_floor_kernel<<<static_cast<unsigned>((*ns_b + 255) / 256), 256, 0, st>>>(
        static_cast<uint64_t*>(qb), *ns_b, kSeedFloor);
    ++*launches;
  }
  CUDA_TRY(cudaGetLastError());
  scamp_c_args a2 = *a;
  a2.timeseries_a = static_cast<double*>(pa);
  a2.len_a = static_cast<uint64_t>(na);
  a2.timeseries_b = a->has_b ? static_cast<double*>(pb) : nullptr;
  a2.len_b = static_cast<uint64_t>(nb);
  a2.window = static_cast<uint64_t>(m2);
  a2.precision_type = SCAMP_PRECISION_MIXED;
  a2.profile_type = SCAMP_PROFILE_1NN_INDEX;
  a2.anchor_interval = 0;
  a2.silent_mode = 1;
  scamp_c_result r2{};
  rc = run_device(ws, &a2, &r2, static_cast<double*>(pa),
                  a->has_b ? static_cast<double*>(pb) : static_cast<double*>(pa),
                  static_cast<uint64_t*>(qa), static_cast<uint64_t*>(qb), nullptr, nullptr,
                  nullptr, nullptr, st, msg, true);
  if (rc) return rc;
  *launches += r2.gpu_launches;
  *seed_a = static_cast<uint64_t*>(qa);
  *seed_b = static_cast<uint64_t*>(qb);
  return SCAMP_OK;
}

int run_device(Workspace& ws, const scamp_c_args* a, scamp_c_result* res,
               const double* dA, const double* dB, uint64_t* dprof_a,
               uint64_t* dprof_b, double* dsum_a, double* dsum_b,
               double* dcorr_a, double* dcorr_b, cudaStream_t st,
               std::string* msg, bool nested, const ExtraOut* ex) {
  scamp_c_args a_local;
  if (a->profile_type == SCAMP_PROFILE_MATRIX_SUMMARY) {
    // matrix summaries reduce along the columns only (src/common.cpp:98-105)
    a_local = *a;
    a_local.computing_rows = 0;
    a_local.keep_rows_separate = 0;
    a = &a_local;
  }
  Plan plan = make_plan(a);
  // 1NN (float best correlation, no index) runs as 1NN_INDEX on the keys;
  // the k-best and matrix-summary types run the FP64 visit kernel
  const bool max_only = a->profile_type == SCAMP_PROFILE_1NN;
  const bool is_1nn = a->profile_type == SCAMP_PROFILE_1NN_INDEX || max_only;
  const bool mixed = a->precision_type == SCAMP_PRECISION_MIXED ||
                     a->precision_type == SCAMP_PRECISION_SINGLE;
  // MATRIX_SUMMARY grid: rows are windows of B (of A in a self-join),
  // columns windows of A.  The mixed form takes the band kernel's per-cell
  // maxima when grid entries span enough windows that most of its 8 x 15
  // blocks fall inside one; else (and in FP64) the visit kernel serves it.
  const bool is_mat = a->profile_type == SCAMP_PROFILE_MATRIX_SUMMARY;
  const int64_t mat_rpc = is_mat ? (plan.ns_b + a->matrix_height - 1) / a->matrix_height : 1;
  const int64_t mat_cpc = is_mat ? (plan.ns_a + a->matrix_width - 1) / a->matrix_width : 1;
  const bool mat_mixed = is_mat && mixed && mat_rpc >= kMatMixedMinSpan &&
                         mat_cpc >= kMatMixedMinSpan && std::max(plan.ns_a, plan.ns_b) < (int64_t{1} << 31) &&
                         static_cast<int64_t>(a->matrix_height) * a->matrix_width < (int64_t{1} << 31);
  // APPROX_ALL_NEIGHBORS in the mixed form: the band kernel with k-best
  // lists (up to knn_mixed_max_k() entries); else the visit kernel
  const bool is_knn = a->profile_type == SCAMP_PROFILE_APPROX_ALL_NEIGHBORS;
  const bool knn_mixed = is_knn && mixed && a->max_matches_per_column >= 1 &&
                         a->max_matches_per_column <= knn_mixed_max_k();
  const bool visit = (is_knn && !knn_mixed) || (is_mat && !mat_mixed);
  const bool ultra = a->precision_type == SCAMP_PRECISION_ULTRA;
  const int64_t m = plan.m;
  const int64_t na = static_cast<int64_t>(a->len_a);
  const int64_t nb = a->has_b ? static_cast<int64_t>(a->len_b) : na;
  uint32_t launches = 0;
  int rc;

  if (!nested) {
    ws.timed_kernel = false;
    ws.timed_verify = false;
    // the tensor-core anchors' one-time self-check (before this join's own
    // statistics, whose buffers it borrows)
    if (mixed && !visit && ws.tc_state == 0 && a->anchor_mode != 1 &&
        (a->anchor_mode == 2 || m >= kTcMinWindow)) {
      if ((rc = tc_self_check(ws, st, msg))) return rc;
    }
    CUDA_TRY(cudaEventRecord(ws.ev0, st));
  }

  // ---- seeds: block-averaged pre-pass (mixed 1NN joins that pay for it) ----
  NvtxRange nvtx_join(nested ? "seeding pre-pass join" : "join");
  uint64_t *seed_a = nullptr, *seed_b = nullptr;
  int64_t seed_ns_a = 0, seed_ns_b = 0;
  if (!nested && mixed && is_1nn && seedable(a, plan)) {
    if ((rc = seed_prepass(ws, a, plan, dA, dB, st, &seed_a, &seed_b, &seed_ns_a, &seed_ns_b,
                           &launches, msg)))
      return rc;
  }

  // ---- statistics ----
  nvtxRangePushA("statistics");
  SeriesBufs sa{}, sb{};
  sa.bshift = sb.bshift = block_shift(m);
  if ((rc = alloc_series(ws, 0, na, plan.ns_a, &sa, msg))) return rc;
  const int chunk = 64;
  {
    const int64_t threads = (plan.ns_a + chunk - 1) / chunk;
    stats_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(
        dA, na, m, ultra ? 1 : 0, chunk, sa.bshift, sa.T, sa.T32, sa.bhi, sa.blo, sa.mu_rel,
        sa.mean, sa.inv, sa.df, sa.dg, sa.inv32, sa.df32, sa.dg32);
    launches += 1;
  }
  if (a->has_b) {
    if ((rc = alloc_series(ws, 1, nb, plan.ns_b, &sb, msg))) return rc;
    const int64_t threads = (plan.ns_b + chunk - 1) / chunk;
    stats_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(
        dB, nb, m, ultra ? 1 : 0, chunk, sb.bshift, sb.T, sb.T32, sb.bhi, sb.blo, sb.mu_rel,
        sb.mean, sb.inv, sb.df, sb.dg, sb.inv32, sb.df32, sb.dg32);
    launches += 1;
  } else {
    sb = sa;
  }
  // ULTRA: the reference's combined update terms (combined_stats_kernel):
  // A's "A" terms, B's "B" terms; a self-join's rows take the "B" terms of A,
  // held in series B's (otherwise unused) df/dg buffers.
  double *ultra_row_df = nullptr, *ultra_row_dg = nullptr;
  if (ultra) {
    combined_stats_kernel<<<static_cast<unsigned>((plan.ns_a + 255) / 256), 256, 0, st>>>(
        sa.T, na, m, sa.mean, 0, sa.df, sa.dg);
    ++launches;
    if (a->has_b) {
      combined_stats_kernel<<<static_cast<unsigned>((plan.ns_b + 255) / 256), 256, 0, st>>>(
          sb.T, nb, m, sb.mean, 1, sb.df, sb.dg);
    } else {
      void* p;
      if ((rc = ensure(ws, S_DF_B, plan.ns_a * 8, &p, msg))) return rc;
      ultra_row_df = static_cast<double*>(p);
      if ((rc = ensure(ws, S_DG_B, plan.ns_a * 8, &p, msg))) return rc;
      ultra_row_dg = static_cast<double*>(p);
      combined_stats_kernel<<<static_cast<unsigned>((plan.ns_a + 255) / 256), 256, 0, st>>>(
          sa.T, na, m, sa.mean, 1, ultra_row_df, ultra_row_dg);
    }
    ++launches;
  }
  CUDA_TRY(cudaGetLastError());
  nvtxRangePop();
  SeriesDev devA = to_dev(sa, na, plan.ns_a);
  SeriesDev devB = to_dev(sb, nb, plan.ns_b);
  SeriesDev devArows = devA;  // series A in the row role
  if (ultra_row_df) {
    devArows.df = ultra_row_df;
    devArows.dg = ultra_row_dg;
  }

  // ---- profiles: packed entries -> merge keys ----
  const KeyLayout kl = make_key_layout(std::max(plan.ns_a, plan.ns_b));
  uint64_t* keys[2] = {nullptr, nullptr};
  double* sums[2] = {dsum_a, dsum_b};
  uint64_t* profs[2] = {dprof_a, dprof_b};
  const int64_t nsz[2] = {plan.ns_a, plan.ns_b};
  bool used[2] = {false, false};
  for (const auto& q : plan.probs) {
    if (q.col_target >= 0) used[q.col_target] = true;
    if (q.row_target >= 0) used[q.row_target] = true;
  }
  float* maxs[2] = {ex ? ex->max[0] : nullptr, ex ? ex->max[1] : nullptr};
  unsigned long long* vkeys[2] = {nullptr, nullptr};
  unsigned* vmat = nullptr;
  const int64_t knn_k = a->max_matches_per_column;
  const int64_t mat_n = static_cast<int64_t>(a->matrix_height) * a->matrix_width;
  if (is_knn) {
    for (int s = 0; s < 2; ++s) {
      if (!used[s]) continue;
      if (!ex || !ex->knn[s]) { *msg = "Error: profile buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
      void* p;
      if ((rc = ensure(ws, s == 0 ? S_KNN_A : S_KNN_B, nsz[s] * knn_k * 8, &p, msg))) return rc;
      vkeys[s] = static_cast<unsigned long long*>(p);
      profile_to_keys_kernel<<<static_cast<unsigned>((nsz[s] * knn_k + 255) / 256), 256, 0, st>>>(
          ex->knn[s], reinterpret_cast<uint64_t*>(vkeys[s]), nsz[s] * knn_k, kl);
      ++launches;
    }
  } else if (is_mat) {
    if (!ex || !ex->matrix) { *msg = "Error: profile buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
    void* p;
    if ((rc = ensure(ws, S_MAT, mat_n * 4, &p, msg))) return rc;
    vmat = static_cast<unsigned*>(p);
    floats_to_ord_kernel<<<static_cast<unsigned>((mat_n + 255) / 256), 256, 0, st>>>(
        ex->matrix, vmat, mat_n);
    ++launches;
  } else if (is_1nn) {
    for (int s = 0; s < 2; ++s) {
      if (max_only) {
        if (!used[s] && !(s == 0 && maxs[0])) continue;
        if (!maxs[s]) { *msg = "Error: profile buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
      } else {
        if (!used[s] && !(s == 0 && profs[0])) continue;
        if (!profs[s]) { *msg = "Error: profile buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
      }
      void* p;
      if ((rc = ensure(ws, s == 0 ? S_KEY_A : S_KEY_B, nsz[s] * 8, &p, msg))) return rc;
      keys[s] = static_cast<uint64_t*>(p);
      if (max_only)
        floats_to_keys_kernel<<<static_cast<unsigned>((nsz[s] + 255) / 256), 256, 0, st>>>(
            maxs[s], keys[s], nsz[s], kl);
      else
        profile_to_keys_kernel<<<static_cast<unsigned>((nsz[s] + 255) / 256), 256, 0, st>>>(
            profs[s], keys[s], nsz[s], kl);
      ++launches;
    }
  } else {
    for (int s = 0; s < 2; ++s)
      if (used[s] && !sums[s]) { *msg = "Error: sum buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
  }

  // ---- seeds merged into the keys ----
  if (seed_a) {
    const int64_t excl = plan.self_join ? plan.m / 4 : -1;
    auto launch_seed = [&](const SeriesDev& X, const SeriesDev& Y, const uint64_t* paa,
                           int64_t ns_paa, uint64_t* kx, uint64_t* ky) {
      const SeedArgs S{X, Y, paa, ns_paa, kx, ky, excl, m, kl, kSeedFloor, seed_factor(m)};
      const int64_t blocks = std::min<int64_t>((X.ns + 7) / 8, static_cast<int64_t>(ws.sms) * 16);
      seed_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(S);
      ++launches;
    };
    if (plan.self_join) {
      launch_seed(devA, devA, seed_a, seed_ns_a, keys[0], keys[0]);
    } else {
      launch_seed(devA, devB, seed_a, seed_ns_a, keys[0], seed_b ? keys[1] : nullptr);
      if (seed_b) launch_seed(devB, devA, seed_b, seed_ns_b, keys[1], keys[0]);
    }
    CUDA_TRY(cudaGetLastError());
  }

  // ---- work plan ----
  // Kernel choice: FP64 form, or the mixed band kernel (FP32 filter; for
  // 1NN_INDEX its candidates are verified, for SUM_THRESH the filter
  // threshold is the sum threshold and every cell above it is accumulated).
  // The k-best and matrix-summary types run the FP64 visit kernel.
  enum { K_FP64, K_MIXED, K_VISIT } kind = visit ? K_VISIT : !mixed ? K_FP64 : K_MIXED;
  // (SUM_THRESH keeps the per-cell filter unless asked: its fast path adds
  // the blocks that lie wholly above the threshold, which needs per-cell r)
  const bool coarse = kind == K_MIXED && !is_mat && !is_knn &&
                      (a->filter_mode == 2 ||
                       (a->filter_mode == 0 && is_1nn && m >= kCoarseFilterMinWindow));
  const void* kfn = kind == K_VISIT ? reinterpret_cast<const void*>(join_visit_kernel)
                  : kind == K_FP64 ? reinterpret_cast<const void*>(join_fp64_kernel)
                  : is_mat ? reinterpret_cast<const void*>(join_mixed_mat_kernel)
                  : is_knn ? reinterpret_cast<const void*>(join_mixed_knn_kernel)
                  : is_1nn ? (coarse ? reinterpret_cast<const void*>(join_mixed_1nn_coarse_kernel)
                                     : reinterpret_cast<const void*>(join_mixed_1nn_kernel))
                           : (coarse ? reinterpret_cast<const void*>(join_mixed_sum_coarse_kernel)
                                     : reinterpret_cast<const void*>(join_mixed_sum_kernel));
  const int W = kind == K_VISIT ? visit_band_width()
              : kind == K_FP64 ? fp64_band_width() : mixed_1nn_band_width();
  const int slab = kind == K_MIXED ? mixed_1nn_slab_rows() : fp64_slab_rows();
  const int nthreads = kind == K_VISIT ? visit_threads()
                     : kind == K_FP64 ? fp64_threads() : mixed_1nn_threads();
  const size_t smem = kind == K_MIXED ? mixed_1nn_smem_bytes() : 0;
  if (smem > 0)
    CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem)));
  int occ = 1;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, nthreads, smem));
  occ = std::max(occ, 1);
  const int64_t resident = static_cast<int64_t>(ws.sms) * occ;
  // Segment length K: the anchor interval for the mixed form, the seed
  // interval (fp64_segment) for FP64.  Both shrink (down to one slab) when
  // the join is too small to give every resident CTA ~8 units.
  int64_t K;
  const double cells_d = static_cast<double>(plan.cells);
  const int64_t k_lb = static_cast<int64_t>(cells_d / (8.0 * resident * 2.0 * W));
  if (kind == K_MIXED) {
    K = a->anchor_interval > 0 ? a->anchor_interval
                               : (is_1nn ? default_anchor_interval(m) : short_anchor_interval(m));
  } else {
    K = fp64_segment(m);
  }
  K = std::min(K, std::max<int64_t>(k_lb, slab));
  K = std::max<int64_t>(slab, (K / slab) * slab);
  {
    // The mixed 1NN kernel pairs the two segments of a unit; their column
    // spans must be a whole number of FP32-copy blocks apart.
    const int64_t blk = 1ll << block_shift(m);
    if (K % blk) K = std::max<int64_t>(blk, (K / blk) * blk);
  }
  // Tensor-core anchors need an anchor interval of whole 1024-column tiles.
  const bool tc_eligible = kind == K_MIXED && !nested && ws.tc_state == 1 &&
                           (m + 15) / 16 * 16 <= anchor_max_window() &&
                           (a->anchor_mode == 2 || (a->anchor_mode == 0 && m >= kTcMinWindow));
  if (tc_eligible && K >= 1024) K = K / 1024 * 1024;

  JoinParams P{};
  std::vector<int64_t> prefix;
  prefix.push_back(0);
  int64_t band_total = 0;
  P.nprob = 0;
  for (const auto& q : plan.probs) {
    Problem& pr = P.prob[P.nprob++];
    pr.R = q.rows_series == 0 ? devArows : devB;
    pr.C = q.cols_series == 0 ? devA : devB;
    pr.d_lo = q.d_lo; pr.d_hi = q.d_hi; pr.x_lo = q.x_lo; pr.x_hi = q.x_hi;
    pr.key_col = is_1nn && q.col_target >= 0 ? keys[q.col_target] : nullptr;
    pr.key_row = is_1nn && q.row_target >= 0 ? keys[q.row_target] : nullptr;
    if (knn_mixed) {
      pr.key_col = q.col_target >= 0 ? reinterpret_cast<uint64_t*>(vkeys[q.col_target]) : nullptr;
      pr.key_row = q.row_target >= 0 ? reinterpret_cast<uint64_t*>(vkeys[q.row_target]) : nullptr;
    }
    pr.sum_col = !is_1nn && q.col_target >= 0 ? sums[q.col_target] : nullptr;
    pr.sum_row = !is_1nn && q.row_target >= 0 ? sums[q.row_target] : nullptr;
    pr.band_begin = band_total;
    pr.nbands = (q.d_hi - q.d_lo + W - 1) / W;
    pr.m = m;
    pr.seg_len = K;
    for (int64_t b = 0; b < pr.nbands; ++b) {
      const int64_t D0 = q.d_lo + b * W;
      const int64_t rows = band_rows(q.n_r, q.n_c, D0);
      const int64_t units = (rows + 2 * K - 1) / (2 * K);
      prefix.push_back(prefix.back() + units);
    }
    band_total += pr.nbands;
  }
  P.total_bands = band_total;
  P.total_units = prefix.back();
  P.m = m;
  P.seg_len = K;
  P.band_width = W;
  P.profile_type = is_1nn ? SCAMP_PROFILE_1NN_INDEX : a->profile_type;
  // a join without seeds starts cold: the band kernel refreshes its ring
  // columns' bests every slab (seeded joins start near their final bests)
  P.refresh_cols = (kind == K_MIXED && ((is_1nn && !seed_a) || knn_mixed)) ? 1 : 0;
  P.knn_k = knn_mixed ? static_cast<int>(knn_k) : 0;
  P.threshold = a->distance_threshold;
  P.kl = kl;
  if (mat_mixed) {
    P.mat = vmat;
    P.mat_w = a->matrix_width;
    P.rows_per_cell = mat_rpc;
    P.cols_per_cell = mat_cpc;
    // ceil(2^64 / d) for d >= 2
    P.rpc_magic = UINT64_MAX / static_cast<uint64_t>(mat_rpc) + 1;
    P.cpc_magic = UINT64_MAX / static_cast<uint64_t>(mat_cpc) + 1;
    for (int p = 0; p < P.nprob; ++p) {
      P.mat_col[p] = plan.probs[p].col_target == 0 ? 1 : 0;
      P.mat_row[p] = plan.probs[p].row_target == 0 ? 1 : 0;
    }
  }
  // Tensor-core anchors (anchor_tc.cu): mixed joins of long windows whose
  // anchor interval is a multiple of the contraction's 1024-column tiles.
  const bool use_tc = tc_eligible && K % 1024 == 0;
  {
    // FP32 anchor: blocks of up to 2^bshift terms, then the block sums; the
    // tensor-core contraction instead rounds its hi*hi accumulator m/16 times
    // (the five small products go to a second accumulator).
    const double blk = static_cast<double>(1 << sa.bshift);
    const double e = use_tc ? std::sqrt(m / 16.0 + 1.0) + std::sqrt(std::ceil(m / blk) + 1.0) + 1.0
                            : std::sqrt(std::min<double>(m, blk)) + std::sqrt(std::ceil(m / blk) + 1.0);
    P.anchor_vcoef = static_cast<float>(e * e / 8.0);  // per 8-row step units
    for (int p = 0; p < P.nprob; ++p) P.prob[p].anchor_vcoef = P.anchor_vcoef;
  }

  if (!a->silent_mode) {
    std::printf("scamp_gb300: %s %s join, m=%lld, %s, %llu cells, %lld units of %d diagonals x 2x%lld rows\n",
                plan.self_join ? "self" : "AB", is_1nn ? "1NN_INDEX" : "SUM_THRESH",
                static_cast<long long>(m), mixed ? "mixed" : "fp64",
                static_cast<unsigned long long>(plan.cells),
                static_cast<long long>(P.total_units), W, static_cast<long long>(K));
  }

  if (P.total_units > 0) {
    NvtxRange nvtx_band("anchors, band kernel, verification");
    void* p;
    if ((rc = ensure(ws, S_PREFIX, prefix.size() * 8, &p, msg))) return rc;
    int64_t* dprefix = static_cast<int64_t*>(p);
    CUDA_TRY(cudaMemcpyAsync(dprefix, prefix.data(), prefix.size() * 8, cudaMemcpyHostToDevice, st));
    if ((rc = ensure(ws, S_COUNTER, 64, &p, msg))) return rc;
    CUDA_TRY(cudaMemsetAsync(p, 0, 64, st));
    P.band_unit_prefix = dprefix;
    P.unit_counter = static_cast<unsigned long long*>(p);
    P.counters = static_cast<unsigned long long*>(p) + 1;
    P.error_flag = reinterpret_cast<int*>(static_cast<char*>(p) + 48);
    if (kind == K_MIXED) {
      // random-walk-like series ask for ~7 (K = 512) to ~18 (K = 1024)
      // 1NN requests per window
      // (k-best lists: a window keeps k candidates open, and cold lists
      // ask for more)
      int64_t want = std::max<int64_t>(kMinVerifyReqs, 32 * (nsz[0] + nsz[1]) *
                                                           (knn_mixed ? 4 * knn_k : 1));
      want = std::max<int64_t>(want, ws.vreq_seen + ws.vreq_seen / 4);
      want = std::max<int64_t>(std::min<int64_t>(want, kMaxVerifyReqs), ws.vreq_cap);
      void* q;
      if ((rc = ensure(ws, S_VREQ, static_cast<size_t>(want) * sizeof(VerifyReq), &q, msg)))
        return rc;
      ws.vreq_cap = want;
      P.vreq = static_cast<VerifyReq*>(q);
      P.vreq_cap = want;
    }
    const int64_t grid = std::min<int64_t>(resident, P.total_units);
    if (!nested) {
      CUDA_TRY(cudaEventRecord(ws.evk0, st));
      ws.timed_kernel = true;
    }
    auto launch_band = [&](const JoinParams& Q, int64_t g) {
      if (is_mat)
        join_mixed_mat_kernel<<<static_cast<unsigned>(g), nthreads, smem, st>>>(Q);
      else if (is_knn)
        join_mixed_knn_kernel<<<static_cast<unsigned>(g), nthreads, smem, st>>>(Q);
      else if (is_1nn && coarse)
        join_mixed_1nn_coarse_kernel<<<static_cast<unsigned>(g), nthreads, smem, st>>>(Q);
      else if (is_1nn)
        join_mixed_1nn_kernel<<<static_cast<unsigned>(g), nthreads, smem, st>>>(Q);
      else if (coarse)
        join_mixed_sum_coarse_kernel<<<static_cast<unsigned>(g), nthreads, smem, st>>>(Q);
      else
        join_mixed_sum_kernel<<<static_cast<unsigned>(g), nthreads, smem, st>>>(Q);
      ++launches;
    };
    if (kind == K_MIXED && use_tc) {
      // Chunks of unit rows (every band's units ub in [u0, u0 + U)): the
      // tensor-core contraction fills the chunk's anchor table (anchor rows
      // 2 u0 .. 2 (u0 + U) - 1 of every problem), then one band-kernel launch
      // runs the chunk's units with their anchors read from it.
      int64_t wp[kMaxProblems] = {0, 0}, wsum = 0, urows = 0;
      for (int p = 0; p < P.nprob; ++p) {
        wp[p] = P.prob[p].nbands * W;
        wsum += wp[p];
        const int64_t rows0 = band_rows(P.prob[p].R.ns, P.prob[p].C.ns, P.prob[p].d_lo);
        urows = std::max<int64_t>(urows, (rows0 + 2 * K - 1) / (2 * K));
      }
      int64_t U = static_cast<int64_t>(kTcTableBudget / (8.0 * static_cast<double>(wsum)));
      U = std::max<int64_t>(kTcMinChunkRows, U / kTcMinChunkRows * kTcMinChunkRows);
      void* tp;
      if ((rc = ensure(ws, S_TC_TAB, static_cast<size_t>(2 * U * wsum) * 4, &tp, msg))) return rc;
      float* tab = static_cast<float*>(tp);
      std::vector<int64_t> cpre;
      for (int64_t u0 = 0, Uc = U; u0 < urows; u0 += Uc, Uc = U) {
        cpre.assign(1, 0);
        for (int p = 0; p < P.nprob; ++p) {
          const Problem& pr = P.prob[p];
          for (int64_t b = 0; b < pr.nbands; ++b) {
            const int64_t rows = band_rows(pr.R.ns, pr.C.ns, pr.d_lo + b * W);
            const int64_t ub = (rows + 2 * K - 1) / (2 * K);
            cpre.push_back(cpre.back() + std::max<int64_t>(0, std::min<int64_t>(ub - u0, Uc)));
          }
        }
        const int64_t cunits = cpre.back();
        if (cunits == 0) continue;
        JoinParams Q = P;
        Q.total_units = cunits;
        Q.unit_row0 = u0;
        float* tp_p = tab;
        for (int p = 0; p < P.nprob; ++p) {
          const int64_t s0 = 2 * u0;
          const int64_t srows = std::max<int64_t>(
              0, std::min<int64_t>(2 * Uc, (band_rows(P.prob[p].R.ns, P.prob[p].C.ns, P.prob[p].d_lo) +
                                           K - 1) / K - s0));
          Q.prob[p].anchor_tab = tp_p;
          Q.prob[p].tab_wp = wp[p];
          Q.prob[p].tab_s0 = s0;
          if (srows > 0 && (rc = tc_anchor_chunk(ws, P.prob[p], K, s0, srows, wp[p], tp_p,
                                                 P.error_flag, ws.tc_desc_mode, st, msg)))
            return rc;
          launches += srows > 0 ? 2 : 0;
          tp_p += 2 * Uc * wp[p];
        }
        CUDA_TRY(cudaMemcpyAsync(dprefix, cpre.data(), cpre.size() * 8, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemsetAsync(P.unit_counter, 0, 8, st));
        launch_band(Q, std::min<int64_t>(resident, cunits));
        if (u0 + Uc < urows && !is_mat) {
          // the chunk's deferred verifications now, so that the request
          // buffer only ever holds one chunk's requests (a long join's would
          // overflow it); the last chunk's go to the verification below
          verify_requests_kernel<<<static_cast<unsigned>(ws.sms * 8), 256, 0, st>>>(P);
          ++launches;
          // a chunk that filled more than half of the buffer: later chunks
          // take fewer unit rows (their tables fit the one allocated)
          unsigned long long nreq = 0;
          CUDA_TRY(cudaMemcpyAsync(&nreq, P.counters + 3, 8, cudaMemcpyDeviceToHost, st));
          CUDA_TRY(cudaStreamSynchronize(st));
          ws.vreq_seen = std::max<int64_t>(ws.vreq_seen, static_cast<int64_t>(nreq));
          while (2 * static_cast<int64_t>(nreq) > P.vreq_cap && U > kTcMinChunkRows / 2) {
            U /= 2;
            nreq /= 2;
          }
          CUDA_TRY(cudaMemsetAsync(P.counters + 3, 0, 8, st));
        }
      }
      CUDA_TRY(cudaGetLastError());
    } else if (kind == K_MIXED) {
      launch_band(P, grid);
    }
    if (kind == K_MIXED) {
      if (!nested) {
        CUDA_TRY(cudaEventRecord(ws.evkv, st));
        ws.timed_verify = true;
      }
      // (the matrix form makes no requests: it publishes its maxima directly)
      if (!is_mat) {
        verify_requests_kernel<<<static_cast<unsigned>(ws.sms * 8), 256, 0, st>>>(P);
        ++launches;
      }
    } else if (kind == K_VISIT) {
      VisitArgs V{};
      V.mode = a->profile_type == SCAMP_PROFILE_APPROX_ALL_NEIGHBORS ? 0 : 1;
      V.topk[0] = vkeys[0];
      V.topk[1] = vkeys[1];
      V.k = static_cast<int>(knn_k);
      V.mat = vmat;
      V.mat_w = a->matrix_width;
      // grid rows: windows of B (of A in a self-join), columns: windows of A
      V.rows_per_cell = V.mode == 1 ? (nsz[1] + a->matrix_height - 1) / a->matrix_height : 1;
      V.cols_per_cell = V.mode == 1 ? (nsz[0] + a->matrix_width - 1) / a->matrix_width : 1;
      for (int p = 0; p < P.nprob; ++p) {
        V.col_target[p] = plan.probs[p].col_target;
        V.row_target[p] = plan.probs[p].row_target;
      }
      join_visit_kernel<<<static_cast<unsigned>(grid), nthreads, 0, st>>>(P, V);
      ++launches;
    } else {
      join_fp64_kernel<<<static_cast<unsigned>(grid), nthreads, 0, st>>>(P);
      ++launches;
    }
    CUDA_TRY(cudaGetLastError());
    if (!nested) CUDA_TRY(cudaEventRecord(ws.evk1, st));
  }

  // ---- FP64 re-evaluation of every reported cell (1NN types) ----
  if (is_1nn) {
    NvtxRange nvtx_eval("FP64 re-evaluation");
    EvalPair E{};
    E.m = m;
    E.kl = kl;
    for (int s = 0; s < 2; ++s) {
      if (!keys[s]) continue;
      EvalSide& es = E.side[s];
      es.keys = keys[s];
      es.prof_in = max_only ? nullptr : profs[s];
      es.max_in = max_only ? maxs[s] : nullptr;
      es.X = s == 0 ? devA : devB;
      es.Y = plan.self_join ? devA : (s == 0 ? devB : devA);
      es.ns = nsz[s];
      es.m = m;
    }
    const int64_t nwin = E.side[0].ns + E.side[1].ns;
    if (nwin > 0) {
      const int64_t blocks = std::min<int64_t>((nwin + 31) / 32, static_cast<int64_t>(ws.sms) * 16);
      final_eval_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(E);
      ++launches;
    }
  }

  // ---- FP64 re-evaluation of the mixed form's k-best lists ----
  if (knn_mixed) {
    NvtxRange nvtx_eval("FP64 re-evaluation");
    for (int s = 0; s < 2; ++s) {
      if (!vkeys[s] || nsz[s] == 0) continue;
      EvalSide es{};
      es.keys = reinterpret_cast<uint64_t*>(vkeys[s]);
      es.prof_in = ex->knn[s];
      es.X = s == 0 ? devA : devB;
      es.Y = plan.self_join ? devA : (s == 0 ? devB : devA);
      es.ns = nsz[s];
      es.m = m;
      const int64_t blocks = std::min<int64_t>((nsz[s] + 31) / 32, static_cast<int64_t>(ws.sms) * 16);
      knn_final_eval_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(
          es, static_cast<int>(knn_k), a->distance_threshold, kl);
      ++launches;
    }
  }

  // ---- keys -> packed entries (+ optional double correlations) ----
  for (int s = 0; s < 2; ++s) {
    if (!vkeys[s]) continue;
    keys_to_profile_kernel<<<static_cast<unsigned>((nsz[s] * knn_k + 255) / 256), 256, 0, st>>>(
        reinterpret_cast<const uint64_t*>(vkeys[s]), ex->knn[s], nullptr, nsz[s] * knn_k, kl);
    ++launches;
  }
  if (vmat) {
    ord_to_floats_kernel<<<static_cast<unsigned>((mat_n + 255) / 256), 256, 0, st>>>(
        vmat, ex->matrix, mat_n);
    ++launches;
  }
  if (is_1nn) {
    double* corr[2] = {dcorr_a, dcorr_b};
    for (int s = 0; s < 2; ++s) {
      if (!keys[s]) continue;
      if (max_only)
        keys_to_floats_kernel<<<static_cast<unsigned>((nsz[s] + 255) / 256), 256, 0, st>>>(
            keys[s], maxs[s], corr[s], nsz[s], kl);
      else
        keys_to_profile_kernel<<<static_cast<unsigned>((nsz[s] + 255) / 256), 256, 0, st>>>(
            keys[s], profs[s], corr[s], nsz[s], kl);
      ++launches;
    }
  }
  CUDA_TRY(cudaGetLastError());
  if (!nested) CUDA_TRY(cudaEventRecord(ws.ev1, st));
  if (res) {
    res->comparisons = plan.cells;
    res->gpu_launches = launches;
    // accuracy fields; the mixed form's tracked margin is read with the
    // work counters (read_times)
    const bool fp64_final = is_1nn || knn_mixed;  // values recomputed in FP64
    res->max_abs_r_err = fp64_final ? final_eval_bound(m, kl.frac_bits) : (kind == K_MIXED ? 0.0 : -1.0);
    res->max_tie_margin = (fp64_final && kind == K_MIXED) ? 0.0 : -1.0;
  }
  if (!nested) {
    ws.tracked_sum_margin = !is_1nn && !knn_mixed && kind == K_MIXED;
    ws.tracked_tie_margin = (is_1nn || knn_mixed) && kind == K_MIXED;
  }
  return SCAMP_OK;
}

// Timing fields, work counters and the device error word of the last join
// (SCAMP_ERR_DEVICE_TIMEOUT when a bounded wait on the device gave up).
int read_times(Workspace& ws, scamp_c_result* res, std::string* msg = nullptr) {
  res->steps = res->slow_steps = res->verifications = 0;
  res->inplace_verifications = 0;
  int status = SCAMP_OK;
  if (ws.timed_kernel && ws.bufs.size() > S_COUNTER && ws.bufs[S_COUNTER].p) {
    unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (cudaMemcpy(c, ws.bufs[S_COUNTER].p, sizeof(c), cudaMemcpyDeviceToHost) == cudaSuccess) {
      res->steps = c[1];
      res->slow_steps = c[2];
      res->verifications = c[3];
      res->inplace_verifications = static_cast<uint32_t>(std::min<unsigned long long>(c[7], UINT32_MAX));
      ws.vreq_seen = std::max<int64_t>(ws.vreq_seen, static_cast<int64_t>(c[4] + c[7]));
      float tm;
      const uint32_t bits = static_cast<uint32_t>(c[5]);
      std::memcpy(&tm, &bits, 4);
      if (ws.tracked_tie_margin) res->max_tie_margin = tm;
      if (ws.tracked_sum_margin) res->max_abs_r_err = tm;
      if (static_cast<uint32_t>(c[6]) != 0) {
        status = SCAMP_ERR_DEVICE_TIMEOUT;
        if (msg) *msg = "Error: a wait on the tensor cores timed out on the device";
      }
    }
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, ws.ev0, ws.ev1);
  res->elapsed_ms = ms;
  res->join_kernel_ms = 0;
  res->verify_kernel_ms = 0;
  if (ws.timed_kernel) {
    float k = 0;
    cudaEventElapsedTime(&k, ws.evk0, ws.evk1);
    res->join_kernel_ms = k;
    if (ws.timed_verify) {
      cudaEventElapsedTime(&k, ws.evkv, ws.evk1);
      res->verify_kernel_ms = k;
    }
  }
  return status;
}

int init_workspace(int device, Workspace** out, std::string* msg) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    *msg = "Error: no CUDA device available (this engine has no CPU fallback)";
    return SCAMP_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev || device >= 64) {
    *msg = "Error: invalid device ordinal";
    return SCAMP_ERR_INVALID_ARGS;
  }
  Workspace& ws = g_ws[device];
  CUDA_TRY(cudaSetDevice(device));
  if (ws.device < 0) {
    CUDA_TRY(cudaDeviceGetAttribute(&ws.sms, cudaDevAttrMultiProcessorCount, device));
    CUDA_TRY(cudaStreamCreateWithFlags(&ws.stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&ws.ev0));
    CUDA_TRY(cudaEventCreate(&ws.ev1));
    CUDA_TRY(cudaEventCreate(&ws.evk0));
    CUDA_TRY(cudaEventCreate(&ws.evk1));
    CUDA_TRY(cudaEventCreate(&ws.evkv));
    ws.device = device;
  }
  *out = &ws;
  return SCAMP_OK;
}

}  // namespace
}  // namespace scamp_gb300

using namespace scamp_gb300;

extern "C" int scamp_gb300_validate(const scamp_c_args* args, char* errbuf, size_t errlen) {
  std::string msg;
  const int rc = validate(args, &msg);
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

extern "C" uint64_t scamp_gb300_count_cells(const scamp_c_args* args) {
  std::string msg;
  if (validate(args, &msg)) return 0;
  return make_plan(args).cells;
}

extern "C" int scamp_gb300_gpu_supported(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n > 0 ? 1 : 0;
}

extern "C" const char* scamp_gb300_version(void) { return "scamp_gb300 0.1.0 (sm_103a)"; }

extern "C" int scamp_gb300_anchor_check(int device, double* max_err, int* available,
                                        char* errbuf, size_t errlen) {
  std::string msg;
  Workspace* ws;
  int rc = init_workspace(device, &ws, &msg);
  if (rc == SCAMP_OK) {
    std::lock_guard<std::mutex> lock(ws->mu);
    ws->tc_state = 0;
    rc = tc_self_check(*ws, ws->stream, &msg);
    if (rc == SCAMP_OK) {
      if (max_err) *max_err = ws->tc_check_err;
      if (available) *available = ws->tc_state == 1 ? 1 : 0;
    }
  }
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

extern "C" int scamp_gb300_wait_limit_check(int device, char* errbuf, size_t errlen) {
  std::string msg;
  Workspace* ws;
  int rc = init_workspace(device, &ws, &msg);
  if (rc == SCAMP_OK) {
    std::lock_guard<std::mutex> lock(ws->mu);
    rc = tc_self_check(*ws, ws->stream, &msg, true);
  }
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

namespace scamp_gb300 {
// The statistics kernel of the joins on one host series, results copied back.
int window_stats(Workspace& ws, const double* series, int64_t n, int64_t m, int ultra,
                 double* mean, double* invnorm, double* df, double* dg, std::string* msg) {
  cudaStream_t st = ws.stream;
  const int64_t ns = n - m + 1;
  void* p;
  int rc;
  if ((rc = ensure(ws, S_RAW_A, n * 8, &p, msg))) return rc;
  double* raw = static_cast<double*>(p);
  CUDA_TRY(cudaMemcpyAsync(raw, series, n * 8, cudaMemcpyHostToDevice, st));
  SeriesBufs sb{};
  sb.bshift = block_shift(m);
  if ((rc = alloc_series(ws, 0, n, ns, &sb, msg))) return rc;
  const int chunk = 64;
  const int64_t threads = (ns + chunk - 1) / chunk;
  stats_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(
      raw, n, m, ultra, chunk, sb.bshift, sb.T, sb.T32, sb.bhi, sb.blo, sb.mu_rel, sb.mean,
      sb.inv, sb.df, sb.dg, sb.inv32, sb.df32, sb.dg32);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(mean, sb.mean, ns * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(invnorm, sb.inv, ns * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(df, sb.df, ns * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(dg, sb.dg, ns * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return SCAMP_OK;
}
}  // namespace scamp_gb300

extern "C" int scamp_gb300_window_stats(int device, const double* series, int64_t n,
                                        int64_t window, int high_precision_norms,
                                        double* mean, double* invnorm, double* df, double* dg,
                                        char* errbuf, size_t errlen) {
  std::string msg;
  if (!series || !mean || !invnorm || !df || !dg || window < 3 || n < window) {
    set_err(errbuf, errlen, "Error: window statistics need a series of at least `window` >= 3 "
                            "samples and four output arrays");
    return SCAMP_ERR_INVALID_ARGS;
  }
  Workspace* ws;
  int rc = init_workspace(device, &ws, &msg);
  if (rc == SCAMP_OK) {
    std::lock_guard<std::mutex> lock(ws->mu);
    rc = window_stats(*ws, series, n, window, high_precision_norms ? 1 : 0, mean, invnorm, df,
                      dg, &msg);
  }
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

extern "C" int scamp_gb300_pipe_peak(int device, int kind, double* ops_per_s) {
  if (!ops_per_s || (kind != 0 && kind != 1)) return SCAMP_ERR_INVALID_ARGS;
  return measure_pipe_peak(device, kind, ops_per_s) ? SCAMP_ERR_CUDA : SCAMP_OK;
}

extern "C" int scamp_gb300_join_dev(const scamp_c_args* args, scamp_c_result* res,
                                    void* stream, char* errbuf, size_t errlen) {
  std::string msg;
  int rc = validate(args, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  Workspace* ws;
  if ((rc = init_workspace(args->device, &ws, &msg))) { set_err(errbuf, errlen, msg); return rc; }
  std::lock_guard<std::mutex> lock(ws->mu);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ExtraOut ex;
  ex.max[0] = res->max_a;
  ex.max[1] = res->max_b;
  ex.knn[0] = res->knn_a;
  ex.knn[1] = res->knn_b;
  ex.matrix = res->matrix;
  rc = run_device(*ws, args, res, args->timeseries_a, args->has_b ? args->timeseries_b : args->timeseries_a,
                  res->profile_a, res->profile_b, res->sum_a, res->sum_b, res->corr_a, res->corr_b, st, &msg,
                  false, &ex);
  if (rc == SCAMP_OK) {
    cudaError_t e = cudaEventSynchronize(ws->ev1);
    if (e != cudaSuccess) { msg = std::string("CUDA error: ") + cudaGetErrorString(e); rc = SCAMP_ERR_CUDA; }
    else {
      rc = read_times(*ws, res, &msg);
    }
  }
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

extern "C" int scamp_gb300_join(const scamp_c_args* args, scamp_c_result* res,
                                char* errbuf, size_t errlen) {
  std::string msg;
  int rc = validate(args, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  if (!res) { set_err(errbuf, errlen, "Error: result struct missing"); return SCAMP_ERR_INVALID_ARGS; }
  Workspace* ws;
  if ((rc = init_workspace(args->device, &ws, &msg))) { set_err(errbuf, errlen, msg); return rc; }
  std::lock_guard<std::mutex> lock(ws->mu);
  cudaStream_t st = ws->stream;
  const bool is_1nn = args->profile_type == SCAMP_PROFILE_1NN_INDEX;
  const bool max_only = args->profile_type == SCAMP_PROFILE_1NN;
  const bool knn = args->profile_type == SCAMP_PROFILE_APPROX_ALL_NEIGHBORS;
  const bool matrix = args->profile_type == SCAMP_PROFILE_MATRIX_SUMMARY;
  const int64_t na = static_cast<int64_t>(args->len_a);
  const int64_t nb = args->has_b ? static_cast<int64_t>(args->len_b) : 0;
  const int64_t nsa = na - static_cast<int64_t>(args->window) + 1;
  const int64_t nsb = args->has_b ? nb - static_cast<int64_t>(args->window) + 1 : nsa;
  auto fail = [&](int code) { set_err(errbuf, errlen, msg); return code; };
#define HOST_CUDA(expr)                                                       \
  do {                                                                        \
    cudaError_t e_ = (expr);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      msg = std::string("CUDA error: ") + cudaGetErrorString(e_);             \
      return fail(SCAMP_ERR_CUDA);                                            \
    }                                                                         \
  } while (0)
  NvtxRange nvtx_call("scamp_gb300_join");
  void *pa, *pb = nullptr;
  if ((rc = ensure(*ws, S_RAW_A, na * 8, &pa, &msg))) return fail(rc);
  HOST_CUDA(cudaMemcpyAsync(pa, args->timeseries_a, na * 8, cudaMemcpyHostToDevice, st));
  if (args->has_b) {
    if ((rc = ensure(*ws, S_RAW_B, nb * 8, &pb, &msg))) return fail(rc);
    HOST_CUDA(cudaMemcpyAsync(pb, args->timeseries_b, nb * 8, cudaMemcpyHostToDevice, st));
  }
  const bool want_b = args->keep_rows_separate != 0 && !matrix;
  uint64_t *dprof[2] = {nullptr, nullptr};
  double *dsum[2] = {nullptr, nullptr}, *dcorr[2] = {nullptr, nullptr};
  ExtraOut ex;
  float* hmax[2] = {res->max_a, res->max_b};
  uint64_t* hknn[2] = {res->knn_a, res->knn_b};
  const int64_t kk = args->max_matches_per_column;
  const int64_t mat_n = static_cast<int64_t>(args->matrix_height) * args->matrix_width;
  if (matrix) {
    void* p;
    if (!res->matrix) { msg = "Error: profile buffer missing"; return fail(SCAMP_ERR_INVALID_ARGS); }
    if ((rc = ensure(*ws, S_MAX_A, mat_n * 4, &p, &msg))) return fail(rc);
    ex.matrix = static_cast<float*>(p);
    HOST_CUDA(cudaMemcpyAsync(p, res->matrix, mat_n * 4, cudaMemcpyHostToDevice, st));
  }
  uint64_t* hprof[2] = {res->profile_a, res->profile_b};
  double* hsum[2] = {res->sum_a, res->sum_b};
  double* hcorr[2] = {res->corr_a, res->corr_b};
  const int64_t nsz[2] = {nsa, nsb};
  for (int s = 0; s < 2 && !matrix; ++s) {
    if (s == 1 && !want_b) continue;
    void* p;
    if (knn) {
      if (!hknn[s]) { msg = "Error: profile buffer missing"; return fail(SCAMP_ERR_INVALID_ARGS); }
      if ((rc = ensure(*ws, s ? S_PROF_B : S_PROF_A, nsz[s] * kk * 8, &p, &msg))) return fail(rc);
      ex.knn[s] = static_cast<uint64_t*>(p);
      HOST_CUDA(cudaMemcpyAsync(p, hknn[s], nsz[s] * kk * 8, cudaMemcpyHostToDevice, st));
    } else if (max_only) {
      if (!hmax[s]) { msg = "Error: profile buffer missing"; return fail(SCAMP_ERR_INVALID_ARGS); }
      if ((rc = ensure(*ws, s ? S_MAX_B : S_MAX_A, nsz[s] * 4, &p, &msg))) return fail(rc);
      ex.max[s] = static_cast<float*>(p);
      HOST_CUDA(cudaMemcpyAsync(p, hmax[s], nsz[s] * 4, cudaMemcpyHostToDevice, st));
      if (hcorr[s]) {
        if ((rc = ensure(*ws, s ? S_CORR_B : S_CORR_A, nsz[s] * 8, &p, &msg))) return fail(rc);
        dcorr[s] = static_cast<double*>(p);
      }
    } else if (is_1nn) {
      if (!hprof[s]) { msg = "Error: profile buffer missing"; return fail(SCAMP_ERR_INVALID_ARGS); }
      if ((rc = ensure(*ws, s ? S_PROF_B : S_PROF_A, nsz[s] * 8, &p, &msg))) return fail(rc);
      dprof[s] = static_cast<uint64_t*>(p);
      HOST_CUDA(cudaMemcpyAsync(p, hprof[s], nsz[s] * 8, cudaMemcpyHostToDevice, st));
      if (hcorr[s]) {
        if ((rc = ensure(*ws, s ? S_CORR_B : S_CORR_A, nsz[s] * 8, &p, &msg))) return fail(rc);
        dcorr[s] = static_cast<double*>(p);
      }
    } else {
      if (!hsum[s]) { msg = "Error: sum buffer missing"; return fail(SCAMP_ERR_INVALID_ARGS); }
      if ((rc = ensure(*ws, s ? S_SUM_B : S_SUM_A, nsz[s] * 8, &p, &msg))) return fail(rc);
      dsum[s] = static_cast<double*>(p);
      HOST_CUDA(cudaMemcpyAsync(p, hsum[s], nsz[s] * 8, cudaMemcpyHostToDevice, st));
    }
  }
  rc = run_device(*ws, args, res, static_cast<double*>(pa),
                  args->has_b ? static_cast<double*>(pb) : static_cast<double*>(pa),
                  dprof[0], dprof[1], dsum[0], dsum[1], dcorr[0], dcorr[1], st, &msg,
                  false, &ex);
  if (rc) return fail(rc);
  if (matrix) HOST_CUDA(cudaMemcpyAsync(res->matrix, ex.matrix, mat_n * 4, cudaMemcpyDeviceToHost, st));
  for (int s = 0; s < 2 && !matrix; ++s) {
    if (s == 1 && !want_b) continue;
    if (knn) {
      HOST_CUDA(cudaMemcpyAsync(hknn[s], ex.knn[s], nsz[s] * kk * 8, cudaMemcpyDeviceToHost, st));
    } else if (max_only) {
      HOST_CUDA(cudaMemcpyAsync(hmax[s], ex.max[s], nsz[s] * 4, cudaMemcpyDeviceToHost, st));
      if (hcorr[s]) HOST_CUDA(cudaMemcpyAsync(hcorr[s], dcorr[s], nsz[s] * 8, cudaMemcpyDeviceToHost, st));
    } else if (is_1nn) {
      HOST_CUDA(cudaMemcpyAsync(hprof[s], dprof[s], nsz[s] * 8, cudaMemcpyDeviceToHost, st));
      if (hcorr[s]) HOST_CUDA(cudaMemcpyAsync(hcorr[s], dcorr[s], nsz[s] * 8, cudaMemcpyDeviceToHost, st));
    } else {
      HOST_CUDA(cudaMemcpyAsync(hsum[s], dsum[s], nsz[s] * 8, cudaMemcpyDeviceToHost, st));
    }
  }
  HOST_CUDA(cudaStreamSynchronize(st));
  if ((rc = read_times(*ws, res, &msg))) return fail(rc);
  return SCAMP_OK;
#undef HOST_CUDA
}

// ---------------------------------------------------------------------------
// Join without allocation (scamp_gb300_join_dev_noalloc).
//
// Some callers cannot let the engine allocate device memory at join time: a
// host whose device memory is all handed to its own pool before any work
// starts, or a loop that must never wait on the allocator (cudaMalloc and
// cudaFree can synchronise the whole device and stall every other stream).
// For them this entry runs the FP64 join with every intermediate buffer
// (statistics, merge keys, the work-queue prefix and counters) carved from
// one static device array, so that nothing is allocated per call.  The array
// bounds each series to kNoAllocMaxSamples samples.
// ---------------------------------------------------------------------------
namespace scamp_gb300 {
namespace {

constexpr int64_t kNoAllocMaxSamples = int64_t{1} << 16;
constexpr int64_t kNoAllocPrefixCap = 1024;   // band prefix entries
constexpr size_t kNoAllocAlign = 256;

constexpr size_t noalloc_round(size_t b) { return (b + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
// One series: T (8n), mean/inv/df/dg (4 x 8n), inv32/df32/dg32 (3 x 4n),
// T32 (4n), bhi/blo (2 x 4 x (n/32 + 1)), mu_rel (4n); windows <= samples.
constexpr size_t noalloc_series_bytes(int64_t n) {
  return noalloc_round(8 * n) + 4 * noalloc_round(8 * n) + 3 * noalloc_round(4 * n) +
         noalloc_round(4 * n) + 2 * noalloc_round(4 * (n / 32 + 1)) + noalloc_round(4 * n);
}
// counters (64 B, zeroed per call) | band prefix | two merge-key arrays | series A | series B
constexpr size_t kNoAllocScratchBytes =
    noalloc_round(64) + noalloc_round(8 * kNoAllocPrefixCap) +
    2 * noalloc_round(8 * kNoAllocMaxSamples) + 2 * noalloc_series_bytes(kNoAllocMaxSamples);

// About 8.6 MB per device, reserved when the module is loaded on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  int sms = 0;
  int occ = 1;                       // resident join_fp64_kernel CTAs per SM
};
NoAllocDevice g_noalloc_dev[64];
std::mutex g_noalloc_mu;

// Once per device, with that device current: the scratch's device address,
// the SM count and the FP64 join kernel's occupancy.  The first call on a
// device therefore makes runtime calls (module load, symbol lookup) that
// should happen before any stream capture is started.
int noalloc_setup(int device, NoAllocDevice** out, std::string* msg) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    *msg = "Error: no CUDA device available (this engine has no CPU fallback)";
    return SCAMP_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev || device >= 64) {
    *msg = "Error: invalid CUDA device ordinal";
    return SCAMP_ERR_INVALID_ARGS;
  }
  CUDA_TRY(cudaSetDevice(device));
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoAllocDevice& d = g_noalloc_dev[device];
  if (!d.scratch) {
    void* p = nullptr;
    CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    CUDA_TRY(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, device));
    int occ = 1;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ, reinterpret_cast<const void*>(join_fp64_kernel), fp64_threads(), 0));
    d.occ = std::max(occ, 1);
    d.scratch = static_cast<unsigned char*>(p);
  }
  *out = &d;
  return SCAMP_OK;
}

// Hands out consecutive 256-byte-aligned pieces of the scratch.
struct Carver {
  unsigned char* p;
  template <typename T>
  T* take(size_t bytes) {
    T* r = reinterpret_cast<T*>(p);
    p += noalloc_round(bytes);
    return r;
  }
};

SeriesBufs carve_series(Carver& c, int64_t n, int bshift) {
  SeriesBufs s{};
  s.bshift = bshift;
  s.T = c.take<double>(8 * n);
  s.mean = c.take<double>(8 * n);
  s.inv = c.take<double>(8 * n);
  s.df = c.take<double>(8 * n);
  s.dg = c.take<double>(8 * n);
  s.inv32 = c.take<float>(4 * n);
  s.df32 = c.take<float>(4 * n);
  s.dg32 = c.take<float>(4 * n);
  s.T32 = c.take<float>(4 * n);
  s.bhi = c.take<float>(4 * (n / 32 + 1));
  s.blo = c.take<float>(4 * (n / 32 + 1));
  s.mu_rel = c.take<float>(4 * n);
  return s;
}

// Band prefix of the no-allocation join on the device: entry g + 1 is the
// number of units in bands 0 .. g (the count make_plan's problems give, as
// run_device() builds it on the host).  One block of kNoAllocPrefixCap
// threads, thread g for band g.
__global__ void __launch_bounds__(kNoAllocPrefixCap)
noalloc_prefix_kernel(JoinParams P, int64_t K, int W, int64_t* __restrict__ prefix) {
  __shared__ int64_t part[kNoAllocPrefixCap];
  const int g = threadIdx.x;
  int64_t units = 0;
  if (g < P.total_bands) {
    int p = 0;
    while (p + 1 < P.nprob && g >= P.prob[p + 1].band_begin) ++p;
    const Problem& pr = P.prob[p];
    const int64_t D0 = pr.d_lo + (g - pr.band_begin) * W;
    const int64_t rows = band_rows(pr.R.ns, pr.C.ns, D0);
    units = (rows + 2 * K - 1) / (2 * K);
  }
  part[g] = units;
  __syncthreads();
  // inclusive scan (Hillis-Steele)
  for (int o = 1; o < kNoAllocPrefixCap; o <<= 1) {
    const int64_t v = g >= o ? part[g - o] : 0;
    __syncthreads();
    part[g] += v;
    __syncthreads();
  }
  if (g == 0) prefix[0] = 0;
  if (g < P.total_bands) prefix[g + 1] = part[g];
}

// The FP64 join of run_device() on the static scratch: the same kernels,
// launch shapes and segment length, so the results equal
// scamp_gb300_join_dev's.  Ordered on `st`; nothing is synchronised.
int run_device_noalloc(const NoAllocDevice& dv, const scamp_c_args* a, scamp_c_result* res,
                       cudaStream_t st, std::string* msg) {
  const int64_t na = static_cast<int64_t>(a->len_a);
  const int64_t nb = a->has_b ? static_cast<int64_t>(a->len_b) : na;
  if (na > kNoAllocMaxSamples || nb > kNoAllocMaxSamples) {
    *msg = "Error: the no-allocation join takes series of at most 65536 samples "
           "(use scamp_gb300_join_dev for longer series)";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (a->precision_type != SCAMP_PRECISION_DOUBLE && a->precision_type != SCAMP_PRECISION_ULTRA) {
    *msg = "Error: the no-allocation join runs the FP64 form only (precision double or ultra)";
    return SCAMP_ERR_INVALID_ARGS;
  }
  if (a->profile_type != SCAMP_PROFILE_1NN_INDEX && a->profile_type != SCAMP_PROFILE_SUM_THRESH) {
    *msg = "Error: the no-allocation join serves 1NN_INDEX and SUM_THRESH";
    return SCAMP_ERR_INVALID_ARGS;
  }
  const Plan plan = make_plan(a);
  const bool is_1nn = a->profile_type == SCAMP_PROFILE_1NN_INDEX;
  const bool ultra = a->precision_type == SCAMP_PRECISION_ULTRA;
  const int64_t m = plan.m;
  const int W = fp64_band_width();
  const int slab = fp64_slab_rows();
  const int nthreads = fp64_threads();

  Carver cv{dv.scratch};
  unsigned long long* counters = cv.take<unsigned long long>(64);
  int64_t* dprefix = cv.take<int64_t>(8 * kNoAllocPrefixCap);
  uint64_t* keys_mem[2] = {cv.take<uint64_t>(8 * kNoAllocMaxSamples),
                           cv.take<uint64_t>(8 * kNoAllocMaxSamples)};
  const int bshift = block_shift(m);
  SeriesBufs sa = carve_series(cv, kNoAllocMaxSamples, bshift);
  SeriesBufs sb = carve_series(cv, kNoAllocMaxSamples, bshift);
  const SeriesBufs sb_carved = sb;

  uint32_t launches = 0;
  const int chunk = 64;
  const double* dA = a->timeseries_a;
  const double* dB = a->has_b ? a->timeseries_b : a->timeseries_a;
  {
    const int64_t threads = (plan.ns_a + chunk - 1) / chunk;
    stats_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(
        dA, na, m, ultra ? 1 : 0, chunk, sa.bshift, sa.T, sa.T32, sa.bhi, sa.blo, sa.mu_rel,
        sa.mean, sa.inv, sa.df, sa.dg, sa.inv32, sa.df32, sa.dg32);
    ++launches;
  }
  if (a->has_b) {
    const int64_t threads = (plan.ns_b + chunk - 1) / chunk;
    stats_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(
        dB, nb, m, ultra ? 1 : 0, chunk, sb.bshift, sb.T, sb.T32, sb.bhi, sb.blo, sb.mu_rel,
        sb.mean, sb.inv, sb.df, sb.dg, sb.inv32, sb.df32, sb.dg32);
    ++launches;
  } else {
    sb = sa;
  }
  // ULTRA update terms as in run_device; a self-join's row terms go to the
  // second carved series' df/dg, unused by a self-join
  bool ultra_rows = false;
  if (ultra) {
    combined_stats_kernel<<<static_cast<unsigned>((plan.ns_a + 255) / 256), 256, 0, st>>>(
        sa.T, na, m, sa.mean, 0, sa.df, sa.dg);
    ++launches;
    if (a->has_b) {
      combined_stats_kernel<<<static_cast<unsigned>((plan.ns_b + 255) / 256), 256, 0, st>>>(
          sb.T, nb, m, sb.mean, 1, sb.df, sb.dg);
    } else {
      combined_stats_kernel<<<static_cast<unsigned>((plan.ns_a + 255) / 256), 256, 0, st>>>(
          sa.T, na, m, sa.mean, 1, sb_carved.df, sb_carved.dg);
      ultra_rows = true;
    }
    ++launches;
  }
  CUDA_TRY(cudaGetLastError());
  const SeriesDev devA = to_dev(sa, na, plan.ns_a);
  const SeriesDev devB = to_dev(sb, nb, plan.ns_b);
  SeriesDev devArows_nd = devA;  // series A in the row role
  if (ultra_rows) {
    devArows_nd.df = sb_carved.df;
    devArows_nd.dg = sb_carved.dg;
  }

  const KeyLayout kl = make_key_layout(std::max(plan.ns_a, plan.ns_b));
  uint64_t* profs[2] = {res->profile_a, res->profile_b};
  double* sums[2] = {res->sum_a, res->sum_b};
  uint64_t* keys[2] = {nullptr, nullptr};
  const int64_t nsz[2] = {plan.ns_a, plan.ns_b};
  bool used[2] = {false, false};
  for (const auto& q : plan.probs) {
    if (q.col_target >= 0) used[q.col_target] = true;
    if (q.row_target >= 0) used[q.row_target] = true;
  }
  for (int s = 0; s < 2; ++s) {
    // the profiles run_device() converts: every target, and profile A
    const bool conv = used[s] || (s == 0 && profs[0]);
    if (is_1nn && conv && !profs[s]) { *msg = "Error: profile buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
    if (!is_1nn && used[s] && !sums[s]) { *msg = "Error: sum buffer missing"; return SCAMP_ERR_INVALID_ARGS; }
  }
  if (is_1nn) {
    for (int s = 0; s < 2; ++s) {
      if (!used[s] && !(s == 0 && profs[0])) continue;
      keys[s] = keys_mem[s];
      profile_to_keys_kernel<<<static_cast<unsigned>((nsz[s] + 255) / 256), 256, 0, st>>>(
          profs[s], keys[s], nsz[s], kl);
      ++launches;
    }
  }

  const int64_t resident = static_cast<int64_t>(dv.sms) * dv.occ;
  // segment length: the FP64 rule of run_device()
  const double cells_d = static_cast<double>(plan.cells);
  const int64_t k_lb = static_cast<int64_t>(cells_d / (8.0 * resident * 2.0 * W));
  int64_t K = fp64_segment(m);
  K = std::min(K, std::max<int64_t>(k_lb, slab));
  K = std::max<int64_t>(slab, (K / slab) * slab);
  {
    const int64_t blk = 1ll << block_shift(m);
    if (K % blk) K = std::max<int64_t>(blk, (K / blk) * blk);
  }

  JoinParams P{};
  // The band prefix is counted here (for the total and the grid) and built
  // again on the device by noalloc_prefix_kernel from the same problems, so
  // that no host memory is copied.
  int64_t np = 1, units_total = 0;
  int64_t band_total = 0;
  for (const auto& q : plan.probs) {
    Problem& pr = P.prob[P.nprob++];
    pr.R = q.rows_series == 0 ? devArows_nd : devB;
    pr.C = q.cols_series == 0 ? devA : devB;
    pr.d_lo = q.d_lo; pr.d_hi = q.d_hi; pr.x_lo = q.x_lo; pr.x_hi = q.x_hi;
    pr.key_col = is_1nn && q.col_target >= 0 ? keys[q.col_target] : nullptr;
    pr.key_row = is_1nn && q.row_target >= 0 ? keys[q.row_target] : nullptr;
    pr.sum_col = !is_1nn && q.col_target >= 0 ? sums[q.col_target] : nullptr;
    pr.sum_row = !is_1nn && q.row_target >= 0 ? sums[q.row_target] : nullptr;
    pr.band_begin = band_total;
    pr.nbands = (q.d_hi - q.d_lo + W - 1) / W;
    if (np + pr.nbands > kNoAllocPrefixCap) {
      *msg = "Error: join too large for the no-allocation work queue";
      return SCAMP_ERR_INVALID_ARGS;
    }
    for (int64_t b = 0; b < pr.nbands; ++b) {
      const int64_t D0 = q.d_lo + b * W;
      const int64_t rows = band_rows(q.n_r, q.n_c, D0);
      units_total += (rows + 2 * K - 1) / (2 * K);
      ++np;
    }
    band_total += pr.nbands;
  }
  P.total_bands = band_total;
  P.total_units = units_total;
  P.m = m;
  P.seg_len = K;
  P.band_width = W;
  P.profile_type = a->profile_type;
  P.threshold = a->distance_threshold;
  P.kl = kl;

  if (P.total_units > 0) {
    noalloc_prefix_kernel<<<1, kNoAllocPrefixCap, 0, st>>>(P, K, W, dprefix);
    ++launches;
    // the unit queue head and the work counters must start at zero
    CUDA_TRY(cudaMemsetAsync(counters, 0, 64, st));
    P.band_unit_prefix = dprefix;
    P.unit_counter = counters;
    P.counters = counters + 1;
    P.error_flag = reinterpret_cast<int*>(counters + 6);
    const int64_t grid = std::min<int64_t>(resident, P.total_units);
    join_fp64_kernel<<<static_cast<unsigned>(grid), nthreads, 0, st>>>(P);
    ++launches;
    CUDA_TRY(cudaGetLastError());
  }
  if (is_1nn) {
    // the FP64 re-evaluation of run_device(), so that both entries report
    // the same values
    EvalPair E{};
    E.m = m;
    E.kl = kl;
    for (int s = 0; s < 2; ++s) {
      if (!keys[s]) continue;
      EvalSide& es = E.side[s];
      es.keys = keys[s];
      es.prof_in = profs[s];
      es.max_in = nullptr;
      es.X = s == 0 ? devA : devB;
      es.Y = plan.self_join ? devA : (s == 0 ? devB : devA);
      es.ns = nsz[s];
      es.m = m;
    }
    const int64_t nwin = E.side[0].ns + E.side[1].ns;
    if (nwin > 0) {
      const int64_t blocks = std::min<int64_t>((nwin + 31) / 32, static_cast<int64_t>(dv.sms) * 16);
      final_eval_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(E);
      ++launches;
    }
    double* corr[2] = {res->corr_a, res->corr_b};
    for (int s = 0; s < 2; ++s) {
      if (!keys[s]) continue;
      keys_to_profile_kernel<<<static_cast<unsigned>((nsz[s] + 255) / 256), 256, 0, st>>>(
          keys[s], profs[s], corr[s], nsz[s], kl);
      ++launches;
    }
  }
  CUDA_TRY(cudaGetLastError());
  res->comparisons = plan.cells;
  res->gpu_launches = launches;
  res->elapsed_ms = res->join_kernel_ms = 0;
  res->steps = res->slow_steps = res->verifications = 0;
  res->max_abs_r_err = is_1nn ? final_eval_bound(m, kl.frac_bits) : -1.0;
  res->max_tie_margin = -1.0;
  return SCAMP_OK;
}

}  // namespace
}  // namespace scamp_gb300

extern "C" int scamp_gb300_join_dev_noalloc(const scamp_c_args* args, scamp_c_result* res,
                                            void* stream, char* errbuf, size_t errlen) {
  std::string msg;
  int rc = validate(args, &msg);
  if (rc == SCAMP_OK && !res) { msg = "Error: result struct missing"; rc = SCAMP_ERR_INVALID_ARGS; }
  NoAllocDevice* dv = nullptr;
  if (rc == SCAMP_OK) rc = noalloc_setup(args->device, &dv, &msg);
  if (rc == SCAMP_OK) rc = run_device_noalloc(*dv, args, res, static_cast<cudaStream_t>(stream), &msg);
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

// ---------------------------------------------------------------------------
// Batched self-joins (scamp_gb300_join_batch): many independent series, each
// its own band problem, all in one persistent launch of the mixed 1NN band
// kernel.  Series, statistics, keys and profiles of the whole batch are
// concatenated in one workspace arena; one batched statistics launch, one
// key conversion each way and one verification launch serve every series.
// ---------------------------------------------------------------------------
namespace scamp_gb300 {
namespace {

struct BatchSeries {
  int64_t n, m, ns, excl, K;
  int bshift;
  int64_t off_n, off_ns, off_blk;
  uint64_t cells;
  // block-averaged pre-pass (f = 0: not seeded): f samples per block, the
  // averaged series' length, window, windows, exclusion, segment length
  int f;
  int64_t n2, m2, ns2, excl2, K2;
  int bshift2;
  int64_t off_n2, off_ns2, off_blk2;
};

// Device arrays of a batch's concatenated series.
struct BatchArrays {
  double *raw, *T, *mean, *inv, *df, *dg;
  float *inv32, *df32, *dg32, *T32, *bhi, *blo, *murel;
  uint64_t* keys;
};

// One series' view of the concatenated arrays.
SeriesDev batch_series_dev(const BatchArrays& A, int64_t off_n, int64_t off_ns, int64_t off_blk,
                           int bshift, int64_t n, int64_t ns) {
  SeriesDev sd;
  sd.T = A.T + off_n; sd.mean = A.mean + off_ns; sd.inv = A.inv + off_ns;
  sd.df = A.df + off_ns; sd.dg = A.dg + off_ns;
  sd.inv32 = A.inv32 + off_ns; sd.df32 = A.df32 + off_ns; sd.dg32 = A.dg32 + off_ns;
  sd.T32 = A.T32 + off_n; sd.bhi = A.bhi + off_blk; sd.blo = A.blo + off_blk;
  sd.mu_rel = A.murel + off_ns; sd.bshift = bshift; sd.n = n; sd.ns = ns;
  return sd;
}

StatsJob batch_stats_job(const BatchArrays& A, int64_t off_n, int64_t off_ns, int64_t off_blk,
                         int bshift, int64_t n, int64_t m) {
  StatsJob j;
  j.T_raw = A.raw + off_n;
  j.n = n;
  j.m = m;
  j.bshift = bshift;
  j.T_clean = A.T + off_n;
  j.mean = A.mean + off_ns;
  j.inv = A.inv + off_ns;
  j.df = A.df + off_ns;
  j.dg = A.dg + off_ns;
  j.T32 = A.T32 + off_n;
  j.bhi = A.bhi + off_blk;
  j.blo = A.blo + off_blk;
  j.mu_rel = A.murel + off_ns;
  j.inv32 = A.inv32 + off_ns;
  j.df32 = A.df32 + off_ns;
  j.dg32 = A.dg32 + off_ns;
  return j;
}

// Band problem of one series of a batch (a self-join into its keys) and its
// band unit prefix entries.
Problem batch_problem(const SeriesDev& sd, uint64_t* keys, int64_t excl, int64_t m, int64_t K,
                      int64_t band_begin, int W, std::vector<int64_t>* bpre) {
  Problem pr{};
  pr.R = sd;
  pr.C = sd;
  pr.d_lo = excl;
  pr.d_hi = sd.ns;
  pr.x_lo = pr.x_hi = 0;
  pr.key_col = pr.key_row = keys;  // self-join: rows and columns into one profile
  pr.band_begin = band_begin;
  pr.nbands = (pr.d_hi - pr.d_lo + W - 1) / W;
  pr.m = m;
  pr.seg_len = K;
  const double blk = static_cast<double>(1 << sd.bshift);
  const double e = std::sqrt(std::min<double>(m, blk)) + std::sqrt(std::ceil(m / blk) + 1.0);
  pr.anchor_vcoef = static_cast<float>(e * e / 8.0);
  for (int64_t g = 0; g < pr.nbands; ++g) {
    const int64_t D0 = pr.d_lo + g * W;
    const int64_t rows = band_rows(sd.ns, sd.ns, D0);
    bpre->push_back(bpre->back() + (rows + 2 * K - 1) / (2 * K));
  }
  return pr;
}

// Segment length of one series of a batch: `pref` (the autotuned value for
// its window, 0 = none) or the cold-start anchor interval, reduced for short
// series so that a band's rows split into at least two segments.
int64_t batch_segment(int64_t m, int64_t ns, int slab, int64_t pref) {
  int64_t K = pref > 0 ? pref : cold_anchor_interval(m);
  const int64_t half = std::max<int64_t>(slab, (ns / 2 / slab) * slab);
  K = std::min(K, half);
  const int64_t blk = int64_t{1} << block_shift(m);
  if (K % blk) K = std::max<int64_t>(blk, (K / blk) * blk);
  return K;
}

// Runs one batch.  `force_K` > 0 sets every series' segment length (the
// autotuner's trials); 0 takes the tuned value of the series' window, else the
// anchor-interval rule.
//
// The host gathers the inputs and builds every launch's arguments first, then
// copies them over; the device part (statistics, keys, diagonal seeds, the
// persistent band kernel, verification, keys back to profiles) is one CUDA
// graph, captured once per batch layout and replayed while the layout (sizes,
// arena and request-buffer addresses, grid) repeats.
int run_batch(Workspace& ws, const scamp_c_args* args, scamp_c_result* res, int count,
              cudaStream_t st, std::string* msg, int64_t force_K = 0) {
  int rc;
  ws.timed_kernel = false;
  ws.timed_verify = false;
  ws.tracked_tie_margin = ws.tracked_sum_margin = false;
  std::vector<BatchSeries> ser(count);
  int64_t Nn = 0, Nns = 0, Nblk = 0, ns_max = 1;
  int64_t N2n = 0, N2ns = 0, N2blk = 0;  // the pre-pass's series
  int nseed = 0;
  bool want_corr = false;
  for (int k = 0; k < count; ++k) {
    const scamp_c_args* a = &args[k];
    BatchSeries& b = ser[k];
    b.n = static_cast<int64_t>(a->len_a);
    b.m = static_cast<int64_t>(a->window);
    b.ns = b.n - b.m + 1;
    b.excl = b.m / 4;  // src/tile.cpp:14
    b.bshift = block_shift(b.m);
    int64_t pref = force_K;
    if (pref <= 0) {
      const auto it = ws.batch_seg.find(b.m);
      pref = it == ws.batch_seg.end() ? 0 : it->second;
    }
    b.K = batch_segment(b.m, b.ns, mixed_1nn_slab_rows(), pref);
    b.off_n = Nn;
    b.off_ns = Nns;
    b.off_blk = Nblk;
    b.cells = b.ns > b.excl ? diag_cells(b.ns, b.ns, b.excl, b.ns) : 0;
    Nn += b.n;
    Nns += b.ns;
    Nblk += (b.n >> b.bshift) + 1;
    ns_max = std::max(ns_max, b.ns);
    // the pre-pass: series averaged over blocks of f samples, window m / f
    b.f = 0;
    if (b.cells > 0) {
      const int f = seed_factor(b.m);
      const int64_t n2 = b.n / f, m2 = b.m / f;
      const int64_t ns2 = n2 - m2 + 1, excl2 = m2 / 4;
      if (b.m >= kSeedMinWindow && ns2 > excl2 && diag_cells(ns2, ns2, excl2, ns2) > 0) {
        b.f = f;
        b.n2 = n2;
        b.m2 = m2;
        b.ns2 = ns2;
        b.excl2 = excl2;
        b.bshift2 = block_shift(m2);
        b.K2 = batch_segment(m2, ns2, mixed_1nn_slab_rows(), 0);
        b.off_n2 = N2n;
        b.off_ns2 = N2ns;
        b.off_blk2 = N2blk;
        N2n += n2;
        N2ns += ns2;
        N2blk += (n2 >> b.bshift2) + 1;
        ++nseed;
      }
    }
    want_corr = want_corr || res[k].corr_a != nullptr;
  }
  // ---- arena ----
  size_t total = 0;
  auto sz = [&](size_t b) { const size_t r = (b + 255) / 256 * 256; total += r; return r; };
  const size_t b_raw = sz(8 * Nn), b_T = sz(8 * Nn), b_mean = sz(8 * Nns), b_inv = sz(8 * Nns),
               b_df = sz(8 * Nns), b_dg = sz(8 * Nns), b_inv32 = sz(4 * Nns), b_df32 = sz(4 * Nns),
               b_dg32 = sz(4 * Nns), b_T32 = sz(4 * Nn), b_bhi = sz(4 * Nblk), b_blo = sz(4 * Nblk),
               b_murel = sz(4 * Nns), b_keys = sz(8 * Nns), b_prof = sz(8 * Nns),
               b_corr = sz(want_corr ? 8 * Nns : 8), b_jobs = sz(sizeof(StatsJob) * count),
               b_jpre = sz(8 * (count + 1)), b_probs = sz(sizeof(Problem) * count),
               b_counter = sz(64), b_wpre = sz(8 * (count + 1)),
               b_eval = sz(sizeof(EvalSide) * count);
  // band prefix: sized after the problems are known
  int64_t bands_max = 0, bands2_max = 0;
  for (const auto& b : ser) {
    bands_max += (b.ns + mixed_1nn_band_width() - 1) / mixed_1nn_band_width();
    if (b.f) bands2_max += (b.ns2 + mixed_1nn_band_width() - 1) / mixed_1nn_band_width();
  }
  const size_t b_bpre = sz(8 * (bands_max + 1));
  // the pre-pass's arrays
  const size_t s_raw = sz(8 * N2n), s_T = sz(8 * N2n), s_mean = sz(8 * N2ns), s_inv = sz(8 * N2ns),
               s_df = sz(8 * N2ns), s_dg = sz(8 * N2ns), s_inv32 = sz(4 * N2ns),
               s_df32 = sz(4 * N2ns), s_dg32 = sz(4 * N2ns), s_T32 = sz(4 * N2n),
               s_bhi = sz(4 * N2blk), s_blo = sz(4 * N2blk), s_murel = sz(4 * N2ns),
               s_keys = sz(8 * N2ns), s_jobs = sz(sizeof(StatsJob) * nseed),
               s_jpre = sz(8 * (nseed + 1)), s_probs = sz(sizeof(Problem) * nseed),
               s_counter = sz(64), s_wpre = sz(8 * (nseed + 1)), s_bpre = sz(8 * (bands2_max + 1)),
               s_paa = sz(sizeof(PaaJob) * nseed), s_paapre = sz(8 * (nseed + 1)),
               s_seed = sz(sizeof(BatchSeedJob) * nseed);
  void* arena;
  if ((rc = ensure(ws, S_BATCH, total, &arena, msg))) return rc;
  unsigned char* cur = static_cast<unsigned char*>(arena);
  auto take = [&](size_t bytes) { unsigned char* r = cur; cur += bytes; return r; };
  double* d_raw = reinterpret_cast<double*>(take(b_raw));
  double* d_T = reinterpret_cast<double*>(take(b_T));
  double* d_mean = reinterpret_cast<double*>(take(b_mean));
  double* d_inv = reinterpret_cast<double*>(take(b_inv));
  double* d_df = reinterpret_cast<double*>(take(b_df));
  double* d_dg = reinterpret_cast<double*>(take(b_dg));
  float* d_inv32 = reinterpret_cast<float*>(take(b_inv32));
  float* d_df32 = reinterpret_cast<float*>(take(b_df32));
  float* d_dg32 = reinterpret_cast<float*>(take(b_dg32));
  float* d_T32 = reinterpret_cast<float*>(take(b_T32));
  float* d_bhi = reinterpret_cast<float*>(take(b_bhi));
  float* d_blo = reinterpret_cast<float*>(take(b_blo));
  float* d_murel = reinterpret_cast<float*>(take(b_murel));
  uint64_t* d_keys = reinterpret_cast<uint64_t*>(take(b_keys));
  uint64_t* d_prof = reinterpret_cast<uint64_t*>(take(b_prof));
  double* d_corr = reinterpret_cast<double*>(take(b_corr));
  StatsJob* d_jobs = reinterpret_cast<StatsJob*>(take(b_jobs));
  int64_t* d_jpre = reinterpret_cast<int64_t*>(take(b_jpre));
  Problem* d_probs = reinterpret_cast<Problem*>(take(b_probs));
  unsigned long long* d_counter = reinterpret_cast<unsigned long long*>(take(b_counter));
  int64_t* d_bpre = reinterpret_cast<int64_t*>(take(b_bpre));
  int64_t* d_wpre = reinterpret_cast<int64_t*>(take(b_wpre));
  EvalSide* d_eval = reinterpret_cast<EvalSide*>(take(b_eval));
  BatchArrays A2;
  A2.raw = reinterpret_cast<double*>(take(s_raw));
  A2.T = reinterpret_cast<double*>(take(s_T));
  A2.mean = reinterpret_cast<double*>(take(s_mean));
  A2.inv = reinterpret_cast<double*>(take(s_inv));
  A2.df = reinterpret_cast<double*>(take(s_df));
  A2.dg = reinterpret_cast<double*>(take(s_dg));
  A2.inv32 = reinterpret_cast<float*>(take(s_inv32));
  A2.df32 = reinterpret_cast<float*>(take(s_df32));
  A2.dg32 = reinterpret_cast<float*>(take(s_dg32));
  A2.T32 = reinterpret_cast<float*>(take(s_T32));
  A2.bhi = reinterpret_cast<float*>(take(s_bhi));
  A2.blo = reinterpret_cast<float*>(take(s_blo));
  A2.murel = reinterpret_cast<float*>(take(s_murel));
  A2.keys = reinterpret_cast<uint64_t*>(take(s_keys));
  StatsJob* d_jobs2 = reinterpret_cast<StatsJob*>(take(s_jobs));
  int64_t* d_jpre2 = reinterpret_cast<int64_t*>(take(s_jpre));
  Problem* d_probs2 = reinterpret_cast<Problem*>(take(s_probs));
  unsigned long long* d_counter2 = reinterpret_cast<unsigned long long*>(take(s_counter));
  int64_t* d_wpre2 = reinterpret_cast<int64_t*>(take(s_wpre));
  int64_t* d_bpre2 = reinterpret_cast<int64_t*>(take(s_bpre));
  PaaJob* d_paa = reinterpret_cast<PaaJob*>(take(s_paa));
  int64_t* d_paapre = reinterpret_cast<int64_t*>(take(s_paapre));
  BatchSeedJob* d_seed = reinterpret_cast<BatchSeedJob*>(take(s_seed));
  BatchArrays A1{d_raw, d_T, d_mean, d_inv, d_df, d_dg, d_inv32, d_df32, d_dg32, d_T32,
                 d_bhi, d_blo, d_murel, d_keys};

  // ---- host side: inputs gathered, every launch's arguments built ----
  void *hp_raw, *hp_prof, *hp_corr = nullptr;
  if ((rc = ensure_pinned(ws, 0, std::max<size_t>(Nn * 8, 8), &hp_raw, msg))) return rc;
  if ((rc = ensure_pinned(ws, 1, std::max<size_t>(Nns * 8, 8), &hp_prof, msg))) return rc;
  if (want_corr && (rc = ensure_pinned(ws, 2, std::max<size_t>(Nns * 8, 8), &hp_corr, msg))) return rc;
  double* h_raw = static_cast<double*>(hp_raw);
  uint64_t* h_prof = static_cast<uint64_t*>(hp_prof);
  double* h_corr = static_cast<double*>(hp_corr);
  for (int k = 0; k < count; ++k) {
    std::memcpy(h_raw + ser[k].off_n, args[k].timeseries_a, ser[k].n * 8);
    std::memcpy(h_prof + ser[k].off_ns, res[k].profile_a, ser[k].ns * 8);
  }
  const int chunk = 64;
  std::vector<StatsJob> jobs(count);
  std::vector<int64_t> jpre(count + 1, 0);
  for (int k = 0; k < count; ++k) {
    const BatchSeries& b = ser[k];
    jobs[k] = batch_stats_job(A1, b.off_n, b.off_ns, b.off_blk, b.bshift, b.n, b.m);
    const int64_t threads = (b.ns + chunk - 1) / chunk;
    jpre[k + 1] = jpre[k] + (threads + 127) / 128;
  }
  const KeyLayout kl = make_key_layout(ns_max);
  const int W = mixed_1nn_band_width();
  std::vector<Problem> probs;
  probs.reserve(count);
  std::vector<int64_t> bpre;
  bpre.push_back(0);
  int64_t band_total = 0;
  for (int k = 0; k < count; ++k) {
    const BatchSeries& b = ser[k];
    if (b.cells == 0) continue;
    const SeriesDev sd = batch_series_dev(A1, b.off_n, b.off_ns, b.off_blk, b.bshift, b.n, b.ns);
    const Problem pr = batch_problem(sd, d_keys + b.off_ns, b.excl, b.m, b.K, band_total, W, &bpre);
    band_total += pr.nbands;
    probs.push_back(pr);
  }
  // the pre-pass: averaged copies, their statistics jobs, band problems, and
  // the seeding jobs that carry its partners back to the series' keys
  std::vector<PaaJob> paa_jobs;
  std::vector<StatsJob> jobs2;
  std::vector<Problem> probs2;
  std::vector<BatchSeedJob> seed_jobs;
  // wpre2: the averaged windows' prefix (diagonal seeds and seeding jobs)
  std::vector<int64_t> paapre(1, 0), jpre2(1, 0), wpre2(1, 0), bpre2(1, 0);
  int64_t band_total2 = 0;
  for (int k = 0; k < count; ++k) {
    const BatchSeries& b = ser[k];
    if (!b.f) continue;
    paa_jobs.push_back(PaaJob{d_raw + b.off_n, A2.raw + b.off_n2, b.n2, b.f});
    paapre.push_back(paapre.back() + b.n2);
    jobs2.push_back(batch_stats_job(A2, b.off_n2, b.off_ns2, b.off_blk2, b.bshift2, b.n2, b.m2));
    jpre2.push_back(jpre2.back() + ((b.ns2 + chunk - 1) / chunk + 127) / 128);
    const SeriesDev sd2 = batch_series_dev(A2, b.off_n2, b.off_ns2, b.off_blk2, b.bshift2, b.n2, b.ns2);
    const Problem pr2 = batch_problem(sd2, A2.keys + b.off_ns2, b.excl2, b.m2, b.K2, band_total2, W,
                                      &bpre2);
    band_total2 += pr2.nbands;
    probs2.push_back(pr2);
    wpre2.push_back(wpre2.back() + b.ns2);
    BatchSeedJob sj;
    sj.X = batch_series_dev(A1, b.off_n, b.off_ns, b.off_blk, b.bshift, b.n, b.ns);
    sj.key = d_keys + b.off_ns;
    sj.paa_key = A2.keys + b.off_ns2;
    sj.ns_paa = b.ns2;
    sj.excl = b.excl;
    sj.m = b.m;
    sj.f = b.f;
    seed_jobs.push_back(sj);
  }
  // seeds from each series' nearest allowed diagonal (diag_seed_kernel),
  // and the FP64 re-evaluation of every reported cell (final_eval_batch_kernel)
  std::vector<int64_t> wpre(probs.size() + 1, 0);
  for (size_t p = 0; p < probs.size(); ++p) wpre[p + 1] = wpre[p] + probs[p].R.ns;
  std::vector<EvalSide> evs(probs.size());
  for (size_t p = 0; p < probs.size(); ++p) {
    EvalSide& e = evs[p];
    e.keys = probs[p].key_col;
    e.prof_in = d_prof + (probs[p].key_col - d_keys);
    e.max_in = nullptr;
    e.X = e.Y = probs[p].R;
    e.ns = probs[p].R.ns;
    e.m = probs[p].m;
  }
  const int64_t eval_blocks = std::max<int64_t>(
      std::min<int64_t>((wpre.back() + 31) / 32, static_cast<int64_t>(ws.sms) * 16), 1);
  const int64_t seed_blocks = std::max<int64_t>(
      std::min<int64_t>((wpre.back() + 255) / 256, static_cast<int64_t>(ws.sms) * 32), 1);
  JoinParams P{};
  int64_t grid = 0;
  const size_t smem = mixed_1nn_smem_bytes();
  const void* kfn = reinterpret_cast<const void*>(join_mixed_1nn_kernel);
  if (!probs.empty()) {
    P.nprob = 0;
    P.batch = d_probs;
    P.nbatch = static_cast<int64_t>(probs.size());
    P.band_unit_prefix = d_bpre;
    P.total_bands = band_total;
    P.total_units = bpre.back();
    P.unit_counter = d_counter;
    P.counters = d_counter + 1;
    P.error_flag = reinterpret_cast<int*>(d_counter + 6);
    P.profile_type = SCAMP_PROFILE_1NN_INDEX;
    P.kl = kl;
    P.refresh_cols = 1;  // batches start cold (diagonal seeds only)
    int64_t want = std::max<int64_t>(kMinVerifyReqs, 32 * Nns);
    want = std::max<int64_t>(want, ws.vreq_seen + ws.vreq_seen / 4);
    want = std::max<int64_t>(std::min<int64_t>(want, kMaxVerifyReqs), ws.vreq_cap);
    void* q;
    if ((rc = ensure(ws, S_VREQ, static_cast<size_t>(want) * sizeof(VerifyReq), &q, msg))) return rc;
    ws.vreq_cap = want;
    P.vreq = static_cast<VerifyReq*>(q);
    P.vreq_cap = want;
    CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int occ = 1;
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, mixed_1nn_threads(), smem));
    grid = std::min<int64_t>(static_cast<int64_t>(ws.sms) * std::max(occ, 1), P.total_units);
  }
  // the pre-pass join: the same kernel over the averaged series, into their
  // own keys (started at the seed floor); its unverified candidates keep
  // their lower bounds, which is all a seed needs (the partner), so it has
  // no verification launch.  It shares the request buffer: the main join's
  // requests are counted from 0 after it.
  JoinParams P2{};
  int64_t grid2 = 0;
  const int64_t nseed_jobs = static_cast<int64_t>(seed_jobs.size());
  if (nseed_jobs > 0 && !probs.empty()) {
    P2 = P;
    P2.batch = d_probs2;
    P2.nbatch = static_cast<int64_t>(probs2.size());
    P2.band_unit_prefix = d_bpre2;
    P2.total_bands = band_total2;
    P2.total_units = bpre2.back();
    P2.unit_counter = d_counter2;
    P2.counters = d_counter2 + 1;
    P2.error_flag = reinterpret_cast<int*>(d_counter2 + 6);
    grid2 = std::min<int64_t>(grid > 0 ? grid : 1, std::max<int64_t>(P2.total_units, 1));
  }
  const bool seeded = grid2 > 0 && P2.total_units > 0;
  const int64_t paa_blocks = std::max<int64_t>(
      std::min<int64_t>((paapre.back() + 255) / 256, static_cast<int64_t>(ws.sms) * 16), 1);
  const int64_t fill2_blocks = std::max<int64_t>(
      std::min<int64_t>((N2ns + 255) / 256, static_cast<int64_t>(ws.sms) * 16), 1);
  const int64_t seed2_blocks = std::max<int64_t>(
      std::min<int64_t>((wpre2.back() + 255) / 256, static_cast<int64_t>(ws.sms) * 32), 1);
  const int64_t bseed_blocks = std::max<int64_t>(
      std::min<int64_t>((wpre2.back() + 7) / 8, static_cast<int64_t>(ws.sms) * 16), 1);

  // ---- copies in ----
  CUDA_TRY(cudaEventRecord(ws.ev0, st));
  if (seeded) {
    CUDA_TRY(cudaMemcpyAsync(d_paa, paa_jobs.data(), sizeof(PaaJob) * nseed_jobs,
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_paapre, paapre.data(), 8 * paapre.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_jobs2, jobs2.data(), sizeof(StatsJob) * nseed_jobs,
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_jpre2, jpre2.data(), 8 * jpre2.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_probs2, probs2.data(), sizeof(Problem) * probs2.size(),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_wpre2, wpre2.data(), 8 * wpre2.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_bpre2, bpre2.data(), 8 * bpre2.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_seed, seed_jobs.data(), sizeof(BatchSeedJob) * nseed_jobs,
                             cudaMemcpyHostToDevice, st));
  }
  CUDA_TRY(cudaMemcpyAsync(d_raw, h_raw, Nn * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d_prof, h_prof, Nns * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(StatsJob) * count, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d_jpre, jpre.data(), 8 * (count + 1), cudaMemcpyHostToDevice, st));
  if (!probs.empty()) {
    CUDA_TRY(cudaMemcpyAsync(d_probs, probs.data(), sizeof(Problem) * probs.size(),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_wpre, wpre.data(), 8 * wpre.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_bpre, bpre.data(), 8 * bpre.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_eval, evs.data(), sizeof(EvalSide) * evs.size(),
                             cudaMemcpyHostToDevice, st));
  }

  // ---- device part: one graph ----
  uint32_t launches = probs.empty() ? 3 : (seeded ? 13 : 7);
  const std::vector<int64_t> key = {
      reinterpret_cast<int64_t>(arena), Nn, Nns, Nblk, count, want_corr ? 1 : 0, bands_max,
      jpre[count], kl.idx_bits, static_cast<int64_t>(probs.size()), seed_blocks, band_total,
      P.total_units, grid, reinterpret_cast<int64_t>(P.vreq), P.vreq_cap,
      static_cast<int64_t>(smem), reinterpret_cast<int64_t>(st), seeded ? 1 : 0, N2n, N2ns, N2blk,
      nseed_jobs, bands2_max, band_total2, P2.total_units, grid2};
  if (!ws.batch_exec || ws.batch_key != key) {
    auto enqueue = [&]() -> cudaError_t {
      cudaError_t e;
      stats_batch_kernel<<<static_cast<unsigned>(jpre[count]), 128, 0, st>>>(d_jobs, d_jpre, count, 0,
                                                                              chunk);
      profile_to_keys_kernel<<<static_cast<unsigned>((Nns + 255) / 256), 256, 0, st>>>(d_prof, d_keys,
                                                                                       Nns, kl);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      if (seeded) {
        const int nj = static_cast<int>(nseed_jobs);
        paa_batch_kernel<<<static_cast<unsigned>(paa_blocks), 256, 0, st>>>(d_paa, d_paapre, nj);
        stats_batch_kernel<<<static_cast<unsigned>(jpre2.back()), 128, 0, st>>>(d_jobs2, d_jpre2, nj, 0,
                                                                                 chunk);
        fill_key_floor_kernel<<<static_cast<unsigned>(fill2_blocks), 256, 0, st>>>(A2.keys, N2ns,
                                                                                    kSeedFloor, kl);
        diag_seed_kernel<<<static_cast<unsigned>(seed2_blocks), 256, 0, st>>>(d_probs2, d_wpre2, nj, kl);
        if ((e = cudaMemsetAsync(d_counter2, 0, 64, st)) != cudaSuccess) return e;
        join_mixed_1nn_kernel<<<static_cast<unsigned>(grid2), mixed_1nn_threads(), smem, st>>>(P2);
        batch_seed_kernel<<<static_cast<unsigned>(bseed_blocks), 256, 0, st>>>(d_seed, d_wpre2, nj,
                                                                                kl, kSeedFloor);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
      }
      if (!probs.empty()) {
        diag_seed_kernel<<<static_cast<unsigned>(seed_blocks), 256, 0, st>>>(
            d_probs, d_wpre, static_cast<int>(probs.size()), kl);
        if ((e = cudaMemsetAsync(d_counter, 0, 64, st)) != cudaSuccess) return e;
        if ((e = cudaEventRecordWithFlags(ws.evk0, st, cudaEventRecordExternal)) != cudaSuccess) return e;
        join_mixed_1nn_kernel<<<static_cast<unsigned>(grid), mixed_1nn_threads(), smem, st>>>(P);
        if ((e = cudaEventRecordWithFlags(ws.evkv, st, cudaEventRecordExternal)) != cudaSuccess) return e;
        verify_requests_kernel<<<static_cast<unsigned>(ws.sms * 8), 256, 0, st>>>(P);
        if ((e = cudaEventRecordWithFlags(ws.evk1, st, cudaEventRecordExternal)) != cudaSuccess) return e;
        final_eval_batch_kernel<<<static_cast<unsigned>(eval_blocks), 256, 0, st>>>(
            d_eval, d_wpre, static_cast<int>(probs.size()), kl);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
      }
      keys_to_profile_kernel<<<static_cast<unsigned>((Nns + 255) / 256), 256, 0, st>>>(
          d_keys, d_prof, want_corr ? d_corr : nullptr, Nns, kl);
      return cudaGetLastError();
    };
    if (ws.batch_exec) {
      CUDA_TRY(cudaStreamSynchronize(st));
      cudaGraphExecDestroy(ws.batch_exec);
      ws.batch_exec = nullptr;
      ws.batch_key.clear();
    }
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const cudaError_t ce = enqueue();
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(st, &graph);
    cudaError_t ie = cudaSuccess;
    if (ce == cudaSuccess && ee == cudaSuccess) ie = cudaGraphInstantiate(&ws.batch_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    const cudaError_t bad = ce != cudaSuccess ? ce : (ee != cudaSuccess ? ee : ie);
    if (bad != cudaSuccess) {
      ws.batch_exec = nullptr;
      *msg = std::string("CUDA error: ") + cudaGetErrorString(bad) + " while building the batch graph";
      return SCAMP_ERR_CUDA;
    }
    ws.batch_key = key;
  }
  CUDA_TRY(cudaGraphLaunch(ws.batch_exec, st));
  ws.timed_kernel = ws.timed_verify = !probs.empty();

  // ---- copies out ----
  CUDA_TRY(cudaMemcpyAsync(h_prof, d_prof, Nns * 8, cudaMemcpyDeviceToHost, st));
  if (want_corr) {
    CUDA_TRY(cudaMemcpyAsync(h_corr, d_corr, Nns * 8, cudaMemcpyDeviceToHost, st));
  }
  CUDA_TRY(cudaEventRecord(ws.ev1, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  for (int k = 0; k < count; ++k) {
    std::memcpy(res[k].profile_a, h_prof + ser[k].off_ns, ser[k].ns * 8);
    if (res[k].corr_a) std::memcpy(res[k].corr_a, h_corr + ser[k].off_ns, ser[k].ns * 8);
  }
  scamp_c_result tot{};
  read_times(ws, &tot);
  if (!probs.empty()) {
    // the batch's work counters live in its arena, not in the join counters
    unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (cudaMemcpy(c, d_counter, sizeof(c), cudaMemcpyDeviceToHost) == cudaSuccess) {
      tot.steps = c[1];
      tot.slow_steps = c[2];
      tot.verifications = c[3];
      tot.inplace_verifications = static_cast<uint32_t>(std::min<unsigned long long>(c[7], UINT32_MAX));
      ws.vreq_seen = std::max<int64_t>(ws.vreq_seen, static_cast<int64_t>(c[4] + c[7]));
      const uint32_t bits = static_cast<uint32_t>(c[5]);
      float tm;
      std::memcpy(&tm, &bits, 4);
      tot.max_tie_margin = tm;
    }
  }
  for (int k = 0; k < count; ++k) {
    res[k].elapsed_ms = tot.elapsed_ms;
    res[k].join_kernel_ms = tot.join_kernel_ms;
    res[k].verify_kernel_ms = tot.verify_kernel_ms;
    res[k].comparisons = ser[k].cells;
    res[k].gpu_launches = launches;
    res[k].steps = tot.steps;
    res[k].slow_steps = tot.slow_steps;
    res[k].verifications = tot.verifications;
    res[k].inplace_verifications = tot.inplace_verifications;
    res[k].max_abs_r_err = final_eval_bound(ser[k].m, kl.frac_bits);
    res[k].max_tie_margin = tot.max_tie_margin;
  }
  return SCAMP_OK;
}

// Autotuner of the batched join's tile height.  A band unit is W diagonals x
// two segments of K rows; K is also the mixed form's anchor interval.  For
// each window length among the series (all of them, or with `retune` = 0 the
// ones not tuned yet), it runs the band kernel on a sample of those series
// (in batch order, until kTuneCells comparisons) at K = the cold-start
// anchor interval, half and a quarter of it (never below 256 rows), twice each,
// and keeps the K with the shortest band + verification kernel time; a
// shorter K must win by 2% to replace a longer one.  Candidates stop at the
// cold-start value: on a sample, longer intervals time within a few percent
// of it, yet on the whole 4096-series batch they were 6% slower.  The
// sample's profiles are scratch.
constexpr uint64_t kTuneCells = uint64_t{1} << 34;

int tune_batch(Workspace& ws, const scamp_c_args* args, int count, bool retune,
               std::string* msg) {
  std::map<int64_t, std::vector<int>> by_window;
  for (int k = 0; k < count; ++k) by_window[static_cast<int64_t>(args[k].window)].push_back(k);
  for (const auto& w : by_window) {
    const int64_t m = w.first;
    if (!retune && ws.batch_seg.count(m)) continue;
    std::vector<scamp_c_args> sa;
    uint64_t cells = 0;
    for (int k : w.second) {
      if (cells >= kTuneCells) break;
      const int64_t ns = static_cast<int64_t>(args[k].len_a) - m + 1;
      if (ns <= m / 4) continue;
      sa.push_back(args[k]);
      cells += diag_cells(ns, ns, m / 4, ns);
    }
    const int64_t k_rule = cold_anchor_interval(m);
    if (sa.empty()) {
      ws.batch_seg[m] = k_rule;
      continue;
    }
    std::vector<scamp_c_result> sr(sa.size());
    std::vector<std::vector<uint64_t>> prof(sa.size());
    for (size_t k = 0; k < sa.size(); ++k) {
      prof[k].resize(sa[k].len_a - sa[k].window + 1);
      sr[k] = scamp_c_result{};
      sr[k].profile_a = prof[k].data();
    }
    const uint64_t no_match = (uint64_t{0xFFFFFFFF} << 32) | 0xC0000000u;  // {-2.0f, 0xFFFFFFFF}
    int64_t best = k_rule;
    double best_ms = 0;
    for (int64_t K = k_rule; K >= std::min<int64_t>(k_rule, 256); K /= 2) {
      if (K < k_rule / 4) break;
      double t = -1;
      for (int rep = 0; rep < 2; ++rep) {
        for (auto& p : prof) std::fill(p.begin(), p.end(), no_match);
        const int rc = run_batch(ws, sa.data(), sr.data(), static_cast<int>(sa.size()), ws.stream, msg, K);
        if (rc) return rc;
        const double ms = sr[0].join_kernel_ms;
        if (t < 0 || ms < t) t = ms;
      }
      if (K == k_rule || t < 0.98 * best_ms) {
        best = K;
        best_ms = t;
      }
      if (K <= 256) break;
    }
    ws.batch_seg[m] = best;
  }
  return SCAMP_OK;
}

// Checks shared by scamp_gb300_join_batch and scamp_gb300_tune_batch (`res`
// null: no result buffers to check).
int validate_batch(const scamp_c_args* args, const scamp_c_result* res, int count,
                   std::string* msg) {
  for (int k = 0; k < count; ++k) {
    const scamp_c_args* a = &args[k];
    std::string m;
    int rc = validate(a, &m);
    if (rc == SCAMP_OK) {
      if (a->has_b || a->is_aligned || a->keep_rows_separate || !a->computing_rows ||
          !a->computing_columns || a->distributed_start_row >= 0 || a->distributed_start_col >= 0)
        m = "Error: batched joins are plain self-joins (rows and columns into profile A)";
      else if (a->profile_type != SCAMP_PROFILE_1NN_INDEX)
        m = "Error: batched joins compute 1NN_INDEX profiles";
      else if (a->precision_type != SCAMP_PRECISION_MIXED && a->precision_type != SCAMP_PRECISION_SINGLE)
        m = "Error: batched joins run the mixed form (precision single or mixed)";
      else if (a->device != args[0].device)
        m = "Error: a batch runs on one device";
      else if (res && !res[k].profile_a)
        m = "Error: profile buffer missing";
      if (!m.empty()) rc = SCAMP_ERR_INVALID_ARGS;
    }
    if (rc) {
      *msg = "series " + std::to_string(k) + ": " + m;
      return rc;
    }
  }
  return SCAMP_OK;
}

}  // namespace
}  // namespace scamp_gb300

extern "C" int scamp_gb300_join_batch(const scamp_c_args* args, scamp_c_result* res, int count,
                                      char* errbuf, size_t errlen) {
  std::string msg;
  if (!args || !res || count <= 0) {
    set_err(errbuf, errlen, "Error: empty batch");
    return SCAMP_ERR_INVALID_ARGS;
  }
  int rc = validate_batch(args, res, count, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  Workspace* ws;
  rc = init_workspace(args[0].device, &ws, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  std::lock_guard<std::mutex> lock(ws->mu);
  rc = run_batch(*ws, args, res, count, ws->stream, &msg);
  if (rc) set_err(errbuf, errlen, msg);
  return rc;
}

extern "C" int scamp_gb300_tune_batch(const scamp_c_args* args, int count, int retune,
                                      int64_t* segment, char* errbuf, size_t errlen) {
  std::string msg;
  if (!args || count <= 0) {
    set_err(errbuf, errlen, "Error: empty batch");
    return SCAMP_ERR_INVALID_ARGS;
  }
  int rc = validate_batch(args, nullptr, count, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  Workspace* ws;
  rc = init_workspace(args[0].device, &ws, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  std::lock_guard<std::mutex> lock(ws->mu);
  rc = tune_batch(*ws, args, count, retune != 0, &msg);
  if (rc) { set_err(errbuf, errlen, msg); return rc; }
  if (segment) {
    for (int k = 0; k < count; ++k) {
      const int64_t m = static_cast<int64_t>(args[k].window);
      const auto it = ws->batch_seg.find(m);
      segment[k] = batch_segment(m, static_cast<int64_t>(args[k].len_a) - m + 1, mixed_1nn_slab_rows(),
                                 it == ws->batch_seg.end() ? 0 : it->second);
    }
  }
  return SCAMP_OK;
}
