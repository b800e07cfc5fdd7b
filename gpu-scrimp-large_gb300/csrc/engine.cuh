// engine.cuh -- device-side types and helpers shared by the join kernels.
//
// Terminology follows the reference (zpzim/GPU-SCRIMP-LARGE): a join compares
// every window ("subsequence") of a row series with every window of a column
// series; cell (i, j) lies on diagonal d = j - i; its covariance advances along
// the diagonal with cov(i+1, j+1) = cov(i, j) + df_c[j]*dg_r[i] + df_r[i]*dg_c[j]
// (src/cpu_kernels.cpp:166-171, src/kernels_compute.h:425-435) and its Pearson
// correlation is r = cov * invnorm_c[j] * invnorm_r[i].
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace scamp_gb300 {

// ---------------------------------------------------------------------------
// Profile keys.
//
// The 1NN_INDEX profile is merged on device with one 64-bit atomicMax per
// update.  key = (q << idx_bits) | (idx_mask - index), where
// q = floor((r + 2) * 2^F), F = 62 - idx_bits, is an order-preserving
// fixed-point image of the correlation r in [-2, 2).  A larger r gives a
// larger key; equal q resolve to the smaller index.  Key 0 is "no match"
// (the reference's {-2.0f, 0xFFFFFFFF}, src/common.cpp:294-299).  NaN maps
// to q = 0, so a NaN correlation never wins (the reference's strict '>'
// compare, src/kernel_gpu_utils.h:138-179).  With idx_bits = 27 (series up to
// 2^27 windows) the key resolves r to 2^-35 ~ 2.9e-11.
// ---------------------------------------------------------------------------
struct KeyLayout {
  int idx_bits;           // bits for the index
  int frac_bits;          // F = 62 - idx_bits
  uint64_t idx_mask;      // (1 << idx_bits) - 1
};

// q from the raw bits of a double, integer pipe only (the FP64 pipe is the
// bottleneck of the FP64 form, so no FP64 instruction is spent here).
__device__ __forceinline__ uint64_t q_from_double_bits(uint64_t bits, int F) {
  const uint32_t hi = static_cast<uint32_t>(bits >> 32);
  const int e = static_cast<int>((hi >> 20) & 0x7FF);
  // NaN / inf / |r| >= 2 never occur for valid cells; treat as no match.
  if (e >= 1024) return 0;
  const uint64_t sig = (bits & 0x000FFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0);
  // |r| * 2^F = sig * 2^(e - 1075 + F); shift right by s = 1075 - F - e.
  const int s = 1075 - F - e;
  uint64_t mag = (s >= 64) ? 0 : (s >= 0 ? (sig >> s) : (sig << (-s)));
  const uint64_t two = 2ull << F;  // 2 * 2^F
  return (bits >> 63) ? (two - mag) : (two + mag);
}

__device__ __forceinline__ uint64_t q_from_float_bits(uint32_t bits, int F) {
  const int e = static_cast<int>((bits >> 23) & 0xFF);
  if (e >= 128) return 0;  // NaN, inf, |r| >= 2
  const uint64_t sig = (bits & 0x7FFFFFu) | (e ? (1u << 23) : 0);
  const int s = 150 - F - e;
  uint64_t mag = (s >= 64) ? 0 : (s >= 0 ? (sig >> s) : (sig << (-s)));
  const uint64_t two = 2ull << F;
  return (bits >> 31) ? (two - mag) : (two + mag);
}

__device__ __forceinline__ uint64_t make_key(uint64_t q, int64_t index,
                                             const KeyLayout& kl) {
  return q == 0 ? 0ull
                : (q << kl.idx_bits) | (kl.idx_mask - static_cast<uint64_t>(index));
}

__host__ __device__ __forceinline__ double key_to_corr(uint64_t key,
                                                       const KeyLayout& kl) {
  const uint64_t q = key >> kl.idx_bits;
  return static_cast<double>(q) / static_cast<double>(1ull << kl.frac_bits) - 2.0;
}

__host__ __device__ __forceinline__ int64_t key_to_index(uint64_t key,
                                                         const KeyLayout& kl) {
  return static_cast<int64_t>(kl.idx_mask - (key & kl.idx_mask));
}

// ---------------------------------------------------------------------------
// Series statistics resident in HBM (one set per input series).
// ---------------------------------------------------------------------------
struct SeriesDev {
  const double* T;     // cleaned series (non-finite -> 0), n samples
  const double* mean;  // window means, ns
  const double* inv;   // inverse norms, NaN for NaN / flat windows, ns
  const double* df;    // (T[i+m]-T[i])/2, 0 at the last window
  const double* dg;    // (T[i+m]-mu[i+1]) + (T[i]-mu[i]), 0 at the last window
  const float* inv32;  // FP32 copies for the mixed form
  const float* df32;
  const float* dg32;
  // FP32 copy of the series relative to local offsets: the samples of block
  // b = t >> bshift are stored as (float)(T[t] - boff[b]), boff[b] being the
  // block's first sample, kept as an unevaluated float sum bhi[b] + blo[b].
  // mu_rel[w] = (float)(mean[w] - boff[w >> bshift]).  Every quantity stays
  // within the local variation of the series, so FP32 keeps its precision
  // even where the series' level wanders far from any global offset.
  const float* T32;
  const float* bhi;
  const float* blo;
  const float* mu_rel;
  int bshift;
  int64_t n;
  int64_t ns;
};

// One band problem: the cells (i, i + d) for d in [d_lo, d_hi) of a
// (rows x cols) matrix.  A self-join is one problem; an AB-join is two (the
// part above the main diagonal, and the part below it run transposed, as the
// reference does, src/tile.cpp:645-707).
struct Problem {
  SeriesDev R;  // row series
  SeriesDev C;  // column series
  int64_t d_lo, d_hi;   // diagonal range
  int64_t x_lo, x_hi;   // excluded diagonals (is_aligned), empty if x_lo >= x_hi
  uint64_t* key_col;    // 1NN_INDEX target of column results (or null)
  uint64_t* key_row;    // 1NN_INDEX target of row results (or null)
  double* sum_col;      // SUM_THRESH targets
  double* sum_row;
  int64_t band_begin;   // first global band of this problem
  int64_t nbands;
  int64_t m;            // window length
  int64_t seg_len;      // K: rows per segment (mixed 1NN kernel)
  float anchor_vcoef;   // initial drift estimate of an anchor / cov^2 (mixed 1NN)
  // Tensor-core anchors (anchor_tc.cu), or null: row s - tab_s0 of the table
  // holds the anchors cov(sK, sK + d) of the diagonals d_lo .. d_lo + tab_wp
  // - 1, blocks of 1024 diagonals stored residue-major.
  const float* anchor_tab;
  int64_t tab_wp;
  int64_t tab_s0;
};

constexpr int kMaxProblems = 2;

// A cell of the mixed 1NN join whose FP32 value is not trusted, settled after
// the join by verify_requests_kernel.
struct VerifyReq {
  uint64_t i;   // row window (low 40 bits) | problem index << 40
  uint32_t d;   // diagonal: column window = i + d
  float ub;     // upper bound of the cell's r (FP32 value + margin)
};

// Everything a join kernel needs, passed by value.
struct JoinParams {
  Problem prob[kMaxProblems];
  int nprob;
  // Batched joins (mixed 1NN kernel): when nbatch > 0 the problems are the
  // device array batch[0 .. nbatch) instead of prob[].
  const Problem* batch;
  int64_t nbatch;
  const int64_t* band_unit_prefix;  // [total_bands + 1] unit offsets
  int64_t unit_row0;                // first unit of every band in this launch (chunked joins)
  int64_t total_bands;
  int64_t total_units;
  unsigned long long* unit_counter; // persistent work queue head
  // [steps, slow steps, verifications, requests, largest trusted margin
  // (float bits, mixed form), (error word), candidates verified in place
  // because the request buffer was full]
  unsigned long long* counters;
  VerifyReq* vreq;                  // verification requests (mixed 1NN)
  int64_t vreq_cap;
  int* error_flag;                  // device error word (0 = ok)
  int64_t m;                        // window length
  int64_t seg_len;                  // K: rows per segment (two per unit)
  int64_t band_width;               // W: diagonals per band
  int profile_type;                 // 1 = 1NN_INDEX, 2 = SUM_THRESH
  double threshold;
  KeyLayout kl;
  float anchor_vcoef;               // initial drift estimate of an anchor / cov^2
  int refresh_cols;                 // mixed 1NN: refresh kept ring columns' bests per slab
  // MATRIX_SUMMARY, mixed form: the grid (order-preserving images of
  // floats, mat_w entries per grid row), windows per grid row and column
  // with their division magics ceil(2^64 / d), and per problem whether its
  // column results (cell (i, j) -> grid (i / rpc, j / cpc)) and its row
  // results (-> grid (j / rpc, i / cpc)) enter the grid.
  // APPROX_ALL_NEIGHBORS, mixed form: k > 0 makes key_row / key_col lists
  // of k keys per window (largest first) instead of one key
  int knn_k;
  unsigned* mat;
  int64_t mat_w;
  int64_t rows_per_cell, cols_per_cell;
  uint64_t rpc_magic, cpc_magic;
  int mat_col[kMaxProblems], mat_row[kMaxProblems];
};

// Outputs of the two experimental profile types (join_visit.cu).
struct VisitArgs {
  int mode;                        // 0: k best matches per window, 1: matrix summary
  unsigned long long* topk[2];     // k keys per window of A / B, largest first
  int k;
  unsigned* mat;                   // matrix entries (ordered images of floats)
  int64_t mat_w;
  int64_t rows_per_cell, cols_per_cell;
  int col_target[kMaxProblems];    // 0 = A, 1 = B, -1 = none, per problem
  int row_target[kMaxProblems];
};

// Locates global band `g` and unit-within-band for unit index `u`.
__device__ __forceinline__ void decode_unit(const JoinParams& P, int64_t u,
                                            int* prob, int64_t* band,
                                            int64_t* unit_in_band) {
  // binary search: largest g with prefix[g] <= u
  int64_t lo = 0, hi = P.total_bands;
  while (hi - lo > 1) {
    int64_t mid = (lo + hi) >> 1;
    if (P.band_unit_prefix[mid] <= u) lo = mid; else hi = mid;
  }
  int p = 0;
  if (P.nbatch > 0) {
    // largest problem whose first band is <= lo
    int64_t a = 0, b = P.nbatch;
    while (b - a > 1) {
      const int64_t mid = (a + b) >> 1;
      if (P.batch[mid].band_begin <= lo) a = mid; else b = mid;
    }
    p = static_cast<int>(a);
    *band = lo - P.batch[p].band_begin;
  } else {
    while (p + 1 < P.nprob && lo >= P.prob[p + 1].band_begin) ++p;
    *band = lo - P.prob[p].band_begin;
  }
  *prob = p;
  *unit_in_band = u - P.band_unit_prefix[lo] + P.unit_row0;
}

__device__ __forceinline__ const Problem& problem_of(const JoinParams& P, int p) {
  return P.nbatch > 0 ? P.batch[p] : P.prob[p];
}

// Rows of band b (first diagonal D0): every row whose cell on D0 is inside.
__host__ __device__ __forceinline__ int64_t band_rows(int64_t n_r, int64_t n_c,
                                                      int64_t D0) {
  int64_t r = n_c - D0;
  return r < n_r ? r : n_r;
}

// ---------------------------------------------------------------------------
// Kernels (launch wrappers live in engine.cu).
// ---------------------------------------------------------------------------
// One series of a batched statistics launch.
struct StatsJob {
  const double* T_raw;
  int64_t n, m;
  int bshift;
  double *T_clean, *mean, *inv, *df, *dg;
  float *T32, *bhi, *blo, *mu_rel, *inv32, *df32, *dg32;
};
// Block b of the launch works for job j with block_prefix[j] <= b < block_prefix[j + 1].
__global__ void stats_batch_kernel(const StatsJob* __restrict__ jobs,
                                   const int64_t* __restrict__ block_prefix, int njobs,
                                   int ultra, int chunk);

__global__ void stats_kernel(const double* __restrict__ T_raw, int64_t n,
                             int64_t m, int ultra, int chunk, int bshift,
                             double* __restrict__ T_clean, float* __restrict__ T32,
                             float* __restrict__ bhi, float* __restrict__ blo,
                             float* __restrict__ mu_rel,
                             double* __restrict__ mean, double* __restrict__ inv,
                             double* __restrict__ df, double* __restrict__ dg,
                             float* __restrict__ inv32, float* __restrict__ df32,
                             float* __restrict__ dg32);

// ULTRA update terms of one series: role_b 0 gives the "A" terms, 1 the "B"
// terms (stats.cu); T is the cleaned series, mean its window means.
__global__ void combined_stats_kernel(const double* __restrict__ T, int64_t n, int64_t m,
                                      const double* __restrict__ mean, int role_b,
                                      double* __restrict__ df, double* __restrict__ dg);
__global__ void join_fp64_kernel(JoinParams P);
__global__ void join_visit_kernel(JoinParams P, VisitArgs V);
__global__ void floats_to_ord_kernel(const float* __restrict__ in, unsigned* __restrict__ out,
                                     int64_t n);
__global__ void ord_to_floats_kernel(const unsigned* __restrict__ in, float* __restrict__ out,
                                     int64_t n);
__global__ void join_mixed_1nn_kernel(JoinParams P);  // mixed 1NN_INDEX
__global__ void join_mixed_sum_kernel(JoinParams P);  // mixed SUM_THRESH
// the same with the per-step covariance bound as the fast path's filter
__global__ void join_mixed_1nn_coarse_kernel(JoinParams P);
__global__ void join_mixed_sum_coarse_kernel(JoinParams P);
__global__ void join_mixed_mat_kernel(JoinParams P);  // mixed MATRIX_SUMMARY
__global__ void join_mixed_knn_kernel(JoinParams P);  // mixed APPROX_ALL_NEIGHBORS
__global__ void verify_requests_kernel(JoinParams P);

// Tensor-core anchors of one problem's chunk of anchor rows (anchor_tc.cu).
struct AnchorArgs {
  SeriesDev R, C;          // row and column series
  int64_t m, m_pad;        // window; terms padded to a multiple of 16
  int64_t K;               // anchor interval (a multiple of 1024)
  int64_t d_lo;            // first diagonal of the problem
  int64_t s0, nrows;       // anchor rows s0 .. s0 + nrows - 1
  int64_t rows_pad;        // nrows rounded up to the tile's 32 rows
  int64_t wp_pad;          // diagonals per table row (multiple of 1024)
  int64_t col_tiles;       // 1024-column tiles per group of 32 rows
  __nv_bfloat16* wsplit;   // [3][rows_pad][m_pad] split anchor windows, each
                           // 64-term block centred by its own mean
  float* xsum;             // [rows_pad] sums of those block-centred values
  float* xi;               // [rows_pad][nsub] the block means
  int64_t nsub;            // 64-term blocks per window (m_pad / 64, rounded up)
  float* table;            // [nrows][wp_pad]
  int* error_flag;         // set when a wait on the tensor cores gives up
  int desc_mode;           // shared-memory descriptor orientation (self-check)
  int wait_test;           // 1: issue no MMA, so every bounded wait runs out
                           // (the wait-limit self-test)
};
__global__ void anchor_split_kernel(AnchorArgs A);
__global__ void anchor_gemm_kernel(AnchorArgs A);
// FP64 check of a table: every `stride`-th entry against a direct FP64 dot;
// out[0] = max |table - cov| inv_r inv_c (as ordered bits), out[1] = count.
__global__ void anchor_check_kernel(AnchorArgs A, int64_t stride, unsigned long long* out);

// Seeds of the mixed 1NN join from a block-averaged pre-pass.
struct SeedArgs {
  SeriesDev X;            // windows seeded
  SeriesDev Y;            // their partners' series
  const uint64_t* paa;    // packed profile of X's block-averaged windows
  int64_t ns_paa;
  uint64_t* key_x;        // X's profile keys
  uint64_t* key_y;        // Y's profile keys, or null
  int64_t excl;           // self-join: |i - j| >= excl; -1 for AB joins
  int64_t m;
  KeyLayout kl;
  float floor;            // pre-pass entries not above it found no partner
  int factor;             // samples per block-averaged sample
};
__global__ void paa_kernel(const double* __restrict__ T, int64_t n_out, int f,
                           double* __restrict__ out);
__global__ void fill_floor_kernel(uint64_t* __restrict__ p, int64_t n, float floor);
__global__ void seed_kernel(SeedArgs S);
__global__ void diag_seed_kernel(const Problem* __restrict__ probs,
                                 const int64_t* __restrict__ win_prefix, int nprob, KeyLayout kl);

// Block-averaged pre-pass of a batch: one series' averaged copy.
struct PaaJob {
  const double* src;      // the series (raw samples)
  double* dst;            // n_out block means (NaN where a block holds a non-finite sample)
  int64_t n_out;
  int f;                  // samples per block
};
// Output sample t of the launch belongs to job p, out_prefix[p] <= t < out_prefix[p + 1].
__global__ void paa_batch_kernel(const PaaJob* __restrict__ jobs,
                                 const int64_t* __restrict__ out_prefix, int njobs);
// Keys {r = floor, index 0}: the pre-pass only looks for partners above floor.
__global__ void fill_key_floor_kernel(uint64_t* __restrict__ keys, int64_t n, float floor,
                                      KeyLayout kl);
// Seeds of one series of a batch from its pre-pass (self-join).
struct BatchSeedJob {
  SeriesDev X;               // the series' windows
  uint64_t* key;             // its profile keys
  const uint64_t* paa_key;   // keys of its block-averaged windows
  int64_t ns_paa;
  int64_t excl, m;
  int f;
};
// Warp w of the launch seeds averaged window w - paa_prefix[p] of job p.
__global__ void batch_seed_kernel(const BatchSeedJob* __restrict__ jobs,
                                  const int64_t* __restrict__ paa_prefix, int njobs,
                                  KeyLayout kl, float floor);

// FP64 re-evaluation of the reported 1NN cells (final_eval.cu): one side is
// one profile's keys, with the series of its windows (X) and of its
// partners (Y).  prof_in / max_in: the profile given on input (its entries
// that the join did not change keep their value); either may be null.
struct EvalSide {
  uint64_t* keys;
  const uint64_t* prof_in;
  const float* max_in;
  SeriesDev X, Y;
  int64_t ns, m;
};
struct EvalPair {
  EvalSide side[2];  // ns = 0 for a side that is not reported
  int64_t m;
  KeyLayout kl;
};
__global__ void final_eval_kernel(EvalPair E);
// The k-best lists of one side (k keys per window): every entry the join
// made is recomputed in FP64 and each list re-sorted; entries of the input
// list (prof_in, k packed entries per window) are kept as they are, entries
// whose FP64 value is not above `thr` dropped.
__global__ void knn_final_eval_kernel(EvalSide S, int k, double thr, KeyLayout kl);
int knn_mixed_max_k();  // longest list the mixed k-best form keeps
__global__ void final_eval_batch_kernel(const EvalSide* __restrict__ sides,
                                        const int64_t* __restrict__ win_prefix, int nsides,
                                        KeyLayout kl);

__global__ void floats_to_keys_kernel(const float* __restrict__ in, uint64_t* __restrict__ keys,
                                      int64_t n, KeyLayout kl);
__global__ void keys_to_floats_kernel(const uint64_t* __restrict__ keys, float* __restrict__ out,
                                      double* __restrict__ corr, int64_t n, KeyLayout kl);
__global__ void profile_to_keys_kernel(const uint64_t* __restrict__ in,
                                       uint64_t* __restrict__ keys, int64_t n,
                                       KeyLayout kl);
__global__ void keys_to_profile_kernel(const uint64_t* __restrict__ keys,
                                       uint64_t* __restrict__ out,
                                       double* __restrict__ corr, int64_t n,
                                       KeyLayout kl);

}  // namespace scamp_gb300
