// join_mixed_1nn.cu -- the mixed-precision band kernel: FP32 filter over an
// FP32 recurrence, exact path for the blocks it flags.  One body, five
// instantiations: 1NN_INDEX (per-cell and per-step-bound filters),
// SUM_THRESH, APPROX_ALL_NEIGHBORS (k-best lists) and MATRIX_SUMMARY.
//
// Work decomposition as in join_fp64.cu (persistent kernel over a device
// queue of units = band of kBand diagonals x two row segments of seg_len
// rows; every thread advances kDiags diagonals in both segments as packed
// f32x2 pairs, .x = first segment, .y = second).
//
// Per cell the hot loop issues exactly the reference's arithmetic
// (src/kernels_compute.h:425-435): two FMAs advance the covariance and two
// multiplies form r = cov * invnorm_col * invnorm_row -- as f32x2 pair
// instructions, so the FP32 pipe, not the issue slot, bounds the loop.  What
// the reference does per cell on top of that -- compare, select, index
// bookkeeping (src/kernels_compute.h:25-113) -- is reduced to one running
// maximum of the whole 8x8x2 block per thread (3-input max.f32, two cells per
// instruction).
//
// 1NN_INDEX: a block whose maximum could beat the smallest best-so-far among
// its rows and columns, less an error margin, is queued for the exact path.
// The margin bounds the FP32 drift since the diagonal's anchor: per diagonal
// the kernel accumulates cov^2 and per thread the squared bound of the
// increments |df_c dg_r| + |df_r dg_c|, and uses
//   margin = C * 2^-24 * sqrt(rows * (sum cov^2 + sum inc^2)) * inv_c * inv_r.
// Each warp drains its queue cooperatively (8 lanes per queued block, both
// segments of a diagonal per lane as an f32x2 pair): cells that may improve
// their row or column are published with their FP32 value when the margin is
// below kTrust; otherwise the lower bound r - margin is published and the
// cell goes to a request buffer that verify_requests_kernel settles after the
// join with a direct dot product of the two centred windows.  The k-best
// form filters at each window's k-th best and inserts into its lists instead.
//
// SUM_THRESH (the reference's sum of every r above the threshold,
// src/kernels_compute.h:87-113 and 380-392), join_mixed_sum_kernel: every
// cell is decided in the main loop.  A cell above the threshold by more than
// the step's margin adds its FP32 r to its row's and its column's slab sums
// in shared memory (flushed to the FP64 profile by atomicAdd when the row's
// slab ends or the column leaves the column ring); the rare cells within the
// margin are settled by their own margin (sum_near): by the FP32 r within
// kTrust, else by a verification request that verify_requests_kernel adds if
// its directly computed r is above the threshold.
//
// MATRIX_SUMMARY: each thread keeps the running maximum of the grid entry its
// blocks fall in and publishes it when they move on (mat_cells_block routes
// the cells of a block that crosses a grid boundary).
//
// Anchors and verifications read an FP32 copy of each series stored relative
// to local block offsets (stats.cu), with every factor centred by its
// window's mean, so FP32 keeps its precision wherever the series wanders.
#include <cstdint>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kDiags = 8;
constexpr int kBand = kThreads * kDiags;  // 1024 diagonals per unit
constexpr int kRows = 8;                  // rows per step
constexpr int kSlab = 128;                // rows staged per slab
constexpr int kSteps = kSlab / kRows;
constexpr int kCols = kSlab + kBand;      // staged columns per slab
constexpr int kBlocks = kCols / 8;        // 8-column blocks
// The staged columns form a ring over the unit's rows: slab q holds unit
// columns 128 q .. 128 q + kCols - 1 at ring columns (128 q + c) mod kCols, so
// a slab stages only the kSlab columns entering it.  Ring columns
// 0 .. kGhost - 1 are repeated after the end, so that a step's 15-column
// window never wraps.
constexpr int kGhost = 16;
constexpr int kPadG = kCols + kGhost + (kCols + kGhost) / 8;
constexpr int kAnchorChunk = 512;         // row-window samples per anchor pass
constexpr int kYSpan = kBand + kAnchorChunk + 16;     // staged column samples
constexpr int kYPad = (kYSpan / 8) * 10;              // padded: 10 pairs per 8
// blocks hold >= 32 samples: the span plus the block after its end
constexpr int kSpanBlk = kYSpan / 32 + 3;
constexpr int kQueue = 16;                // queued blocks per warp
constexpr float kEps = 5.9604645e-8f;     // 2^-24
constexpr float kBoundC = 4.0f;
// kBoundC * kEps * sqrt(kRows), widened by 2^-16 (see the step's threshold)
static_assert(kRows == 8, "kStepMarginC holds sqrt(8)");
constexpr float kStepMarginC = kBoundC * kEps * 2.8284271f * 1.0000153f;
// A candidate whose drift margin exceeds kTrust is verified by a direct dot
// product.  The margin is a statistical bound; 5e-6 leaves room for it to be
// exceeded (measured: max |r| error 6.6e-6 at 2048 rows per anchor, where
// kTrust = 8e-6 let one cell reach 1.07e-5).
constexpr float kTrust = 5e-6f;
constexpr float kNoTarget = 3.0e38f;      // best of a side that is not computed

typedef unsigned long long u64;

__device__ __forceinline__ u64 f2u(float2 v) {
  return (static_cast<u64>(__float_as_uint(v.y)) << 32) | __float_as_uint(v.x);
}
__device__ __forceinline__ float2 u2f(u64 v) {
  return make_float2(__uint_as_float(static_cast<uint32_t>(v)),
                     __uint_as_float(static_cast<uint32_t>(v >> 32)));
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2u(a)), "l"(f2u(b)), "l"(f2u(c)));
  return u2f(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2u(a)), "l"(f2u(b)));
  return u2f(d);
}
__device__ __forceinline__ float max3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
// PTX sqrt.approx.f32: an approximate square root (a few ulp); sqrt(0) = 0.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float qnan() { return __int_as_float(0x7FC00000); }

// Largest |cov| over the 8 diagonals, per segment (NaN entries ignored).
__device__ __forceinline__ float2 absmax8(const float2 (&c)[8]) {
  float x = max3(fabsf(c[0].x), fabsf(c[1].x), fabsf(c[2].x));
  float y = max3(fabsf(c[0].y), fabsf(c[1].y), fabsf(c[2].y));
  x = max3(x, fabsf(c[3].x), fabsf(c[4].x));
  y = max3(y, fabsf(c[3].y), fabsf(c[4].y));
  x = max3(x, fabsf(c[5].x), fabsf(c[6].x));
  y = max3(y, fabsf(c[5].y), fabsf(c[6].y));
  return make_float2(fmaxf(x, fabsf(c[7].x)), fmaxf(y, fabsf(c[7].y)));
}

// Correlation encoded by a profile key, rounded down (a filter threshold may
// only be lower than the true best).  Integer pipe only.
__device__ __forceinline__ float key_corr_floor(u64 key, const KeyLayout& kl) {
  const u64 q = key >> kl.idx_bits;
  if (q == 0) return -3.0f;                                 // no match yet
  const int p = 63 - __clzll(static_cast<long long>(q));    // leading bit
  const int e = p - kl.frac_bits;                           // (r + 2) in [2^e, 2^(e+1))
  const uint32_t mant = static_cast<uint32_t>((q << (63 - p)) >> 40) & 0x7FFFFFu;
  const float v = __uint_as_float((static_cast<uint32_t>(e + 127) << 23) | mant);
  return v - 2.0f;                                          // exact for v in [1, 4)
}

// A block queued for the exact path: the owner's covariances at the END of
// the step (the drain rewinds them), the step's drift estimate (largest
// sum cov^2 over the owner's diagonals plus the increment bound) and the
// block's position.
struct SlowItem {
  float2 cov[kDiags];  // covariances after the item's last step
  float2 vw;
  int s;      // first step within the slab | number of steps (1 or 2) << 8 |
              // segments to walk << 16 (bits 0-1 first step, 2-3 second)
  int owner;  // thread index of the owner
};

// CTA-uniform context of the exact path, kept in shared memory.
struct SlowCtx {
  const Problem* pr;
  int64_t rbase[2];
  int64_t D0;  // first diagonal of the unit; thread t owns D0 + t*kDiags ..
  int ring0;   // ring column of the slab's first staged column
  // SUM_THRESH: cells with r > thr add r to their row's and column's sums
  // (r_best / c_best hold the slab's float sums instead of bests)
  bool sum_mode;
  float thr;
  int64_t m;
  KeyLayout kl;
  int prob;                        // index of the problem in JoinParams
  VerifyReq* vreq;                 // deferred verification requests
  unsigned long long* vcount;      // their count (may exceed vcap)
  int64_t vcap;
  unsigned long long* tmargin;     // largest drift margin of a trusted FP32 value (float bits)
  unsigned long long* overflow;    // candidates verified in place (request buffer full)
  // MATRIX_SUMMARY: the grid and its geometry (JoinParams), the current
  // problem's targets
  int knn_k;  // APPROX_ALL_NEIGHBORS: list length (0 otherwise)
  unsigned* mat;
  int64_t mat_w;
  int64_t rpc, cpc;
  uint64_t rpc_magic, cpc_magic;
  bool mcol, mrow;
};

struct Smem {
  union {
    struct {
      // {df.x, df.y} and {dg.x, dg.y} per staged column pair: separate
      // 8-byte arrays, so that 64-bit loads at a stride of 9 slots meet no
      // bank conflict
      float2 c_df[kPadG];
      float2 c_dg[kPadG];
      float2 c_iv[kPadG];  // {inv.x, inv.y}
    } s;
    struct {
      float2 xr[kAnchorChunk];    // centred row windows of both segments (chunk)
      float2 yc[kYPad];           // column samples (block-relative), padded
      float2 cb[2][kSpanBlk];     // {bhi, blo} of the blocks of the staged span
    } a;
  } u;
  float2 c_best[kCols];
  // per 8-column ring block (entry kBlocks repeats block 0): smallest best,
  // largest inverse norm, largest |df|, |dg|
  float2 c_blkmin[kBlocks + 1];
  float2 c_blkmax_iv[kBlocks + 1];
  float4 c_blkmax_fg[kBlocks + 1];
  float4 r_fg[kSlab];
  float2 r_iv[kSlab];
  float2 r_best[kSlab];
  float2 r_stepmin[kSteps];
  float2 r_stepmax_iv[kSteps];
  float4 r_stepmax_fg[kSteps];
  SlowItem queue[kWarps][kQueue];
  Problem prob;  // the current unit's band problem
  long long unit, band, unit_in_band;
  int prob_index;
  SlowCtx cx;
};

// Filter-table entry: smallest best, largest inverse norm, largest |df|,
// |dg| (per segment), over a set of columns or rows.
struct TableEntry {
  float2 mn, mx;
  float4 mf;
};

// One column's or row's entry; a NaN inverse norm (window that cannot match)
// counts as 0, as fmaxf against a 0 start would.
__device__ __forceinline__ TableEntry table_entry(float4 f, float2 iv, float2 best) {
  TableEntry e;
  e.mn = best;
  e.mx = make_float2(fmaxf(0.f, iv.x), fmaxf(0.f, iv.y));
  e.mf = make_float4(fabsf(f.x), fabsf(f.y), fabsf(f.z), fabsf(f.w));
  return e;
}

__device__ __forceinline__ void combine(TableEntry& a, const TableEntry& b) {
  a.mn = make_float2(fminf(a.mn.x, b.mn.x), fminf(a.mn.y, b.mn.y));
  a.mx = make_float2(fmaxf(a.mx.x, b.mx.x), fmaxf(a.mx.y, b.mx.y));
  a.mf = make_float4(fmaxf(a.mf.x, b.mf.x), fmaxf(a.mf.y, b.mf.y),
                     fmaxf(a.mf.z, b.mf.z), fmaxf(a.mf.w, b.mf.w));
}

// Reduces an entry over aligned groups of 8 lanes (whole warp active).
__device__ __forceinline__ void reduce8(TableEntry& e) {
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    TableEntry x;
    x.mn.x = __shfl_xor_sync(0xffffffffu, e.mn.x, o);
    x.mn.y = __shfl_xor_sync(0xffffffffu, e.mn.y, o);
    x.mx.x = __shfl_xor_sync(0xffffffffu, e.mx.x, o);
    x.mx.y = __shfl_xor_sync(0xffffffffu, e.mx.y, o);
    x.mf.x = __shfl_xor_sync(0xffffffffu, e.mf.x, o);
    x.mf.y = __shfl_xor_sync(0xffffffffu, e.mf.y, o);
    x.mf.z = __shfl_xor_sync(0xffffffffu, e.mf.z, o);
    x.mf.w = __shfl_xor_sync(0xffffffffu, e.mf.w, o);
    combine(e, x);
  }
}

template <int P>
struct Parity {
  static constexpr int value = P;
};

static_assert(kSlab == kThreads, "one staged row per thread");
static_assert(kCols % kThreads == 0, "whole warps stage the columns");

// Four CTAs per SM: 4 x (shared memory + 1 KB reserved) within 228 KB.
static_assert(sizeof(Smem) + 1024 <= 228 * 1024 / 4, "shared memory exceeds 4 CTAs/SM");

__device__ __forceinline__ int padc(int c) { return c + (c >> 3); }
// Ring column of slab-relative column c (0 <= c < kCols).
__device__ __forceinline__ int ringc(int ring0, int c) {
  const int r = ring0 + c;
  return r >= kCols ? r - kCols : r;
}

// {df.x, df.y, dg.x, dg.y} of the staged column in padded slot `slot`.
__device__ __forceinline__ float4 col_fg(const Smem& sm, int slot) {
  const float2 a = sm.u.s.c_df[slot], b = sm.u.s.c_dg[slot];
  return make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ int pady2(int x) { return x + (x >> 3) * 2; }

// Offset of block b relative to block b0, as the float sum of the two
// blocks' hi/lo parts: exact while the two offsets are within a factor of two.
__device__ __forceinline__ float block_delta(const SeriesDev& S, int64_t b, int64_t b0) {
  return (S.bhi[b] - S.bhi[b0]) + (S.blo[b] - S.blo[b0]);
}

// Partial covariance of row window i and column window j over the terms
// t in [tb, te), FP32: each factor formed as (sample relative to its block
// offset) + (block offset - window mean), summed per run of terms that share
// both blocks.
__device__ __forceinline__ float cov_part(const SeriesDev& R, const SeriesDev& C,
                                          int64_t i, int64_t j, int64_t tb, int64_t te_all) {
  const int sh = R.bshift;
  const int64_t bi = i >> sh, bj = j >> sh;
  const float mri = R.mu_rel[i], mcj = C.mu_rel[j];
  float acc = 0.f;
  int64_t t = tb;
  while (t < te_all) {
    const int64_t br = (i + t) >> sh, bc = (j + t) >> sh;
    int64_t te = ((br + 1) << sh) - i;
    const int64_t te2 = ((bc + 1) << sh) - j;
    if (te2 < te) te = te2;
    if (te_all < te) te = te_all;
    const float xc = block_delta(R, br, bi) - mri;
    const float yc = block_delta(C, bc, bj) - mcj;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
    int64_t u = t;
    for (; u + 3 < te; u += 4) {
      p0 = fmaf(R.T32[i + u] + xc, C.T32[j + u] + yc, p0);
      p1 = fmaf(R.T32[i + u + 1] + xc, C.T32[j + u + 1] + yc, p1);
      p2 = fmaf(R.T32[i + u + 2] + xc, C.T32[j + u + 2] + yc, p2);
      p3 = fmaf(R.T32[i + u + 3] + xc, C.T32[j + u + 3] + yc, p3);
    }
    for (; u < te; ++u) p0 = fmaf(R.T32[i + u] + xc, C.T32[j + u] + yc, p0);
    acc += (p0 + p1) + (p2 + p3);
    t = te;
  }
  return acc;
}

// The same covariance computed by a whole warp: lane l sums the terms
// t = l, l + 32, ...; the partial sums meet in a shuffle reduction.
__device__ __forceinline__ float verify_cov_warp(const SeriesDev& R, const SeriesDev& C,
                                                 int64_t i, int64_t j, int64_t m, int lane) {
  const int sh = R.bshift;
  const int64_t bi = i >> sh, bj = j >> sh;
  const float mri = R.mu_rel[i], mcj = C.mu_rel[j];
  const float hr0 = R.bhi[bi], lr0 = R.blo[bi], hc0 = C.bhi[bj], lc0 = C.blo[bj];
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int64_t t0 = lane; t0 < m; t0 += 128) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t t = t0 + 32 * u;
      if (t < m) {
        const int64_t br = (i + t) >> sh, bc = (j + t) >> sh;
        const float x = R.T32[i + t] + (((R.bhi[br] - hr0) + (R.blo[br] - lr0)) - mri);
        const float y = C.T32[j + t] + (((C.bhi[bc] - hc0) + (C.blo[bc] - lc0)) - mcj);
        acc[u] = fmaf(x, y, acc[u]);
      }
    }
  }
  float a = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  return a;
}

// The whole covariance, one lane (the diagonal seeds).
__device__ __noinline__ float verify_cov_lane(const SeriesDev& R, const SeriesDev& C,
                                              int64_t i, int64_t j, int64_t m) {
  return cov_part(R, C, i, j, 0, m);
}


__device__ __forceinline__ void publish(Smem& sm, const SlowCtx& cx, float rv, int64_t i,
                                        int64_t j, int rslot, int cslot, int g) {
  const Problem& pr = *cx.pr;
  const float rb = g ? sm.r_best[rslot].y : sm.r_best[rslot].x;
  const float cb = g ? sm.c_best[cslot].y : sm.c_best[cslot].x;
  if (rv > rb) {
    atomicMax(reinterpret_cast<u64*>(pr.key_row + i),
              make_key(q_from_float_bits(__float_as_uint(rv), cx.kl.frac_bits), j, cx.kl));
    // The float copies only filter candidates; a racing store of a smaller
    // value costs extra work later, never a wrong result.
    if (g) sm.r_best[rslot].y = rv; else sm.r_best[rslot].x = rv;
  }
  if (rv > cb) {
    atomicMax(reinterpret_cast<u64*>(pr.key_col + j),
              make_key(q_from_float_bits(__float_as_uint(rv), cx.kl.frac_bits), i, cx.kl));
    if (g) sm.c_best[cslot].y = rv; else sm.c_best[cslot].x = rv;
  }
}

// Inserts `key` into a list of k keys kept largest first: each slot keeps
// the larger of its key and the incoming one and passes the smaller on, so
// after every insertion slot s holds the (s+1)-th largest key inserted.
__device__ __forceinline__ void topk_insert(u64* slots, int k, u64 key) {
  for (int s = 0; s < k && key != 0; ++s) {
    const u64 old = atomicMax(slots + s, key);
    if (old < key) key = old;
  }
}

// A list's filter value: its k-th best (rounded down), at least the threshold.
__device__ __forceinline__ float knn_floor(const uint64_t* list, int k, float thr,
                                           const KeyLayout& kl) {
  return fmaxf(key_corr_floor(list[k - 1], kl), thr);
}

// APPROX_ALL_NEIGHBORS counterpart of publish(): a cell above its row's
// (column's) k-th best enters that window's list; the shared filter value
// then follows the list's new k-th entry.
__device__ __noinline__ void knn_publish(Smem& sm, const SlowCtx& cx, float rv, int64_t i,
                                         int64_t j, int rslot, int cslot, int g) {
  if (!(rv > cx.thr)) return;
  const Problem& pr = *cx.pr;
  const int k = cx.knn_k;
  const float rb = g ? sm.r_best[rslot].y : sm.r_best[rslot].x;
  const float cb = g ? sm.c_best[cslot].y : sm.c_best[cslot].x;
  const uint64_t q = q_from_float_bits(__float_as_uint(rv), cx.kl.frac_bits);
  if (rv > rb && pr.key_row) {
    u64* list = reinterpret_cast<u64*>(pr.key_row + i * k);
    topk_insert(list, k, make_key(q, j, cx.kl));
    const float nb = knn_floor(pr.key_row + i * k, k, cx.thr, cx.kl);
    if (g) sm.r_best[rslot].y = nb; else sm.r_best[rslot].x = nb;
  }
  if (rv > cb && pr.key_col) {
    u64* list = reinterpret_cast<u64*>(pr.key_col + j * k);
    topk_insert(list, k, make_key(q, i, cx.kl));
    const float nb = knn_floor(pr.key_col + j * k, k, cx.thr, cx.kl);
    if (g) sm.c_best[cslot].y = nb; else sm.c_best[cslot].x = nb;
  }
}

// One cell of the exact path: publish (or add) its FP32 value when that is
// safe, else queue a verification request at `slot`.
__device__ __forceinline__ void exact_cell(Smem& sm, const SlowCtx& cx, float rv, float mk,
                                           bool cand, bool req, unsigned long long slot,
                                           int64_t i, int64_t j, int rslot, int cslot, int g,
                                           float& add, float& tmax, int& nreq) {
  if (!cand) return;
  if (req) {
    ++nreq;
    if (slot < static_cast<unsigned long long>(cx.vcap)) {
      // (1NN: the lower bound raises the filters at once; a k-best list
      // would keep it beside the verified value)
      if (!cx.sum_mode && !cx.knn_k) publish(sm, cx, rv - mk, i, j, rslot, cslot, g);
      VerifyReq q;
      q.i = static_cast<uint64_t>(i) | (static_cast<uint64_t>(cx.prob) << 40);
      q.d = static_cast<uint32_t>(j - i);
      q.ub = rv + mk;
      cx.vreq[slot] = q;
    } else {
      // request buffer full: verified in place by this lane (slow: the
      // counted overflow makes later joins size the buffer for it)
      const Problem& pr = *cx.pr;
      // (the dot inline: a call from here makes every band kernel that
      // calls the exact path keep more registers live across it)
      const float ev = (cov_part(pr.R, pr.C, i, j, 0, cx.m) * pr.C.inv32[j]) * pr.R.inv32[i];
      atomicAdd(cx.overflow, 1ull);
      if (cx.sum_mode) add = ev > cx.thr ? ev : 0.f;
      else if (cx.knn_k) knn_publish(sm, cx, ev, i, j, rslot, cslot, g);
      else publish(sm, cx, ev, i, j, rslot, cslot, g);
    }
  } else if (cx.sum_mode) {
    add = rv > cx.thr ? rv : 0.f;
    if (add != 0.f) tmax = fmaxf(tmax, mk);
  } else {
    if (cx.knn_k) knn_publish(sm, cx, rv, i, j, rslot, cslot, g);
    else publish(sm, cx, rv, i, j, rslot, cslot, g);
    tmax = fmaxf(tmax, mk);
  }
}

// Exact path of queued blocks, 8 lanes per block (four blocks per pass):
// lane k holds the covariances of diagonal k in both segments (an f32x2
// pair, as the fast path holds them) at the block's end and visits the
// block's rows (8 per step), each with the covariance the fast path used
// there.  kMerged (the per-cell-filter kernels): one pass, rows last to
// first, stepping the covariance back over each row before checking it.
// Otherwise (the per-step-bound kernels) the covariance is first rewound to
// the block's start, then the rows are checked first to last (measured: the
// one-pass form is 6-7% faster on the AB and batched joins of short windows,
// 1.3% slower on the self-join of 1024-sample windows).  Every cell that may
// improve its row or column is published with its FP32 value when its
// margin is within kTrust.  A cell with a larger margin is published with the lower bound
// rv - margin (so the filters rise at once) and appended to the
// verification requests, which verify_requests_kernel settles after the
// join.  Returns the lane's number of requests.
template <bool kMerged>
__device__ __noinline__ int drain_queue(Smem& sm, int warp, int count, int lane) {
  __syncwarp();  // the queue was written by other lanes
  const SlowCtx& cx = sm.cx;
  const int k = lane & 7;
  int nreq = 0;
  float tmax = 0.f;  // largest margin of a value published or added unverified
  for (int p = 0; p < count; p += 4) {
    // every lane runs the pass (warp-wide request reservation); a lane
    // without a block carries the first queued one and checks nothing
    const int item = p + (lane >> 3);
    const bool act = item < count;
    const SlowItem& it = sm.queue[warp][act ? item : 0];
    float2 c = it.cov[k];
    const float2 vw = it.vw;
    const int s0 = it.s & 255;
    const int nrows = act ? kRows * ((it.s >> 8) & 255) : 0;
    const int msk = (it.s >> 16) & 15;  // segments to walk, per step of the block
    // the blocks of a pass may differ in length: the row loop below runs
    // the longest on every lane (its ballots need the whole warp)
    const int nrows_w = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(nrows)));
    const int r0 = s0 * kRows;
    const int cb0 = 8 * (s0 + it.owner) + k;  // staged column at row 0
    if constexpr (!kMerged) {
#pragma unroll 8
      for (int rr = nrows - 1; rr >= 0; --rr) {
        const float4 rf = sm.r_fg[r0 + rr];
        const float4 cf = col_fg(sm, padc(ringc(cx.ring0, cb0 + rr)));
        c = fma2(make_float2(-rf.x, -rf.y), make_float2(cf.z, cf.w), c);
        c = fma2(make_float2(-cf.x, -cf.y), make_float2(rf.z, rf.w), c);
      }
    }
    const float2 vk = make_float2(kBoundC * kEps * sqrtf(kRows * vw.x),
                                  kBoundC * kEps * sqrtf(kRows * vw.y));
    const int64_t jd = cx.D0 + it.owner * kDiags + k;  // the lane's diagonal
    // kMerged, rows last to first: stepping back over row rr leaves c at the
    // covariance the fast path used in row rr (the order of a block's rows
    // does not matter: updates are atomic maxima or sums, and every floor
    // read is a value already published)
#pragma unroll 1
    for (int rw = kMerged ? nrows_w - 1 : 0; kMerged ? rw >= 0 : rw < nrows_w;
         rw += kMerged ? -1 : 1) {
      const bool live = rw < nrows;
      const int rr = live ? rw : 0;  // rows past the block's end read row 0
      const int cs = cb0 + rr;
      const int rcs = ringc(cx.ring0, cs);  // its ring column
      const float4 rf = sm.r_fg[r0 + rr];
      const float4 cf = col_fg(sm, padc(rcs));
      if constexpr (kMerged) {
        if (live) {
          c = fma2(make_float2(-rf.x, -rf.y), make_float2(cf.z, cf.w), c);
          c = fma2(make_float2(-cf.x, -cf.y), make_float2(rf.z, rf.w), c);
        }
      }
      const float2 ivr = sm.r_iv[r0 + rr];
      const float2 ivc = sm.u.s.c_iv[padc(rcs)];
      const float2 rv = mul2(mul2(c, ivc), ivr);  // the fast path's rounding
      const float2 mk = mul2(mul2(vk, ivc), ivr);
      const float2 rb = sm.r_best[r0 + rr];
      const float2 cbv = sm.c_best[rcs];
      // the value to beat: the row's and column's bests, or the threshold
      const float tx = cx.sum_mode ? cx.thr : fminf(rb.x, cbv.x);
      const float ty = cx.sum_mode ? cx.thr : fminf(rb.y, cbv.y);
      const int sm2 = msk >> (2 * (rw >> 3));
      const bool cx_ = live && (sm2 & 1) && rv.x + mk.x > tx;
      const bool cy_ = live && (sm2 & 2) && rv.y + mk.y > ty;
      // SUM_THRESH: a cell surely above the threshold counts with its FP32 r
      const bool qx = cx_ && mk.x > kTrust && !(cx.sum_mode && rv.x - mk.x > tx);
      const bool qy = cy_ && mk.y > kTrust && !(cx.sum_mode && rv.y - mk.y > ty);
      const unsigned mx = __ballot_sync(0xffffffffu, qx), my = __ballot_sync(0xffffffffu, qy);
      unsigned long long sx = 0, sy = 0;
      if (mx | my) {
        const int leader = __ffs(mx | my) - 1;
        unsigned long long base = 0;
        if (lane == leader)
          base = atomicAdd(cx.vcount, static_cast<unsigned long long>(__popc(mx) + __popc(my)));
        base = __shfl_sync(0xffffffffu, base, leader);
        const unsigned lt = (1u << lane) - 1u;
        sx = base + __popc(mx & lt) + __popc(my & lt);
        sy = sx + (qx ? 1u : 0u);
      }
      float ax = 0.f, ay = 0.f;  // SUM_THRESH: what the cells add to their rows and column
      if (cx_ || cy_) {
        const int64_t i0 = cx.rbase[0] + r0 + rr, i1 = cx.rbase[1] + r0 + rr;
        exact_cell(sm, cx, rv.x, mk.x, cx_, qx, sx, i0, i0 + jd, r0 + rr, rcs, 0, ax, tmax, nreq);
        exact_cell(sm, cx, rv.y, mk.y, cy_, qy, sy, i1, i1 + jd, r0 + rr, rcs, 1, ay, tmax, nreq);
      }
      if (cx.sum_mode) {
        // the 8 diagonals of a block meet in one row: reduce over its lanes
        // (k = lane bits 0-2) before the shared-memory atomics
        if (ax != 0.f) atomicAdd(&sm.c_best[rcs].x, ax);
        if (ay != 0.f) atomicAdd(&sm.c_best[rcs].y, ay);
        float2 rs = make_float2(ax, ay);
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
          rs.x += __shfl_xor_sync(0xffffffffu, rs.x, o);
          rs.y += __shfl_xor_sync(0xffffffffu, rs.y, o);
        }
        if (k == 0) {
          if (rs.x != 0.f) atomicAdd(&sm.r_best[r0 + rr].x, rs.x);
          if (rs.y != 0.f) atomicAdd(&sm.r_best[r0 + rr].y, rs.y);
        }
      }
      if constexpr (!kMerged) {
        c = fma2(make_float2(cf.x, cf.y), make_float2(rf.z, rf.w), c);
        c = fma2(make_float2(rf.x, rf.y), make_float2(cf.z, cf.w), c);
      }
    }
  }
  // the trusted margins, one atomic per drain (non-negative floats order as
  // their bit patterns)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) tmax = fmaxf(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
  if (lane == 0 && tmax > 0.f) atomicMax(cx.tmargin, static_cast<unsigned long long>(__float_as_uint(tmax)));
  __syncwarp();
  return nreq;
}

// SUM_THRESH: the cells of a thread-step that lie within the step's margin
// m of the threshold (flags fx, fy per segment; rare), walked again by their
// lane alone from the step's start (rewound from the covariances at its
// end, as the exact path rewinds).  Each such cell is decided by its own
// margin mk = vk inv_c inv_r (vk per segment, the exact path's formula): by
// its FP32 r when mk is within kTrust, else by a verification request (a
// full request buffer verifies it in place).  Adds go straight to the slab's
// shared-memory sums.  Returns the lane's number of requests.
__device__ __noinline__ int sum_near(Smem& sm, const float2 (&cov_end)[kDiags], int s, int t,
                                     bool fx, bool fy, float2 m, float2 vk) {
  const SlowCtx& cx = sm.cx;
  const int r0 = s * kRows;
  const int cb0 = 8 * (s + t);
  float2 c[kDiags];
#pragma unroll
  for (int k = 0; k < kDiags; ++k) c[k] = cov_end[k];
#pragma unroll 1
  for (int rr = kRows - 1; rr >= 0; --rr) {
    const float4 rf = sm.r_fg[r0 + rr];
#pragma unroll
    for (int k = 0; k < kDiags; ++k) {
      const float4 cf = col_fg(sm, padc(ringc(cx.ring0, cb0 + rr + k)));
      c[k] = fma2(make_float2(-rf.x, -rf.y), make_float2(cf.z, cf.w), c[k]);
      c[k] = fma2(make_float2(-cf.x, -cf.y), make_float2(rf.z, rf.w), c[k]);
    }
  }
  int nreq = 0;
  float tmax = 0.f;
#pragma unroll 1
  for (int rr = 0; rr < kRows; ++rr) {
    const float4 rf = sm.r_fg[r0 + rr];
    const float2 ivr = sm.r_iv[r0 + rr];
#pragma unroll 1
    for (int k = 0; k < kDiags; ++k) {
      const int rcx = ringc(cx.ring0, cb0 + rr + k);
      const int slot = padc(rcx);
      const float2 ivc = sm.u.s.c_iv[slot];
      const float2 r2 = mul2(mul2(c[k], ivc), ivr);
      const float2 mk2 = mul2(mul2(vk, ivc), ivr);
#pragma unroll 1
      for (int g = 0; g < 2; ++g) {
        const float r = g ? r2.y : r2.x;
        if (!((g ? fy : fx) && fabsf(r - cx.thr) <= (g ? m.y : m.x))) continue;  // NaN: skip
        const float mk = g ? mk2.y : mk2.x;
        float add = 0.f;
        if (mk <= kTrust) {
          if (r > cx.thr) {
            add = r;
            tmax = fmaxf(tmax, mk);
          }
        } else {
          const int64_t i = cx.rbase[g] + r0 + rr;
          const int64_t j = i + cx.D0 + t * kDiags + k;
          const unsigned long long sl = atomicAdd(cx.vcount, 1ull);
          ++nreq;
          if (sl < static_cast<unsigned long long>(cx.vcap)) {
            VerifyReq q;
            q.i = static_cast<uint64_t>(i) | (static_cast<uint64_t>(cx.prob) << 40);
            q.d = static_cast<uint32_t>(j - i);
            q.ub = r + mk;
            cx.vreq[sl] = q;
          } else {
            // request buffer full: verified in place (counted)
            const Problem& pr = *cx.pr;
            const float ev = (cov_part(pr.R, pr.C, i, j, 0, cx.m) * pr.C.inv32[j]) * pr.R.inv32[i];
            atomicAdd(cx.overflow, 1ull);
            if (ev > cx.thr) add = ev;
          }
        }
        if (add != 0.f) {
          atomicAdd(g ? &sm.r_best[r0 + rr].y : &sm.r_best[r0 + rr].x, add);
          atomicAdd(g ? &sm.c_best[rcx].y : &sm.c_best[rcx].x, add);
        }
      }
      const float4 cf = col_fg(sm, slot);
      c[k] = fma2(make_float2(cf.x, cf.y), make_float2(rf.z, rf.w), c[k]);
      c[k] = fma2(make_float2(rf.x, rf.y), make_float2(cf.z, cf.w), c[k]);
    }
  }
  if (tmax > 0.f) atomicMax(cx.tmargin, static_cast<unsigned long long>(__float_as_uint(tmax)));
  return nreq;
}

// MATRIX_SUMMARY: a thread's running maxima (per segment and target).
struct MatRun {
  int cell[2][2];
  float mx[2][2];
};

// Order-preserving uint32 image of a float (not NaN).
__device__ __forceinline__ unsigned ord_float(float x) {
  const unsigned b = __float_as_uint(x);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// n / d for n < 2^32 and d >= 2 from M = ceil(2^64 / d): exact while
// n d < 2^64 (floor(n M / 2^64) = n / d + n e / (d 2^64), e = M d - 2^64 < d).
__device__ __forceinline__ int64_t div_magic(int64_t n, uint64_t M) {
  return static_cast<int64_t>(__umul64hi(static_cast<uint64_t>(n), M));
}

// MATRIX_SUMMARY: a thread-step whose block crosses a grid boundary (flags
// fx, fy per segment) is walked again from the step's start (rewound from
// the covariances at its end, as the exact path rewinds), and every cell
// above the threshold goes to its own grid entry.
__device__ __noinline__ void mat_cells_block(Smem& sm, const float2 (&cov_end)[kDiags], int s,
                                             int t, bool fx, bool fy) {
  const SlowCtx& cx = sm.cx;
  const int r0 = s * kRows;
  const int cb0 = 8 * (s + t);
  float2 c[kDiags];
#pragma unroll
  for (int k = 0; k < kDiags; ++k) c[k] = cov_end[k];
#pragma unroll 1
  for (int rr = kRows - 1; rr >= 0; --rr) {
    const float4 rf = sm.r_fg[r0 + rr];
#pragma unroll
    for (int k = 0; k < kDiags; ++k) {
      const float4 cf = col_fg(sm, padc(ringc(cx.ring0, cb0 + rr + k)));
      c[k] = fma2(make_float2(-rf.x, -rf.y), make_float2(cf.z, cf.w), c[k]);
      c[k] = fma2(make_float2(-cf.x, -cf.y), make_float2(rf.z, rf.w), c[k]);
    }
  }
#pragma unroll 1
  for (int rr = 0; rr < kRows; ++rr) {
    const float4 rf = sm.r_fg[r0 + rr];
    const float2 dfr = make_float2(rf.x, rf.y), dgr = make_float2(rf.z, rf.w);
    const float2 ivr = sm.r_iv[r0 + rr];
#pragma unroll
    for (int k = 0; k < kDiags; ++k) {
      const int slot = padc(ringc(cx.ring0, cb0 + rr + k));
      const float2 r2 = mul2(mul2(c[k], sm.u.s.c_iv[slot]), ivr);
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const float r = g ? r2.y : r2.x;
        if ((g ? fy : fx) && r > cx.thr) {  // false for NaN
          const int64_t i = cx.rbase[g] + r0 + rr;
          const int64_t j = i + cx.D0 + t * kDiags + k;
          if (cx.mcol)
            atomicMax(cx.mat + div_magic(i, cx.rpc_magic) * cx.mat_w + div_magic(j, cx.cpc_magic),
                      ord_float(r));
          if (cx.mrow)
            atomicMax(cx.mat + div_magic(j, cx.rpc_magic) * cx.mat_w + div_magic(i, cx.cpc_magic),
                      ord_float(r));
        }
      }
      const float4 cf = col_fg(sm, slot);
      c[k] = fma2(make_float2(cf.x, cf.y), dgr, c[k]);
      c[k] = fma2(dfr, make_float2(cf.z, cf.w), c[k]);
    }
  }
}

// The band kernel's body; kSum selects SUM_THRESH (separate instantiations,
// so the 1NN_INDEX form carries none of the sum bookkeeping).  kCoarse
// selects the fast path's filter:
//   false: per cell, r = (cov * inv_c) * inv_r, the block's largest r
//          against the threshold (8 packed multiplies per row);
//   true:  per step, the block's largest covariance times the largest
//          inverse norms of its columns and rows -- an upper bound of every
//          r in the block, which spares the per-cell multiplies.  It is
//          tight where the inverse norms of neighbouring windows are close
//          (long windows); a block it flags goes to the exact path, which
//          checks every cell with its own r.
// kMat selects MATRIX_SUMMARY (running grid maxima), kKnn the k-best lists
// (filters at each window's k-th best); both take the per-cell filter.
template <bool kSum, bool kCoarse, bool kMat = false, bool kKnn = false>
__device__ __forceinline__ void band_body(const JoinParams& P) {
  static_assert(!(kMat && (kSum || kCoarse)), "the matrix form takes per-cell maxima");
  static_assert(!(kKnn && (kSum || kCoarse || kMat)), "the k-best form is a 1NN variant");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  constexpr bool sum_mode = kSum;
  const float thr = static_cast<float>(P.threshold);
  // a window's filter value: its best (1NN), or its list's k-th best, at
  // least the threshold (k-best lists of kk keys per window)
  const int kk = kKnn ? P.knn_k : 1;
  auto best_floor = [&](const uint64_t* keys, int64_t w) -> float {
    const float v = key_corr_floor(keys[w * kk + (kk - 1)], P.kl);
    return kKnn ? fmaxf(v, thr) : v;
  };
  unsigned long long n_steps = 0, n_slow = 0, n_verify = 0;
  int qn = 0;  // queued blocks of this warp (warp-uniform)
  float tfast = 0.f;  // SUM_THRESH: largest margin of a block added on the fast path
  // MATRIX_SUMMARY: per segment (x, y) and target (column, row results) the
  // grid entry the thread's recent blocks fell in and their largest r, kept
  // in the exact path's queue space (the matrix form queues nothing)
  static_assert(sizeof(MatRun) * kThreads <= sizeof(SlowItem) * kWarps * kQueue,
                "matrix state exceeds the queue space");
  MatRun& mrun = reinterpret_cast<MatRun*>(&sm.queue[0][0])[t];
  if constexpr (kMat) {
#pragma unroll
    for (int g = 0; g < 2; ++g)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        mrun.cell[g][h] = -1;
        mrun.mx[g][h] = -3.f;
      }
  }

  for (;;) {
    if (t == 0) {
      const long long uu = static_cast<long long>(atomicAdd(P.unit_counter, 1ull));
      sm.unit = uu;
      if (uu < P.total_units) {
        int pi;
        int64_t bb, ubb;
        decode_unit(P, uu, &pi, &bb, &ubb);
        sm.prob = problem_of(P, pi);
        sm.prob_index = pi;
        sm.band = bb;
        sm.unit_in_band = ubb;
      }
    }
    __syncthreads();
    const int64_t u = sm.unit;
    if (u >= P.total_units) break;
    const Problem& pr = sm.prob;
    const int64_t K = pr.seg_len;  // per problem: batched joins mix windows
    const int64_t m = pr.m;
    const int64_t band = sm.band, ub = sm.unit_in_band;
    const int64_t D0 = pr.d_lo + band * kBand;
    const int64_t rows_b = band_rows(pr.R.ns, pr.C.ns, D0);
    int64_t seg_row[2], seg_len[2];
    seg_row[0] = ub * 2 * K;
    seg_row[1] = seg_row[0] + K;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int64_t l = rows_b - seg_row[g];
      seg_len[g] = l < 0 ? 0 : (l > K ? K : l);
    }
    const int64_t d_my = D0 + t * kDiags;
    const int sh = pr.C.bshift;

    // ---------------- anchors ----------------
    // With the thread's first column window j0 and
    // Y(p) = T32c[p] + (boff_c[p >> bshift] - mu_j0) (the column samples
    // centred by that window's mean, shared by the thread's 8 windows):
    //   anchor_k = sum_t xc_t * Y(j_k + t) - (mu_jk - mu_j0) * sum_t xc_t
    // where xc is the row window centred by its FP64 mean.  The two segments
    // run as f32x2 pairs: their column spans are seg_len apart, a multiple of
    // the block size, so both halves cross block boundaries together.  The
    // row windows and the CTA's column spans are staged in shared memory.
    float2 acc2[kDiags];
    float2 xsum2 = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < kDiags; ++k) acc2[k] = make_float2(0.f, 0.f);
    int64_t jb[2], b0s[2];
    float mu0[2];
    float2 o0[2];                 // {bhi, blo} of the block of mu_j0
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      jb[g] = seg_row[g] + d_my;  // the thread's first column window
      const int64_t jc = jb[g] < pr.C.ns ? jb[g] : pr.C.ns - 1;
      b0s[g] = jc >> sh;
      mu0[g] = pr.C.mu_rel[jc];   // mu_j0 - boff_c[b0]
      o0[g] = make_float2(pr.C.bhi[b0s[g]], pr.C.blo[b0s[g]]);
    }
    const bool live1 = seg_len[1] > 0;
    const int64_t nblk_c = (pr.C.n + (int64_t{1} << sh) - 1) >> sh;
    int64_t span_b0 = 0;
    // anchors from the tensor-core table (anchor_tc.cu) when the join has one
    const bool tab = pr.anchor_tab != nullptr;
    if (tab) {
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const bool live = g == 0 ? seg_len[0] > 0 : live1;
        const float* rowp = pr.anchor_tab + (seg_row[g] / K - pr.tab_s0) * pr.tab_wp +
                            band * kBand + t;
#pragma unroll
        for (int k = 0; k < kDiags; ++k) {
          const float v = (live && jb[g] + k < pr.C.ns) ? rowp[k * 128] : 0.f;
          if (g) acc2[k].y = v; else acc2[k].x = v;
        }
      }
    }
    for (int64_t t0 = 0; t0 < (tab ? 0 : m); t0 += kAnchorChunk) {
      const int chunk = static_cast<int>((m - t0) < kAnchorChunk ? (m - t0) : kAnchorChunk);
      {
        const int64_t i0 = seg_row[0], i1 = seg_row[1];
        const int64_t bi0 = i0 >> sh, bi1 = i1 >> sh;
        const float mr0 = pr.R.mu_rel[i0], mr1 = live1 ? pr.R.mu_rel[i1] : 0.f;
        for (int x = t; x < chunk; x += kThreads) {
          const int64_t p0 = i0 + t0 + x, p1 = i1 + t0 + x;
          float2 v;
          v.x = pr.R.T32[p0] + (block_delta(pr.R, p0 >> sh, bi0) - mr0);
          v.y = live1 ? pr.R.T32[p1] + (block_delta(pr.R, p1 >> sh, bi1) - mr1) : 0.f;
          sm.u.a.xr[x] = v;
        }
        const int64_t cb0 = i0 + D0 + t0, cb1 = i1 + D0 + t0;
        for (int x = t; x < kBand + chunk + 16; x += kThreads) {
          const int64_t p0 = cb0 + x, p1 = cb1 + x;
          float2 v;
          v.x = p0 < pr.C.n ? pr.C.T32[p0] : 0.f;
          v.y = (live1 && p1 < pr.C.n) ? pr.C.T32[p1] : 0.f;
          sm.u.a.yc[pady2(x)] = v;
        }
        if (t < 2 * kSpanBlk) {
          const int g = t >= kSpanBlk, x = t - g * kSpanBlk;
          const int64_t b = ((g ? cb1 : cb0) >> sh) + x;
          const bool ok = (g == 0 || live1) && b < nblk_c;
          sm.u.a.cb[g][x] = ok ? make_float2(pr.C.bhi[b], pr.C.blo[b]) : make_float2(0.f, 0.f);
        }
        span_b0 = cb0 >> sh;
      }
      __syncthreads();
      const int64_t plim0 = pr.C.n;
      int64_t cur_b = -1;                        // block of the cached corrections
      float2 dlo = make_float2(0.f, 0.f), dhi = make_float2(0.f, 0.f);
      for (int c0 = 0; c0 < chunk; c0 += 32) {
        float2 part[kDiags];
#pragma unroll
        for (int k = 0; k < kDiags; ++k) part[k] = make_float2(0.f, 0.f);
        float2 xs = make_float2(0.f, 0.f);
        const int c1 = (c0 + 32 < chunk) ? c0 + 32 : chunk;
        // groups of 8 row samples: 16 column samples cover the 8 windows;
        // 16 consecutive samples touch at most two blocks (blocks hold >= 32)
        for (int xg = c0; xg < c1; xg += 8) {
          const int64_t pg = jb[0] + t0 + xg;
          const int64_t bf = pg >> sh;
          if (bf != cur_b) {
            // the same sums as block_delta(), from the staged offsets; the
            // second segment's blocks sit at the same span positions
            cur_b = bf;
            const int x = static_cast<int>(bf - span_b0);
            const float2 l0 = sm.u.a.cb[0][x], h0 = sm.u.a.cb[0][x + 1];
            const float2 l1 = sm.u.a.cb[1][x], h1 = sm.u.a.cb[1][x + 1];
            dlo.x = (pg < plim0) ? ((l0.x - o0[0].x) + (l0.y - o0[0].y)) - mu0[0] : 0.f;
            dhi.x = (((bf + 1) << sh) < plim0) ? ((h0.x - o0[0].x) + (h0.y - o0[0].y)) - mu0[0] : 0.f;
            dlo.y = (live1 && pg + K < plim0) ? ((l1.x - o0[1].x) + (l1.y - o0[1].y)) - mu0[1] : 0.f;
            dhi.y = (live1 && ((bf + 1) << sh) + K < plim0)
                        ? ((h1.x - o0[1].x) + (h1.y - o0[1].y)) - mu0[1] : 0.f;
          }
          const int nb = static_cast<int>(((bf + 1) << sh) - pg);  // samples left in block bf
          const int o = pady2(t * kDiags + xg);      // 16-byte aligned slot
          float2 y[16];
#pragma unroll
          for (int q = 0; q < 16; q += 2) {
            const float4 v = *reinterpret_cast<const float4*>(&sm.u.a.yc[o + q + (q >> 3) * 2]);
            y[q] = make_float2(v.x, v.y);
            y[q + 1] = make_float2(v.z, v.w);
          }
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const float2 d = q < nb ? dlo : dhi;
            y[q] = make_float2(y[q].x + d.x, y[q].y + d.y);
          }
#pragma unroll
          for (int v = 0; v < 8; ++v) {
            if (xg + v < c1) {
              const float2 xv = sm.u.a.xr[xg + v];
              xs = make_float2(xs.x + xv.x, xs.y + xv.y);
#pragma unroll
              for (int k = 0; k < kDiags; ++k) part[k] = fma2(xv, y[v + k], part[k]);
            }
          }
        }
#pragma unroll
        for (int k = 0; k < kDiags; ++k)
          acc2[k] = make_float2(acc2[k].x + part[k].x, acc2[k].y + part[k].y);
        xsum2 = make_float2(xsum2.x + xs.x, xsum2.y + xs.y);
      }
      __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < kDiags; ++k) {
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const int64_t j = jb[g] + k;
        if (tab || j >= pr.C.ns || (g == 1 && !live1)) continue;
        const float ek = (pr.C.mu_rel[j] + block_delta(pr.C, j >> sh, b0s[g])) - mu0[g];
        if (g) acc2[k].y = fmaf(-ek, xsum2.y, acc2[k].y);
        else acc2[k].x = fmaf(-ek, xsum2.x, acc2[k].x);
      }
    }
    float2 cov[kDiags];
#pragma unroll
    for (int k = 0; k < kDiags; ++k) {
      const int64_t d = d_my + k;
      const bool valid = d < pr.d_hi && !(d >= pr.x_lo && d < pr.x_hi);
      // An excluded diagonal carries NaN: every r on it is NaN and never wins.
      cov[k] = valid ? acc2[k] : make_float2(qnan(), qnan());
    }
    // Drift state of the thread, per segment: the sum over steps of the
    // largest cov^2 among its diagonals (an upper bound of every diagonal's
    // own sum), starting from the anchors' rounding; and the sum of squared
    // increment bounds.
    float2 Vt;
    {
      const float2 cm = absmax8(cov);
      Vt = make_float2(pr.anchor_vcoef * cm.x * cm.x, pr.anchor_vcoef * cm.y * cm.y);
    }
    float2 W = make_float2(0.f, 0.f);

    if (t == 0) {
      // read by the exact path only after the slab's first barrier
      SlowCtx& cx = sm.cx;
      cx.pr = &sm.prob;
      cx.D0 = D0;
      cx.m = m;
      cx.kl = P.kl;
      cx.prob = sm.prob_index;
      cx.vreq = P.vreq;
      cx.vcount = P.counters + 3;
      cx.vcap = P.vreq_cap;
      cx.tmargin = P.counters + 4;
      cx.overflow = P.counters + 6;
      cx.sum_mode = kSum;
      cx.thr = static_cast<float>(P.threshold);
      cx.knn_k = kKnn ? P.knn_k : 0;
      if constexpr (kMat) {
        cx.mat = P.mat;
        cx.mat_w = P.mat_w;
        cx.rpc = P.rows_per_cell;
        cx.cpc = P.cols_per_cell;
        cx.rpc_magic = P.rpc_magic;
        cx.cpc_magic = P.cpc_magic;
        cx.mcol = P.mat_col[sm.prob_index] != 0;
        cx.mrow = P.mat_row[sm.prob_index] != 0;
      }
    }

    // ---------------- slabs ----------------
    const int64_t nslabs = (seg_len[0] + kSlab - 1) / kSlab;
    for (int64_t q = 0; q < nslabs; ++q) {
      int64_t rbase[2], rend[2], cbase_g[2];
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        rbase[g] = seg_row[g] + q * kSlab;
        rend[g] = seg_row[g] + seg_len[g];
        cbase_g[g] = rbase[g] + D0;
        if (t == 0) sm.cx.rbase[g] = rbase[g];
      }
      const int ring0 = static_cast<int>((q * kSlab) % kCols);
      const int rq = ring0 >> 3;  // ring block of the slab's first column
      if (t == 0) sm.cx.ring0 = ring0;
      // Staging, coalesced: thread t stages columns t, t + kThreads, ... and
      // row t.  The filter tables are reduced on the way, 8 lanes (8
      // consecutive columns or rows) at a time: per 8-column block and per
      // 8-row step the smallest best, the largest inverse norm and the
      // largest |df|, |dg|.
      if (!sum_mode && q > 0 && P.refresh_cols && pr.key_col) {
        // Joins that start cold (no seeds): the columns kept from the last
        // slab take their bests from the profile keys, which other CTAs
        // raise quickly at the start; ring columns otherwise keep the bests
        // staged when they entered.
#pragma unroll 2
        for (int c = t; c < kCols - kSlab; c += kThreads) {
          const int rc = ringc(ring0, c);
          float2 cb = sm.c_best[rc];
          if (cb.x != kNoTarget) cb.x = fmaxf(cb.x, best_floor(pr.key_col, cbase_g[0] + c));
          if (cb.y != kNoTarget) cb.y = fmaxf(cb.y, best_floor(pr.key_col, cbase_g[1] + c));
          sm.c_best[rc] = cb;
          float2 mn = cb;
#pragma unroll
          for (int o = 1; o < 8; o <<= 1) {
            mn.x = fminf(mn.x, __shfl_xor_sync(0xffffffffu, mn.x, o));
            mn.y = fminf(mn.y, __shfl_xor_sync(0xffffffffu, mn.y, o));
          }
          if ((lane & 7) == 0) {
            const int b = rc >> 3;
            sm.c_blkmin[b] = mn;
            if (b == 0) sm.c_blkmin[kBlocks] = mn;
          }
        }
      }
#pragma unroll 3
      for (int c = (q == 0 ? 0 : kCols - kSlab) + t; c < kCols; c += kThreads) {
        const int rc = ringc(ring0, c);
        const int64_t j0 = cbase_g[0] + c, j1 = cbase_g[1] + c;
        const bool ok0 = seg_len[0] > 0 && j0 < pr.C.ns;
        const bool ok1 = seg_len[1] > 0 && j1 < pr.C.ns;
        float4 f;
        f.x = ok0 ? pr.C.df32[j0] : 0.f;
        f.y = ok1 ? pr.C.df32[j1] : 0.f;
        f.z = ok0 ? pr.C.dg32[j0] : 0.f;
        f.w = ok1 ? pr.C.dg32[j1] : 0.f;
        const float2 iv = make_float2(ok0 ? pr.C.inv32[j0] : qnan(), ok1 ? pr.C.inv32[j1] : qnan());
        // A window that cannot match (padding, NaN or flat) must not lower
        // the filter threshold: its best is "unreachable".
        float2 cbv;
        if (sum_mode) {
          // the ring column's previous occupant (kCols columns earlier)
          // leaves: its sums go to the profile, the new one starts at 0
          if (q > 0 && pr.sum_col) {
            const float2 old = sm.c_best[rc];
            const int64_t o0 = j0 - kCols, o1 = j1 - kCols;
            if (old.x != 0.f && o0 >= 0 && o0 < pr.C.ns) atomicAdd(pr.sum_col + o0, static_cast<double>(old.x));
            if (old.y != 0.f && o1 >= 0 && o1 < pr.C.ns) atomicAdd(pr.sum_col + o1, static_cast<double>(old.y));
          }
          cbv = make_float2(0.f, 0.f);
        } else {
          cbv.x = (pr.key_col && ok0 && !isnan(iv.x)) ? best_floor(pr.key_col, j0) : kNoTarget;
          cbv.y = (pr.key_col && ok1 && !isnan(iv.y)) ? best_floor(pr.key_col, j1) : kNoTarget;
        }
        sm.u.s.c_df[padc(rc)] = make_float2(f.x, f.y);
        sm.u.s.c_dg[padc(rc)] = make_float2(f.z, f.w);
        sm.u.s.c_iv[padc(rc)] = iv;
        if (rc < kGhost) {
          sm.u.s.c_df[padc(rc + kCols)] = make_float2(f.x, f.y);
          sm.u.s.c_dg[padc(rc + kCols)] = make_float2(f.z, f.w);
          sm.u.s.c_iv[padc(rc + kCols)] = iv;
        }
        sm.c_best[rc] = cbv;
        TableEntry e = table_entry(f, iv, cbv);
        reduce8(e);  // 8 lanes = one aligned ring block
        if ((lane & 7) == 0) {
          const int b = rc >> 3;
          sm.c_blkmin[b] = e.mn;
          sm.c_blkmax_iv[b] = e.mx;
          sm.c_blkmax_fg[b] = e.mf;
          if (b == 0) {
            sm.c_blkmin[kBlocks] = e.mn;
            sm.c_blkmax_iv[kBlocks] = e.mx;
            sm.c_blkmax_fg[kBlocks] = e.mf;
          }
        }
      }
      {
        const int r = t;  // kSlab == kThreads
        const int64_t i0 = rbase[0] + r, i1 = rbase[1] + r;
        const bool ok0 = i0 < rend[0], ok1 = i1 < rend[1];
        float4 f;
        f.x = ok0 ? pr.R.df32[i0] : 0.f;
        f.y = ok1 ? pr.R.df32[i1] : 0.f;
        f.z = ok0 ? pr.R.dg32[i0] : 0.f;
        f.w = ok1 ? pr.R.dg32[i1] : 0.f;
        const float2 iv = make_float2(ok0 ? pr.R.inv32[i0] : qnan(), ok1 ? pr.R.inv32[i1] : qnan());
        float2 rbv;
        if (sum_mode) {
          rbv = make_float2(0.f, 0.f);
        } else {
          rbv.x = (pr.key_row && ok0 && !isnan(iv.x)) ? best_floor(pr.key_row, i0) : kNoTarget;
          rbv.y = (pr.key_row && ok1 && !isnan(iv.y)) ? best_floor(pr.key_row, i1) : kNoTarget;
        }
        sm.r_fg[r] = f;
        sm.r_iv[r] = iv;
        sm.r_best[r] = rbv;
        TableEntry e = table_entry(f, iv, rbv);
        reduce8(e);
        if ((lane & 7) == 0) {
          sm.r_stepmin[r >> 3] = e.mn;
          sm.r_stepmax_iv[r >> 3] = e.mx;
          sm.r_stepmax_fg[r >> 3] = e.mf;
        }
      }
      __syncthreads();
      // ---------------- steps ----------------
      // Steps run in pairs.  The thread's column window is carried from the
      // first step of a pair to the second (the last 7 columns of step s are
      // the first 7 of step s + 1): column x of step s sits in slot
      // (8 * (s & 1) + x) & 15, so every slot index is a constant.  The exact
      // path runs only between pairs: a step whose trigger finds the warp's
      // queue full is recorded in `pend` and queued after the pair as a
      // two-step (or one-step) block.
      float4 cfw[16];
      float2 ciw[16];
      int pend = -1;
      // segments of the pending block, per step (bits 0-1, 2-3; SUM_THRESH,
      // every segment otherwise)
      int pmsk = 15;
      float2 vlast = make_float2(0.f, 0.f);
      auto step = [&](const int s, auto parity) {
        [[maybe_unused]] constexpr int P = decltype(parity)::value;
        const int r0 = s * kRows;
        // ring block of the step's first column 8(s + t)
        const int rb = (rq + s + t) < kBlocks ? (rq + s + t) : (rq + s + t - kBlocks);
        const int base = 9 * rb;  // its padded slot
        // filter threshold and margin: the step's 15 columns lie in ring
        // blocks rb and rb + 1
        const float2 bm0 = sm.c_blkmin[rb], bm1 = sm.c_blkmin[rb + 1];
        const float2 bm = make_float2(fminf(bm0.x, bm1.x), fminf(bm0.y, bm1.y));
        const float2 rsm = sm.r_stepmin[s];
        const float2 ic0 = sm.c_blkmax_iv[rb], ic1 = sm.c_blkmax_iv[rb + 1];
        const float2 icm = make_float2(fmaxf(ic0.x, ic1.x), fmaxf(ic0.y, ic1.y));
        const float2 irm = sm.r_stepmax_iv[s];
        {
          const float2 cm = absmax8(cov);
          Vt = fma2(cm, cm, Vt);
        }
        {
          // bound of |df_c dg_r| + |df_r dg_c| over the step's cells
          const float4 cf0 = sm.c_blkmax_fg[rb], cf1 = sm.c_blkmax_fg[rb + 1];
          const float4 cfm = make_float4(fmaxf(cf0.x, cf1.x), fmaxf(cf0.y, cf1.y),
                                         fmaxf(cf0.z, cf1.z), fmaxf(cf0.w, cf1.w));
          const float4 rfm = sm.r_stepmax_fg[s];
          const float2 inc = fma2(make_float2(rfm.x, rfm.y), make_float2(cfm.z, cfm.w),
                                  mul2(make_float2(rfm.z, rfm.w), make_float2(cfm.x, cfm.y)));
          W = fma2(inc, inc, W);
        }
        const float vx = Vt.x + W.x, vy = Vt.y + W.y;
        // threshold - margin, the margin as the exact path forms it per cell
        // (C eps sqrt(rows v) inv_c inv_r) but with the block's largest
        // inverse norms, an approximate square root and a 2^-16 allowance
        // for both
        const float2 mg = mul2(mul2(make_float2(sqrt_approx(vx), sqrt_approx(vy)), icm), irm);
        const float2 tb = sum_mode ? make_float2(thr, thr)
                                   : make_float2(fminf(bm.x, rsm.x), fminf(bm.y, rsm.y));
        const float2 tt = fma2(make_float2(-kStepMarginC, -kStepMarginC), mg, tb);
        const float tx = tt.x, ty = tt.y;

        // fast path: recurrence + block maximum
        float bx = -3.f, by = -3.f;
        if constexpr (kCoarse) {
          // largest covariance of the block (NaN diagonals ignored), then
          // the bound max(cov, 0) * max inv_c * max inv_r of every r in it
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            {
              const int x = rr + kDiags - 1;
              cfw[(8 * P + x) & 15] = col_fg(sm, base + x + (x >> 3));
            }
            const float4 rf = sm.r_fg[r0 + rr];
            const float2 dfr = make_float2(rf.x, rf.y), dgr = make_float2(rf.z, rf.w);
            {
              const float ax = max3(cov[0].x, cov[1].x, cov[2].x);
              const float ay = max3(cov[0].y, cov[1].y, cov[2].y);
              const float cx3 = max3(cov[3].x, cov[4].x, cov[5].x);
              const float cy3 = max3(cov[3].y, cov[4].y, cov[5].y);
              bx = max3(bx, cov[6].x, cov[7].x);
              by = max3(by, cov[6].y, cov[7].y);
              bx = max3(bx, ax, cx3);
              by = max3(by, ay, cy3);
            }
#pragma unroll
            for (int k = 0; k < kDiags; ++k) {
              const float4 c4 = cfw[(8 * P + rr + k) & 15];
              cov[k] = fma2(make_float2(c4.x, c4.y), dgr, cov[k]);
              cov[k] = fma2(dfr, make_float2(c4.z, c4.w), cov[k]);
            }
          }
          const float2 bnd = mul2(mul2(make_float2(fmaxf(bx, 0.f), fmaxf(by, 0.f)), icm), irm);
          bx = bnd.x;
          by = bnd.y;
        } else if constexpr (kSum) {
          // SUM_THRESH: every cell's r (rounded as the exact path rounds it)
          // against the threshold, where the segment's step margin is within
          // kTrust (elsewhere `the` is out of reach and the segment goes to
          // the exact path if it reaches the threshold); row sums per step
          // row, column sums per step column, reduced after the step.  The
          // column values come straight from shared memory (no carried
          // window: its registers hold the sums).
          // a cell above the threshold by more than the step's margin (which
          // bounds every cell's own margin) adds its r; cells within it are
          // rare and settled by sum_near after the step
          const float2 smg = mul2(make_float2(kStepMarginC, kStepMarginC), mg);
          const float thx = thr + smg.x, thy = thr + smg.y;
          float2 dmin = make_float2(3.f, 3.f);  // nearest |r - thr| of the step
          float2 rsum[kRows];
          float2 cacc[kRows + kDiags - 1];
#pragma unroll
          for (int x = 0; x < kRows + kDiags - 1; ++x) cacc[x] = make_float2(0.f, 0.f);
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            const float4 rf = sm.r_fg[r0 + rr];
            const float2 dfr = make_float2(rf.x, rf.y), dgr = make_float2(rf.z, rf.w);
            const float2 ivr = sm.r_iv[r0 + rr];
            rsum[rr] = make_float2(0.f, 0.f);
#pragma unroll
            for (int k = 0; k < kDiags; ++k) {
              const int x = rr + k;
              const int slot = base + x + (x >> 3);
              const float4 c4 = col_fg(sm, slot);
              const float2 r2 = mul2(mul2(cov[k], sm.u.s.c_iv[slot]), ivr);
              bx = fmaxf(bx, r2.x);  // NaN cells are ignored
              by = fmaxf(by, r2.y);
              dmin = make_float2(fminf(dmin.x, fabsf(r2.x - thr)), fminf(dmin.y, fabsf(r2.y - thr)));
              const float ax = r2.x > thx ? r2.x : 0.f;
              const float ay = r2.y > thy ? r2.y : 0.f;
              rsum[rr] = make_float2(rsum[rr].x + ax, rsum[rr].y + ay);
              cacc[x] = make_float2(cacc[x].x + ax, cacc[x].y + ay);
              cov[k] = fma2(make_float2(c4.x, c4.y), dgr, cov[k]);
              cov[k] = fma2(dfr, make_float2(c4.z, c4.w), cov[k]);
            }
          }
          // rows: a reduce-scatter over the warp (lanes 4 r .. 4 r + 3 end
          // with row r's total), one shared-memory atomic per row
          {
            float2 w4[4], w2[2];
            const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const float2 snd = b16 ? rsum[i] : rsum[i + 4];
              const float2 kp = b16 ? rsum[i + 4] : rsum[i];
              w4[i] = make_float2(kp.x + __shfl_xor_sync(0xffffffffu, snd.x, 16),
                                  kp.y + __shfl_xor_sync(0xffffffffu, snd.y, 16));
            }
#pragma unroll
            for (int i = 0; i < 2; ++i) {
              const float2 snd = b8 ? w4[i] : w4[i + 2];
              const float2 kp = b8 ? w4[i + 2] : w4[i];
              w2[i] = make_float2(kp.x + __shfl_xor_sync(0xffffffffu, snd.x, 8),
                                  kp.y + __shfl_xor_sync(0xffffffffu, snd.y, 8));
            }
            const float2 snd = b4 ? w2[0] : w2[1];
            float2 z = b4 ? w2[1] : w2[0];
            z.x += __shfl_xor_sync(0xffffffffu, snd.x, 4);
            z.y += __shfl_xor_sync(0xffffffffu, snd.y, 4);
            z.x += __shfl_xor_sync(0xffffffffu, z.x, 2);
            z.y += __shfl_xor_sync(0xffffffffu, z.y, 2);
            z.x += __shfl_xor_sync(0xffffffffu, z.x, 1);
            z.y += __shfl_xor_sync(0xffffffffu, z.y, 1);
            const int row = (b16 ? 4 : 0) + (b8 ? 2 : 0) + (b4 ? 1 : 0);
            if ((lane & 3) == 0) {
              if (z.x != 0.f) atomicAdd(&sm.r_best[r0 + row].x, z.x);
              if (z.y != 0.f) atomicAdd(&sm.r_best[r0 + row].y, z.y);
            }
          }
          // columns: thread t's step columns 8..14 are thread t + 1's 0..6
#pragma unroll
          for (int x = 0; x < kDiags - 1; ++x) {
            const float ux = __shfl_up_sync(0xffffffffu, cacc[8 + x].x, 1);
            const float uy = __shfl_up_sync(0xffffffffu, cacc[8 + x].y, 1);
            if (lane > 0) cacc[x] = make_float2(cacc[x].x + ux, cacc[x].y + uy);
          }
#pragma unroll
          for (int x = 0; x < kRows + kDiags - 1; ++x) {
            if (x < 8 || lane == 31) {
              const int rcx = ringc(ring0, 8 * (s + t) + x);
              if (cacc[x].x != 0.f) atomicAdd(&sm.c_best[rcx].x, cacc[x].x);
              if (cacc[x].y != 0.f) atomicAdd(&sm.c_best[rcx].y, cacc[x].y);
            }
          }
          const bool nx = dmin.x <= smg.x, ny = dmin.y <= smg.y;
          if (nx || ny) {
            const float2 vk = make_float2(kBoundC * kEps * sqrtf(kRows * vx),
                                          kBoundC * kEps * sqrtf(kRows * vy));
            n_verify += sum_near(sm, cov, s, t, nx, ny, smg, vk);
          }
          // the largest margin of a value added from FP32 by this step
          if (bx > thx) tfast = fmaxf(tfast, smg.x);
          if (by > thy) tfast = fmaxf(tfast, smg.y);
        } else {
          float2 rprev;
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            {
              const int x = rr + kDiags - 1;
              cfw[(8 * P + x) & 15] = col_fg(sm, base + x + (x >> 3));
              ciw[(8 * P + x) & 15] = sm.u.s.c_iv[base + x + (x >> 3)];
            }
            const float4 rf = sm.r_fg[r0 + rr];
            const float2 dfr = make_float2(rf.x, rf.y), dgr = make_float2(rf.z, rf.w);
            const float2 ivr = sm.r_iv[r0 + rr];
            // the row's largest cov * inv_c, times inv_r (> 0): the largest r
            // of the row, rounded exactly as (cov * inv_c) * inv_r per cell
            float mx = -3.f, my = -3.f;
#pragma unroll
            for (int k = 0; k < kDiags; k += 2) {
              const float2 pa = mul2(cov[k], ciw[(8 * P + rr + k) & 15]);
              const float2 pb = mul2(cov[k + 1], ciw[(8 * P + rr + k + 1) & 15]);
              mx = max3(mx, pa.x, pb.x);
              my = max3(my, pa.y, pb.y);
            }
            const float2 rm = mul2(make_float2(mx, my), ivr);
            if (rr & 1) {
              bx = max3(bx, rprev.x, rm.x);
              by = max3(by, rprev.y, rm.y);
            } else {
              rprev = rm;
            }
#pragma unroll
            for (int k = 0; k < kDiags; ++k) {
              const float4 c4 = cfw[(8 * P + rr + k) & 15];
              cov[k] = fma2(make_float2(c4.x, c4.y), dgr, cov[k]);
              cov[k] = fma2(dfr, make_float2(c4.z, c4.w), cov[k]);
            }
          }
        }
        bool trig = bx > tx || by > ty;
        if constexpr (kMat) {
          // a block inside one grid entry (per target) raises the thread's
          // running maximum of that entry, published when the thread's
          // blocks move on; a block across a grid boundary routes each cell
          trig = false;
          const float2 smg = mul2(make_float2(kStepMarginC, kStepMarginC), mg);
          bool nonuni[2] = {false, false};
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            const float bm = g ? by : bx;
            if (!(bm > thr)) continue;
            tfast = fmaxf(tfast, g ? smg.y : smg.x);
            const int64_t i0 = rbase[g] + r0, j0 = i0 + d_my;
            const int64_t rpc = sm.cx.rpc, cpc = sm.cx.cpc;
            int cell[2] = {-1, -1};
            bool uni = true;
            if (sm.cx.mcol) {
              const int64_t qa = div_magic(i0, sm.cx.rpc_magic), qb = div_magic(j0, sm.cx.cpc_magic);
              uni = uni && i0 - qa * rpc + (kRows - 1) < rpc &&
                    j0 - qb * cpc + (kRows + kDiags - 2) < cpc;
              cell[0] = static_cast<int>(qa * sm.cx.mat_w + qb);
            }
            if (sm.cx.mrow) {
              const int64_t qa = div_magic(j0, sm.cx.rpc_magic), qb = div_magic(i0, sm.cx.cpc_magic);
              uni = uni && j0 - qa * rpc + (kRows + kDiags - 2) < rpc &&
                    i0 - qb * cpc + (kRows - 1) < cpc;
              cell[1] = static_cast<int>(qa * sm.cx.mat_w + qb);
            }
            if (!uni) {
              nonuni[g] = true;
              continue;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              if (cell[h] < 0) continue;
              const int cur = mrun.cell[g][h];
              if (cell[h] != cur) {
                if (cur >= 0) atomicMax(sm.cx.mat + cur, ord_float(mrun.mx[g][h]));
                mrun.cell[g][h] = cell[h];
                mrun.mx[g][h] = bm;
              } else {
                mrun.mx[g][h] = fmaxf(mrun.mx[g][h], bm);
              }
            }
          }
          if (nonuni[0] || nonuni[1]) mat_cells_block(sm, cov, s, t, nonuni[0], nonuni[1]);
        }
        // segments the exact path walks (bit 0: first, bit 1: second)
        [[maybe_unused]] int smask = 3;
        if constexpr (kSum && !kCoarse) {
          // SUM_THRESH: every cell was decided above (sum_near for the ones
          // near the threshold); the exact path is not needed
          trig = false;
          smask = 0;
        }
        if constexpr (kSum && !kCoarse) {
          // A step of a pair whose first step is pending joins that pending
          // two-step block (its segments in mask bits 2, 3); others queue in
          // rank order while there is room, else become the pending step.
          // (The sums must not walk a segment twice.)
          const bool want_q = trig && pend < 0;
          if (trig && pend >= 0) pmsk |= smask << 2;
          const unsigned tmask = __ballot_sync(0xffffffffu, want_q);
          if (tmask) {
            const int rank = __popc(tmask & ((1u << lane) - 1u));
            if (want_q) {
              if (qn + rank < kQueue) {
                SlowItem& it = sm.queue[warp][qn + rank];
#pragma unroll
                for (int k = 0; k < kDiags; ++k) it.cov[k] = cov[k];
                it.vw = make_float2(vx, vy);
                it.s = s | (1 << 8) | (smask << 16);
                it.owner = t;
              } else {
                pend = s;
                pmsk = smask;
              }
            }
            const int nq = qn + __popc(tmask);
            qn = nq < kQueue ? nq : kQueue;
          }
          n_slow += trig ? 1u : 0u;
        } else {
          // queue the triggered lanes in rank order while there is room;
          // the exact path walks both segments of every step of the block
          // (a cell of 1NN_INDEX published twice changes nothing)
          const unsigned tmask = __ballot_sync(0xffffffffu, trig);
          if (tmask) {
            const int rank = __popc(tmask & ((1u << lane) - 1u));
            if (trig) {
              if (qn + rank < kQueue) {
                SlowItem& it = sm.queue[warp][qn + rank];
#pragma unroll
                for (int k = 0; k < kDiags; ++k) it.cov[k] = cov[k];
                it.vw = make_float2(vx, vy);
                it.s = s | (1 << 8) | (15 << 16);
                it.owner = t;
              } else if (pend < 0) {
                pend = s;
              }
            }
            const int nq = qn + __popc(tmask);
            qn = nq < kQueue ? nq : kQueue;
            n_slow += trig ? 1u : 0u;
          }
        }
        vlast = make_float2(vx, vy);
      };
#pragma unroll 1
      for (int s = 0; s < kSteps; s += 2) {
        {
          const int rb = (rq + s + t) < kBlocks ? (rq + s + t) : (rq + s + t - kBlocks);
          if constexpr (!(kSum && !kCoarse)) {
#pragma unroll
            for (int x = 0; x < kDiags - 1; ++x) {
              cfw[x] = col_fg(sm, 9 * rb + x);  // padc(ring column 8 rb + x), x < 8
              if constexpr (!kCoarse) ciw[x] = sm.u.s.c_iv[9 * rb + x];
            }
          }
        }
        step(s, Parity<0>());
        step(s + 1, Parity<1>());
        // between pairs: drain a half-full queue (every queue at the slab's
        // end), then queue and drain the steps that found it full
        const unsigned pmask = __ballot_sync(0xffffffffu, pend >= 0);
        if (pmask || qn >= kQueue / 2 || (qn && s + 2 == kSteps)) {
          if (qn) {
            n_verify += drain_queue<!kCoarse>(sm, warp, qn, lane);
            qn = 0;
          }
          const int np = __popc(pmask);
          const int rank = __popc(pmask & ((1u << lane) - 1u));
          for (int done = 0; done < np; done += kQueue) {
            if (pend >= 0 && rank >= done && rank < done + kQueue) {
              SlowItem& it = sm.queue[warp][rank - done];
#pragma unroll
              for (int k = 0; k < kDiags; ++k) it.cov[k] = cov[k];
              it.vw = vlast;
              it.s = pend | ((s + 2 - pend) << 8) | (pmsk << 16);
              it.owner = t;
            }
            const int take = (np - done) < kQueue ? (np - done) : kQueue;
            n_verify += drain_queue<!kCoarse>(sm, warp, take, lane);
          }
          pend = -1;
        }
      }
      n_steps += kSteps;
      __syncthreads();
      if (sum_mode && pr.sum_row) {
        // the slab's row sums (thread t: row t; it restages row t next)
        const float2 v = sm.r_best[t];
        const int64_t i0 = rbase[0] + t, i1 = rbase[1] + t;
        if (v.x != 0.f && i0 < rend[0]) atomicAdd(pr.sum_row + i0, static_cast<double>(v.x));
        if (v.y != 0.f && i1 < rend[1]) atomicAdd(pr.sum_row + i1, static_cast<double>(v.y));
      }
      if (sum_mode && pr.sum_col && q + 1 == nslabs) {
        // unit end: every column left in the ring
        for (int c = t; c < kCols; c += kThreads) {
          const float2 v = sm.c_best[ringc(ring0, c)];
          const int64_t j0 = cbase_g[0] + c, j1 = cbase_g[1] + c;
          if (v.x != 0.f && j0 < pr.C.ns) atomicAdd(pr.sum_col + j0, static_cast<double>(v.x));
          if (v.y != 0.f && j1 < pr.C.ns) atomicAdd(pr.sum_col + j1, static_cast<double>(v.y));
        }
      }
      // The flushes read the unit's Problem in shared memory, which thread 0
      // overwrites when it fetches the next unit.
      if (sum_mode && q + 1 == nslabs) __syncthreads();
    }
  }
  // per-CTA totals of the work counters
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    n_steps += __shfl_xor_sync(0xffffffffu, n_steps, o);
    n_slow += __shfl_xor_sync(0xffffffffu, n_slow, o);
    n_verify += __shfl_xor_sync(0xffffffffu, n_verify, o);
  }
  if (lane == 0 && P.counters) {
    atomicAdd(P.counters + 0, n_steps);
    atomicAdd(P.counters + 1, n_slow);
    atomicAdd(P.counters + 2, n_verify);
  }
  if constexpr (kMat) {
#pragma unroll
    for (int g = 0; g < 2; ++g)
#pragma unroll
      for (int h = 0; h < 2; ++h)
        if (mrun.cell[g][h] >= 0) atomicMax(P.mat + mrun.cell[g][h], ord_float(mrun.mx[g][h]));
  }
  if constexpr (kSum || kMat) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tfast = fmaxf(tfast, __shfl_xor_sync(0xffffffffu, tfast, o));
    if (lane == 0 && P.counters && tfast > 0.f)
      atomicMax(P.counters + 4, static_cast<unsigned long long>(__float_as_uint(tfast)));
  }
}

}  // namespace

size_t mixed_1nn_smem_bytes() { return sizeof(Smem); }

__global__ void __launch_bounds__(kThreads, 4) join_mixed_1nn_kernel(JoinParams P) {
  band_body<false, false>(P);
}

__global__ void __launch_bounds__(kThreads, 4) join_mixed_sum_kernel(JoinParams P) {
  band_body<true, false>(P);
}

__global__ void __launch_bounds__(kThreads, 4) join_mixed_mat_kernel(JoinParams P) {
  band_body<false, false, true>(P);
}

__global__ void __launch_bounds__(kThreads, 4) join_mixed_knn_kernel(JoinParams P) {
  band_body<false, false, false, true>(P);
}

__global__ void __launch_bounds__(kThreads, 4) join_mixed_1nn_coarse_kernel(JoinParams P) {
  band_body<false, true>(P);
}

__global__ void __launch_bounds__(kThreads, 4) join_mixed_sum_coarse_kernel(JoinParams P) {
  band_body<true, true>(P);
}

// Settles the verification requests of the band kernels, one warp per
// cell.  A request whose upper bound rv + margin no longer exceeds the
// current best of its row or column cannot change the profile and is
// skipped; otherwise the cell's covariance is computed directly from the
// FP32 series copies (each factor centred per window) and its r merged into
// both profiles.  Runs after the join on the same stream; the request count
// is read on the device.
__global__ void __launch_bounds__(256)
verify_requests_kernel(JoinParams P) {
  const int lane = threadIdx.x & 31;
  const unsigned long long total = P.counters[3];
  const int64_t n = total < static_cast<unsigned long long>(P.vreq_cap)
                        ? static_cast<int64_t>(total) : P.vreq_cap;
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  for (int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
       w < n; w += nwarps) {
    const VerifyReq rq = P.vreq[w];
    const Problem& pr = problem_of(P, static_cast<int>(rq.i >> 40));
    const int64_t i = static_cast<int64_t>(rq.i & ((uint64_t{1} << 40) - 1));
    const int64_t j = i + rq.d;
    if (P.profile_type == 2) {  // SUM_THRESH: the cell counts if above it
      const float cv = verify_cov_warp(pr.R, pr.C, i, j, pr.m, lane);
      const float rv = (cv * pr.C.inv32[j]) * pr.R.inv32[i];
      if (lane == 0 && rv > static_cast<float>(P.threshold)) {
        if (pr.sum_row) atomicAdd(pr.sum_row + i, static_cast<double>(rv));
        if (pr.sum_col) atomicAdd(pr.sum_col + j, static_cast<double>(rv));
      }
      continue;
    }
    if (P.knn_k > 0) {  // APPROX_ALL_NEIGHBORS: into the k-best lists
      const int k = P.knn_k;
      const float thr = static_cast<float>(P.threshold);
      // decided by lane 0 for the warp: the lists change under other
      // warps' (and lane 0's own) atomics, and the lanes' loads of them need
      // not agree, while the shuffles of the dot need every lane
      bool ro = pr.key_row && rq.ub > knn_floor(pr.key_row + i * k, k, thr, P.kl);
      bool co = pr.key_col && rq.ub > knn_floor(pr.key_col + j * k, k, thr, P.kl);
      ro = __shfl_sync(0xffffffffu, ro, 0);
      co = __shfl_sync(0xffffffffu, co, 0);
      if (!ro && !co) continue;
      const float cv = verify_cov_warp(pr.R, pr.C, i, j, pr.m, lane);
      if (lane == 0) {
        const float rv = (cv * pr.C.inv32[j]) * pr.R.inv32[i];
        if (rv > thr) {
          const uint64_t q = q_from_float_bits(__float_as_uint(rv), P.kl.frac_bits);
          if (ro && rv > knn_floor(pr.key_row + i * k, k, thr, P.kl))
            topk_insert(reinterpret_cast<u64*>(pr.key_row + i * k), k, make_key(q, j, P.kl));
          if (co && rv > knn_floor(pr.key_col + j * k, k, thr, P.kl))
            topk_insert(reinterpret_cast<u64*>(pr.key_col + j * k), k, make_key(q, i, P.kl));
        }
      }
      continue;
    }
    // warp-uniform by lane 0's view, as above
    bool row_open = pr.key_row && rq.ub > key_corr_floor(pr.key_row[i], P.kl);
    bool col_open = pr.key_col && rq.ub > key_corr_floor(pr.key_col[j], P.kl);
    row_open = __shfl_sync(0xffffffffu, row_open, 0);
    col_open = __shfl_sync(0xffffffffu, col_open, 0);
    if (!row_open && !col_open) continue;
    const float cv = verify_cov_warp(pr.R, pr.C, i, j, pr.m, lane);
    if (lane == 0) {
      const float rv = (cv * pr.C.inv32[j]) * pr.R.inv32[i];
      const uint64_t q = q_from_float_bits(__float_as_uint(rv), P.kl.frac_bits);
      if (row_open) atomicMax(reinterpret_cast<u64*>(pr.key_row + i), make_key(q, j, P.kl));
      if (col_open) atomicMax(reinterpret_cast<u64*>(pr.key_col + j), make_key(q, i, P.kl));
    }
  }
}

// ---------------------------------------------------------------------------
// Seeds of the mixed 1NN join (an approximate pre-pass in the manner of
// SCRIMP++'s PreSCRIMP).  A join of the series averaged over blocks of f
// samples (window m / f) gives every block-averaged window a likely partner;
// each full-resolution window i = f i' + o then gets the exact correlation of
// the cell on the same diagonal, (i, f idx(i') + o), merged into the profile
// keys before the band kernel runs.  Every seed is a real cell's r, so the
// join's result is unchanged; its filters simply start high, which spares
// most of the exact-path work of the first bands.
// ---------------------------------------------------------------------------

// out[k] = mean of T[f k .. f k + f), NaN when any of them is not finite.
__global__ void paa_kernel(const double* __restrict__ T, int64_t n_out, int f,
                           double* __restrict__ out) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n_out) return;
  double sum = 0.0;
  bool finite = true;
  for (int u = 0; u < f; ++u) {
    const double v = T[static_cast<int64_t>(f) * k + u];
    finite = finite && isfinite(v);
    sum += v;
  }
  out[k] = finite ? sum / f : __longlong_as_double(0x7FF8000000000000ll);
}

// Packed entries {r = floor, index 0}: the pre-pass only looks for partners
// above `floor`, which spares it the cold start of a join from "no match".
__global__ void fill_floor_kernel(uint64_t* __restrict__ p, int64_t n, float floor) {
  const int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) p[k] = __float_as_uint(floor);
}

// One warp per window i of X: its seed partner from the block-averaged
// profile, the exact r of that cell, merged into X's keys (and Y's).
__global__ void __launch_bounds__(256) seed_kernel(SeedArgs S) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  for (int64_t i = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
       i < S.X.ns; i += nwarps) {
    const int64_t ib = i / S.factor;
    const int64_t ip = ib < S.ns_paa ? ib : S.ns_paa - 1;
    const uint64_t packed = S.paa[ip];
    if (!(__uint_as_float(static_cast<uint32_t>(packed)) > S.floor)) continue;  // no partner found
    const int64_t j = S.factor * static_cast<int64_t>(packed >> 32) + (i - S.factor * ip);
    if (j >= S.Y.ns) continue;
    if (S.excl >= 0 && (j - i < S.excl && i - j < S.excl)) continue;  // trivial match
    const float ivx = S.X.inv32[i], ivy = S.Y.inv32[j];
    if (isnan(ivx) || isnan(ivy)) continue;
    const float cv = verify_cov_warp(S.X, S.Y, i, j, S.m, lane);
    if (lane == 0) {
      const uint64_t q = q_from_float_bits(__float_as_uint((cv * ivy) * ivx), S.kl.frac_bits);
      atomicMax(reinterpret_cast<u64*>(S.key_x + i), make_key(q, j, S.kl));
      if (S.key_y) atomicMax(reinterpret_cast<u64*>(S.key_y + j), make_key(q, i, S.kl));
    }
  }
}

// Seeds of self-joins from diagonals near the exclusion zone, one thread per
// window: cells (i, i + d_lo + 16 s), s < kDiagSeeds, are real cells of the
// join, so their r are valid starting bests for window i (as a row) and the
// partner windows (as columns).  Where the series moves slowly against the
// window length (random walks) they are close to the final bests, and the
// filter starts high instead of sending every block of the first slabs to
// the exact path.  win_prefix[p] is the first global window of problem p.
constexpr int kDiagSeeds = 8;
constexpr int kDiagSeedStep = 16;
__global__ void __launch_bounds__(256) diag_seed_kernel(const Problem* __restrict__ probs,
                                                        const int64_t* __restrict__ win_prefix,
                                                        int nprob, KeyLayout kl) {
  const int64_t total = win_prefix[nprob];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < total;
       w += stride) {
    int lo = 0, hi = nprob;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (win_prefix[mid] <= w) lo = mid; else hi = mid;
    }
    const Problem& pr = probs[lo];
    const int64_t i = w - win_prefix[lo];
    if (i >= pr.R.ns) continue;
    const float ivx = pr.R.inv32[i];
    if (isnan(ivx)) continue;
    uint64_t best = 0;
    for (int s = 0; s < kDiagSeeds; ++s) {
      const int64_t j = i + pr.d_lo + static_cast<int64_t>(s) * kDiagSeedStep;
      if (j >= pr.C.ns) break;
      const float ivy = pr.C.inv32[j];
      if (isnan(ivy)) continue;
      const float cv = verify_cov_lane(pr.R, pr.C, i, j, pr.m);
      const uint64_t q = q_from_float_bits(__float_as_uint((cv * ivy) * ivx), kl.frac_bits);
      if (pr.key_col) atomicMax(reinterpret_cast<u64*>(pr.key_col + j), make_key(q, i, kl));
      const uint64_t kr = make_key(q, j, kl);
      best = kr > best ? kr : best;
    }
    if (pr.key_row && best) atomicMax(reinterpret_cast<u64*>(pr.key_row + i), best);
  }
}

// Largest p with prefix[p] <= t (prefix[0] = 0, p < n).
__device__ __forceinline__ int job_of(const int64_t* __restrict__ prefix, int n, int64_t t) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void paa_batch_kernel(const PaaJob* __restrict__ jobs,
                                 const int64_t* __restrict__ out_prefix, int njobs) {
  const int64_t total = out_prefix[njobs];
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
       t += stride) {
    const int p = job_of(out_prefix, njobs, t);
    const PaaJob& J = jobs[p];
    const int64_t k = t - out_prefix[p];
    double sum = 0.0;
    bool finite = true;
    for (int u = 0; u < J.f; ++u) {
      const double v = J.src[static_cast<int64_t>(J.f) * k + u];
      finite = finite && isfinite(v);
      sum += v;
    }
    J.dst[k] = finite ? sum / J.f : __longlong_as_double(0x7FF8000000000000ll);
  }
}

__global__ void fill_key_floor_kernel(uint64_t* __restrict__ keys, int64_t n, float floor,
                                      KeyLayout kl) {
  const uint64_t key = make_key(q_from_float_bits(__float_as_uint(floor), kl.frac_bits), 0, kl);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride)
    keys[k] = key;
}

// One warp per block-averaged window i' of a series (PreSCRIMP-style seeds
// with a neighbourhood refinement): its pre-pass partner j' puts the windows
// i = f i' + o (o < f) near diagonal D = f (j' - i'); lane l takes diagonal
// D + l - 15 (|l - 15| < f), computes its first cell's covariance directly
// (FP32, centred) and walks the block's rows with the FP32 recurrence; per
// row the warp keeps the best of its cells, merged into that window's key.
// Every seed is a real cell's r, so the join's result does not depend on
// them; good seeds only spare the join's exact path the records a cold start
// sets (a short series' best improves about ln(n) times as the bands sweep
// outward).
__global__ void __launch_bounds__(256) batch_seed_kernel(const BatchSeedJob* __restrict__ jobs,
                                                         const int64_t* __restrict__ paa_prefix,
                                                         int njobs, KeyLayout kl, float floor) {
  const int lane = threadIdx.x & 31;
  const int64_t total = paa_prefix[njobs];
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  const uint64_t q_floor = q_from_float_bits(__float_as_uint(floor), kl.frac_bits);
  for (int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w < total;
       w += nwarps) {
    const int p = job_of(paa_prefix, njobs, w);
    const BatchSeedJob& J = jobs[p];
    const int64_t ip = w - paa_prefix[p];
    const uint64_t pk = J.paa_key[ip];
    if ((pk >> kl.idx_bits) <= q_floor) continue;  // no partner above the floor (warp-uniform)
    const int64_t jp = static_cast<int64_t>(kl.idx_mask - (pk & kl.idx_mask));
    const int f = J.f;
    const int64_t ns = J.X.ns;
    const int64_t i0 = static_cast<int64_t>(f) * ip;
    const int delta = lane - 15;
    const int64_t d = static_cast<int64_t>(f) * (jp - ip) + delta;
    // rows o in [o_lo, o_hi) of this lane's diagonal are cells of the join
    int64_t o_lo = 0, o_hi = 0;
    if (lane < 31 && (delta < f && -delta < f) && (d >= J.excl || -d >= J.excl)) {
      o_lo = -(i0 + d) > 0 ? -(i0 + d) : 0;
      o_hi = f;
      if (ns - i0 < o_hi) o_hi = ns - i0;
      if (ns - i0 - d < o_hi) o_hi = ns - i0 - d;
    }
    float cov = 0.f;
    if (o_lo < o_hi) cov = cov_part(J.X, J.X, i0 + o_lo, i0 + o_lo + d, 0, J.m);
    for (int o = 0; o < f; ++o) {
      const int64_t i = i0 + o, j = i + d;
      const bool valid = o >= o_lo && o < o_hi;
      uint64_t key = 0;
      if (valid) {
        const float ivi = J.X.inv32[i], ivj = J.X.inv32[j];
        if (!isnan(ivi) && !isnan(ivj))
          key = make_key(q_from_float_bits(__float_as_uint((cov * ivj) * ivi), kl.frac_bits), j, kl);
        if (o + 1 < o_hi)
          cov = fmaf(J.X.df32[i], J.X.dg32[j], fmaf(J.X.df32[j], J.X.dg32[i], cov));
      }
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        const uint64_t other = __shfl_xor_sync(0xffffffffu, key, s);
        key = other > key ? other : key;
      }
      if (lane == 0 && key && i < ns) atomicMax(reinterpret_cast<u64*>(J.key + i), key);
    }
  }
}

int mixed_1nn_band_width() { return kBand; }
int mixed_1nn_slab_rows() { return kSlab; }
int mixed_1nn_threads() { return kThreads; }

}  // namespace scamp_gb300
