// join_fp64.cu -- the plain (all-FP64) form of the SCAMP join.
//
// Replaces the reference's do_tile (src/kernels.cu:22-167) and its tile
// scheduler (src/SCAMP.cpp:25-169, src/tile.cpp:546-707).  One persistent
// kernel walks a device-side work queue of units; a unit is a band of
// kFp64Band diagonals times two segments of seg_len rows (the segments run
// interleaved, which doubles the independent FP64 chains per thread).  Each
// segment starts from an FP64 direct-dot seed (the reference's QT seed,
// src/qt_helper.cpp:52-72), then every cell costs exactly four FP64-pipe
// instructions: two DFMA for the recurrence and two for r = cov*inv_c*inv_r.
// GB300 issues FP64 at 1/62 of its FP32 rate (measured), so everything else
// -- compares, index tracking, key packing -- runs on the integer pipe, which
// has ample spare issue slots.
//
// Profile updates follow the reference's semantics (strict '>' with NaN never
// winning, src/kernel_gpu_utils.h:138-179; SUM_THRESH adds r when r > thr,
// src/kernels_compute.h:88-113) but merge through order-preserving 64-bit
// keys: per-slab maxima are staged in shared memory and published with one
// global atomicMax per improved entry (the reference's packed-u64 CAS loop,
// src/kernel_gpu_utils.h:261-307, becomes a single atomic).
#include <cstdint>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr int kThreads = 128;
constexpr int kDiags = 4;             // diagonals per thread
constexpr int kBand = kThreads * kDiags;  // diagonals per unit
constexpr int kRows = 4;              // rows per step
constexpr int kSlab = 64;             // rows staged per slab
constexpr int kCols = kSlab + kBand;  // columns staged per slab

__device__ __forceinline__ double fmul_dfma(double a, double b) {
  // a*b issued as a DFMA with -0 addend (exact, keeps -0): on GB300 DFMA
  // retires faster than DMUL (measured).
  double r;
  asm("fma.rn.f64 %0, %1, %2, 0d8000000000000000;" : "=d"(r) : "d"(a), "d"(b));
  return r;
}

__device__ __forceinline__ uint64_t umax64(uint64_t a, uint64_t b) {
  return a > b ? a : b;
}

// Ordered integer image of a double; NaN maps below everything.
__device__ __forceinline__ int64_t ord_double(double x) {
  const int64_t b = __double_as_longlong(x);
  if ((b & 0x7FF0000000000000ll) == 0x7FF0000000000000ll) return INT64_MIN;
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFll);
}

struct SmemFp64 {
  double df_r[2][kSlab], dg_r[2][kSlab], iv_r[2][kSlab];
  double df_c[2][kCols], dg_c[2][kCols], iv_c[2][kCols];
  union {
    struct {
      unsigned long long col[2][kCols];
      unsigned long long row[2][kSlab];
    } key;
    struct {
      double col[2][kCols];
      double row[2][kSlab];
    } sum;
  } prof;
  unsigned char dirty_col[2][kCols];
  unsigned char dirty_row[2][kSlab];
  long long unit;
};

// FP64 direct-dot seed: cov of row window i and column window j, each centred
// by its own mean (the reference's QT seed, src/qt_helper.cpp:52-72).  Four
// interleaved accumulators keep the FP64 pipe fed.
__device__ double seed_fp64(const SeriesDev& R, const SeriesDev& C, int64_t i,
                            int64_t j, int64_t m) {
  const double mr = R.mean[i], mc = C.mean[j];
  const double* __restrict__ tr = R.T + i;
  const double* __restrict__ tc = C.T + j;
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  int64_t t = 0;
  for (; t + 4 <= m; t += 4) {
    a0 = fma(tr[t] - mr, tc[t] - mc, a0);
    a1 = fma(tr[t + 1] - mr, tc[t + 1] - mc, a1);
    a2 = fma(tr[t + 2] - mr, tc[t + 2] - mc, a2);
    a3 = fma(tr[t + 3] - mr, tc[t + 3] - mc, a3);
  }
  for (; t < m; ++t) a0 = fma(tr[t] - mr, tc[t] - mc, a0);
  return (a0 + a1) + (a2 + a3);
}

}  // namespace

__global__ void __launch_bounds__(kThreads)
join_fp64_kernel(JoinParams P) {
  __shared__ SmemFp64 sm;
  const int t = threadIdx.x;
  const int lane = t & 31;
  const bool is_1nn = P.profile_type == 1;
  const double thr = P.threshold;
  const int64_t ord_thr = ord_double(thr);
  const int64_t K = P.seg_len;

  for (;;) {
    if (t == 0) sm.unit = static_cast<long long>(atomicAdd(P.unit_counter, 1ull));
    __syncthreads();
    const int64_t u = sm.unit;
    __syncthreads();
    if (u >= P.total_units) break;

    int pi;
    int64_t band, ub;
    decode_unit(P, u, &pi, &band, &ub);
    const Problem& pr = P.prob[pi];
    const int64_t D0 = pr.d_lo + band * kBand;
    const int64_t rows_b = band_rows(pr.R.ns, pr.C.ns, D0);
    int64_t seg_row[2], seg_len[2];
    seg_row[0] = ub * 2 * K;
    seg_row[1] = seg_row[0] + K;
    for (int g = 0; g < 2; ++g) {
      int64_t l = rows_b - seg_row[g];
      seg_len[g] = l < 0 ? 0 : (l > K ? K : l);
    }
    const int64_t d_my = D0 + t * kDiags;

    // Seeds for this thread's diagonals.
    double cov[2][kDiags];
    for (int g = 0; g < 2; ++g) {
      for (int k = 0; k < kDiags; ++k) {
        const int64_t d = d_my + k;
        const int64_t i = seg_row[g];
        cov[g][k] = 0;
        if (seg_len[g] > 0 && d < pr.d_hi && i + d < pr.C.ns)
          cov[g][k] = seed_fp64(pr.R, pr.C, i, i + d, P.m);
      }
    }
    // Per-diagonal validity (diagonal range and the is_aligned exclusion).
    bool dvalid[kDiags];
    for (int k = 0; k < kDiags; ++k) {
      const int64_t d = d_my + k;
      dvalid[k] = d < pr.d_hi && !(d >= pr.x_lo && d < pr.x_hi);
    }

    const int64_t nslabs = (seg_len[0] + kSlab - 1) / kSlab;
    for (int64_t q = 0; q < nslabs; ++q) {
      // ---- stage rows, columns and profile entries of this slab ----
      for (int g = 0; g < 2; ++g) {
        const int64_t rbase = seg_row[g] + q * kSlab;
        const int64_t rend = seg_row[g] + seg_len[g];
        for (int x = t; x < kSlab; x += kThreads) {
          const int64_t i = rbase + x;
          const bool ok = i < rend;
          sm.df_r[g][x] = ok ? pr.R.df[i] : 0.0;
          sm.dg_r[g][x] = ok ? pr.R.dg[i] : 0.0;
          sm.iv_r[g][x] = ok ? pr.R.inv[i] : __longlong_as_double(0x7FF8000000000000ll);
          if (is_1nn) {
            sm.prof.key.row[g][x] = (ok && pr.key_row) ? pr.key_row[i] : 0ull;
          } else {
            sm.prof.sum.row[g][x] = 0.0;
          }
          sm.dirty_row[g][x] = 0;
        }
        const int64_t cbase = rbase + D0;
        for (int x = t; x < kCols; x += kThreads) {
          const int64_t j = cbase + x;
          const bool ok = j < pr.C.ns;
          sm.df_c[g][x] = ok ? pr.C.df[j] : 0.0;
          sm.dg_c[g][x] = ok ? pr.C.dg[j] : 0.0;
          sm.iv_c[g][x] = ok ? pr.C.inv[j] : __longlong_as_double(0x7FF8000000000000ll);
          if (is_1nn) {
            sm.prof.key.col[g][x] = (ok && pr.key_col) ? pr.key_col[j] : 0ull;
          } else {
            sm.prof.sum.col[g][x] = 0.0;
          }
          sm.dirty_col[g][x] = 0;
        }
      }
      __syncthreads();

      // ---- compute kSlab rows in steps of kRows ----
      for (int r0 = 0; r0 < kSlab; r0 += kRows) {
        const int cb = r0 + t * kDiags;  // first staged column of this step
        if (is_1nn) {
          uint64_t cbest[2][kDiags + kRows - 1];
          uint64_t rbest[2][kRows];
#pragma unroll
          for (int g = 0; g < 2; ++g) {
#pragma unroll
            for (int c = 0; c < kDiags + kRows - 1; ++c) cbest[g][c] = 0;
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) rbest[g][rr] = 0;
          }
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            const int64_t row0 = seg_row[g] + q * kSlab + r0;
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) {
              const double dfr = sm.df_r[g][r0 + rr];
              const double dgr = sm.dg_r[g][r0 + rr];
              const double ivr = sm.iv_r[g][r0 + rr];
              const int64_t i = row0 + rr;
#pragma unroll
              for (int k = 0; k < kDiags; ++k) {
                const int c = cb + rr + k;
                const double r = fmul_dfma(fmul_dfma(cov[g][k], sm.iv_c[g][c]), ivr);
                uint64_t qv = q_from_double_bits(__double_as_longlong(r), P.kl.frac_bits);
                if (!dvalid[k]) qv = 0;
                const int64_t j = i + d_my + k;
                rbest[g][rr] = umax64(rbest[g][rr], make_key(qv, j, P.kl));
                cbest[g][rr + k] = umax64(cbest[g][rr + k], make_key(qv, i, P.kl));
                cov[g][k] = fma(sm.df_c[g][c], dgr, cov[g][k]);
                cov[g][k] = fma(dfr, sm.dg_c[g][c], cov[g][k]);
              }
            }
          }
          // publish column maxima to shared memory
          if (pr.key_col) {
#pragma unroll
            for (int g = 0; g < 2; ++g) {
#pragma unroll
              for (int c = 0; c < kDiags + kRows - 1; ++c) {
                const uint64_t v = cbest[g][c];
                unsigned long long* slot = &sm.prof.key.col[g][cb + c];
                if (v > *slot) {
                  if (atomicMax(slot, static_cast<unsigned long long>(v)) < v)
                    sm.dirty_col[g][cb + c] = 1;
                }
              }
            }
          }
          // row maxima: warp reduction, then one shared atomic per warp
          if (pr.key_row) {
#pragma unroll
            for (int g = 0; g < 2; ++g) {
#pragma unroll
              for (int rr = 0; rr < kRows; ++rr) {
                uint64_t v = rbest[g][rr];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                  v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
                if (lane == 0) {
                  unsigned long long* slot = &sm.prof.key.row[g][r0 + rr];
                  if (v > *slot) {
                    if (atomicMax(slot, static_cast<unsigned long long>(v)) < v)
                      sm.dirty_row[g][r0 + rr] = 1;
                  }
                }
              }
            }
          }
        } else {
          // SUM_THRESH: sum r over cells with r > threshold.
          double csum[2][kDiags + kRows - 1];
          double rsum[2][kRows];
#pragma unroll
          for (int g = 0; g < 2; ++g) {
#pragma unroll
            for (int c = 0; c < kDiags + kRows - 1; ++c) csum[g][c] = 0;
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) rsum[g][rr] = 0;
          }
#pragma unroll
          for (int g = 0; g < 2; ++g) {
#pragma unroll
            for (int rr = 0; rr < kRows; ++rr) {
              const double dfr = sm.df_r[g][r0 + rr];
              const double dgr = sm.dg_r[g][r0 + rr];
              const double ivr = sm.iv_r[g][r0 + rr];
#pragma unroll
              for (int k = 0; k < kDiags; ++k) {
                const int c = cb + rr + k;
                const double r = fmul_dfma(fmul_dfma(cov[g][k], sm.iv_c[g][c]), ivr);
                const bool take = dvalid[k] && ord_double(r) > ord_thr;
                if (take) {
                  rsum[g][rr] += r;
                  csum[g][rr + k] += r;
                }
                cov[g][k] = fma(sm.df_c[g][c], dgr, cov[g][k]);
                cov[g][k] = fma(dfr, sm.dg_c[g][c], cov[g][k]);
              }
            }
          }
          if (pr.sum_col) {
#pragma unroll
            for (int g = 0; g < 2; ++g)
#pragma unroll
              for (int c = 0; c < kDiags + kRows - 1; ++c)
                if (csum[g][c] != 0.0) atomicAdd(&sm.prof.sum.col[g][cb + c], csum[g][c]);
          }
          if (pr.sum_row) {
#pragma unroll
            for (int g = 0; g < 2; ++g)
#pragma unroll
              for (int rr = 0; rr < kRows; ++rr) {
                double v = rsum[g][rr];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0 && v != 0.0) atomicAdd(&sm.prof.sum.row[g][r0 + rr], v);
              }
          }
        }
      }
      __syncthreads();

      // ---- publish the slab's improved entries to the global profile ----
      for (int g = 0; g < 2; ++g) {
        const int64_t rbase = seg_row[g] + q * kSlab;
        const int64_t rend = seg_row[g] + seg_len[g];
        const int64_t cbase = rbase + D0;
        if (is_1nn) {
          if (pr.key_col)
            for (int x = t; x < kCols; x += kThreads)
              if (sm.dirty_col[g][x] && cbase + x < pr.C.ns)
                atomicMax(reinterpret_cast<unsigned long long*>(&pr.key_col[cbase + x]),
                          sm.prof.key.col[g][x]);
          if (pr.key_row)
            for (int x = t; x < kSlab; x += kThreads)
              if (sm.dirty_row[g][x] && rbase + x < rend)
                atomicMax(reinterpret_cast<unsigned long long*>(&pr.key_row[rbase + x]),
                          sm.prof.key.row[g][x]);
        } else {
          if (pr.sum_col)
            for (int x = t; x < kCols; x += kThreads) {
              const double v = sm.prof.sum.col[g][x];
              if (v != 0.0 && cbase + x < pr.C.ns) atomicAdd(&pr.sum_col[cbase + x], v);
            }
          if (pr.sum_row)
            for (int x = t; x < kSlab; x += kThreads) {
              const double v = sm.prof.sum.row[g][x];
              if (v != 0.0 && rbase + x < rend) atomicAdd(&pr.sum_row[rbase + x], v);
            }
        }
      }
      __syncthreads();
    }
  }
}

int fp64_band_width() { return kBand; }
int fp64_slab_rows() { return kSlab; }
int fp64_threads() { return kThreads; }

}  // namespace scamp_gb300
