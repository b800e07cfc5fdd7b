// join_mixed.cu -- the mixed-precision form of the SCAMP join.
//
// Same work decomposition as join_fp64.cu (persistent kernel, device work
// queue of units = band x two row segments), with the hot loop in FP32:
//  - each thread advances kDiags diagonals in BOTH segments of its unit at
//    once, as packed f32x2 pairs (.x = first segment, .y = second), so every
//    recurrence and product instruction (fma.rn.f32x2 / mul.rn.f32x2) does
//    two cells' work from one issue slot;
//  - every segment starts from an anchor: the covariance of its first row
//    computed as an FP32 dot product of FP64-centred data (row window centred
//    by its own mean, column span by one constant per CTA and then by each
//    window's mean), accumulated in blocks of 32 terms;  the segment length
//    (anchor_interval rows) bounds the FP32 drift of the recurrence.
// The reference's MIXED mode (src/kernels.cu:192-197) keeps the recurrence in
// FP64; this form keeps FP64 only for the statistics, the centring and the
// final key conversion.
#include <cstdint>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr int kThreads = 128;
constexpr int kDiags = 8;
constexpr int kBand = kThreads * kDiags;  // 1024 diagonals per unit
constexpr int kRows = 8;                  // rows per step
constexpr int kSlab = 128;                // rows staged per slab
constexpr int kCols = kSlab + kBand;      // staged columns per slab
constexpr int kAnchorChunk = 1024;        // window samples staged per pass

typedef unsigned long long u64;

__device__ __forceinline__ u64 f2_to_u64(float2 v) {
  return (static_cast<u64>(__float_as_uint(v.y)) << 32) | __float_as_uint(v.x);
}
__device__ __forceinline__ float2 u64_to_f2(u64 v) {
  return make_float2(__uint_as_float(static_cast<uint32_t>(v)),
                     __uint_as_float(static_cast<uint32_t>(v >> 32)));
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  u64 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_to_u64(a)), "l"(f2_to_u64(b)), "l"(f2_to_u64(c)));
  return u64_to_f2(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  u64 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_to_u64(a)), "l"(f2_to_u64(b)));
  return u64_to_f2(d);
}

struct SmemMixed {
  float2 df_r[kSlab], dg_r[kSlab], iv_r[kSlab];
  float2 df_c[kCols], dg_c[kCols], iv_c[kCols];
  union {
    struct {
      u64 col[2][kCols];
      u64 row[2][kSlab];
    } key;
    struct {
      float col[2][kCols];
      float row[2][kSlab];
    } sum;
    struct {  // anchor staging (used before the first slab)
      float xr[2][kAnchorChunk];
      float yc[2][kBand + kAnchorChunk];
    } anc;
  } u;
  float best_col[2][kCols];  // float copy of the staged column maxima
  float best_row[2][kSlab];
  unsigned char dirty_col[2][kCols];
  unsigned char dirty_row[2][kSlab];
  long long unit;
};

__device__ __forceinline__ float nanf_() { return __int_as_float(0x7FC00000); }

}  // namespace

size_t mixed_smem_bytes() { return sizeof(SmemMixed); }

__global__ void __launch_bounds__(kThreads)
join_mixed_kernel(JoinParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemMixed& sm = *reinterpret_cast<SmemMixed*>(smem_raw);
  const int t = threadIdx.x;
  const int lane = t & 31;
  const bool is_1nn = P.profile_type == 1;
  const float thr = static_cast<float>(P.threshold);
  const int64_t K = P.seg_len;
  const int64_t m = P.m;

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

    // ---------------- anchors ----------------
    float acc[2][kDiags];
    float e_k[2][kDiags];
    double cta_c[2];
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int64_t cb = seg_row[g] + D0;  // column of the band's first diagonal
      cta_c[g] = (seg_len[g] > 0 && cb < pr.C.ns) ? pr.C.mean[cb] : 0.0;
#pragma unroll
      for (int k = 0; k < kDiags; ++k) {
        acc[g][k] = 0.f;
        const int64_t j = seg_row[g] + d_my + k;
        e_k[g][k] = (seg_len[g] > 0 && j < pr.C.ns)
                        ? static_cast<float>(pr.C.mean[j] - cta_c[g]) : 0.f;
      }
    }
    for (int64_t t0 = 0; t0 < m; t0 += kAnchorChunk) {
      const int chunk = static_cast<int>((m - t0) < kAnchorChunk ? (m - t0) : kAnchorChunk);
      for (int g = 0; g < 2; ++g) {
        const int64_t i = seg_row[g];
        const bool live = seg_len[g] > 0;
        const double mu_r = live ? pr.R.mean[i] : 0.0;
        for (int x = t; x < chunk; x += kThreads)
          sm.u.anc.xr[g][x] = live ? static_cast<float>(pr.R.T[i + t0 + x] - mu_r) : 0.f;
        const int64_t cb = i + D0 + t0;
        for (int x = t; x < kBand + chunk; x += kThreads) {
          const int64_t j = cb + x;
          sm.u.anc.yc[g][x] = (live && j < pr.C.n) ? static_cast<float>(pr.C.T[j] - cta_c[g]) : 0.f;
        }
      }
      __syncthreads();
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const float* __restrict__ xr = sm.u.anc.xr[g];
        const float* __restrict__ yc = sm.u.anc.yc[g] + t * kDiags;
        for (int b0 = 0; b0 < chunk; b0 += 32) {
          float part[kDiags];
#pragma unroll
          for (int k = 0; k < kDiags; ++k) part[k] = 0.f;
          const int b1 = (b0 + 32 < chunk) ? b0 + 32 : chunk;
          for (int tt = b0; tt < b1; ++tt) {
            const float xv = xr[tt];
#pragma unroll
            for (int k = 0; k < kDiags; ++k)
              part[k] = fmaf(xv, yc[tt + k] - e_k[g][k], part[k]);
          }
#pragma unroll
          for (int k = 0; k < kDiags; ++k) acc[g][k] += part[k];
        }
      }
      __syncthreads();
    }
    float2 cov[kDiags];
#pragma unroll
    for (int k = 0; k < kDiags; ++k) cov[k] = make_float2(acc[0][k], acc[1][k]);

    bool dvalid[kDiags];
#pragma unroll
    for (int k = 0; k < kDiags; ++k) {
      const int64_t d = d_my + k;
      dvalid[k] = d < pr.d_hi && !(d >= pr.x_lo && d < pr.x_hi);
    }

    // ---------------- slabs ----------------
    const int64_t nslabs = (seg_len[0] + kSlab - 1) / kSlab;
    for (int64_t q = 0; q < nslabs; ++q) {
      int64_t rbase[2], rend[2], cbase[2];
      for (int g = 0; g < 2; ++g) {
        rbase[g] = seg_row[g] + q * kSlab;
        rend[g] = seg_row[g] + seg_len[g];
        cbase[g] = rbase[g] + D0;
      }
      for (int x = t; x < kSlab; x += kThreads) {
        float2 f, gg, iv;
        const int64_t i0 = rbase[0] + x, i1 = rbase[1] + x;
        const bool ok0 = i0 < rend[0], ok1 = i1 < rend[1];
        f.x = ok0 ? pr.R.df32[i0] : 0.f;  f.y = ok1 ? pr.R.df32[i1] : 0.f;
        gg.x = ok0 ? pr.R.dg32[i0] : 0.f; gg.y = ok1 ? pr.R.dg32[i1] : 0.f;
        iv.x = ok0 ? pr.R.inv32[i0] : nanf_(); iv.y = ok1 ? pr.R.inv32[i1] : nanf_();
        sm.df_r[x] = f; sm.dg_r[x] = gg; sm.iv_r[x] = iv;
        for (int g = 0; g < 2; ++g) {
          const int64_t i = g ? i1 : i0;
          const bool ok = g ? ok1 : ok0;
          if (is_1nn) {
            const u64 kv = (ok && pr.key_row) ? pr.key_row[i] : 0ull;
            sm.u.key.row[g][x] = kv;
            sm.best_row[g][x] = kv ? static_cast<float>(key_to_corr(kv, P.kl)) : -3.f;
          } else {
            sm.u.sum.row[g][x] = 0.f;
          }
          sm.dirty_row[g][x] = 0;
        }
      }
      for (int x = t; x < kCols; x += kThreads) {
        float2 f, gg, iv;
        const int64_t j0 = cbase[0] + x, j1 = cbase[1] + x;
        const bool ok0 = j0 < pr.C.ns && seg_len[0] > 0, ok1 = j1 < pr.C.ns && seg_len[1] > 0;
        f.x = ok0 ? pr.C.df32[j0] : 0.f;  f.y = ok1 ? pr.C.df32[j1] : 0.f;
        gg.x = ok0 ? pr.C.dg32[j0] : 0.f; gg.y = ok1 ? pr.C.dg32[j1] : 0.f;
        iv.x = ok0 ? pr.C.inv32[j0] : nanf_(); iv.y = ok1 ? pr.C.inv32[j1] : nanf_();
        sm.df_c[x] = f; sm.dg_c[x] = gg; sm.iv_c[x] = iv;
        for (int g = 0; g < 2; ++g) {
          const int64_t j = g ? j1 : j0;
          const bool ok = g ? ok1 : ok0;
          if (is_1nn) {
            const u64 kv = (ok && pr.key_col) ? pr.key_col[j] : 0ull;
            sm.u.key.col[g][x] = kv;
            sm.best_col[g][x] = kv ? static_cast<float>(key_to_corr(kv, P.kl)) : -3.f;
          } else {
            sm.u.sum.col[g][x] = 0.f;
          }
          sm.dirty_col[g][x] = 0;
        }
      }
      __syncthreads();

      for (int r0 = 0; r0 < kSlab; r0 += kRows) {
        const int cb = r0 + t * kDiags;
        if (is_1nn) {
          float cbv[2][kDiags + kRows - 1];
          int cbi[2][kDiags + kRows - 1];
          float rbv[2][kRows];
          int rbk[2][kRows];
#pragma unroll
          for (int c = 0; c < kDiags + kRows - 1; ++c) {
            cbv[0][c] = cbv[1][c] = -3.f;
            cbi[0][c] = cbi[1][c] = 0;
          }
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            rbv[0][rr] = rbv[1][rr] = -3.f;
            rbk[0][rr] = rbk[1][rr] = 0;
          }
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            const float2 dfr = sm.df_r[r0 + rr];
            const float2 dgr = sm.dg_r[r0 + rr];
            const float2 ivr = sm.iv_r[r0 + rr];
#pragma unroll
            for (int k = 0; k < kDiags; ++k) {
              const int c = cb + rr + k;
              const float2 dfc = sm.df_c[c], dgc = sm.dg_c[c], ivc = sm.iv_c[c];
              float2 r = mul2(mul2(cov[k], ivc), ivr);
              if (!dvalid[k]) r = make_float2(nanf_(), nanf_());
              if (r.x > rbv[0][rr]) { rbv[0][rr] = r.x; rbk[0][rr] = k; }
              if (r.y > rbv[1][rr]) { rbv[1][rr] = r.y; rbk[1][rr] = k; }
              if (r.x > cbv[0][rr + k]) { cbv[0][rr + k] = r.x; cbi[0][rr + k] = rr; }
              if (r.y > cbv[1][rr + k]) { cbv[1][rr + k] = r.y; cbi[1][rr + k] = rr; }
              cov[k] = fma2(dfc, dgr, cov[k]);
              cov[k] = fma2(dfr, dgc, cov[k]);
            }
          }
          if (pr.key_col) {
#pragma unroll
            for (int g = 0; g < 2; ++g) {
#pragma unroll
              for (int c = 0; c < kDiags + kRows - 1; ++c) {
                const float v = cbv[g][c];
                if (v > sm.best_col[g][cb + c]) {
                  const int64_t i = rbase[g] + r0 + cbi[g][c];
                  const u64 key = make_key(q_from_float_bits(__float_as_uint(v), P.kl.frac_bits), i, P.kl);
                  if (atomicMax(&sm.u.key.col[g][cb + c], key) < key) {
                    // The float copy only filters candidates; a racing store of
                    // a smaller value costs extra atomics, never a wrong result.
                    sm.dirty_col[g][cb + c] = 1;
                    sm.best_col[g][cb + c] = v;
                  }
                }
              }
            }
          }
          if (pr.key_row) {
#pragma unroll
            for (int g = 0; g < 2; ++g) {
#pragma unroll
              for (int rr = 0; rr < kRows; ++rr) {
                float v = rbv[g][rr];
                int64_t j = static_cast<int64_t>(t * kDiags + rbk[g][rr]);
                // warp argmax (smallest column on ties)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                  const float ov = __shfl_xor_sync(0xffffffffu, v, o);
                  const int64_t oj = __shfl_xor_sync(0xffffffffu, j, o);
                  if (ov > v || (ov == v && oj < j)) { v = ov; j = oj; }
                }
                if (lane == 0 && v > sm.best_row[g][r0 + rr]) {
                  const int64_t i = rbase[g] + r0 + rr;
                  const int64_t col = i + D0 + j;
                  const u64 key = make_key(q_from_float_bits(__float_as_uint(v), P.kl.frac_bits), col, P.kl);
                  if (atomicMax(&sm.u.key.row[g][r0 + rr], key) < key) {
                    sm.dirty_row[g][r0 + rr] = 1;
                    sm.best_row[g][r0 + rr] = v;
                  }
                }
              }
            }
          }
        } else {
          float csum[2][kDiags + kRows - 1];
          float rsum[2][kRows];
#pragma unroll
          for (int c = 0; c < kDiags + kRows - 1; ++c) csum[0][c] = csum[1][c] = 0.f;
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) rsum[0][rr] = rsum[1][rr] = 0.f;
#pragma unroll
          for (int rr = 0; rr < kRows; ++rr) {
            const float2 dfr = sm.df_r[r0 + rr];
            const float2 dgr = sm.dg_r[r0 + rr];
            const float2 ivr = sm.iv_r[r0 + rr];
#pragma unroll
            for (int k = 0; k < kDiags; ++k) {
              const int c = cb + rr + k;
              const float2 dfc = sm.df_c[c], dgc = sm.dg_c[c], ivc = sm.iv_c[c];
              const float2 r = mul2(mul2(cov[k], ivc), ivr);
              const float vx = (dvalid[k] && r.x > thr) ? r.x : 0.f;
              const float vy = (dvalid[k] && r.y > thr) ? r.y : 0.f;
              rsum[0][rr] += vx; rsum[1][rr] += vy;
              csum[0][rr + k] += vx; csum[1][rr + k] += vy;
              cov[k] = fma2(dfc, dgr, cov[k]);
              cov[k] = fma2(dfr, dgc, cov[k]);
            }
          }
          if (pr.sum_col) {
#pragma unroll
            for (int g = 0; g < 2; ++g)
#pragma unroll
              for (int c = 0; c < kDiags + kRows - 1; ++c)
                if (csum[g][c] != 0.f) atomicAdd(&sm.u.sum.col[g][cb + c], csum[g][c]);
          }
          if (pr.sum_row) {
#pragma unroll
            for (int g = 0; g < 2; ++g)
#pragma unroll
              for (int rr = 0; rr < kRows; ++rr) {
                float v = rsum[g][rr];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0 && v != 0.f) atomicAdd(&sm.u.sum.row[g][r0 + rr], v);
              }
          }
        }
      }
      __syncthreads();

      for (int g = 0; g < 2; ++g) {
        if (is_1nn) {
          if (pr.key_col)
            for (int x = t; x < kCols; x += kThreads)
              if (sm.dirty_col[g][x] && cbase[g] + x < pr.C.ns)
                atomicMax(reinterpret_cast<u64*>(&pr.key_col[cbase[g] + x]), sm.u.key.col[g][x]);
          if (pr.key_row)
            for (int x = t; x < kSlab; x += kThreads)
              if (sm.dirty_row[g][x] && rbase[g] + x < rend[g])
                atomicMax(reinterpret_cast<u64*>(&pr.key_row[rbase[g] + x]), sm.u.key.row[g][x]);
        } else {
          if (pr.sum_col)
            for (int x = t; x < kCols; x += kThreads) {
              const float v = sm.u.sum.col[g][x];
              if (v != 0.f && cbase[g] + x < pr.C.ns) atomicAdd(&pr.sum_col[cbase[g] + x], static_cast<double>(v));
            }
          if (pr.sum_row)
            for (int x = t; x < kSlab; x += kThreads) {
              const float v = sm.u.sum.row[g][x];
              if (v != 0.f && rbase[g] + x < rend[g]) atomicAdd(&pr.sum_row[rbase[g] + x], static_cast<double>(v));
            }
        }
      }
      __syncthreads();
    }
  }
}

int mixed_band_width() { return kBand; }
int mixed_slab_rows() { return kSlab; }
int mixed_threads() { return kThreads; }

}  // namespace scamp_gb300
