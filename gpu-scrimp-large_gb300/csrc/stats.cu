// stats.cu -- window statistics on device, in compensated FP64.
//
// Replaces the reference's host-side, sequential precompute
// (src/cpu_stats.cpp:11-160, called from src/SCAMP.cpp:195-206) with one
// kernel.  Each thread owns `chunk` consecutive windows: it sums its first
// window directly, then slides (the reference's rolling, TwoSum-compensated
// update), so the rounding error restarts every `chunk` windows instead of
// growing over the whole series.  ULTRA precision sums every window directly
// (the reference's brute-force O(nm) option, src/cpu_stats.cpp:31-41, 85-97).
//
// Semantics kept exactly:
//  - non-finite samples become 0 and poison every window holding them
//    (src/cpu_stats.cpp:11-29);
//  - invnorm = 1/sqrt(ssd), NaN when the window held a non-finite sample or
//    ssd <= 1e-13 (src/cpu_stats.cpp:140-152);
//  - df[i] = (T[i+m]-T[i])/2, dg[i] = (T[i+m]-mu[i+1]) + (T[i]-mu[i]), and
//    df = dg = 0 at the last window (src/cpu_stats.cpp:154-157).
#include <cmath>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr double kFlatnessEpsilon = 1e-13;  // src/cpu_stats.cpp:4

__device__ __forceinline__ double clean(double x) {
  return isfinite(x) ? x : 0.0;
}

// TwoSum accumulate (Knuth): s + c += x.
__device__ __forceinline__ void acc2(double& s, double& c, double x) {
  const double t = s + x;
  const double z = t - s;
  c += (s - (t - z)) + (x - z);
  s = t;
}

}  // namespace

// Statistics of windows [tid * chunk, (tid + 1) * chunk) of one series.
__device__ __forceinline__ void stats_body(int64_t tid, const double* __restrict__ T_raw, int64_t n,
                             int64_t m, int ultra, int chunk, int bshift,
                             double* __restrict__ T_clean, float* __restrict__ T32,
                             float* __restrict__ bhi, float* __restrict__ blo,
                             float* __restrict__ mu_rel,
                             double* __restrict__ mean, double* __restrict__ inv,
                             double* __restrict__ df, double* __restrict__ dg,
                             float* __restrict__ inv32, float* __restrict__ df32,
                             float* __restrict__ dg32) {
  const int64_t ns = n - m + 1;
  const int64_t w0 = tid * chunk;
  if (w0 >= ns) return;
  const int64_t w1 = (w0 + chunk < ns) ? w0 + chunk : ns;

  // Cleaned samples owned by this chunk (the last chunk also owns the tail).
  // Block offsets are the blocks' first (cleaned) samples.
  auto block_off = [&](int64_t b) { return clean(T_raw[b << bshift]); };
  {
    const int64_t s_end = (w1 == ns) ? n : w1;
    for (int64_t t = w0; t < s_end; ++t) {
      const double c = clean(T_raw[t]);
      T_clean[t] = c;
      const int64_t b = t >> bshift;
      const double o = block_off(b);
      T32[t] = static_cast<float>(c - o);
      if ((b << bshift) == t) {
        const float hi = static_cast<float>(o);
        bhi[b] = hi;
        blo[b] = static_cast<float>(o - static_cast<double>(hi));
      }
    }
  }

  // Mean and NaN status of window w0, and the position of the last
  // non-finite sample seen so far.
  int64_t last_bad = -1;
  double ps = 0, pc = 0;
  for (int64_t t = 0; t < m; ++t) {
    const double x = T_raw[w0 + t];
    if (!isfinite(x)) last_bad = w0 + t;
    acc2(ps, pc, clean(x));
  }
  // The mean is carried as mu + mu_lo: the low part restores the digits the
  // division drops, which matters for series with a large offset relative
  // to their variation (dg subtracts the mean from the raw samples).
  const double md = static_cast<double>(m);
  double mu = (ps + pc) / md;
  double mu_lo = (fma(-mu, md, ps) + pc) / md;

  // ssd of window w0, direct.
  double ss = 0, sc = 0;
  for (int64_t t = 0; t < m; ++t) {
    const double v = clean(T_raw[w0 + t]) - mu;
    acc2(ss, sc, v * v);
  }

  for (int64_t w = w0; w < w1; ++w) {
    // Mean of window w+1 (needed by dg[w]).
    double mu_next = 0, mu_next_lo = 0;
    int64_t last_bad_next = last_bad;
    const bool has_next = (w + 1 < ns);
    double ps_n = ps, pc_n = pc;
    if (has_next) {
      const double x_out = clean(T_raw[w]);
      const double x_in_raw = T_raw[w + m];
      if (!isfinite(x_in_raw)) last_bad_next = w + m;
      const double x_in = clean(x_in_raw);
      if (ultra) {
        double s2 = 0, c2 = 0;
        for (int64_t t = 0; t < m; ++t) acc2(s2, c2, clean(T_raw[w + 1 + t]));
        ps_n = s2;
        pc_n = c2;
      } else {
        acc2(ps_n, pc_n, -x_out);
        acc2(ps_n, pc_n, x_in);
      }
      mu_next = (ps_n + pc_n) / md;
      mu_next_lo = (fma(-mu_next, md, ps_n) + pc_n) / md;
    }

    // Window w statistics.  A near-flat ssd from the recurrence is summed
    // again directly, so the flatness rule sees no accumulated residue.
    double ssd = ss + sc;
    if (ssd <= 1e3 * kFlatnessEpsilon && !ultra) {
      double s2 = 0, c2 = 0;
      for (int64_t t = 0; t < m; ++t) {
        const double v = (clean(T_raw[w + t]) - mu) - mu_lo;
        acc2(s2, c2, v * v);
      }
      ssd = s2 + c2;
    }
    const bool nan_window = last_bad >= w;  // a non-finite sample in [w, w+m)
    double iv;
    if (nan_window || !(ssd > kFlatnessEpsilon)) {
      iv = nan("");
    } else {
      iv = 1.0 / sqrt(ssd);
    }
    double f = 0, g = 0;
    if (has_next) {
      const double a = clean(T_raw[w]);
      const double b = clean(T_raw[w + m]);
      f = (b - a) / 2.0;
      g = ((b - mu_next) - mu_next_lo) + ((a - mu) - mu_lo);
    }
    mean[w] = mu;
    mu_rel[w] = static_cast<float>((mu - block_off(w >> bshift)) + mu_lo);
    inv[w] = iv;
    df[w] = f;
    dg[w] = g;
    inv32[w] = static_cast<float>(iv);
    df32[w] = static_cast<float>(f);
    dg32[w] = static_cast<float>(g);

    if (!has_next) break;
    // Advance ssd to window w+1: the reference's recurrence
    // (src/cpu_stats.cpp:114-117), accumulated with compensation; ULTRA
    // recomputes it directly.
    if (ultra) {
      double s2 = 0, c2 = 0;
      for (int64_t t = 0; t < m; ++t) {
        const double v = clean(T_raw[w + 1 + t]) - mu_next;
        acc2(s2, c2, v * v);
      }
      ss = s2;
      sc = c2;
    } else {
      // With the means' low parts, so that a large offset's rounded mean
      // does not leave a per-step residue (b - a)(delta_w + delta_w+1).
      const double a = clean(T_raw[w]);
      const double b = clean(T_raw[w + m]);
      acc2(ss, sc, (((a - mu) - mu_lo) + ((b - mu_next) - mu_next_lo)) * (b - a));
    }
    ps = ps_n;
    pc = pc_n;
    mu = mu_next;
    mu_lo = mu_next_lo;
    last_bad = last_bad_next;
  }
}


__global__ void stats_kernel(const double* __restrict__ T_raw, int64_t n,
                             int64_t m, int ultra, int chunk, int bshift,
                             double* __restrict__ T_clean, float* __restrict__ T32,
                             float* __restrict__ bhi, float* __restrict__ blo,
                             float* __restrict__ mu_rel,
                             double* __restrict__ mean, double* __restrict__ inv,
                             double* __restrict__ df, double* __restrict__ dg,
                             float* __restrict__ inv32, float* __restrict__ df32,
                             float* __restrict__ dg32) {
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  stats_body(tid, T_raw, n, m, ultra, chunk, bshift, T_clean, T32, bhi, blo, mu_rel, mean, inv,
             df, dg, inv32, df32, dg32);
}

__global__ void stats_batch_kernel(const StatsJob* __restrict__ jobs,
                                   const int64_t* __restrict__ block_prefix, int njobs,
                                   int ultra, int chunk) {
  const int64_t b = blockIdx.x;
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (block_prefix[mid] <= b) lo = mid; else hi = mid;
  }
  const StatsJob& j = jobs[lo];
  const int64_t tid = (b - block_prefix[lo]) * blockDim.x + threadIdx.x;
  stats_body(tid, j.T_raw, j.n, j.m, ultra, chunk, j.bshift, j.T_clean, j.T32, j.bhi, j.blo,
             j.mu_rel, j.mean, j.inv, j.df, j.dg, j.inv32, j.df32, j.dg32);
}

// ULTRA's update terms (the reference's compute_combined_stats_cpu,
// src/cpu_stats.cpp:162-196, used by src/tile.cpp:404-409).  With the
// covariance written against a constant c for one window,
//   cov(i+1, j+1) = cov(i, j) + (x[i+m] - mu[i+1]) (y[j+m] - c)
//                             - (x[i] - mu[i]) (y[j] - c),
// exact for c = mean(y[j+1 .. j+m-1]), the (m-1)-sample mean.  One side of a
// band takes the "A" terms of its series,
//   df = -(x[i] - mu[i]),  dg = x[i+m] - mu[i+1],
// the other the "B" terms,
//   df = y[j+m] - mu'[j+1],  dg = y[j] - mu'[j+1],
// so that df_c dg_r + df_r dg_c is the update above.  mu' is summed directly
// per window (TwoSum-compensated).  The last window's terms are 0 (the
// recurrence never leaves it).
__global__ void combined_stats_kernel(const double* __restrict__ T, int64_t n, int64_t m,
                                      const double* __restrict__ mean, int role_b,
                                      double* __restrict__ df, double* __restrict__ dg) {
  const int64_t ns = n - m + 1;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  if (i == ns - 1) {
    df[i] = 0.0;
    dg[i] = 0.0;
    return;
  }
  if (!role_b) {
    df[i] = -(T[i] - mean[i]);
    dg[i] = T[i + m] - mean[i + 1];
    return;
  }
  double s = 0.0, c = 0.0;
  for (int64_t t = i + 1; t < i + m; ++t) acc2(s, c, T[t]);
  const double mu1 = (s + c) / static_cast<double>(m - 1);
  df[i] = T[i + m] - mu1;
  dg[i] = T[i] - mu1;
}

}  // namespace scamp_gb300
