// final_eval.cu -- FP64 re-evaluation of every reported 1NN cell.
//
// Both join forms choose each window's best partner from a recurrence (FP64
// in the plain form, FP32 behind a filter in the mixed form).  Before the
// profile is written back, this kernel recomputes the correlation of every
// (window, reported partner) pair directly: centred FP64 dot product and
// centred sums of squares of the two windows, r = dot / sqrt(sxx * syy), so
// the value a join reports does not carry the recurrence's drift or the
// statistics' rounding.  This is the reference's correlation formula
// (src/cpu_kernels.cpp:166-171 with the norms of src/cpu_stats.cpp:85-97,
// the brute-force ULTRA statistics) evaluated once per reported cell.
//
// Error bound (per reported value, against the exact correlation of the two
// FP64 windows): every centred term x_t = fl(T - mu) carries one rounding;
// each of a group's 8 lanes sums its terms by FMA into two accumulators of
// at most ceil(m / 16) terms, one add joins them, three shuffle levels add
// the lanes' sums, and the quotient takes three more roundings, so with
// gamma_k = k u / (1 - k u), u = 2^-53:
//   |r_hat - r| <= 2 gamma_{ceil(m/16) + 10}
// (the dot's error is gamma_k * sum |x y| <= gamma_k ||x|| ||y||; each sum of
// squares is off by at most gamma_k of itself).  The 64-bit key then keeps r
// to 2^-F.  The host adds the two (final_eval_bound).
//
// Entries the join did not change (a best-so-far entry given on input, whose
// index may refer to another join) are left as they are.
#include <cstdint>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr int kLanes = 8;  // lanes per window: four windows per warp

// Direct FP64 correlation of window i of X with window j of Y by kLanes
// lanes (a lane sums every kLanes-th term, the partial sums meet in a
// shuffle tree); the value is valid in the group's first lane (NaN when a
// window has no spread).
__device__ __forceinline__ double corr_group_fp64(const SeriesDev& X, const SeriesDev& Y,
                                                  int64_t i, int64_t j, int64_t m, int sub,
                                                  bool first) {
  const double mx = X.mean[i], my = Y.mean[j];
  const double* __restrict__ tx = X.T + i;
  const double* __restrict__ ty = Y.T + j;
  double sxy = 0.0, sxx = 0.0, syy = 0.0, sxy2 = 0.0, sxx2 = 0.0, syy2 = 0.0;
  int64_t t = sub;
  for (; t + kLanes < m; t += 2 * kLanes) {
    const double x0 = tx[t] - mx, y0 = ty[t] - my;
    const double x1 = tx[t + kLanes] - mx, y1 = ty[t + kLanes] - my;
    sxy = fma(x0, y0, sxy);
    sxx = fma(x0, x0, sxx);
    syy = fma(y0, y0, syy);
    sxy2 = fma(x1, y1, sxy2);
    sxx2 = fma(x1, x1, sxx2);
    syy2 = fma(y1, y1, syy2);
  }
  if (t < m) {
    const double x0 = tx[t] - mx, y0 = ty[t] - my;
    sxy = fma(x0, y0, sxy);
    sxx = fma(x0, x0, sxx);
    syy = fma(y0, y0, syy);
  }
  sxy += sxy2;
  sxx += sxx2;
  syy += syy2;
#pragma unroll
  for (int o = kLanes / 2; o > 0; o >>= 1) {
    sxy += __shfl_xor_sync(0xffffffffu, sxy, o);
    sxx += __shfl_xor_sync(0xffffffffu, sxx, o);
    syy += __shfl_xor_sync(0xffffffffu, syy, o);
  }
  return first ? sxy / sqrt(sxx * syy) : 0.0;
}

// The key an input profile entry turns into (profile_to_keys_kernel,
// floats_to_keys_kernel): 0 when there is no entry.
__device__ __forceinline__ uint64_t initial_key(const EvalSide& s, int64_t w, const KeyLayout& kl) {
  if (s.prof_in) {
    const uint64_t e = s.prof_in[w];
    const uint32_t cbits = static_cast<uint32_t>(e);
    const uint32_t idx = static_cast<uint32_t>(e >> 32);
    if (!(__uint_as_float(cbits) >= -1.0f) || static_cast<uint64_t>(idx) > kl.idx_mask) return 0;
    return make_key(q_from_float_bits(cbits, kl.frac_bits), idx, kl);
  }
  if (s.max_in) {
    const float c = s.max_in[w];
    if (!(c >= -1.0f)) return 0;
    return make_key(q_from_float_bits(__float_as_uint(c), kl.frac_bits), 0, kl);
  }
  return 0;
}

// Window w of side s, evaluated by the kLanes lanes of group `sub`; every
// lane of the warp calls it (the shuffle tree needs them), `active` marks the
// groups with a window.
__device__ __forceinline__ void eval_window(const EvalSide& s, int64_t w, int64_t m,
                                            const KeyLayout& kl, int sub, bool active) {
  uint64_t k = active ? s.keys[w] : 0;
  if (k != 0 && k == initial_key(s, w, kl)) k = 0;
  int64_t j = k ? key_to_index(k, kl) : 0;
  if (j < 0 || j >= s.Y.ns) k = 0;
  // groups with nothing to do still take part in the shuffles (no terms)
  const bool work = k != 0;
  const double r = corr_group_fp64(s.X, s.Y, work ? w : 0, work ? j : 0, work ? m : 0, sub,
                                   sub == 0);
  if (sub == 0 && work && !isnan(r)) {
    // |r| <= 1 up to rounding; the key holds r in [-2, 2)
    const double rc = r > 1.0 ? 1.0 : (r < -1.0 ? -1.0 : r);
    s.keys[w] = make_key(q_from_double_bits(__double_as_longlong(rc), kl.frac_bits), j, kl);
  }
}

// The key entry `e` of an input k-best list turns into: 0 when empty.
__device__ __forceinline__ uint64_t list_entry_key(uint64_t e, const KeyLayout& kl) {
  const uint32_t cbits = static_cast<uint32_t>(e);
  const uint32_t idx = static_cast<uint32_t>(e >> 32);
  if (!(__uint_as_float(cbits) >= -1.0f) || static_cast<uint64_t>(idx) > kl.idx_mask) return 0;
  return make_key(q_from_float_bits(cbits, kl.frac_bits), idx, kl);
}

constexpr int kKnnMaxK = 64;  // longest list the mixed k-best form keeps

}  // namespace

int knn_mixed_max_k() { return kKnnMaxK; }

// k-best lists: kLanes lanes per window, its k entries in turn (the slot loop
// is warp-uniform, so the shuffle tree always has its lanes), then the
// group's first lane re-sorts the list, largest key first (ties: the smaller
// index, which the key's index field orders first).
__global__ void __launch_bounds__(256) knn_final_eval_kernel(EvalSide S, int k, double thr,
                                                             KeyLayout kl) {
  const int lane = threadIdx.x & 31;
  const int sub = lane & (kLanes - 1);
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  constexpr int kGroups = 32 / kLanes;
  for (int64_t g0 = ((static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * kGroups;
       g0 < S.ns; g0 += nwarps * kGroups) {
    const int64_t w = g0 + lane / kLanes;
    const bool active = w < S.ns;
    uint64_t* list = S.keys + (active ? w : 0) * k;
    for (int s = 0; s < k; ++s) {
      uint64_t key = active ? list[s] : 0;
      if (key != 0 && S.prof_in) {
        // an entry of the given list stays as it is
        for (int t = 0; t < k; ++t)
          if (list_entry_key(S.prof_in[w * k + t], kl) == key) {
            key = 0;
            break;
          }
      }
      const int64_t j = key ? key_to_index(key, kl) : 0;
      const bool work = key != 0 && j >= 0 && j < S.Y.ns;
      const double r = corr_group_fp64(S.X, S.Y, work ? w : 0, work ? j : 0, work ? S.m : 0, sub,
                                       sub == 0);
      if (sub == 0 && work) {
        const double rc = r > 1.0 ? 1.0 : (r < -1.0 ? -1.0 : r);
        list[s] = (!isnan(r) && r > thr)
                      ? make_key(q_from_double_bits(__double_as_longlong(rc), kl.frac_bits), j, kl)
                      : 0;
      }
    }
    if (sub == 0 && active) {
      uint64_t v[kKnnMaxK];
      const int kc = k < kKnnMaxK ? k : kKnnMaxK;
      for (int s = 0; s < kc; ++s) {
        const uint64_t x = list[s];
        int p = s;
        while (p > 0 && v[p - 1] < x) {
          v[p] = v[p - 1];
          --p;
        }
        v[p] = x;
      }
      for (int s = 0; s < kc; ++s) list[s] = v[s];
    }
  }
}

// Groups of kLanes lanes, one window each, over up to two profile sides (a
// single join).  The loop bound is warp-uniform: a warp's four groups stay
// together for the shuffles.
__global__ void __launch_bounds__(256) final_eval_kernel(EvalPair E) {
  const int lane = threadIdx.x & 31;
  const int sub = lane & (kLanes - 1);
  const int64_t total = E.side[0].ns + E.side[1].ns;
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  constexpr int kGroups = 32 / kLanes;
  for (int64_t g0 = ((static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * kGroups;
       g0 < total; g0 += nwarps * kGroups) {
    const int64_t g = g0 + lane / kLanes;
    const bool active = g < total;
    const int s = (active && g >= E.side[0].ns) ? 1 : 0;
    const int64_t w = active ? g - (s ? E.side[0].ns : 0) : 0;
    eval_window(E.side[s], w, E.m, E.kl, sub, active);
  }
}

// The same over a batch: side k covers windows win_prefix[k] ..
// win_prefix[k + 1] - 1 of the launch.
__global__ void __launch_bounds__(256) final_eval_batch_kernel(const EvalSide* __restrict__ sides,
                                                               const int64_t* __restrict__ win_prefix,
                                                               int nsides, KeyLayout kl) {
  const int lane = threadIdx.x & 31;
  const int sub = lane & (kLanes - 1);
  const int64_t total = win_prefix[nsides];
  const int64_t nwarps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  constexpr int kGroups = 32 / kLanes;
  for (int64_t g0 = ((static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * kGroups;
       g0 < total; g0 += nwarps * kGroups) {
    const int64_t g = g0 + lane / kLanes;
    const bool active = g < total;
    int lo = 0;
    if (active) {
      int hi = nsides;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (win_prefix[mid] <= g) lo = mid; else hi = mid;
      }
    }
    const EvalSide& s = sides[lo];
    eval_window(s, active ? g - win_prefix[lo] : 0, s.m, kl, sub, active);
  }
}

}  // namespace scamp_gb300
