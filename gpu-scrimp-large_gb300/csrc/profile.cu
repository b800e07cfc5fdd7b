// profile.cu -- conversion between the reference's packed 1NN_INDEX entries
// (src/common.h:70-74: float32 correlation in the low word, uint32 index in
// the high word) and the engine's order-preserving merge keys (engine.cuh).
#include "engine.cuh"

namespace scamp_gb300 {

__global__ void profile_to_keys_kernel(const uint64_t* __restrict__ in,
                                       uint64_t* __restrict__ keys, int64_t n,
                                       KeyLayout kl) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint64_t e = in[i];
  const uint32_t cbits = static_cast<uint32_t>(e);
  const uint32_t idx = static_cast<uint32_t>(e >> 32);
  const float c = __uint_as_float(cbits);
  // Entries below -1 are "no match" (src/scamp_utils.cpp:129-131).
  if (!(c >= -1.0f) || static_cast<uint64_t>(idx) > kl.idx_mask) {
    keys[i] = 0;
    return;
  }
  keys[i] = make_key(q_from_float_bits(cbits, kl.frac_bits), idx, kl);
}

__global__ void keys_to_profile_kernel(const uint64_t* __restrict__ keys,
                                       uint64_t* __restrict__ out,
                                       double* __restrict__ corr, int64_t n,
                                       KeyLayout kl) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = keys[i];
  uint64_t e;
  double r;
  if (k == 0) {
    r = -2.0;
    e = (0xFFFFFFFFull << 32) | __float_as_uint(-2.0f);
  } else {
    r = key_to_corr(k, kl);
    const uint32_t idx = static_cast<uint32_t>(key_to_index(k, kl));
    e = (static_cast<uint64_t>(idx) << 32) | __float_as_uint(static_cast<float>(r));
  }
  if (out) out[i] = e;
  if (corr) corr[i] = r;
}

// The reference's 1NN profile (PROFILE_TYPE_1NN, float per window, -2.0 =
// none; src/common.cpp:290-292, merged by elementwise max, :388-391) to keys
// and back.  A best-so-far value carries index 0.
__global__ void floats_to_keys_kernel(const float* __restrict__ in, uint64_t* __restrict__ keys,
                                      int64_t n, KeyLayout kl) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float c = in[i];
  keys[i] = (c >= -1.0f) ? make_key(q_from_float_bits(__float_as_uint(c), kl.frac_bits), 0, kl)
                         : 0;
}

__global__ void keys_to_floats_kernel(const uint64_t* __restrict__ keys, float* __restrict__ out,
                                      double* __restrict__ corr, int64_t n, KeyLayout kl) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = keys[i];
  const double r = k == 0 ? -2.0 : key_to_corr(k, kl);
  out[i] = static_cast<float>(r);
  if (corr) corr[i] = r;
}

}  // namespace scamp_gb300
