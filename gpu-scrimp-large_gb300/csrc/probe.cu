// probe.cu -- measured pipe throughput, the denominator of the roofline
// fraction this engine reports (the join is bound by the FP32 / FP64 FMA
// pipe, not by HBM or tensor cores).  Each thread runs independent FMA
// chains long enough that launch overhead is negligible.
#include <cuda_runtime.h>

#include <cstdint>

namespace scamp_gb300 {

namespace {
constexpr int kChains = 8;

__global__ void probe_ffma2(float* out, int iters, float a, float b) {
  unsigned long long v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    float2 f = make_float2(threadIdx.x * 1e-3f + c, c * 0.5f);
    v[c] = *reinterpret_cast<unsigned long long*>(&f);
  }
  float2 af = make_float2(a, a), bf = make_float2(b, b);
  const unsigned long long ra = *reinterpret_cast<unsigned long long*>(&af);
  const unsigned long long rb = *reinterpret_cast<unsigned long long*>(&bf);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c)
      asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(v[c]) : "l"(ra), "l"(rb));
  }
  float s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    float2 f = *reinterpret_cast<float2*>(&v[c]);
    s += f.x + f.y;
  }
  if (s == 1234.5f) out[threadIdx.x] = s;  // never true; keeps the chains live
}

__global__ void probe_dfma(float* out, int iters, double a, double b) {
  double v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3 + c;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = fma(v[c], a, b);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 1234.5) out[threadIdx.x] = static_cast<float>(s);
}
}  // namespace

// Returns lane-operations per second (one FMA = one op) for kind 0 (FP32,
// packed pairs count as two) or kind 1 (FP64).  0 on success.
int measure_pipe_peak(int device, int kind, double* ops_per_s) {
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return 1;
  float* out = nullptr;
  if (cudaMalloc(&out, 256 * sizeof(float)) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 256, blocks = sms * 8;
  const int iters = kind == 0 ? 100000 : 2000;
  auto launch = [&](int it) {
    if (kind == 0)
      probe_ffma2<<<blocks, threads>>>(out, it, 1.0001f, 0.5f);
    else
      probe_dfma<<<blocks, threads>>>(out, it, 1.0001, 0.5);
  };
  launch(iters / 10);  // warm-up
  float best_ms = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    launch(iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) best_ms = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return 1;
  const double lanes = static_cast<double>(threads) * blocks;
  const double ops = lanes * iters * kChains * (kind == 0 ? 2.0 : 1.0);
  *ops_per_s = ops / (best_ms * 1e-3);
  return 0;
}

}  // namespace scamp_gb300
