// join_visit.cu -- the two experimental profile types of the reference,
// computed exactly, in FP64:
//
//  - APPROX_ALL_NEIGHBORS (pyscamp selfjoin_knn / abjoin_knn): for every
//    window, its k best matches above the threshold.  The reference keeps
//    per-tile match lists and raises per-column thresholds when a tile's
//    list overflows (src/tile.cpp:419-544, src/common.cpp:199-262), so its
//    lists may miss matches; these are the exact k best.
//  - MATRIX_SUMMARY (pyscamp selfjoin_matrix / abjoin_matrix): a height x
//    width grid over the distance matrix (rows: windows of B, columns:
//    windows of A), each entry the largest correlation above the threshold
//    among its cells.  The reference writes each tile column's best match
//    only (src/kernels_smem.h:282-330), a lower bound of this maximum.
//
// One thread walks one diagonal of a band unit (the FP64 form's work queue),
// both segments in turn: a direct FP64 seed (the reference's QT seed,
// src/qt_helper.cpp:52-72), then r = cov * inv_c * inv_r and the recurrence
// cov += df_c dg_r + df_r dg_c per cell (src/cpu_kernels.cpp:166-171).
//
// Top-k lists hold k order-preserving keys per window, largest first; a
// candidate enters through a chain of atomicMax: each slot keeps the larger
// of its value and the incoming one and passes the smaller on, so after all
// insertions slot s holds the (s+1)-th largest key inserted.  Matrix entries
// are order-preserving uint32 images of floats; a thread keeps the running
// maximum of the grid cell its diagonal is in and publishes it with one
// atomicMax when the diagonal leaves the grid cell.
#include <cstdint>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr int kVisitThreads = 256;  // one diagonal per thread

// Order-preserving uint32 image of a float (NaN excluded by the callers).
__device__ __forceinline__ unsigned ord_float(float x) {
  const unsigned b = __float_as_uint(x);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ __forceinline__ double seed_dot(const SeriesDev& R, const SeriesDev& C,
                                           int64_t i, int64_t j, int64_t m) {
  const double mr = R.mean[i], mc = C.mean[j];
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  int64_t t = 0;
  for (; t + 3 < m; t += 4) {
    s0 = fma(R.T[i + t] - mr, C.T[j + t] - mc, s0);
    s1 = fma(R.T[i + t + 1] - mr, C.T[j + t + 1] - mc, s1);
    s2 = fma(R.T[i + t + 2] - mr, C.T[j + t + 2] - mc, s2);
    s3 = fma(R.T[i + t + 3] - mr, C.T[j + t + 3] - mc, s3);
  }
  for (; t < m; ++t) s0 = fma(R.T[i + t] - mr, C.T[j + t] - mc, s0);
  return (s0 + s1) + (s2 + s3);
}

__device__ __forceinline__ void topk_insert(unsigned long long* slots, int k,
                                            unsigned long long key) {
  for (int s = 0; s < k && key != 0; ++s) {
    const unsigned long long old = atomicMax(slots + s, key);
    if (old < key) key = old;  // the displaced key moves on
  }
}

// x / div and x % div of a position that advances by one.
struct Walk {
  int64_t q, r, div;
  __device__ __forceinline__ Walk(int64_t x, int64_t dv) : q(x / dv), r(x % dv), div(dv) {}
  __device__ __forceinline__ void next() {
    if (++r == div) {
      r = 0;
      ++q;
    }
  }
};

// Running maximum of one grid cell along a diagonal.
struct CellMax {
  int64_t cell = -1;
  float v = -3.f;
  __device__ __forceinline__ void add(unsigned* mat, int64_t c, float r) {
    if (c != cell) {
      if (cell >= 0 && v > -2.f) atomicMax(mat + cell, ord_float(v));
      cell = c;
      v = -3.f;
    }
    v = fmaxf(v, r);
  }
  __device__ __forceinline__ void flush(unsigned* mat) {
    if (cell >= 0 && v > -2.f) atomicMax(mat + cell, ord_float(v));
    cell = -1;
  }
};

}  // namespace

int visit_band_width() { return kVisitThreads; }
int visit_threads() { return kVisitThreads; }

__global__ void __launch_bounds__(kVisitThreads)
join_visit_kernel(JoinParams P, VisitArgs V) {
  __shared__ long long s_unit;
  const int t = threadIdx.x;
  const double thr = P.threshold;
  for (;;) {
    if (t == 0) s_unit = static_cast<long long>(atomicAdd(P.unit_counter, 1ull));
    __syncthreads();
    const int64_t u = s_unit;
    __syncthreads();
    if (u >= P.total_units) break;
    int pi;
    int64_t band, ub;
    decode_unit(P, u, &pi, &band, &ub);
    const Problem& pr = P.prob[pi];
    const int64_t K = P.seg_len;
    const int64_t D0 = pr.d_lo + band * kVisitThreads;
    const int64_t d = D0 + t;
    if (d >= pr.d_hi || (d >= pr.x_lo && d < pr.x_hi)) continue;
    const int64_t rows_b = band_rows(pr.R.ns, pr.C.ns, D0);
    const int ct = V.col_target[pi], rt = V.row_target[pi];
    for (int g = 0; g < 2; ++g) {
      const int64_t i0 = (2 * ub + g) * K;
      int64_t i1 = i0 + K;
      if (i1 > rows_b) i1 = rows_b;
      if (i1 > pr.C.ns - d) i1 = pr.C.ns - d;  // this diagonal's last row
      if (i0 >= i1) continue;
      double cov = seed_dot(pr.R, pr.C, i0, i0 + d, P.m);
      CellMax mc, mr;
      // grid coordinates of the cell, kept by counting: (i / rpc, j / cpc)
      // for column results, (j / rpc, i / cpc) for row results
      Walk wi_r(i0, V.rows_per_cell), wj_c(i0 + d, V.cols_per_cell);
      Walk wj_r(i0 + d, V.rows_per_cell), wi_c(i0, V.cols_per_cell);
      for (int64_t i = i0; i < i1; ++i) {
        const int64_t j = i + d;
        const double r = cov * pr.C.inv[j] * pr.R.inv[i];
        if (r > thr) {  // false for NaN (windows that cannot match)
          if (V.mode == 0) {
            const uint64_t q = q_from_double_bits(__double_as_longlong(r), P.kl.frac_bits);
            if (ct >= 0) {
              unsigned long long* sl = V.topk[ct] + j * V.k;
              const unsigned long long key = make_key(q, i, P.kl);
              if (key > sl[V.k - 1]) topk_insert(sl, V.k, key);
            }
            if (rt >= 0) {
              unsigned long long* sl = V.topk[rt] + i * V.k;
              const unsigned long long key = make_key(q, j, P.kl);
              if (key > sl[V.k - 1]) topk_insert(sl, V.k, key);
            }
          } else {
            // grid rows are windows of B, columns windows of A; a target of
            // A takes the cell with A's window as its column
            const float rf = static_cast<float>(r);
            if (ct == 0) mc.add(V.mat, wi_r.q * V.mat_w + wj_c.q, rf);
            if (rt == 0) mr.add(V.mat, wj_r.q * V.mat_w + wi_c.q, rf);
          }
        }
        cov = fma(pr.C.df[j], pr.R.dg[i], cov);
        cov = fma(pr.R.df[i], pr.C.dg[j], cov);
        if (V.mode == 1) {
          wi_r.next();
          wj_c.next();
          wj_r.next();
          wi_c.next();
        }
      }
      if (V.mode == 1) {
        mc.flush(V.mat);
        mr.flush(V.mat);
      }
    }
  }
}

// Matrix entries between floats (-2 = none) and their ordered images.
__global__ void floats_to_ord_kernel(const float* __restrict__ in, unsigned* __restrict__ out,
                                     int64_t n) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = ord_float(in[i]);
}

__global__ void ord_to_floats_kernel(const unsigned* __restrict__ in, float* __restrict__ out,
                                     int64_t n) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const unsigned b = in[i];
  out[i] = __uint_as_float((b & 0x80000000u) ? (b & 0x7FFFFFFFu) : ~b);
}

}  // namespace scamp_gb300
