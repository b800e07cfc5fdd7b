// anchor_tc.cu -- tensor-core anchors of the mixed band kernel.
//
// The mixed form re-anchors every diagonal of a band at rows 0, K, 2K, ...
// (the anchor interval K), with the covariance of the anchor row's window
// and each column window: cov(sK, j) for the columns j = sK + d of the
// band's diagonals d.  This is the job of the reference's QT seed (a
// sliding dot product by cuFFT, src/qt_helper.cpp:75-121; its CPU form is a
// direct dot, src/qt_helper.cpp:52-72).  Over all bands, the anchors of a
// set of anchor rows s form a dense window-block contraction
//     G[s, j] = sum_t x_s(t) y(j + t),
// x_s = the centred anchor window of the row series, y = the column series
// relative to a local offset: a GEMM whose column operand is a Hankel matrix
// shared by every anchor row.  This file computes it on the tensor cores
// (tcgen05.mma, kind::f16, bf16 operands, FP32 accumulation in TMEM) for a
// chunk of anchor rows into an anchor table the band kernel reads.
//
// Split-BF16x3: every FP32 value v (the same FP32 data as the CUDA-core
// anchors: block-relative series, centred by the FP64 means) is split
// exactly into three bf16 terms v = hi + mid + lo (8 significant bits each).
// The six products of order <= 2 (hi*hi; hi*mid, mid*hi; hi*lo, mid*mid,
// lo*hi) are accumulated; the dropped ones are below 2^-24 of each product.
// hi*hi goes to one TMEM accumulator and the five small products to a second;
// both start afresh every 64 terms (four MMAs), and the 64-term sums are
// added in FP32 registers with round-to-nearest.  The tensor core's own
// FP32 accumulation rounds each MMA step toward the partial sum's scale
// (measured: 4.3e-6 of the normalised anchor after 32 steps on one
// accumulator); four steps over 64 terms keep that below the FP32 data's
// own rounding.
//
// Hankel operand without a materialised Hankel tile: the column windows
// j = J0 + 8q + r (q < 128 rows of the MMA's M dimension, r = residue 0..7)
// of a 1024-column tile are, for a fixed residue r, rows of one stream
// z_r[e] = y(J0 + r + e) spaced 8 elements (16 bytes) apart.  In the
// canonical K-major layout a core matrix (8 rows x 16 bytes) of rows
// 8a..8a+7 and terms 8b..8b+7 is then the 128 contiguous bytes at
// z_r + 128a + 16b: one shared-memory descriptor with a 16-byte step along K
// and a 128-byte step along M addresses the whole Hankel operand of residue
// r from its stream.  Eight streams per split (one per residue) replace the
// 1024 x m tile.
//
// Offset-free partial sums: the column operand is the series relative to
// one offset per tile, y = T - y0, so a partial sum over part of a window
// carries (local level - y0) * (sum of x over that part) -- much larger than
// the covariance where the series wanders.  Each 64-term block of an anchor
// window is therefore centred by its own mean xi_b before the split: with
// x' = x - xi_b summing to zero over every block, the tensor cores only see
// offset-free products, and the block means come back in the epilogue as
//     sum_t x(t) y(j+t) = sum_t x'(t) y(j+t) + sum_b xi_b S_b(j),
// S_b(j) the sum of y over block b of window j, from prefix sums of the tile's
// span (double-float, in shared memory).  With S_b(j) - len_b (mu_j - y0) in
// place of S_b(j) (the blocks' xi sum to the window's zero mean) every term
// of the epilogue stays at the covariance's own scale.
//
// Anchor table layout (per problem): row s - s0 of the chunk holds the
// anchors of diagonals d_lo .. d_lo + wp_pad - 1 in blocks of 1024
// diagonals (the band width), each block stored residue-major: diagonal
// d_lo + 1024 b + 8q + r at b * 1024 + 128 r + q.  Thread t of the band
// kernel, whose diagonals are 8t .. 8t + 7 of band b, then reads entry
// 128 k + t for its k-th diagonal: coalesced across the warp.
//
// Waits on the MMA completion barrier are bounded; a wait that gives up
// sets the join's error word (the host returns SCAMP_ERR_DEVICE_TIMEOUT).
#include <cuda_bf16.h>

#include <cstdint>

#include "engine.cuh"

namespace scamp_gb300 {

namespace {

constexpr int kTcThreads = 128;         // four warps: TMEM lanes 0..127
constexpr int kTileCols = 1024;         // columns j per tile (8 residues x 128 rows)
constexpr int kRowsPerTile = 16;        // anchor rows per tile (the MMA's N)
constexpr int kKBlock = 512;            // window terms staged per pass
constexpr int kSub = 64;                // terms per TMEM accumulation
constexpr int kStreamLen = 8 * 127 + kKBlock;  // stream elements a pass reads
constexpr int kStreamPad = kStreamLen + 8;      // padded (16-byte multiple)
constexpr int kTmemCols = 256;          // 8 residues x 2 accumulators x 16 columns
constexpr int kMaxPad = 8192;           // longest window (padded) the contraction serves

// Shared memory of one CTA (dynamic): streams [3 splits][8 residues][kStreamPad]
// bf16, the anchor-window operand [3 splits][kRowsPerTile x kKBlock] bf16 in
// core-matrix layout, the anchor rows' sums, the TMEM address and the barrier.
struct TcSmem {
  __nv_bfloat16 z[3][8][kStreamPad];
  __nv_bfloat16 w[3][kRowsPerTile * kKBlock];
  float xsum[kRowsPerTile];
  uint32_t tmem_base;
  unsigned long long mbar;
  double part[kTcThreads];  // prefix-sum scan of the threads' span pieces
  // followed in the dynamic allocation by: float2 pre[span + 1] (prefix sums
  // of y as hi + lo) and float xi[kRowsPerTile][nsub]
};

// Dynamic shared memory of a contraction with m_pad window terms.
__host__ __device__ inline size_t tc_smem_bytes(int64_t m_pad) {
  const int64_t span = kTileCols + m_pad;
  return sizeof(TcSmem) + static_cast<size_t>(span + 1) * sizeof(float2) +
         static_cast<size_t>(kRowsPerTile * ((m_pad + 63) / 64)) * sizeof(float);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, no swizzle: start address,
// leading-dimension byte offset, stride-dimension byte offset (all >> 4),
// descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t{1} << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A
// and B bf16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                            (static_cast<uint32_t>(kRowsPerTile >> 3) << 17) |
                            (static_cast<uint32_t>(128 >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
      :
      : "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait for barrier phase `parity`: false when it gave up (about two
// seconds of clock64, or 2^26 polls).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const long long t0 = clock64();
  for (int it = 0; it < (1 << 26); ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > (1ll << 32)) break;
  }
  return false;
}

// 16 consecutive FP32 columns of the warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Exact split of an FP32 value into three bf16 terms (each remainder is
// exact in FP32; the last has at most 8 significant bits).
__device__ __forceinline__ void split3(float v, __nv_bfloat16& h, __nv_bfloat16& m,
                                       __nv_bfloat16& l) {
  h = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(h);
  m = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(m);
  l = __float2bfloat16_rn(r2);
}

// Offset of block b relative to block b0 (as the band kernel's anchors).
__device__ __forceinline__ float blk_delta(const SeriesDev& S, int64_t b, int64_t b0) {
  return (S.bhi[b] - S.bhi[b0]) + (S.blo[b] - S.blo[b0]);
}

}  // namespace

// Anchor windows of one problem's chunk, split: row `row` is anchor row
// s = s0 + row, window sK of the row series centred by its FP64 mean, from
// the same block-relative FP32 data the CUDA-core anchors use.  Each 64-term
// block b is centred by its own mean: xi[row][b] = that mean, out[split][row]
// [t] = the split of x(t) - xi_b (rows padded to a multiple of kRowsPerTile,
// terms to m_pad; padding 0), xsum[row] = the sum of x(t) - xi_b (the split
// is exact).  One block per row.
__global__ void __launch_bounds__(256) anchor_split_kernel(AnchorArgs A) {
  __shared__ float xs[kMaxPad];
  __shared__ float red[256];
  const int64_t row = blockIdx.x;
  const int64_t s = A.s0 + row;
  const int64_t i = s * A.K;
  const SeriesDev& R = A.R;
  const bool live = row < A.nrows && i < R.ns;
  const int sh = R.bshift;
  const int64_t bi = live ? (i >> sh) : 0;
  const float mr = live ? R.mu_rel[i] : 0.f;
  for (int64_t t = threadIdx.x; t < A.m_pad; t += blockDim.x)
    xs[t] = (live && t < A.m) ? R.T32[i + t] + (blk_delta(R, (i + t) >> sh, bi) - mr) : 0.f;
  __syncthreads();
  // block means (one thread per 64-term block)
  for (int64_t b = threadIdx.x; b < A.nsub; b += blockDim.x) {
    const int64_t t0 = 64 * b, t1 = (t0 + 64 < A.m) ? t0 + 64 : A.m;
    float sum = 0.f;
    for (int64_t t = t0; t < t1; ++t) sum += xs[t];
    A.xi[row * A.nsub + b] = t1 > t0 ? sum / static_cast<float>(t1 - t0) : 0.f;
  }
  __syncthreads();
  float part = 0.f;
  for (int64_t t = threadIdx.x; t < A.m_pad; t += blockDim.x) {
    const float v = t < A.m ? xs[t] - A.xi[row * A.nsub + (t >> 6)] : 0.f;
    __nv_bfloat16 h, md, l;
    split3(v, h, md, l);
    const int64_t o = row * A.m_pad + t;
    A.wsplit[0 * A.rows_pad * A.m_pad + o] = h;
    A.wsplit[1 * A.rows_pad * A.m_pad + o] = md;
    A.wsplit[2 * A.rows_pad * A.m_pad + o] = l;
    part += v;
  }
  red[threadIdx.x] = part;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) A.xsum[row] = red[0];
}

// The contraction of one problem's chunk into its anchor table.  Tiles:
// (group of kRowsPerTile anchor rows) x (1024 columns); a persistent CTA
// takes tiles in stride.  desc_mode 0: the descriptors' leading offset steps
// along K and the stride offset along M/N (the canonical K-major form);
// desc_mode 1 swaps them (selected once by the host's self-check).
__global__ void __launch_bounds__(kTcThreads, 1) anchor_gemm_kernel(AnchorArgs A) {
  extern __shared__ __align__(1024) unsigned char tc_raw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(tc_raw);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const SeriesDev& C = A.C;
  const int sh = C.bshift;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :
                 : "r"(smem_u32(&sm.tmem_base)), "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" : : "r"(smem_u32(&sm.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = sm.tmem_base;
  uint32_t phase = 0;
  bool ok = true;

  const int64_t groups = A.rows_pad / kRowsPerTile;
  const int64_t col_tiles = A.col_tiles;
  const int64_t ntiles = groups * col_tiles;
  const int64_t kpb = A.K / kTileCols;  // column tiles per anchor row step
  for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int64_t grp = tile / col_tiles, ct = tile - grp * col_tiles;
    const int64_t s_first = A.s0 + grp * kRowsPerTile;
    // columns J0 .. J0 + 1023: diagonal block ct - (s - s_first) kpb of row s
    const int64_t J0 = s_first * A.K + A.d_lo + ct * kTileCols;
    if (J0 >= C.ns) continue;  // no column window of the tile exists (uniform)
    const int64_t bJ0 = (J0 < C.n ? J0 : C.n - 1) >> sh;  // offset block of the tile
    // ---- prefix sums of the span y(J0 + p), p < span, as hi + lo floats ----
    float2* pre = reinterpret_cast<float2*>(tc_raw + sizeof(TcSmem));
    float* xi_s = reinterpret_cast<float*>(pre + (kTileCols + A.m_pad + 1));
    {
      const int64_t span = kTileCols + A.m_pad;
      const int64_t per = (span + kTcThreads - 1) / kTcThreads;
      const int64_t p0 = t * per, p1 = (p0 + per < span) ? p0 + per : span;
      double run = 0.0;
      for (int64_t p = p0; p < p1; ++p) {
        const int64_t g = J0 + p;
        if (g < C.n) run += static_cast<double>(C.T32[g] + blk_delta(C, g >> sh, bJ0));
      }
      sm.part[t] = run;
      __syncthreads();
      if (t == 0) {
        double acc_p = 0.0;
        for (int k = 0; k < kTcThreads; ++k) {
          const double v = sm.part[k];
          sm.part[k] = acc_p;
          acc_p += v;
        }
      }
      __syncthreads();
      run = sm.part[t];
      for (int64_t p = p0; p < p1; ++p) {
        const float hi = static_cast<float>(run);
        pre[p] = make_float2(hi, static_cast<float>(run - hi));
        const int64_t g = J0 + p;
        if (g < C.n) run += static_cast<double>(C.T32[g] + blk_delta(C, g >> sh, bJ0));
      }
      if (p1 == span && p0 < p1) {
        const float hi = static_cast<float>(run);
        pre[span] = make_float2(hi, static_cast<float>(run - hi));
      }
      for (int64_t q = t; q < kRowsPerTile * A.nsub; q += kTcThreads)
        xi_s[q] = A.xi[(grp * kRowsPerTile) * A.nsub + q];
    }
    float acc[8][kRowsPerTile];  // lane q's columns J0 + 8q + r, one per anchor row
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
      for (int n = 0; n < kRowsPerTile; ++n) acc[r][n] = 0.f;
    const uint32_t lane_addr = static_cast<uint32_t>(32 * warp) << 16;
    for (int64_t k0 = 0; k0 < A.m_pad && ok; k0 += kKBlock) {
      // ---- streams z_r[e] = y(J0 + k0 + r + e), split ----
      for (int p = t; p < kStreamLen + 8; p += kTcThreads) {
        const int64_t g = J0 + k0 + p;  // sample of the column series
        float v = 0.f;
        if (g < C.n && k0 + p < A.m + kTileCols) v = C.T32[g] + blk_delta(C, g >> sh, bJ0);
        __nv_bfloat16 h, md, l;
        split3(v, h, md, l);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const int e = p - r;
          if (e >= 0 && e < kStreamPad) {
            sm.z[0][r][e] = h;
            sm.z[1][r][e] = md;
            sm.z[2][r][e] = l;
          }
        }
      }
      // ---- anchor-window operand: the core matrix (8 rows x 8 terms) of
      // rows 8c.. and terms 8b.. at element (c * (kKBlock / 8) + b) * 64 ----
      for (int q = t; q < 3 * kRowsPerTile * (kKBlock / 8); q += kTcThreads) {
        const int split = q / (kRowsPerTile * (kKBlock / 8));
        const int rem = q - split * (kRowsPerTile * (kKBlock / 8));
        const int row = rem / (kKBlock / 8), b = rem - row * (kKBlock / 8);
        const int64_t src = (static_cast<int64_t>(split) * A.rows_pad + grp * kRowsPerTile + row) *
                                A.m_pad + k0 + 8 * b;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (k0 + 8 * b < A.m_pad) v = *reinterpret_cast<const uint4*>(A.wsplit + src);
        const int c = row >> 3, rr = row & 7;
        *reinterpret_cast<uint4*>(&sm.w[split][(c * (kKBlock / 8) + b) * 64 + rr * 8]) = v;
      }
      if (k0 == 0 && t < kRowsPerTile) sm.xsum[t] = A.xsum[grp * kRowsPerTile + t];
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      const int kend = static_cast<int>((A.m_pad - k0) < kKBlock ? (A.m_pad - k0) : kKBlock);
      for (int sb = 0; sb < kend && ok; sb += kSub) {
        // ---- MMAs of 64 terms (one thread) into fresh accumulators ----
        if (t == 0 && !A.wait_test) {
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // A (Hankel): K step 16 B, M step 128 B; B (windows): K step 128 B,
          // N step (kKBlock / 8) * 128 B
          const uint32_t a_k = 16, a_m = 128, b_k = 128, b_n = (kKBlock / 8) * 128;
          const uint32_t a_lbo = A.desc_mode ? a_m : a_k, a_sbo = A.desc_mode ? a_k : a_m;
          const uint32_t b_lbo = A.desc_mode ? b_n : b_k, b_sbo = A.desc_mode ? b_k : b_n;
          const int send = (sb + kSub) < kend ? sb + kSub : kend;
          for (int ks = sb; ks < send; ks += 16) {
            for (int r = 0; r < 8; ++r) {
              const uint32_t d_main = tmem + static_cast<uint32_t>(r * 2 * kRowsPerTile);
              const uint32_t d_corr = d_main + kRowsPerTile;
              // the 6 products of order <= 2: (A split, B split, accumulator)
#pragma unroll
              for (int pr = 0; pr < 6; ++pr) {
                const int sa = pr == 0 ? 0 : pr == 1 ? 0 : pr == 2 ? 1 : pr == 3 ? 0 : pr == 4 ? 1 : 2;
                const int sbs = pr == 0 ? 0 : pr == 1 ? 1 : pr == 2 ? 0 : pr == 3 ? 2 : pr == 4 ? 1 : 0;
                const uint64_t ad = smem_desc(smem_u32(&sm.z[sa][r][ks]), a_lbo, a_sbo);
                const uint64_t bd = smem_desc(smem_u32(&sm.w[sbs][(ks / 8) * 64]), b_lbo, b_sbo);
                const bool first = ks == sb && (pr == 0 || pr == 1);
                mma_bf16(pr == 0 ? d_main : d_corr, ad, bd, first ? 0u : 1u);
              }
            }
          }
          mma_commit(&sm.mbar);
        }
        __syncwarp();
        // every thread waits for the MMAs; the outcome is made uniform over
        // the CTA before any warp-wide TMEM access
        const bool done = mbar_wait(&sm.mbar, phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        ok = __syncthreads_and(done ? 1 : 0) != 0;
        if (!ok) {
          if (t == 0 && A.error_flag) atomicExch(A.error_flag, 1);
          break;
        }
        // ---- the 64-term sums into the registers (round to nearest) ----
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          float mv[16], cv[16];
          tmem_ld16(tmem + lane_addr + static_cast<uint32_t>(r * 2 * kRowsPerTile), mv);
          tmem_ld16(tmem + lane_addr + static_cast<uint32_t>(r * 2 * kRowsPerTile + kRowsPerTile),
                    cv);
#pragma unroll
          for (int n = 0; n < kRowsPerTile; ++n) acc[r][n] += mv[n] + cv[n];
        }
        // the next MMAs overwrite the accumulators: every warp has read them
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
      }
    }
    if (!ok) break;
    // ---- epilogue: lane q of warp w holds columns j = J0 + 8 (32 w + lane) + r ----
    const int q = 32 * warp + lane;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int64_t j = J0 + 8 * q + r;
      const int o = 8 * q + r;  // j - J0
      // cov = sum_t x'(y(j+t) - y0) + sum_b xi_b (S_b(j) - len_b ej) - ej sum x'
      // with ej = mu_j - y0 (y0: the tile's offset block)
      float ej = 0.f;
      if (j < C.ns) ej = C.mu_rel[j] + blk_delta(C, j >> sh, bJ0);
      float corr[kRowsPerTile];
#pragma unroll
      for (int n = 0; n < kRowsPerTile; ++n) corr[n] = -ej * sm.xsum[n];
      for (int64_t b = 0; b < A.nsub; ++b) {
        const int64_t t0 = 64 * b, t1 = (t0 + 64 < A.m) ? t0 + 64 : A.m;
        const float2 pa = pre[o + t0], pb = pre[o + t1];
        const float sbj = ((pb.x - pa.x) + (pb.y - pa.y)) - static_cast<float>(t1 - t0) * ej;
#pragma unroll
        for (int n = 0; n < kRowsPerTile; ++n) corr[n] = fmaf(xi_s[n * A.nsub + b], sbj, corr[n]);
      }
#pragma unroll
      for (int n = 0; n < kRowsPerTile; ++n) {
        const int64_t row = grp * kRowsPerTile + n;
        const int64_t s = A.s0 + row;
        const int64_t b = ct - (s - s_first) * kpb;  // diagonal block of row s
        if (row < A.nrows && b >= 0 && b < A.wp_pad / kTileCols)
          A.table[row * A.wp_pad + b * kTileCols + r * 128 + q] = acc[r][n] + corr[n];
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (!ok) {
    // a wait gave up: wait once more (bounded) for the MMAs in flight before
    // the accumulators are freed
    mbar_wait(&sm.mbar, phase ^ 1u);
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :
                 : "r"(tmem), "r"(kTmemCols)
                 : "memory");
}

size_t anchor_gemm_smem_bytes(int64_t m_pad) { return tc_smem_bytes(m_pad); }
int64_t anchor_max_window() { return kMaxPad; }
int anchor_tile_cols() { return kTileCols; }
int anchor_rows_per_tile() { return kRowsPerTile; }
int anchor_kblock() { return kKBlock; }

}  // namespace scamp_gb300

namespace scamp_gb300 {

// FP64 check of an anchor table (the self-check and the diagnostic entry):
// every `stride`-th entry whose row and column windows exist and are valid,
// against the direct FP64 covariance of the two windows, scaled by both
// inverse norms; out[0] = max error (bits of a non-negative double, so
// integer max orders them), out[1] = entries checked.
__global__ void __launch_bounds__(256) anchor_check_kernel(AnchorArgs A, int64_t stride,
                                                           unsigned long long* out) {
  const int64_t total = A.nrows * A.wp_pad;
  const int64_t step = static_cast<int64_t>(gridDim.x) * blockDim.x * stride;
  for (int64_t e = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * stride;
       e < total; e += step) {
    const int64_t row = e / A.wp_pad, x = e - row * A.wp_pad;
    const int64_t b = x >> 10, r = (x >> 7) & 7, q = x & 127;
    const int64_t d = A.d_lo + 1024 * b + 8 * q + r;
    const int64_t i = (A.s0 + row) * A.K, j = i + d;
    if (i >= A.R.ns || j >= A.C.ns || j < 0) continue;
    const double iv = A.R.inv[i] * A.C.inv[j];
    if (isnan(iv)) continue;
    const double mr = A.R.mean[i], mc = A.C.mean[j];
    double c = 0.0;
    for (int64_t t = 0; t < A.m; ++t) c = fma(A.R.T[i + t] - mr, A.C.T[j + t] - mc, c);
    const double err = fabs(static_cast<double>(A.table[e]) - c) * iv;
    atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(err)));
    atomicAdd(out + 1, 1ull);
  }
}

}  // namespace scamp_gb300
