// Kernel set (d): stochastic reconfiguration in sample space.
//
// The reference solves (S + lambda I) x = F in parameter space with
// S = O_c^H O_c / B and F = O_c^H (E - Ebar) / B
// (optimizers/stochastic_reconfiguration/optimizer.py:55-124). With the P x 2B
// matrix Y = [Re O_c | Im O_c] (parameter-major rows of the per-sample
// log-derivatives) the push-through identity
//     (X^T X + lambda I)^-1 X^T e = X^T (X X^T + lambda I)^-1 e
// moves the solve to the 2B x 2B Gram T = Y^T Y / B:
//   1. centre every row of O over the samples (fk_center_columns);
//   2. T = Y^T Y: FP32 products accumulated in FP32 over chunks of K, chunk
//      sums reduced in FP64 (fk_sr_gram), upper-triangle tiles only;
//   3. (T/B + lambda I) alpha = eps solved by FP64 conjugate gradients with the
//      reference's stopping rule ||r|| <= tol ||eps|| (linear_equations.py:34-137)
//      (fk_sr_solve);
//   4. x = Y alpha / B and theta <- theta - lr x (fk_sr_backmap).
// For real parameters (the AR network) eps = [Re(E - Ebar); Im(E - Ebar)] and
// the update solves the real SR system S = Re<O_c^* O_c>, F = Re<O_c^* E_c>.
#include <mutex>

#include "fk_common.cuh"

namespace fk {

// ---------------------------------------------------------------- centring
__global__ void center_kernel(float* __restrict__ y, int64_t rows, int64_t cols, float* __restrict__ mean) {
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= rows) return;
  float* r = y + row * cols;
  // compensated float32 sums per lane, a float32 tree over the warp (the
  // FP64 pipe of this part is narrow)
  Kahan k;
  for (int64_t j = lane; j < cols; j += 32) k.add(r[j]);
  float s = k.s - k.c;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  float mu = s / (float)cols;
  for (int64_t j = lane; j < cols; j += 32) r[j] -= mu;
  if (mean && lane == 0) mean[row] = mu;
}

// ---------------------------------------------------------------- Gram
// T[i][j] = sum_p Y[p][i] Y[p][j], Y columns: [0,B) from A (row stride B),
// [B,2B) from Bm. 64x64 output tile per CTA (256 threads, 4x4 each), K split
// over blockIdx.z; per CTA the K range is walked in chunks whose FP32 partial
// sums are added into FP64 registers, then atomically into T (FP64).
constexpr int kGT = 64;
constexpr int kGK = 16;
constexpr int kChunk = 2048;

__device__ __forceinline__ float ycol(const float* __restrict__ a, const float* __restrict__ b, int64_t bsz,
                                      int64_t p, int64_t j) {
  return j < bsz ? a[p * bsz + j] : b[p * bsz + (j - bsz)];
}

__global__ void __launch_bounds__(256) gram_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                                   int64_t P, int64_t bsz, int64_t n, int64_t k_per_cta,
                                                   double* __restrict__ t) {
  // upper-triangle tile index -> (ti, tj)
  int64_t ntile = (n + kGT - 1) / kGT;
  int64_t idx = blockIdx.x, ti = 0;
  while (idx >= ntile - ti) {
    idx -= ntile - ti;
    ++ti;
  }
  int64_t tj = ti + idx;
  const int64_t i0 = ti * kGT, j0 = tj * kGT;
  const int64_t k_begin = (int64_t)blockIdx.z * k_per_cta;
  const int64_t k_end = min(P, k_begin + k_per_cta);
  __shared__ float si[kGK][kGT];
  __shared__ float sj[kGK][kGT];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc64[4][4];
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc64[u][v] = 0.0;
  for (int64_t c0 = k_begin; c0 < k_end; c0 += kChunk) {
    const int64_t c1 = min(k_end, c0 + kChunk);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    for (int64_t k0 = c0; k0 < c1; k0 += kGK) {
      for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
        int kk = e / kGT, col = e % kGT;
        int64_t p = k0 + kk;
        bool ok = p < c1;
        si[kk][col] = (ok && i0 + col < n) ? ycol(a, b, bsz, p, i0 + col) : 0.f;
        sj[kk][col] = (ok && j0 + col < n) ? ycol(a, b, bsz, p, j0 + col) : 0.f;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kGK; ++kk) {
        float xi[4], xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          xi[u] = si[kk][ty * 4 + u];
          xj[u] = sj[kk][tx * 4 + u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] += xi[u] * xj[v];
      }
      __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc64[u][v] += (double)acc[u][v];
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      int64_t i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
      if (i < n && j < n && j >= i) atomicAdd(&t[i * n + j], acc64[u][v]);
    }
  }
}

__global__ void mirror_kernel(double* t, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  int64_t i = idx / n, j = idx % n;
  if (j < i) t[i * n + j] = t[j * n + i];
}

// ---------------------------------------------------------------- Gram on tensor cores
// T = Y^T Y (Y = [o_re | o_im], P x n, parameter-major fp32) with tcgen05:
// each fp32 value is split into bf16 hi = bf16(y) and lo = bf16(y - hi), and
// every product is hi*hi + hi*lo + lo*hi (the lo*lo term is below fp32's
// rounding), accumulated in fp32 in TMEM over ranges of at most 4096
// parameters and in fp64 across ranges: three bf16 MMAs per product. Output tiles of 128 (i) x 256 (j) samples on or
// above the diagonal, K = parameters split into ranges (work item = tile x
// range); per range the tile's fp32 sums are added into T with fp64 atomics.
// Roles (13 warps): 8 converter warps load 64 parameters x (128 + 256)
// columns per stage from global memory (32-byte sector loads), split them
// into hi/lo and store them as MN-major operands (8 samples per 16 bytes,
// LBO 128 B along K, SBO 1 KB along the samples) in one of two stages; one
// issuer warp (lane 0) issues 12 MMAs (M128 N256 K16) per stage into one of
// two TMEM accumulators; 4 drain warps read a finished accumulator (the
// lane quarter of their rank in the warpgroup) and add it into T while the
// next item accumulates. Every wait is bounded (mbar_wait).
namespace gram_tc {
constexpr int kM = 128, kN = 256, kK = 64, kStages = 2;
constexpr int kAB = kM * kK * 2;                 // one A half (hi or lo): 16 KB
constexpr int kBB = kN * kK * 2;                 // one B half: 32 KB
constexpr int kStage = 2 * kAB + 2 * kBB;        // 96 KB
constexpr int kConvWarps = 8, kIssuerWarp = 8;
constexpr int kThreads = 32 * 13;
constexpr int kSmem = kStages * kStage + 256;
static_assert((kM / 8 + kN / 8) * kK % (kConvWarps * 32) == 0, "whole chunks per converter thread");
}  // namespace gram_tc

struct GramTcArgs {
  const float* a;   // o_re [P][bsz]
  const float* b;   // o_im [P][bsz] (== a when n == bsz)
  int64_t P, bsz, n;
  int64_t kper;     // parameters per range (multiple of 64)
  int64_t splits;
  int64_t nti, ntj;
  int64_t items;
  double* t;        // n x n, j >= i written
  int* err;
};

// Work item -> tile origin (i0, j0) and parameter range [k0, k1). Tile rows
// ti take j-tiles tj >= ti / 2 (the first 256-wide tile reaching row ti*128).
__device__ __forceinline__ void gram_item(const GramTcArgs& g, int64_t item, int64_t& i0, int64_t& j0, int64_t& k0,
                                          int64_t& k1) {
  // consecutive items (the CTAs running at the same time) share a parameter
  // range, so its rows are read from DRAM once and from L2 by every tile
  const int64_t tiles = g.items / g.splits;
  const int64_t split = item / tiles, tile = item % tiles;
  int64_t ti = 0, rem = tile;
  while (ti < g.nti && rem >= g.ntj - ti / 2) {
    rem -= g.ntj - ti / 2;
    ++ti;
  }
  i0 = ti * gram_tc::kM;
  j0 = (ti / 2 + rem) * gram_tc::kN;
  k0 = split * g.kper;
  k1 = min(g.P, k0 + g.kper);
}

// 8 consecutive columns [c, c+8) of parameter row p: zero outside P x n.
__device__ __forceinline__ void gram_load8(const GramTcArgs& g, int64_t p, int64_t c, float* v) {
  if (p < g.P && c < g.n) {
    const float* src = c < g.bsz ? g.a + p * g.bsz + c : g.b + p * g.bsz + (c - g.bsz);
    const float4 x0 = reinterpret_cast<const float4*>(src)[0];
    const float4 x1 = reinterpret_cast<const float4*>(src)[1];
    v[0] = x0.x; v[1] = x0.y; v[2] = x0.z; v[3] = x0.w;
    v[4] = x1.x; v[5] = x1.y; v[6] = x1.z; v[7] = x1.w;
  } else {
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = 0.f;
  }
}

__device__ __forceinline__ void gram_split_store(const float* v, uint8_t* hi, uint8_t* lo, int off) {
  float h[8], l[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    h[e] = __bfloat162float(__float2bfloat16_rn(v[e]));
    l[e] = v[e] - h[e];
  }
  uint4 uh, ul;
  uh.x = pack_bf16x2(h[0], h[1]); uh.y = pack_bf16x2(h[2], h[3]);
  uh.z = pack_bf16x2(h[4], h[5]); uh.w = pack_bf16x2(h[6], h[7]);
  ul.x = pack_bf16x2(l[0], l[1]); ul.y = pack_bf16x2(l[2], l[3]);
  ul.z = pack_bf16x2(l[4], l[5]); ul.w = pack_bf16x2(l[6], l[7]);
  *reinterpret_cast<uint4*>(hi + off) = uh;
  *reinterpret_cast<uint4*>(lo + off) = ul;
}

__global__ void __launch_bounds__(gram_tc::kThreads, 1) gram_tc_kernel(const __grid_constant__ GramTcArgs g) {
  using namespace gram_tc;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStage);
  uint64_t* full = bars;          // [2] converters -> issuer (8 warp arrivals)
  uint64_t* empty = bars + 2;     // [2] MMAs done with a stage (commit)
  uint64_t* accfull = bars + 4;   // [2] accumulator complete (commit)
  uint64_t* accempty = bars + 6;  // [2] accumulator drained (4 warp arrivals)
  uint64_t* drain = bars + 8;     // every MMA complete before teardown
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 9);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(&full[i], kConvWarps);
      mbar_init(&empty[i], 1);
      mbar_init(&accfull[i], 1);
      mbar_init(&accempty[i], 4);
    }
    mbar_init(drain, 1);
    fence_mbar_init();
  }
  if (warp == kIssuerWarp) {
    tmem_alloc(tslot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool abort = false;

  if (warp < kConvWarps) {
    // ---------------------------------------------------------------- converters
    uint32_t gc = 0;
    for (int64_t it = blockIdx.x; it < g.items && !abort; it += gridDim.x) {
      int64_t i0, j0, k0, k1;
      gram_item(g, it, i0, j0, k0, k1);
      for (int64_t kc = k0; kc < k1 && !abort; kc += kK, ++gc) {
        const uint32_t st = gc % kStages;
        if (gc >= kStages && !mbar_wait(&empty[st], ((gc / kStages) - 1) & 1, g.err)) {
          abort = true;
          break;
        }
        uint8_t* base = smem + st * kStage;
        uint8_t *ahi = base, *alo = base + kAB, *bhi = base + 2 * kAB, *blo = base + 2 * kAB + kBB;
        // A: 16 groups of 8 samples x 64 parameters; B: 32 groups x 64.
        // Consecutive threads take consecutive parameters: conflict-free
        // 16-byte shared stores, one 32-byte sector per global load. All of
        // a thread's loads are issued before the first store, so that their
        // latencies overlap.
        constexpr int kPer = (kM / 8 + kN / 8) * kK / (kConvWarps * 32);
        float v[kPer][8];
#pragma unroll
        for (int r = 0; r < kPer; ++r) {
          const int q = threadIdx.x + r * kConvWarps * 32;
          const int pq = q % kK, grp = q / kK;
          gram_load8(g, kc + pq, grp < kM / 8 ? i0 + 8 * grp : j0 + 8 * (grp - kM / 8), v[r]);
        }
#pragma unroll
        for (int r = 0; r < kPer; ++r) {
          const int q = threadIdx.x + r * kConvWarps * 32;
          const int pq = q % kK, grp = q / kK;
          if (grp < kM / 8)
            gram_split_store(v[r], ahi, alo, (grp * kK + pq) * 16);
          else
            gram_split_store(v[r], bhi, blo, ((grp - kM / 8) * kK + pq) * 16);
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&full[st]);
      }
    }
  } else if (warp == kIssuerWarp) {
    // ---------------------------------------------------------------- issuer
    const uint32_t idesc = umma_idesc_bf16_mn(kM, kN);
    uint32_t gc = 0, li = 0;
    for (int64_t it = blockIdx.x; it < g.items && !abort; it += gridDim.x, ++li) {
      int64_t i0, j0, k0, k1;
      gram_item(g, it, i0, j0, k0, k1);
      const uint32_t buf = li % 2;
      if (li >= 2 && !mbar_wait(&accempty[buf], ((li / 2) - 1) & 1, g.err)) {
        abort = true;
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + buf * kN;
      bool first = true;
      for (int64_t kc = k0; kc < k1; kc += kK, ++gc) {
        const uint32_t st = gc % kStages;
        if (!mbar_wait(&full[st], (gc / kStages) & 1, g.err)) {
          abort = true;
          break;
        }
        tc_fence_after();
        if (lane == 0) {
          const uint32_t base = smem_u32(smem + st * kStage);
          const uint64_t ahi = umma_sdesc(base, 128, kK * 16), alo = umma_sdesc(base + kAB, 128, kK * 16);
          const uint64_t bhi = umma_sdesc(base + 2 * kAB, 128, kK * 16);
          const uint64_t blo = umma_sdesc(base + 2 * kAB + kBB, 128, kK * 16);
#pragma unroll
          for (int ks = 0; ks < kK / 16; ++ks) {
            umma_bf16(d, ahi + ks * 16, bhi + ks * 16, idesc, (first && ks == 0) ? 0u : 1u);
            umma_bf16(d, ahi + ks * 16, blo + ks * 16, idesc, 1u);
            umma_bf16(d, alo + ks * 16, bhi + ks * 16, idesc, 1u);
          }
          umma_commit(&empty[st]);
        }
        __syncwarp();
        first = false;
      }
      if (abort) break;
      if (lane == 0) umma_commit(&accfull[buf]);
      __syncwarp();
    }
    if (lane == 0) {
      umma_commit(drain);
      mbar_wait(drain, 0, g.err);
    }
    __syncwarp();
  } else {
    // ---------------------------------------------------------------- drain
    // a warp reads the TMEM lane quarter of its rank in its warpgroup
    // (warps 9, 10, 11, 12 -> quarters 1, 2, 3, 0)
    const int q4 = warp % 4;
    uint32_t li = 0;
    for (int64_t it = blockIdx.x; it < g.items && !abort; it += gridDim.x, ++li) {
      int64_t i0, j0, k0, k1;
      gram_item(g, it, i0, j0, k0, k1);
      const uint32_t buf = li % 2;
      bool ok = mbar_wait(&accfull[buf], (li / 2) & 1, g.err);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        abort = true;
        break;
      }
      tc_fence_after();
      const int64_t i = i0 + q4 * 32 + lane;
      const uint32_t tl = tmem + buf * kN + ((uint32_t)(q4 * 32) << 16);
      for (int c0 = 0; c0 < kN; c0 += 16) {
        float v[16];
        tmem_ld16(tl + c0, v);
        tmem_ld_wait();
        if (i < g.n) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int64_t j = j0 + c0 + e;
            if (j >= i && j < g.n) atomicAdd(&g.t[i * g.n + j], (double)v[e]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&accempty[buf]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kIssuerWarp) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------- pre-split Gram on tensor cores
// The tensor-core Gram's split operands written once (split_kernel): every
// float32 value of Y (rows x n) as bf16 hi = bf16(y) and lo = bf16(y - hi)
// in a blocked layout in which each operand of a pipeline stage is one
// contiguous run, so that gram_split_kernel streams them with bulk copies
// instead of converting every value again for each tile that reads it
// (n / 128 + n / 256 times). Block (kc, g) holds rows [32 kc, 32 kc + 32) x
// columns [8 g, 8 g + 8), one row per 16 bytes (a row of an MN-major core
// matrix); blocks ordered by kc, then g; rows padded to a multiple of 32 and
// columns to a multiple of 256 with zeros; lo follows hi.
namespace gram_split {
constexpr int kK = 32;                   // parameter rows per stage
constexpr int kBlock = kK * 8 * 2;       // one (kc, g) block: 512 B
constexpr int kStages = 4;
constexpr int kA = (gram_tc::kM / 8) * kBlock;  // 128 samples: 8 KB (hi or lo)
constexpr int kB = (gram_tc::kN / 8) * kBlock;  // 256 samples: 16 KB
constexpr int kStage = 2 * kA + 2 * kB;         // 48 KB
constexpr int kThreads = 32 * 8;                // producer, issuer, 2 idle, 4 drain warps
constexpr int kSmem = kStages * kStage + 256;
}  // namespace gram_split

static int64_t split_rows_pad(int64_t rows) { return (rows + 31) / 32 * 32; }
static int64_t split_cols_pad(int64_t n) { return (n + 255) / 256 * 256; }
static int64_t split_bytes(int64_t rows, int64_t n) { return 2 * split_rows_pad(rows) * split_cols_pad(n) * 2; }

// One thread per (row, group of 8 columns); the 32 threads of a warp write
// the 32 rows of one block (512 contiguous bytes of hi and of lo). Column c
// of Y comes from a[p * ld + c] when c < bsz, from b[p * ld + c - bsz] after.
__global__ void split_kernel(const float* __restrict__ a, const float* __restrict__ b, int64_t ld, int64_t bsz,
                             int64_t rows, int64_t n, int64_t groups, int64_t total, uint4* __restrict__ hi,
                             uint4* __restrict__ lo) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int64_t blk = idx / 32;
  const int r = (int)(idx % 32);
  const int64_t kc = blk / groups, g = blk % groups;
  const int64_t p = kc * 32 + r;
  float v[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int64_t c = g * 8 + e;
    v[e] = (p < rows && c < n) ? (c < bsz ? a[p * ld + c] : b[p * ld + (c - bsz)]) : 0.f;
  }
  float h[8], l[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    h[e] = __bfloat162float(__float2bfloat16_rn(v[e]));
    l[e] = v[e] - h[e];
  }
  uint4 uh, ul;
  uh.x = pack_bf16x2(h[0], h[1]); uh.y = pack_bf16x2(h[2], h[3]);
  uh.z = pack_bf16x2(h[4], h[5]); uh.w = pack_bf16x2(h[6], h[7]);
  ul.x = pack_bf16x2(l[0], l[1]); ul.y = pack_bf16x2(l[2], l[3]);
  ul.z = pack_bf16x2(l[4], l[5]); ul.w = pack_bf16x2(l[6], l[7]);
  hi[idx] = uh;
  lo[idx] = ul;
}

// Centring and split in one pass (center_split_kernel): one CTA per block of
// 32 rows. Each row is centred within its two column groups, [0, bsz) from a
// and [bsz, n) from b (the per-row compensated mean of center_kernel, the
// same arithmetic), optionally written back in place, and split into the
// blocked hi / lo operands: the rows are read from DRAM once (the second
// pass over the CTA's 32 rows hits L2).
__global__ void __launch_bounds__(256) center_split_kernel(float* __restrict__ a, float* __restrict__ b, int64_t ld,
                                                           int64_t bsz, int64_t rows, int64_t n, int64_t groups,
                                                           int write_back, uint4* __restrict__ hi,
                                                           uint4* __restrict__ lo) {
  __shared__ float mean_sm[32][2];
  const int64_t kc = blockIdx.x;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  for (int rr = 0; rr < 4; ++rr) {
    const int r = warp * 4 + rr;
    const int64_t p = kc * 32 + r;
    for (int h = 0; h < 2; ++h) {
      const int64_t c_lo = h == 0 ? 0 : bsz;
      const int64_t c_hi = h == 0 ? (bsz < n ? bsz : n) : n;
      float mu = 0.f;
      if (p < rows && c_hi > c_lo) {
        const float* src = h == 0 ? a + p * ld : b + p * ld;
        const int64_t len = c_hi - c_lo;
        Kahan k;
        for (int64_t j = lane; j < len; j += 32) k.add(src[j]);
        float sum = k.s - k.c;
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        mu = sum / (float)len;
      }
      if (lane == 0) mean_sm[r][h] = mu;
    }
  }
  __syncthreads();
  // 64 columns per pass: thread = (row r, 8-column group gq); the 8 threads
  // of a row read 256 contiguous bytes of it
  const int r = threadIdx.x / 8, gq = threadIdx.x % 8;
  const int64_t p = kc * 32 + r;
  for (int64_t c0 = 0; c0 < groups * 8; c0 += 64) {
    const int64_t c = c0 + 8 * gq;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int64_t col = c + e;
      float x = 0.f;
      if (p < rows && col < n) {
        float* q = col < bsz ? a + p * ld + col : b + p * ld + (col - bsz);
        x = *q - mean_sm[r][col < bsz ? 0 : 1];
        if (write_back) *q = x;
      }
      v[e] = x;
    }
    float hv[8], lv[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      hv[e] = __bfloat162float(__float2bfloat16_rn(v[e]));
      lv[e] = v[e] - hv[e];
    }
    const int64_t idx = ((kc * groups + c / 8) * 32 + r);
    hi[idx] = make_uint4(pack_bf16x2(hv[0], hv[1]), pack_bf16x2(hv[2], hv[3]), pack_bf16x2(hv[4], hv[5]),
                         pack_bf16x2(hv[6], hv[7]));
    lo[idx] = make_uint4(pack_bf16x2(lv[0], lv[1]), pack_bf16x2(lv[2], lv[3]), pack_bf16x2(lv[4], lv[5]),
                         pack_bf16x2(lv[6], lv[7]));
  }
}

struct GramSplitArgs {
  const uint8_t* hi;
  const uint8_t* lo;
  int64_t groups;   // padded columns / 8
  int64_t n;        // columns of Y (T is n x n)
  int64_t kchunks;  // padded rows / 32
  int64_t kper;     // chunks per range
  int64_t splits;
  int64_t nti, ntj;
  int64_t items;
  double* t;
  int* err;
};

__device__ __forceinline__ void gram_split_item(const GramSplitArgs& g, int64_t item, int64_t& i0, int64_t& j0,
                                                int64_t& c0, int64_t& c1) {
  // Range-major, as gram_item: the CTAs running together share a range. Within
  // a range the upper-triangle tiles go in bands of kBand tile rows, column
  // by column within a band, so that the ~152 tiles in flight span about
  // kBand A blocks and 152 / kBand B blocks (their operands shared through
  // L2) instead of a few tile rows with every B block.
  constexpr int64_t kBand = 8;
  const int64_t tiles = g.items / g.splits;
  const int64_t split = item / tiles;
  int64_t rem = item % tiles;
  int64_t b0 = 0;  // first tile row of the band
  for (; b0 < g.nti; b0 += kBand) {
    const int64_t b1 = min(g.nti, b0 + kBand);
    int64_t cnt = 0;
    for (int64_t ti = b0; ti < b1; ++ti) cnt += g.ntj - ti / 2;
    if (rem < cnt) break;
    rem -= cnt;
  }
  const int64_t b1 = min(g.nti, b0 + kBand);
  // column tj holds the band's rows ti < 2 tj + 2 (tj >= ti / 2)
  int64_t tj = b0 / 2;
  for (;;) {
    const int64_t c = min(b1, 2 * tj + 2) - b0;
    if (c == b1 - b0) break;  // full columns from here on
    if (rem < c) break;
    rem -= c;
    ++tj;
  }
  const int64_t full = b1 - b0;
  if (min(b1, 2 * tj + 2) - b0 == full) {
    tj += rem / full;
    rem %= full;
  }
  i0 = (b0 + rem) * gram_tc::kM;
  j0 = tj * gram_tc::kN;
  c0 = split * g.kper;
  c1 = min(g.kchunks, c0 + g.kper);
}

// T += upper triangle of Y^T Y from the split operands: a producer thread
// streams the four operand runs of a stage (A hi, A lo: 128 samples; B hi,
// B lo: 256 samples; 32 parameters) into one of four 48 KB stages with bulk
// copies; the issuer (lane 0) issues hi*hi + hi*lo + lo*hi as M128 N256 K16
// MMAs into one of two TMEM accumulators (FP32 over a range of at most 4096
// parameters); 4 drain warps add finished tiles into T with FP64 atomics.
// Every wait is bounded.
__global__ void __launch_bounds__(gram_split::kThreads, 1) gram_split_kernel(const __grid_constant__ GramSplitArgs g) {
  using namespace gram_split;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStage);
  uint64_t* full = bars;                 // [4] bytes of a stage landed
  uint64_t* empty = bars + kStages;      // [4] MMAs done with a stage (commit)
  uint64_t* accfull = bars + 2 * kStages;
  uint64_t* accempty = accfull + 2;      // [2] drained (4 warp arrivals)
  uint64_t* drain = accempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&accfull[i], 1);
      mbar_init(&accempty[i], 4);
    }
    mbar_init(drain, 1);
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tslot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool abort = false;

  if (warp == 0) {
    // ---------------------------------------------------------------- producer
    if (lane == 0) {
      uint32_t gc = 0;
      for (int64_t it = blockIdx.x; it < g.items && !abort; it += gridDim.x) {
        int64_t i0, j0, c0, c1;
        gram_split_item(g, it, i0, j0, c0, c1);
        for (int64_t kc = c0; kc < c1; ++kc, ++gc) {
          const uint32_t st = gc % kStages;
          if (gc >= kStages && !mbar_wait(&empty[st], ((gc / kStages) - 1) & 1, g.err)) {
            abort = true;
            break;
          }
          uint8_t* base = smem + st * kStage;
          const int64_t oa = (kc * g.groups + i0 / 8) * kBlock;
          const int64_t ob = (kc * g.groups + j0 / 8) * kBlock;
          mbar_arrive_expect_tx(&full[st], kStage);
          bulk_g2s(base, g.hi + oa, kA, &full[st]);
          bulk_g2s(base + kA, g.lo + oa, kA, &full[st]);
          bulk_g2s(base + 2 * kA, g.hi + ob, kB, &full[st]);
          bulk_g2s(base + 2 * kA + kB, g.lo + ob, kB, &full[st]);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------------- issuer
    const uint32_t idesc = umma_idesc_bf16_mn(gram_tc::kM, gram_tc::kN);
    uint32_t gc = 0, li = 0;
    for (int64_t it = blockIdx.x; it < g.items && !abort; it += gridDim.x, ++li) {
      int64_t i0, j0, c0, c1;
      gram_split_item(g, it, i0, j0, c0, c1);
      const uint32_t buf = li % 2;
      if (li >= 2 && !mbar_wait(&accempty[buf], ((li / 2) - 1) & 1, g.err)) {
        abort = true;
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + buf * gram_tc::kN;
      bool first = true;
      for (int64_t kc = c0; kc < c1; ++kc, ++gc) {
        const uint32_t st = gc % kStages;
        if (!mbar_wait(&full[st], (gc / kStages) & 1, g.err)) {
          abort = true;
          break;
        }
        tc_fence_after();
        if (lane == 0) {
          const uint32_t base = smem_u32(smem + st * kStage);
          const uint64_t ahi = umma_sdesc(base, 128, kK * 16), alo = umma_sdesc(base + kA, 128, kK * 16);
          const uint64_t bhi = umma_sdesc(base + 2 * kA, 128, kK * 16);
          const uint64_t blo = umma_sdesc(base + 2 * kA + kB, 128, kK * 16);
#pragma unroll
          for (int ks = 0; ks < kK / 16; ++ks) {
            umma_bf16(d, ahi + ks * 16, bhi + ks * 16, idesc, (first && ks == 0) ? 0u : 1u);
            umma_bf16(d, ahi + ks * 16, blo + ks * 16, idesc, 1u);
            umma_bf16(d, alo + ks * 16, bhi + ks * 16, idesc, 1u);
          }
          umma_commit(&empty[st]);
        }
        __syncwarp();
        first = false;
      }
      if (abort) break;
      if (lane == 0) umma_commit(&accfull[buf]);
      __syncwarp();
    }
    if (lane == 0) {
      umma_commit(drain);
      mbar_wait(drain, 0, g.err);
    }
    __syncwarp();
  } else if (warp >= 4) {
    // ---------------------------------------------------------------- drain
    // warps 4..7 read TMEM lane quarters 0..3
    const int q4 = warp % 4;
    uint32_t li = 0;
    for (int64_t it = blockIdx.x; it < g.items && !abort; it += gridDim.x, ++li) {
      int64_t i0, j0, c0, c1;
      gram_split_item(g, it, i0, j0, c0, c1);
      const uint32_t buf = li % 2;
      bool ok = mbar_wait(&accfull[buf], (li / 2) & 1, g.err);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        abort = true;
        break;
      }
      tc_fence_after();
      const int64_t i = i0 + q4 * 32 + lane;
      const uint32_t tl = tmem + buf * gram_tc::kN + ((uint32_t)(q4 * 32) << 16);
      for (int cq = 0; cq < gram_tc::kN; cq += 16) {
        float v[16];
        tmem_ld16(tl + cq, v);
        tmem_ld_wait();
        if (i < g.n) {
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int64_t j = j0 + cq + e;
            if (j >= i && j < g.n) atomicAdd(&g.t[i * g.n + j], (double)v[e]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&accempty[buf]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------- FP64 CG
// State: x, r, p, q (n each) + scalars s[0]=rr, s[1]=pq, s[2]=rr_new, s[3]=stop
// (1 when converged), s[4]=tol^2 * ||b||^2, s[5]=iterations.
__global__ void cg_init_kernel(const double* __restrict__ rhs, int64_t n, double* x, double* r, double* p,
                               double* s, double tol) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double v = rhs[i];
    x[i] = 0.0;
    r[i] = v;
    p[i] = v;
    acc += v * v;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s[0] = red[0];
    s[1] = 0.0;
    s[2] = 0.0;
    s[3] = red[0] == 0.0 ? 1.0 : 0.0;
    s[4] = tol * tol * red[0];
    s[5] = 0.0;
  }
}

// q = (scale T + shift I) p ; s[1] += p.q   (a warp per row)
__global__ void cg_matvec_kernel(const double* __restrict__ t, int64_t n, double scale, double shift,
                                 const double* __restrict__ p, double* __restrict__ q, double* s) {
  if (s[3] != 0.0) return;
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= n) return;
  const double* tr = t + row * n;
  double acc = 0.0;
  for (int64_t j = lane; j < n; j += 32) acc += tr[j] * p[j];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    double v = scale * acc + shift * p[row];
    q[row] = v;
    atomicAdd(&s[1], v * p[row]);
  }
}

// x += alpha p, r -= alpha q, s[2] += r.r
__global__ void cg_update_kernel(int64_t n, double* x, double* r, const double* p, const double* q, double* s) {
  if (s[3] != 0.0) return;
  __shared__ double red[256];
  double alpha = s[0] / s[1];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    double ri = r[i] - alpha * q[i];
    r[i] = ri;
    acc += ri * ri;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(&s[2], red[0]);
}

// p = r + beta p; roll the scalars; stop when ||r||^2 <= tol^2 ||b||^2
__global__ void cg_direction_kernel(int64_t n, const double* r, double* p, double* s, int last) {
  if (s[3] != 0.0) return;
  double beta = s[2] / s[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = r[i] + beta * p[i];
}

__global__ void cg_roll_kernel(double* s) {
  if (s[3] != 0.0) return;
  s[5] += 1.0;
  s[0] = s[2];
  s[1] = 0.0;
  s[2] = 0.0;
  if (s[0] <= s[4]) s[3] = 1.0;
}

// ---------------------------------------------------------------- back-map
// params[p] -= lr * scale * sum_j Y[p][j] alpha[j]   (a warp per row). The
// update is float32, so the products and sums are too (compensated per lane,
// then a tree over the warp): FP64 stays in the solve, and this part's
// narrow FP64 pipe does not bound the kernel.
// alpha is converted to float once per block into shared memory (a
// double-to-float conversion runs on the FP64 pipe).
constexpr int kBackmapThreads = 1024;
constexpr int64_t kBackmapMaxN = 16384;  // float alpha in shared memory: 64 KB

__global__ void __launch_bounds__(kBackmapThreads) backmap_kernel(const float* __restrict__ a,
                                                                  const float* __restrict__ b, int64_t P, int64_t bsz,
                                                                  int64_t n, const double* __restrict__ alpha,
                                                                  double scale, float lr, float* __restrict__ params,
                                                                  float* __restrict__ x_out) {
  extern __shared__ float alpha_f[];
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) alpha_f[j] = (float)alpha[j];
  __syncthreads();
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= P) return;
  Kahan k;
  for (int64_t j = lane; j < n; j += 32) k.add(ycol(a, b, bsz, row, j) * alpha_f[j]);
  float acc = k.s - k.c;
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    float xv = (float)(scale * (double)acc);
    if (x_out) x_out[row] = xv;
    if (params) params[row] -= lr * xv;
  }
}

// ---------------------------------------------------------------- complex parameters
// For complex parameters (the RBM family) the SR system is Hermitian:
// S = O_c^H O_c / B, F = O_c^H E_c / B (optimizer.py:94-114). With
// O_c = A + iC (A, C real, stored parameter-major [P][B] as o_re, o_im) the
// push-through identity gives x = O_c^H (T/B + lambda I)^-1 E_c / B with the
// B x B Hermitian T = O_c O_c^H = (A^T A + C^T C) + i (C^T A - A^T C) (samples
// as rows here). The 2B x 2B real Gram G of [A | C] holds these blocks:
// Tr = G11 + G22, Ti = G21 - G12. The Hermitian system T z = e is solved as
// the real symmetric positive (semi)definite embedding
//     [[Tr, -Ti], [Ti, Tr]] [zr; zi] = [er; ei],
// written over G in place: each thread owns the four entries (i, j),
// (i, n+j), (n+i, j), (n+i, n+j) of one (i, j), reads them and writes them.
__global__ void hermitian_embed_kernel(double* g, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const int64_t i = idx / n, j = idx % n, m = 2 * n;
  const double g11 = g[i * m + j], g12 = g[i * m + n + j];
  const double g21 = g[(n + i) * m + j], g22 = g[(n + i) * m + n + j];
  const double tr = g11 + g22, ti = g21 - g12;
  g[i * m + j] = tr;
  g[i * m + n + j] = -ti;
  g[(n + i) * m + j] = ti;
  g[(n + i) * m + n + j] = tr;
}

// x = scale * O_c^H z = scale * [(A zr + C zi) + i (A zi - C zr)] per parameter
// (A, C parameter-major rows); params (interleaved re, im) -= lr * x when
// params != NULL, x (interleaved) written to x_out when != NULL. Warp per
// row, float32 compensated sums as in backmap_kernel.
__global__ void __launch_bounds__(kBackmapThreads) complex_backmap_kernel(const float* __restrict__ a,
                                                                          const float* __restrict__ c, int64_t P,
                                                                          int64_t bsz, const double* __restrict__ z,
                                                                          double scale, float lr,
                                                                          float2* __restrict__ params,
                                                                          float2* __restrict__ x_out) {
  extern __shared__ float z_f[];
  for (int64_t j = threadIdx.x; j < 2 * bsz; j += blockDim.x) z_f[j] = (float)z[j];
  __syncthreads();
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= P) return;
  const float* ar = a + row * bsz;
  const float* cr = c + row * bsz;
  Kahan kr, ki;
  for (int64_t j = lane; j < bsz; j += 32) {
    const float av = ar[j], cv = cr[j], zr = z_f[j], zi = z_f[bsz + j];
    kr.add(av * zr + cv * zi);
    ki.add(av * zi - cv * zr);
  }
  float xr = kr.s - kr.c, xi = ki.s - ki.c;
  for (int o = 16; o > 0; o >>= 1) {
    xr += __shfl_xor_sync(0xffffffffu, xr, o);
    xi += __shfl_xor_sync(0xffffffffu, xi, o);
  }
  if (lane == 0) {
    float2 xv = make_float2((float)(scale * (double)xr), (float)(scale * (double)xi));
    if (x_out) x_out[row] = xv;
    if (params) {
      float2 p = params[row];
      params[row] = make_float2(p.x - lr * xv.x, p.y - lr * xv.y);
    }
  }
}

// Both back-maps stage up to 64 KB of float coefficients in shared memory.
static cudaError_t backmap_smem_attr() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(backmap_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(kBackmapMaxN * sizeof(float)));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(complex_backmap_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kBackmapMaxN * sizeof(float)));
  done = e == cudaSuccess;
  return e;
}

}  // namespace fk

using namespace fk;

extern "C" {

int fk_sr_hermitian_embed(double* gram, int64_t n_samples, void* stream) {
  FK_CHECK_ARG(gram && n_samples > 0, "fk_sr_hermitian_embed: bad arguments");
  int64_t nn = n_samples * n_samples;
  hermitian_embed_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(gram,
                                                                                                     n_samples);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_sr_complex_backmap(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples,
                          const double* z, double scale, float lr, float* params, float* x_out, void* stream) {
  FK_CHECK_ARG(o_re && o_im && z && n_params > 0 && n_samples > 0 && (params || x_out),
               "fk_sr_complex_backmap: bad arguments");
  FK_CHECK_ARG(2 * n_samples <= kBackmapMaxN, "fk_sr_complex_backmap: 2 n_samples = %lld exceeds %lld",
               (long long)(2 * n_samples), (long long)kBackmapMaxN);
  FK_CUDA(backmap_smem_attr());
  int64_t threads = n_params * 32;
  complex_backmap_kernel<<<(unsigned)((threads + kBackmapThreads - 1) / kBackmapThreads), kBackmapThreads,
                           (size_t)(2 * n_samples) * sizeof(float), static_cast<cudaStream_t>(stream)>>>(
      o_re, o_im, n_params, n_samples, z, scale, lr, reinterpret_cast<float2*>(params),
      reinterpret_cast<float2*>(x_out));
  FK_CUDA(launched());
  return FK_OK;
}

int fk_center_columns(float* y, int64_t rows, int64_t cols, float* mean, void* stream) {
  FK_CHECK_ARG(y && rows >= 0 && cols > 0, "fk_center_columns: bad arguments");
  if (rows == 0) return FK_OK;
  int64_t threads = rows * 32;
  center_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(y, rows, cols,
                                                                                                 mean);
  FK_CUDA(launched());
  return FK_OK;
}

int64_t fk_sr_gram_workspace_bytes(int64_t n_params, int64_t n_samples) {
  (void)n_params;
  (void)n_samples;
  return 0;
}

}  // extern "C"

// Adds the upper triangle (j >= i) of Y^T Y into gram (CUDA cores), Y =
// [a | b] (b == a when n == bsz), P parameter rows.
static int gram_cc_add(const float* a, const float* b, int64_t P, int64_t bsz, int64_t n, double* gram,
                       cudaStream_t s) {
  int64_t ntile = (n + kGT - 1) / kGT;
  int64_t tiles = ntile * (ntile + 1) / 2;
  // enough K splits to fill the GPU ~4 times over
  int64_t splits = (4 * 152 + tiles - 1) / tiles;
  int64_t kmax = (P + kGK - 1) / kGK;
  if (splits > kmax) splits = kmax;
  if (splits < 1) splits = 1;
  int64_t kper = (P + splits - 1) / splits;
  kper = (kper + kGK - 1) / kGK * kGK;
  dim3 grid((unsigned)tiles, 1, (unsigned)splits);
  gram_kernel<<<grid, 256, 0, s>>>(a, b, P, bsz, n, kper, gram);
  return check_cuda(launched(), "gram_kernel");
}

static int mirror(double* gram, int64_t n, cudaStream_t s) {
  mirror_kernel<<<(unsigned)((n * n + 255) / 256), 256, 0, s>>>(gram, n);
  return check_cuda(launched(), "mirror_kernel");
}

// The same on the tensor cores (n a multiple of 8, a and b 16-byte aligned).
static int gram_tc_add(const float* a_re, const float* a_im, int64_t n_params, int64_t bsz, int64_t n, double* gram,
                       cudaStream_t s) {
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, gram_tc::kSmem);
  });
  FK_CUDA(attr_err);
  GramTcArgs a;
  a.a = a_re;
  a.b = a_im;
  a.P = n_params;
  a.bsz = bsz;
  a.n = n;
  a.nti = (n + gram_tc::kM - 1) / gram_tc::kM;
  a.ntj = (n + gram_tc::kN - 1) / gram_tc::kN;
  int64_t tiles = 0;
  for (int64_t ti = 0; ti < a.nti; ++ti) tiles += a.ntj - ti / 2;
  // parameter ranges of at most 4096 parameters: the tensor core sums a
  // range in fp32 (relative error of a positive sum, e.g. a diagonal entry,
  // about 2e-5 at this length), the ranges are added in fp64; and at least
  // two items per SM
  int64_t splits = (2 * 152 + tiles - 1) / tiles;
  const int64_t min_splits = (n_params + 4095) / 4096;
  if (splits < min_splits) splits = min_splits;
  if (splits < 1) splits = 1;
  a.kper = ((n_params + splits - 1) / splits + gram_tc::kK - 1) / gram_tc::kK * gram_tc::kK;
  a.splits = (n_params + a.kper - 1) / a.kper;
  a.items = tiles * a.splits;
  a.t = gram;
  a.err = device_error_word();
  const int64_t grid = a.items < 152 ? a.items : 152;
  gram_tc_kernel<<<(unsigned)grid, gram_tc::kThreads, gram_tc::kSmem, s>>>(a);
  return check_cuda(launched(), "gram_tc_kernel");
}

static int split_run(const float* a, const float* b, int64_t ld, int64_t bsz, int64_t rows, int64_t n, void* split,
                     cudaStream_t s) {
  const int64_t groups = split_cols_pad(n) / 8;
  const int64_t total = split_rows_pad(rows) * groups;
  uint4* hi = static_cast<uint4*>(split);
  uint4* lo = hi + total;
  split_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(a, b, ld, bsz, rows, n, groups, total, hi, lo);
  return check_cuda(launched(), "split_kernel");
}

static int gram_split_add(const void* split, int64_t rows, int64_t n, double* gram, cudaStream_t s) {
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(gram_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    gram_split::kSmem);
  });
  FK_CUDA(attr_err);
  GramSplitArgs a;
  a.groups = split_cols_pad(n) / 8;
  a.kchunks = split_rows_pad(rows) / 32;
  a.hi = static_cast<const uint8_t*>(split);
  a.lo = a.hi + a.kchunks * a.groups * gram_split::kBlock;
  a.n = n;
  a.nti = (n + gram_tc::kM - 1) / gram_tc::kM;
  a.ntj = (n + gram_tc::kN - 1) / gram_tc::kN;
  int64_t tiles = 0;
  for (int64_t ti = 0; ti < a.nti; ++ti) tiles += a.ntj - ti / 2;
  // ranges of at most 4096 parameters (128 chunks: the FP32 sums in TMEM, as
  // in fk_sr_gram_tc), at least two items per SM
  int64_t splits = (2 * 152 + tiles - 1) / tiles;
  const int64_t min_splits = (a.kchunks + 127) / 128;
  if (splits < min_splits) splits = min_splits;
  if (splits > a.kchunks) splits = a.kchunks;
  a.kper = (a.kchunks + splits - 1) / splits;
  a.splits = (a.kchunks + a.kper - 1) / a.kper;
  a.items = tiles * a.splits;
  a.t = gram;
  a.err = device_error_word();
  const int64_t grid = a.items < 152 ? a.items : 152;
  gram_split_kernel<<<(unsigned)grid, gram_split::kThreads, gram_split::kSmem, s>>>(a);
  return check_cuda(launched(), "gram_split_kernel");
}

extern "C" {

int64_t fk_sr_gram_split_bytes(int64_t rows, int64_t n) {
  if (rows < 0 || n <= 0) return -1;
  return split_bytes(rows, n);
}

int fk_sr_gram_split(const float* a, const float* b, int64_t ld, int64_t bsz, int64_t rows, int64_t n, void* split,
                     int64_t split_bytes_given, void* stream) {
  FK_CHECK_ARG(a && split && rows >= 0 && n > 0 && bsz > 0 && ld >= (b ? bsz : n) && (b || bsz >= n),
               "fk_sr_gram_split: bad arguments");
  FK_CHECK_ARG(((uintptr_t)split % 16) == 0, "fk_sr_gram_split: split must be 16-byte aligned");
  FK_CHECK_ARG(split_bytes_given >= split_bytes(rows, n), "fk_sr_gram_split: split buffer %lld < %lld bytes",
               (long long)split_bytes_given, (long long)split_bytes(rows, n));
  if (rows == 0) return FK_OK;
  return split_run(a, b ? b : a, ld, bsz, rows, n, split, static_cast<cudaStream_t>(stream));
}

int fk_sr_center_split(float* a, float* b, int64_t ld, int64_t bsz, int64_t rows, int64_t n, int32_t write_back,
                       void* split, int64_t split_bytes_given, void* stream) {
  FK_CHECK_ARG(a && split && rows >= 0 && n > 0 && bsz > 0 && bsz <= n && (b || bsz == n) && ld >= bsz &&
                   ld >= n - bsz,
               "fk_sr_center_split: bad arguments");
  FK_CHECK_ARG(((uintptr_t)split % 16) == 0, "fk_sr_center_split: split must be 16-byte aligned");
  FK_CHECK_ARG(split_bytes_given >= split_bytes(rows, n), "fk_sr_center_split: split buffer %lld < %lld bytes",
               (long long)split_bytes_given, (long long)split_bytes(rows, n));
  if (rows == 0) return FK_OK;
  const int64_t groups = split_cols_pad(n) / 8;
  const int64_t kchunks = split_rows_pad(rows) / 32;
  uint4* hi = static_cast<uint4*>(split);
  uint4* lo = hi + kchunks * groups * 32;
  center_split_kernel<<<(unsigned)kchunks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      a, b ? b : a, ld, bsz, rows, n, groups, write_back, hi, lo);
  return check_cuda(launched(), "center_split_kernel");
}

int fk_sr_gram_split_accumulate(const void* split, int64_t rows, int64_t n, double* gram, void* stream) {
  FK_CHECK_ARG(split && gram && rows >= 0 && n > 0 && n <= 65536, "fk_sr_gram_split_accumulate: bad arguments");
  FK_CHECK_ARG(((uintptr_t)split % 16) == 0, "fk_sr_gram_split_accumulate: split must be 16-byte aligned");
  if (rows == 0) return FK_OK;
  return gram_split_add(split, rows, n, gram, static_cast<cudaStream_t>(stream));
}

int fk_sr_gram(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, double* gram,
               int64_t gram_elems, void* stream) {
  FK_CHECK_ARG(o_re && gram && n_params > 0 && n_samples > 0, "fk_sr_gram: bad arguments");
  int64_t n = o_im ? 2 * n_samples : n_samples;
  FK_CHECK_ARG(gram_elems >= n * n, "fk_sr_gram: gram buffer too small (%lld < %lld)", (long long)gram_elems,
               (long long)(n * n));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FK_CUDA(cudaMemsetAsync(gram, 0, (size_t)(n * n) * sizeof(double), s));
  int st = gram_cc_add(o_re, o_im ? o_im : o_re, n_params, n_samples, n, gram, s);
  return st != FK_OK ? st : mirror(gram, n, s);
}

int fk_sr_gram_tc(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, double* gram,
                  int64_t gram_elems, void* stream) {
  FK_CHECK_ARG(o_re && gram && n_params > 0 && n_samples > 0, "fk_sr_gram_tc: bad arguments");
  FK_CHECK_ARG(n_samples % 8 == 0, "fk_sr_gram_tc: n_samples must be a multiple of 8 (got %lld)",
               (long long)n_samples);
  FK_CHECK_ARG(((uintptr_t)o_re % 16) == 0 && (!o_im || ((uintptr_t)o_im % 16) == 0),
               "fk_sr_gram_tc: o_re / o_im must be 16-byte aligned");
  const int64_t n = o_im ? 2 * n_samples : n_samples;
  FK_CHECK_ARG(n <= 65536, "fk_sr_gram_tc: n = %lld exceeds 65536", (long long)n);
  FK_CHECK_ARG(gram_elems >= n * n, "fk_sr_gram_tc: gram buffer too small (%lld < %lld)", (long long)gram_elems,
               (long long)(n * n));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FK_CUDA(cudaMemsetAsync(gram, 0, (size_t)(n * n) * sizeof(double), s));
  int st = gram_tc_add(o_re, o_im ? o_im : o_re, n_params, n_samples, n, gram, s);
  return st != FK_OK ? st : mirror(gram, n, s);
}

int fk_sr_gram_accumulate(const float* y, int64_t rows, int64_t n, double* gram, int32_t tensor_cores,
                          void* stream) {
  FK_CHECK_ARG(y && gram && rows >= 0 && n > 0, "fk_sr_gram_accumulate: bad arguments");
  if (rows == 0) return FK_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!tensor_cores) return gram_cc_add(y, y, rows, n, n, gram, s);
  FK_CHECK_ARG(n % 8 == 0 && ((uintptr_t)y % 16) == 0 && n <= 65536,
               "fk_sr_gram_accumulate: the tensor cores need n a multiple of 8 and <= 65536 (got %lld) and y "
               "16-byte aligned",
               (long long)n);
  return gram_tc_add(y, y, rows, n, n, gram, s);
}

int fk_sr_gram_mirror(double* gram, int64_t n, void* stream) {
  FK_CHECK_ARG(gram && n > 0, "fk_sr_gram_mirror: bad arguments");
  return mirror(gram, n, static_cast<cudaStream_t>(stream));
}

int64_t fk_sr_solve_workspace_bytes(int64_t n) { return (3 * n + 8) * (int64_t)sizeof(double); }

int fk_sr_solve(const double* gram, int64_t n, double scale, double shift, const double* rhs, double tol,
                int32_t max_iter, double* x, double* stats, void* workspace, int64_t workspace_bytes,
                void* stream) {
  FK_CHECK_ARG(gram && rhs && x && n > 0 && max_iter > 0, "fk_sr_solve: bad arguments");
  FK_CHECK_ARG(workspace && workspace_bytes >= fk_sr_solve_workspace_bytes(n), "fk_sr_solve: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* r = static_cast<double*>(workspace);
  double* p = r + n;
  double* q = p + n;
  double* sc = q + n;
  cg_init_kernel<<<1, 1024, 0, st>>>(rhs, n, x, r, p, sc, tol);
  FK_CUDA(launched());
  const unsigned mv_blocks = (unsigned)((n * 32 + 255) / 256);
  const unsigned vec_blocks = (unsigned)((n + 255) / 256 < 152 ? (n + 255) / 256 : 152);
  // Every iteration is launched; once converged the kernels return at once
  // (no host synchronisation inside the solve).
  for (int it = 0; it < max_iter; ++it) {
    cg_matvec_kernel<<<mv_blocks, 256, 0, st>>>(gram, n, scale, shift, p, q, sc);
    cg_update_kernel<<<vec_blocks, 256, 0, st>>>(n, x, r, p, q, sc);
    cg_direction_kernel<<<vec_blocks, 256, 0, st>>>(n, r, p, sc, 0);
    cg_roll_kernel<<<1, 1, 0, st>>>(sc);
    FK_CUDA(launched(4));
  }
  if (stats) {
    // stats = {iterations, ||r||^2, tol^2 ||b||^2}
    FK_CUDA(cudaMemcpyAsync(stats, sc + 5, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 1, sc + 0, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 2, sc + 4, sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  return FK_OK;
}

int fk_sr_backmap(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, const double* alpha,
                  double scale, float lr, float* params, float* x_out, void* stream) {
  FK_CHECK_ARG(o_re && alpha && n_params > 0 && n_samples > 0 && (params || x_out), "fk_sr_backmap: bad arguments");
  int64_t n = o_im ? 2 * n_samples : n_samples;
  FK_CHECK_ARG(n <= kBackmapMaxN, "fk_sr_backmap: n = %lld exceeds %lld", (long long)n, (long long)kBackmapMaxN);
  FK_CUDA(backmap_smem_attr());
  int64_t threads = n_params * 32;
  backmap_kernel<<<(unsigned)((threads + kBackmapThreads - 1) / kBackmapThreads), kBackmapThreads,
                   (size_t)n * sizeof(float), static_cast<cudaStream_t>(stream)>>>(
      o_re, o_im ? o_im : o_re, n_params, n_samples, n, alpha, scale, lr, params, x_out);
  FK_CUDA(launched());
  return FK_OK;
}


}  // extern "C"

// ---------------------------------------------------------------- no-allocation solve
// Some hosts cannot hand this library a workspace: their device memory is
// owned by another allocator (a framework that reserves nearly all of the GPU
// at start-up, so a cudaMalloc would fail), or their policy forbids
// cudaMalloc/cudaFree on the solve path because those calls synchronise the
// device. fk_sr_solve_noalloc serves them with the scratch of the conjugate
// gradients (three vectors of length n plus eight scalars) in a file-scope
// device array of fixed size. The array exists once per device that loads the
// library and stays reserved until the process exits.
namespace fk {

constexpr int64_t kNoAllocMaxN = 8192;  // largest n: 196,672 bytes of scratch
static __device__ __align__(256) double g_sr_noalloc_scratch[3 * kNoAllocMaxN + 8];

// Device address of the scratch array on the current device, looked up once
// per device with that device current (the host-side name is not a device
// pointer and must never be handed to a kernel).
// std::call_once makes the per-device set-up safe when several host threads
// make their first call on a device at the same time. The address belongs to
// the device's current context: after cudaDeviceReset the library must be
// reloaded before this entry point is called again on that device.
constexpr int kNoAllocMaxDevices = 64;

static double* noalloc_scratch() {
  int dev = 0;
  if (check_cuda(cudaGetDevice(&dev), "cudaGetDevice") != FK_OK) return nullptr;
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("fk_sr_solve_noalloc: device index %d out of range", dev);
    return nullptr;
  }
  static std::once_flag once[kNoAllocMaxDevices];
  static double* cached[kNoAllocMaxDevices] = {nullptr};
  static cudaError_t lookup[kNoAllocMaxDevices];
  std::call_once(once[dev], [dev] {
    void* p = nullptr;
    lookup[dev] = cudaGetSymbolAddress(&p, g_sr_noalloc_scratch);
    if (lookup[dev] == cudaSuccess) cached[dev] = static_cast<double*>(p);
  });
  if (check_cuda(lookup[dev], "cudaGetSymbolAddress") != FK_OK) return nullptr;
  return cached[dev];
}

}  // namespace fk

extern "C" int fk_sr_solve_noalloc(const double* gram, int64_t n, double scale, double shift, const double* rhs,
                                   double tol, int32_t max_iter, double* x, double* stats, void* stream) {
  FK_CHECK_ARG(gram && rhs && x && n > 0 && max_iter > 0, "fk_sr_solve_noalloc: bad arguments");
  FK_CHECK_ARG(n <= fk::kNoAllocMaxN,
               "fk_sr_solve_noalloc: n = %lld exceeds the built-in scratch (n <= %lld); use fk_sr_solve with a "
               "workspace",
               (long long)n, (long long)fk::kNoAllocMaxN);
  double* ws = fk::noalloc_scratch();
  if (!ws) return FK_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* r = ws;
  double* p = r + n;
  double* q = p + n;
  double* sc = q + n;
  // cg_init rewrites x, r, p and every scalar before any of them is read, so
  // nothing left in the shared array by an earlier call is ever used.
  fk::cg_init_kernel<<<1, 1024, 0, st>>>(rhs, n, x, r, p, sc, tol);
  FK_CUDA(fk::launched());
  const unsigned mv_blocks = (unsigned)((n * 32 + 255) / 256);
  const unsigned vec_blocks = (unsigned)((n + 255) / 256 < 152 ? (n + 255) / 256 : 152);
  for (int it = 0; it < max_iter; ++it) {
    fk::cg_matvec_kernel<<<mv_blocks, 256, 0, st>>>(gram, n, scale, shift, p, q, sc);
    fk::cg_update_kernel<<<vec_blocks, 256, 0, st>>>(n, x, r, p, q, sc);
    fk::cg_direction_kernel<<<vec_blocks, 256, 0, st>>>(n, r, p, sc, 0);
    fk::cg_roll_kernel<<<1, 1, 0, st>>>(sc);
    FK_CUDA(fk::launched(4));
  }
  if (stats) {
    FK_CUDA(cudaMemcpyAsync(stats, sc + 5, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 1, sc + 0, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 2, sc + 4, sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  return FK_OK;
}
