// Adjoint of log psi through ConvNetAutoregressive2D (hand-written backward).
//
// Seeds w[b] = (w_re, w_im) weight Re and Im log psi of sample b. With
// log psi = sum_sites (Re_s - lse/2, Im_s) (abstract_machine.py:56-57) the
// head gradient per site is
//   dRe_j = w_re (delta_{j,s} - softmax(2 Re)_j),   dIm_j = w_im delta_{j,s}.
// The gradient then runs through the causal convs in reverse, one kernel
// family per op (thread = sample, CTA = tile x lattice row, like the forward):
//   head    : gL, gHp_last = (W_o^T gL) . [relu(Hp) > 0]
//   C^T     : gCat = sum_taps gHp[q - tap] W_c^T, masked by [Cat > 0];
//             X half -> gT at (r, c - s) via W_x^T and [T > 0];
//             Y half -> gVp at (r - 1, c) via W_y^T and [relu(Vp) > 0], plus the
//             stream gradient of V.
//   V^T/H^T : gradients of the conv inputs, plus the residual gradient of the
//             block input, masked by the previous conv's relu.
// Weight gradients are sum_q X[q + tap] (x) G[q] per tap, either summed over
// samples (block reduction + atomics) or kept per sample (param-major
// [num_params][batch], the rows of O_k). Weight normalisation is applied last:
// dv = e^g/|v| (dW - u (u.dW)), dg = e^g (u.dW) (deepar/layers/wrappers.py:123-134).
// Activations are read from the forward/sampler workspace (bf16 or fp32);
// gradients are fp32 throughout.
#include "fk_ar2d.cuh"

#include <type_traits>

#include <stdlib.h>
#include <string.h>

namespace FK_NS {

__device__ __forceinline__ void load_g(const float* t, int64_t tile, int P, int pix, int C, int m, int c0, int n,
                                       float* v) {
  load_row(blk<float>(t, tile, P, pix, C), m, c0, n, v);
}
__device__ __forceinline__ void store_g(float* t, int64_t tile, int P, int pix, int C, int m, int c0, int n,
                                        const float* v) {
  store_row(blk<float>(t, tile, P, pix, C), m, c0, n, v);
}

// acc[ci] += sum_n g[n] W[row0 + ci][n]  (W fp32 [K][N] row-major, rows
// 16-byte aligned: one vector load per four FMAs)
template <int CI, int N>
__device__ __forceinline__ void dot_rows(const float* __restrict__ W, int row0, const float* g, float* acc) {
#pragma unroll 4
  for (int ci = 0; ci < CI; ++ci) {
    const float4* w = reinterpret_cast<const float4*>(W + (int64_t)(row0 + ci) * N);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int n4 = 0; n4 < N / 4; ++n4) {
      float4 v = __ldg(w + n4);
      s0 += g[4 * n4] * v.x + g[4 * n4 + 2] * v.z;
      s1 += g[4 * n4 + 1] * v.y + g[4 * n4 + 3] * v.w;
    }
    acc[ci] += s0 + s1;
  }
}

struct HeadBwdArgs {
  const void* hlast;     // relu(Hp) of the final conv (act type)
  const float* wo;       // [F][4]
  const float* bo;       // [4]
  const int8_t* spins;
  const float2* seeds;   // [batch]
  int64_t batch;
  float* gL;             // [tiles][P][8ch] fp32 (4 used)
  void* ghp;             // [tiles][P][F] (gradient type)
  int updown;            // EqualUpDownSpins mask (from the spins)
};

template <int F, typename T, typename TG>
__global__ void __launch_bounds__(128) head_bwd_kernel(const __grid_constant__ HeadBwdArgs a, int H, int W) {
  const int P = H * W;
  const int64_t tile = blockIdx.x / H;
  const int r = blockIdx.x % H;
  const int m = threadIdx.x;
  const int64_t b = tile * kTile + m;
  float2 w = b < a.batch ? a.seeds[b] : make_float2(0.f, 0.f);
  // EqualUpDownSpins: +1 spins before the row's first site
  int n_up = 0;
  if (a.updown)
    for (int k = 0; k < r * W; ++k) n_up += spin_at(a.spins, a.batch, P, b, k) > 0.f ? 1 : 0;
  for (int c = 0; c < W; ++c) {
    const int pix = r * W + c;
    const int mk = a.updown ? ((2 * n_up >= P ? 1 : 0) | (2 * (pix - n_up) >= P ? 2 : 0)) : 0;
    float g[F];
    load_row(blk<T>(a.hlast, tile, P, pix, F), m, 0, F, g);
    float l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) l[j] = __ldg(a.bo + j);
#pragma unroll 8
    for (int k = 0; k < F; ++k) {
#pragma unroll
      for (int j = 0; j < 4; ++j) l[j] += g[k] * __ldg(a.wo + k * 4 + j);
    }
    // a masked outcome has probability 0 (layers/spins_invariants.py:13-22)
    float pi0 = (mk & 1) ? 0.f : ((mk & 2) ? 1.f : 1.f / (1.f + expf(2.f * (l[1] - l[0]))));
    float pi1 = 1.f - pi0;
    bool up = spin_at(a.spins, a.batch, P, b, pix) > 0.f;
    n_up += up ? 1 : 0;
    float gl[8] = {w.x * ((up ? 1.f : 0.f) - pi0), w.x * ((up ? 0.f : 1.f) - pi1), up ? w.y : 0.f,
                   up ? 0.f : w.y, 0.f, 0.f, 0.f, 0.f};
    store_g(a.gL, tile, P, pix, 8, m, 0, 8, gl);
    float gh[F];
#pragma unroll 8
    for (int k = 0; k < F; ++k) {
      float s = 0.f;
#pragma unroll
      for (int j = 0; j < 4; ++j) s += __ldg(a.wo + k * 4 + j) * gl[j];
      gh[k] = g[k] > 0.f ? s : 0.f;
    }
    store_row(blk<TG>(a.ghp, tile, P, pix, F), m, 0, F, gh);
  }
}

struct CBwdArgs {
  const float* ghp;      // gradient of Hp (masked), F
  const void* cat;       // saved Cat
  const void* t;         // saved T = relu(conv_h)
  const void* rv;        // saved relu(Vp)
  const float* gvpd;     // masked stream gradient of V_{i+1} (NULL on the final conv)
  const float* wc;       // [9F][F]
  const float* wx;       // [F][F/2]
  const float* wy;       // [F][F/2]
  int shift;             // 1 on the final conv (right shift)
  float* gcatm;          // out: masked Cat gradient, F
  float* gt;             // out: gradient of the h-conv pre-activation (masked), F
  float* gvp;            // out: gradient of Vp (masked), F
};

template <int F, typename T>
__global__ void __launch_bounds__(128) c_bwd_kernel(const __grid_constant__ CBwdArgs a, int H, int W) {
  constexpr int F2 = F / 2;
  const int P = H * W;
  const int64_t tile = blockIdx.x / H;
  const int r = blockIdx.x % H;
  const int m = threadIdx.x;
  for (int c = 0; c < W; ++c) {
    const int pix = r * W + c;
    float gcat[F];
#pragma unroll
    for (int k = 0; k < F; ++k) gcat[k] = 0.f;
    for (int t = 0; t < 9; ++t) {
      int rs = r + 2 - t / 3, cs = c + 2 - t % 3;
      if (rs >= H || cs >= W) continue;
      float g[F];
      load_g(a.ghp, tile, P, rs * W + cs, F, m, 0, F, g);
      dot_rows<F, F>(a.wc, t * F, g, gcat);
    }
    float cat[F];
    load_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F, cat);
#pragma unroll
    for (int k = 0; k < F; ++k) gcat[k] = cat[k] > 0.f ? gcat[k] : 0.f;
    store_g(a.gcatm, tile, P, pix, F, m, 0, F, gcat);
    // X half -> T at (r, c - s)
    const int cx = c - a.shift;
    if (cx >= 0) {
      float tt[F], gt[F];
      load_row(blk<T>(a.t, tile, P, r * W + cx, F), m, 0, F, tt);
#pragma unroll
      for (int k = 0; k < F; ++k) gt[k] = 0.f;
      dot_rows<F, F2>(a.wx, 0, gcat, gt);
#pragma unroll
      for (int k = 0; k < F; ++k) gt[k] = tt[k] > 0.f ? gt[k] : 0.f;
      store_g(a.gt, tile, P, r * W + cx, F, m, 0, F, gt);
    }
    if (a.shift && c == W - 1) {
      float z[F];
#pragma unroll
      for (int k = 0; k < F; ++k) z[k] = 0.f;
      store_g(a.gt, tile, P, pix, F, m, 0, F, z);
    }
    // Y half -> Vp at (r - 1, c)
    if (r >= 1) {
      const int py = pix - W;
      float rv[F], gv[F];
      load_row(blk<T>(a.rv, tile, P, py, F), m, 0, F, rv);
      if (a.gvpd) {
        load_g(a.gvpd, tile, P, py, F, m, 0, F, gv);
      } else {
#pragma unroll
        for (int k = 0; k < F; ++k) gv[k] = 0.f;
      }
      float gr[F];
#pragma unroll
      for (int k = 0; k < F; ++k) gr[k] = 0.f;
      dot_rows<F, F2>(a.wy, 0, gcat + F2, gr);
#pragma unroll
      for (int k = 0; k < F; ++k) gv[k] += rv[k] > 0.f ? gr[k] : 0.f;
      store_g(a.gvp, tile, P, py, F, m, 0, F, gv);
    }
    if (r == H - 1) {
      float gv[F];
      if (a.gvpd) {
        load_g(a.gvpd, tile, P, pix, F, m, 0, F, gv);
      } else {
#pragma unroll
        for (int k = 0; k < F; ++k) gv[k] = 0.f;
      }
      store_g(a.gvp, tile, P, pix, F, m, 0, F, gv);
    }
  }
}

struct VHBwdArgs {
  const float* gvp;      // gradient of Vp (masked), F
  const float* gt;       // gradient of the h-conv pre-activation (masked), F
  const float* wv;       // [9F][F]
  const float* wh;       // [3F][F]
  const float* res_v;    // masked stream gradient of the block's second conv (residual path) or NULL
  const float* res_h;
  const void* vprev;     // saved V_{i-1} (relu mask)
  const void* hprev;     // saved H_{i-1}
  float* gvpd_prev;      // out: masked stream gradient of V_{i-1}
  float* ghp_prev;       // out: masked gradient of Hp_{i-1}
};

template <int F, typename T>
__global__ void __launch_bounds__(128) vh_bwd_kernel(const __grid_constant__ VHBwdArgs a, int H, int W) {
  const int P = H * W;
  const int64_t tile = blockIdx.x / H;
  const int r = blockIdx.x % H;
  const int m = threadIdx.x;
  for (int c = 0; c < W; ++c) {
    const int pix = r * W + c;
    float gv[F], gh[F];
#pragma unroll
    for (int k = 0; k < F; ++k) {
      gv[k] = 0.f;
      gh[k] = 0.f;
    }
    for (int t = 0; t < 9; ++t) {  // V taps: (dr, dc) = (t/3 - 2, t%3 - 1)
      int rs = r + 2 - t / 3, cs = c + 1 - t % 3;
      if (rs >= H || cs < 0 || cs >= W) continue;
      float g[F];
      load_g(a.gvp, tile, P, rs * W + cs, F, m, 0, F, g);
      dot_rows<F, F>(a.wv, t * F, g, gv);
    }
    for (int t = 0; t < 3; ++t) {  // H taps: dc = t - 2
      int cs = c + 2 - t;
      if (cs >= W) continue;
      float g[F];
      load_g(a.gt, tile, P, r * W + cs, F, m, 0, F, g);
      dot_rows<F, F>(a.wh, t * F, g, gh);
    }
    if (a.res_v) {
      float x[F];
      load_g(a.res_v, tile, P, pix, F, m, 0, F, x);
#pragma unroll
      for (int k = 0; k < F; ++k) gv[k] += x[k];
      load_g(a.res_h, tile, P, pix, F, m, 0, F, x);
#pragma unroll
      for (int k = 0; k < F; ++k) gh[k] += x[k];
    }
    float v[F], h[F];
    load_row(blk<T>(a.vprev, tile, P, pix, F), m, 0, F, v);
    load_row(blk<T>(a.hprev, tile, P, pix, F), m, 0, F, h);
#pragma unroll
    for (int k = 0; k < F; ++k) {
      gv[k] = v[k] > 0.f ? gv[k] : 0.f;
      gh[k] = h[k] > 0.f ? gh[k] : 0.f;
    }
    store_g(a.gvpd_prev, tile, P, pix, F, m, 0, F, gv);
    store_g(a.ghp_prev, tile, P, pix, F, m, 0, F, gh);
  }
}

// ---------------------------------------------------------------- weight gradients
struct WgArgs {
  int ntaps;
  int dr[9], dc[9];
  const void* X;        // activations (act type), cin channels; NULL -> spins
  const int8_t* spins;
  int cin;
  const void* G;        // blocked (gradient type), gC channels; uses [g0, g0 + N)
  int gC, g0, N;
  float* dW;            // summed raw kernel gradient [ntaps*cin][N]
  float* dB;            // summed bias gradient [N]
  float* O;             // per-sample: O[(o_kernel + k*N + n) * o_ld + o_col + b]
  int64_t o_kernel, o_bias;
  int64_t o_ld, o_col;
  int64_t batch;
  int items;            // work items = ntaps * ceil(cin/8) * ceil(N/8)
  int items_per_cta;
  // Fixed-order mode: each tile writes its sums to part[tile][ntaps*cin*N + N]
  // (kernel then bias) instead of adding them atomically; the tiles are then
  // summed in order (wgrad_part_reduce_kernel).
  float* part;
};

constexpr int kItemsPerCta = 4;

template <typename T, typename TG>
__global__ void __launch_bounds__(128) wgrad_kernel(const __grid_constant__ WgArgs a, int H, int W) {
  __shared__ float red[4][64];
  const int P = H * W;
  const int64_t tile = blockIdx.x;
  const int m = threadIdx.x;
  const int64_t b = tile * kTile + m;
  const int kchunks = (a.cin + 7) / 8;
  const int nchunks = (a.N + 7) / 8;
  for (int it = blockIdx.y * a.items_per_cta; it < a.items && it < (int)(blockIdx.y + 1) * a.items_per_cta; ++it) {
    const int t = it / (kchunks * nchunks);
    const int kc = (it / nchunks) % kchunks;
    const int nc = it % nchunks;
    const bool with_bias = (t == 0 && kc == 0);
    float acc[8][8];
    float gb[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      gb[i] = 0.f;
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    }
    for (int r = 0; r < H; ++r) {
      for (int c = 0; c < W; ++c) {
        float g[8];
        load_row(blk<TG>(a.G, tile, P, r * W + c, a.gC), m, a.g0 + nc * 8, 8, g);
        if (with_bias) {
#pragma unroll
          for (int j = 0; j < 8; ++j) gb[j] += g[j];
        }
        int rs = r + a.dr[t], cs = c + a.dc[t];
        if (rs < 0 || rs >= H || cs < 0 || cs >= W) continue;
        float x[8];
        if (a.X) {
          load_row(blk<T>(a.X, tile, P, rs * W + cs, a.cin), m, kc * 8, 8, x);
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) x[i] = 0.f;
          x[0] = spin_at(a.spins, a.batch, P, b, rs * W + cs);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[i][j] += x[i] * g[j];
        }
      }
    }
    const int kmax = a.cin - kc * 8 < 8 ? a.cin - kc * 8 : 8;
    const int nmax = a.N - nc * 8 < 8 ? a.N - nc * 8 : 8;
    if (a.O) {
      if (b < a.batch) {
        for (int i = 0; i < kmax; ++i) {
          int64_t row = (int64_t)(t * a.cin + kc * 8 + i) * a.N + nc * 8;
          for (int j = 0; j < nmax; ++j) a.O[(a.o_kernel + row + j) * a.o_ld + a.o_col + b] = acc[i][j];
        }
        if (with_bias)
          for (int j = 0; j < nmax; ++j) a.O[(a.o_bias + nc * 8 + j) * a.o_ld + a.o_col + b] = gb[j];
      }
    } else {
      // block reduction over the 128 samples, then one atomic per element
      const int lane = m & 31, warp = m >> 5;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float v = acc[i][j];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          acc[i][j] = v;
        }
      }
      if (lane == 0) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) red[warp][i * 8 + j] = acc[i][j];
      }
      __syncthreads();
      if (m < 64) {
        int i = m / 8, j = m % 8;
        float v = red[0][m] + red[1][m] + red[2][m] + red[3][m];
        if (i < kmax && j < nmax) {
          const int64_t e = (int64_t)(t * a.cin + kc * 8 + i) * a.N + nc * 8 + j;
          if (a.part)
            a.part[tile * ((int64_t)a.ntaps * a.cin * a.N + a.N) + e] = v;
          else
            atomicAdd(&a.dW[e], v);
        }
      }
      __syncthreads();
      if (with_bias) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float v = gb[j];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          gb[j] = v;
        }
        if (lane == 0)
          for (int j = 0; j < 8; ++j) red[warp][j] = gb[j];
        __syncthreads();
        if (m < nmax) {
          const float v = red[0][m] + red[1][m] + red[2][m] + red[3][m];
          if (a.part)
            a.part[tile * ((int64_t)a.ntaps * a.cin * a.N + a.N) + (int64_t)a.ntaps * a.cin * a.N + nc * 8 + m] = v;
          else
            atomicAdd(&a.dB[nc * 8 + m], v);
        }
        __syncthreads();
      }
    }
  }
}

// Weight-normalisation chain rule, all weight-normalised convs in one launch
// (blockIdx.y = conv). Summed: one thread per output channel. Per-sample: one
// thread per (output channel, sample) on the O rows.
struct WnArgs {
  const float* params;
  float* grad;     // summed: flat gradient (kernel slots hold dW on entry)
  float* O;        // per-sample rows (kernel slots hold dW on entry)
  int64_t batch;
  ConvDesc conv[kMaxConvs];
  int64_t o_row[kMaxConvs];  // per-sample: row of O holding the conv's first kernel element
};

__global__ void wn_kernel(const __grid_constant__ WnArgs a) {
  const ConvDesc& cd = a.conv[blockIdx.y];
  const int N = cd.cout, K = cd.K;
  const int64_t p_kernel = cd.p_kernel, p_g = cd.p_g;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t cols = a.O ? (int64_t)N * a.batch : N;
  if (idx >= cols) return;
  // per-sample: consecutive threads take consecutive samples of one channel,
  // so that every access to the parameter-major O rows is coalesced
  int n = a.O ? (int)(idx / a.batch) : (int)idx;
  int64_t b = a.O ? idx % a.batch : 0;
  const float* v = a.params + p_kernel;
  float sq = 0.f;
  for (int k = 0; k < K; ++k) sq += v[(int64_t)k * N + n] * v[(int64_t)k * N + n];
  float inv = rsqrtf(fmaxf(sq, 1e-12f));
  float eg = expf(a.params[p_g + n]);
  const int64_t o_row = a.o_row[blockIdx.y];
  auto at = [&](int k) -> float& {
    return a.O ? a.O[(o_row + (int64_t)k * N + n) * a.batch + b] : a.grad[p_kernel + (int64_t)k * N + n];
  };
  float dot = 0.f;
  for (int k = 0; k < K; ++k) dot += at(k) * v[(int64_t)k * N + n] * inv;
  for (int k = 0; k < K; ++k) {
    float u = v[(int64_t)k * N + n] * inv;
    at(k) = eg * inv * (at(k) - u * dot);
  }
  if (a.O)
    a.O[(o_row + (p_g - p_kernel) + n) * a.batch + b] = eg * dot;
  else
    a.grad[p_g + n] = eg * dot;
}

// Every conv but the head (not weight-normalised).
static int launch_wn(const NetLayout& L, const float* params, float* grad, float* O, int64_t batch, cudaStream_t s) {
  WnArgs* a = new WnArgs;
  a->params = params;
  a->grad = grad;
  a->O = O;
  a->batch = batch;
  int maxc = 0;
  for (int k = 0; k < L.n_convs - 1; ++k) {
    a->conv[k] = L.conv[k];
    a->o_row[k] = L.conv[k].p_kernel;
    maxc = maxc > L.conv[k].cout ? maxc : L.conv[k].cout;
  }
  const int64_t cols = O ? (int64_t)maxc * batch : maxc;
  dim3 grid((unsigned)((cols + 127) / 128), (unsigned)(L.n_convs - 1));
  wn_kernel<<<grid, 128, 0, s>>>(*a);
  delete a;
  return check_cuda(launched(), "wn_kernel");
}

// ---------------------------------------------------------------- SR Gram sink
// Per-sample rows one conv at a time, for the SR Gram without the whole
// [num_params][B] arrays: each conv's rows (kernel, bias, weight-norm gain: a
// contiguous parameter range) go to the next free rows of a buffer whose rows
// hold the columns of every pass ([0, B): seeds (1, 0), [B, 2B): seeds
// (0, 1)). When the next step's convs do not fit, and after the last step,
// the buffered convs get the weight-norm chain rule, every row is centred
// within each pass's columns, and Y^T Y of the buffer is added into the Gram.
struct RowSink {
  const NetLayout* L;
  const float* params;
  float* buf;
  int64_t cap;   // buffer rows
  int64_t used;
  int64_t ld;    // row length: passes x B
  int64_t col;   // first column of the pass being written
  int groups;    // passes
  int tensor_cores;
  void* split;   // tensor cores: the buffer's rows as split operands (fk_sr_gram_split)
  int64_t split_bytes;
  double* gram;
  int n;         // buffered convs
  int conv[kMaxConvs];
  int64_t row[kMaxConvs];
  int64_t at[kMaxConvs];  // buffer row of each conv, -1: not buffered
};

static int64_t conv_rows(const ConvDesc& cd) {
  return (cd.p_g >= 0 ? cd.p_g : cd.p_bias) + cd.cout - cd.p_kernel;
}

static int sink_flush(RowSink& k, cudaStream_t s) {
  if (k.used == 0) return FK_OK;
  const NetLayout& L = *k.L;
  if (L.wn) {
    WnArgs* a = new WnArgs;
    a->params = k.params;
    a->grad = nullptr;
    a->O = k.buf;
    a->batch = k.ld;
    int nw = 0, maxc = 0;
    for (int i = 0; i < k.n; ++i) {
      const ConvDesc& cd = L.conv[k.conv[i]];
      if (cd.p_g < 0) continue;
      a->conv[nw] = cd;
      a->o_row[nw++] = k.row[i];
      maxc = maxc > cd.cout ? maxc : cd.cout;
    }
    if (nw > 0) {
      dim3 grid((unsigned)(((int64_t)maxc * k.ld + 127) / 128), (unsigned)nw);
      wn_kernel<<<grid, 128, 0, s>>>(*a);
    }
    delete a;
    if (nw > 0) FK_CUDA(launched());
  }
  int st;
  if (k.tensor_cores) {
    // the two passes' column groups [0, B) and [B, 2B) centred and split in one pass
    st = fk_sr_center_split(k.buf, k.buf + k.ld / 2, k.ld, k.ld / 2, k.used, k.ld, 0, k.split, k.split_bytes, s);
    if (st == FK_OK) st = fk_sr_gram_split_accumulate(k.split, k.used, k.ld, k.gram, s);
  } else {
    st = fk_center_columns(k.buf, k.used * k.groups, k.ld / k.groups, nullptr, s);
    if (st == FK_OK) st = fk_sr_gram_accumulate(k.buf, k.used, k.ld, k.gram, 0, s);
  }
  for (int i = 0; i < k.n; ++i) k.at[k.conv[i]] = -1;
  k.used = 0;
  k.n = 0;
  return st;
}

// Buffer rows for the convs cs[0..n) not yet buffered, flushing first when
// they do not all fit.
static int sink_reserve(RowSink& k, const int* cs, int n, cudaStream_t s) {
  int64_t need = 0;
  for (int i = 0; i < n; ++i)
    if (k.at[cs[i]] < 0) need += conv_rows(k.L->conv[cs[i]]);
  FK_CHECK_ARG(need <= k.cap, "fk_ar2d_sr_gram: row buffer of %lld rows < %lld rows of one step", (long long)k.cap,
               (long long)need);
  if (k.used + need > k.cap) {
    int st = sink_flush(k, s);
    if (st != FK_OK) return st;
  }
  for (int i = 0; i < n; ++i) {
    if (k.at[cs[i]] >= 0) continue;
    k.at[cs[i]] = k.used;
    k.conv[k.n] = cs[i];
    k.row[k.n++] = k.used;
    k.used += conv_rows(k.L->conv[cs[i]]);
  }
  return FK_OK;
}

// Buffer row of conv `ci`.
static int sink_place(RowSink& k, int ci, int64_t* r0, cudaStream_t s) {
  if (k.at[ci] < 0) {
    int st = sink_reserve(k, &ci, 1, s);
    if (st != FK_OK) return st;
  }
  *r0 = k.at[ci];
  return FK_OK;
}

// Floats of a row buffer holding `rows` rows of n floats, and with the
// tensor cores also their split operands (after the rows, 256-byte aligned).
static int64_t sink_floats(int64_t rows, int64_t n, bool tc) {
  const int64_t f = (rows * n + 63) / 64 * 64;
  return tc ? f + fk_sr_gram_split_bytes(rows, n) / 4 : f;
}

// The convs whose per-sample rows step i of the backward writes (all five
// convs of causal conv i); the head's are written before step n_cc - 1.
static void step_convs(int i, int cs[5]) {
  cs[0] = conv_index(i, kConvC);
  cs[1] = conv_index(i, kConvX);
  cs[2] = conv_index(i, kConvY);
  cs[3] = conv_index(i, kConvH);
  cs[4] = conv_index(i, kConvV);
}

// Rows the buffer needs at least: the largest step (or the head).
static int64_t sink_min_rows(const NetLayout& L) {
  int64_t m = conv_rows(L.conv[L.n_convs - 1]);
  for (int i = 0; i < L.n_cc; ++i) {
    int cs[5];
    step_convs(i, cs);
    int64_t r = 0;
    for (int k = 0; k < 5; ++k) r += conv_rows(L.conv[cs[k]]);
    m = r > m ? r : m;
  }
  return m;
}

// The head and the steps n_cc - 1 .. 0 of one pass, or of two passes over the
// same activations (seeds0 / G0 and seeds1 / G1, their per-sample rows in
// columns [0, B) and [B, 2B) of the sink's buffer). With a sink, the convs of
// a step get their buffer rows before either pass writes them, so that no
// flush falls between the passes.
template <typename GT, typename HeadFn, typename StepFn>
static int run_passes(const NetLayout& L, int64_t batch, RowSink* sink, const float* seeds0, const GT& G0,
                      const float* seeds1, const GT* G1, HeadFn& head, StepFn& step, cudaStream_t s) {
  const int np = G1 ? 2 : 1;
  const float* sd[2] = {seeds0, seeds1};
  const GT* gs[2] = {&G0, G1};
  int st;
  if (sink) {
    const int io = L.n_convs - 1;
    if ((st = sink_reserve(*sink, &io, 1, s)) != FK_OK) return st;
  }
  for (int p = 0; p < np; ++p) {
    if (sink) sink->col = p * batch;
    if ((st = head(sd[p], *gs[p])) != FK_OK) return st;
  }
  for (int i = L.n_cc - 1; i >= 0; --i) {
    if (sink) {
      int cs[5];
      step_convs(i, cs);
      if ((st = sink_reserve(*sink, cs, 5, s)) != FK_OK) return st;
    }
    for (int p = 0; p < np; ++p) {
      if (sink) sink->col = p * batch;
      if ((st = step(i, *gs[p])) != FK_OK) return st;
    }
  }
  return FK_OK;
}

// ---------------------------------------------------------------- driver
constexpr int kGradRing = 3;

struct BwdTensors {
  float* gvpd[40];
  float* ghp[40];
  float* gcatm;
  float* gt;
  float* gvp;
  float* gl;
  int64_t bytes;
};

static int64_t bwd_layout(const NetLayout& L, int64_t batch, char* base, BwdTensors* T) {
  int64_t tiles = (batch + kTile - 1) / kTile;
  int64_t tb = tiles * L.P * (int64_t)kTile * L.F * 4;
  int64_t off = 0;
  auto take = [&](int64_t bytes) -> float* {
    float* p = base ? reinterpret_cast<float*>(base + off) : nullptr;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  BwdTensors tmp;
  BwdTensors* t = T ? T : &tmp;
  memset(t, 0, sizeof(*t));
  // Step i of the backward reads the gradients of causal convs i and i + 1
  // and writes those of i - 1: three buffers per stream, indexed i mod 3.
  for (int i = 0; i < L.n_cc; ++i) {
    t->gvpd[i] = i < kGradRing ? take(tb) : t->gvpd[i % kGradRing];
    t->ghp[i] = i < kGradRing ? take(tb) : t->ghp[i % kGradRing];
  }
  t->gcatm = take(tb);
  t->gt = take(tb);
  t->gvp = take(tb);
  t->gl = take(tiles * L.P * (int64_t)kTile * 8 * 4);
  t->bytes = off;
  return off;
}

static const float* w32(const NetLayout& L, const void* packed, int idx) {
  return reinterpret_cast<const float*>(static_cast<const char*>(packed) + L.conv[idx].w32_off);
}

static void tap_list(int kind, WgArgs& w) {
  if (kind == kConvV) {
    w.ntaps = 9;
    for (int t = 0; t < 9; ++t) {
      w.dr[t] = t / 3 - 2;
      w.dc[t] = t % 3 - 1;
    }
  } else if (kind == kConvH) {
    w.ntaps = 3;
    for (int t = 0; t < 3; ++t) {
      w.dr[t] = 0;
      w.dc[t] = t - 2;
    }
  } else {
    w.ntaps = 9;
    for (int t = 0; t < 9; ++t) {
      w.dr[t] = t / 3 - 2;
      w.dc[t] = t % 3 - 2;
    }
  }
}

// Sums the per-tile partials of the fixed-order mode in tile order.
__global__ void wgrad_part_reduce_kernel(const float* part, int64_t tiles, int kn, int n, float* dW, float* dB) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kn + n) return;
  float s = 0.f;
  for (int64_t t = 0; t < tiles; ++t) s += part[t * (kn + n) + e];
  if (e < kn)
    dW[e] = s;
  else
    dB[e - kn] = s;
}

// Per-sample weight gradients of the tensor-core adjoint's 32-channel convs on
// the tensor cores (wgrad_rows_tc_kernel); FK_AR2D_ROWS=cuda keeps them on the
// CUDA cores (wgrad_kernel on the same 16-bit gradients, for comparisons).
static bool rows_on_tensor_cores() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("FK_AR2D_ROWS");
    v = (e && strcmp(e, "cuda") == 0) ? 0 : 1;
  }
  return v == 1;
}

// Where the per-sample rows of conv cd go: the [num_params][batch] array O,
// or the sink's buffer.
struct RowsTarget {
  float* O;
  int64_t o_kernel, o_bias, o_ld, o_col;
};

static int rows_target(const NetLayout& L, const ConvDesc& cd, float* O, int64_t batch, cudaStream_t s,
                       RowSink* sink, RowsTarget* t) {
  if (sink) {
    int64_t r0 = 0;
    const int st = sink_place(*sink, (int)(&cd - L.conv), &r0, s);
    if (st != FK_OK) return st;
    *t = RowsTarget{sink->buf, r0, r0 + (cd.p_bias - cd.p_kernel), sink->ld, sink->col};
  } else {
    *t = RowsTarget{O, cd.p_kernel, cd.p_bias, batch, 0};
  }
  return FK_OK;
}

template <typename T, typename TG = float>
static int launch_wgrad(const NetLayout& L, WgArgs& w, const ConvDesc& cd, float* grad, float* O, int64_t batch,
                        cudaStream_t s, RowSink* sink = nullptr) {
  int64_t tiles = (batch + kTile - 1) / kTile;
  w.batch = batch;
  w.items = w.ntaps * ((w.cin + 7) / 8) * ((w.N + 7) / 8);
#ifndef FK_TC_FP16
  // per-sample rows of the BF16 path's 64-channel convs (CUDA-core adjoint,
  // float gradients): on the tensor cores, the gradients rounded to bf16
  if (O && std::is_same<T, tc16>::value && std::is_same<TG, float>::value && w.X && w.cin == 64 &&
      (w.N == 32 || w.N == 64) && rows_on_tensor_cores() && wgrad_rows_tc_supported(L.H, L.W, w.N)) {
    RowsTarget tg;
    const int st = rows_target(L, cd, O, batch, s, sink, &tg);
    if (st != FK_OK) return st;
    WgRowsArgs r;
    memset(&r, 0, sizeof(r));
    r.X = w.X;
    r.G = w.G;
    r.cin = 64;
    r.g_float = 1;
    r.gC = w.gC;
    r.g0 = w.g0;
    r.N = w.N;
    r.ntaps = w.ntaps;
    for (int t = 0; t < w.ntaps; ++t) {
      r.dr[t] = w.dr[t];
      r.dc[t] = w.dc[t];
    }
    r.O = tg.O;
    r.o_kernel = tg.o_kernel;
    r.o_bias = tg.o_bias;
    r.o_ld = tg.o_ld;
    r.o_col = tg.o_col;
    r.batch = batch;
    return launch_wgrad_rows_tc(r, L.H, L.W, device_error_word(), s);
  }
#endif
  if (O) {
    RowsTarget t;
    const int st = rows_target(L, cd, O, batch, s, sink, &t);
    if (st != FK_OK) return st;
    w.O = t.O;
    w.o_kernel = t.o_kernel;
    w.o_bias = t.o_bias;
    w.o_ld = t.o_ld;
    w.o_col = t.o_col;
  } else {
    w.dW = grad + cd.p_kernel;
    w.dB = grad + cd.p_bias;
  }
  // per-sample rows: one item per CTA (the CTA count, not the arithmetic,
  // bounds that mode); summed: kItemsPerCta
  w.items_per_cta = O ? 1 : kItemsPerCta;
  dim3 grid((unsigned)tiles, (unsigned)((w.items + w.items_per_cta - 1) / w.items_per_cta));
  wgrad_kernel<T, TG><<<grid, 128, 0, s>>>(w, L.H, L.W);
  if (!w.part || O) return check_cuda(launched(), "wgrad_kernel");
  FK_CUDA(launched());
  const int kn = w.ntaps * w.cin * w.N;
  wgrad_part_reduce_kernel<<<(kn + w.N + 127) / 128, 128, 0, s>>>(w.part, tiles, kn, w.N, w.dW, w.dB);
  return check_cuda(launched(), "wgrad_part_reduce_kernel");
}

template <int F, typename T>
static int backward_impl(const NetLayout& L, const void* packed, const float* params, const int8_t* spins,
                         int64_t batch, const float* seeds, const Tensors& A, const BwdTensors& G0, float* grad,
                         float* O, cudaStream_t s, RowSink* sink = nullptr, const float* seeds1 = nullptr,
                         const BwdTensors* G1 = nullptr) {
  const int64_t tiles = (batch + kTile - 1) / kTile;
  const unsigned rows = (unsigned)(tiles * L.H);
  const int last = L.n_cc - 1;
  // Per-sample rows are written exactly once per (parameter, sample); the
  // summed gradient accumulates with atomics and starts from zero.
  if (!O) FK_CUDA(cudaMemsetAsync(grad, 0, (size_t)L.num_params * sizeof(float), s));
  // head and step i of one pass (seeds, gradient tensors)
  auto head = [&](const float* seeds, const BwdTensors& G) -> int {
    HeadBwdArgs h;
    const int io = L.n_convs - 1;
    h.hlast = A.h[last];
    h.wo = w32(L, packed, io);
    h.bo = reinterpret_cast<const float*>(static_cast<const char*>(packed) + L.conv[io].b_off);
    h.spins = spins;
    h.seeds = reinterpret_cast<const float2*>(seeds);
    h.batch = batch;
    h.gL = G.gl;
    h.ghp = G.ghp[last];
    h.updown = L.updown;
    head_bwd_kernel<F, T, float><<<rows, 128, 0, s>>>(h, L.H, L.W);
    FK_CUDA(launched());
    WgArgs w;
    memset(&w, 0, sizeof(w));
    w.ntaps = 1;
    w.X = A.h[last];
    w.cin = F;
    w.G = G.gl;
    w.gC = 8;
    w.g0 = 0;
    w.N = 4;
    w.spins = spins;
    return launch_wgrad<T>(L, w, L.conv[io], grad, O, batch, s, sink);
  };
  auto step = [&](int i, const BwdTensors& G) -> int {
    int st;
    const ConvDesc& cv = L.conv[conv_index(i, kConvV)];
    const ConvDesc& ch = L.conv[conv_index(i, kConvH)];
    const ConvDesc& cx = L.conv[conv_index(i, kConvX)];
    const ConvDesc& cy = L.conv[conv_index(i, kConvY)];
    const ConvDesc& cc = L.conv[conv_index(i, kConvC)];
    CBwdArgs c;
    c.ghp = G.ghp[i];
    c.cat = A.cat[i];
    c.t = A.t[i];
    c.rv = A.rv[i];
    c.gvpd = (i == last) ? nullptr : G.gvpd[i];
    c.wc = w32(L, packed, conv_index(i, kConvC));
    c.wx = w32(L, packed, conv_index(i, kConvX));
    c.wy = w32(L, packed, conv_index(i, kConvY));
    c.shift = (i == last) ? 1 : 0;
    c.gcatm = G.gcatm;
    c.gt = G.gt;
    c.gvp = G.gvp;
    c_bwd_kernel<F, T><<<rows, 128, 0, s>>>(c, L.H, L.W);
    FK_CUDA(launched());
    // weight gradients of the five convs of causal conv i
    WgArgs w;
    memset(&w, 0, sizeof(w));
    w.spins = spins;
    tap_list(kConvC, w);
    w.X = A.cat[i];
    w.cin = F;
    w.G = G.ghp[i];
    w.gC = F;
    w.N = F;
    if ((st = launch_wgrad<T>(L, w, cc, grad, O, batch, s, sink)) != FK_OK) return st;
    memset(&w, 0, sizeof(w));
    w.spins = spins;
    w.ntaps = 1;
    w.dr[0] = 0;
    w.dc[0] = (i == last) ? -1 : 0;
    w.X = A.t[i];
    w.cin = F;
    w.G = G.gcatm;
    w.gC = F;
    w.g0 = 0;
    w.N = F / 2;
    if ((st = launch_wgrad<T>(L, w, cx, grad, O, batch, s, sink)) != FK_OK) return st;
    w.dr[0] = -1;
    w.dc[0] = 0;
    w.X = A.rv[i];
    w.g0 = F / 2;
    if ((st = launch_wgrad<T>(L, w, cy, grad, O, batch, s, sink)) != FK_OK) return st;
    memset(&w, 0, sizeof(w));
    w.spins = spins;
    tap_list(kConvH, w);
    w.X = i == 0 ? nullptr : A.h[i - 1];
    w.cin = i == 0 ? 1 : F;
    w.G = G.gt;
    w.gC = F;
    w.N = F;
    if ((st = launch_wgrad<T>(L, w, ch, grad, O, batch, s, sink)) != FK_OK) return st;
    tap_list(kConvV, w);
    w.X = i == 0 ? nullptr : A.v[i - 1];
    w.G = G.gvp;
    if ((st = launch_wgrad<T>(L, w, cv, grad, O, batch, s, sink)) != FK_OK) return st;
    if (i > 0) {
      VHBwdArgs v;
      v.gvp = G.gvp;
      v.gt = G.gt;
      v.wv = w32(L, packed, conv_index(i, kConvV));
      v.wh = w32(L, packed, conv_index(i, kConvH));
      // cc i = 2b+1 is the first conv of a block whose second conv (2b+2)
      // adds the block input S_{2b} = S_{i-1} as residual.
      const bool block_first = (i % 2 == 1) && (i + 1 < last);
      v.res_v = block_first ? G.gvpd[i + 1] : nullptr;
      v.res_h = block_first ? G.ghp[i + 1] : nullptr;
      v.vprev = A.v[i - 1];
      v.hprev = A.h[i - 1];
      v.gvpd_prev = G.gvpd[i - 1];
      v.ghp_prev = G.ghp[i - 1];
      vh_bwd_kernel<F, T><<<rows, 128, 0, s>>>(v, L.H, L.W);
      FK_CUDA(launched());
    }
    return FK_OK;
  };
  int st = run_passes(L, batch, sink, seeds, G0, seeds1, G1, head, step, s);
  if (st != FK_OK) return st;
  if (sink) return sink_flush(*sink, s);
  if (L.wn) return launch_wn(L, params, grad, O, batch, s);
  return FK_OK;
}

// ---------------------------------------------------------------- adjoint on tensor cores
// Workspace of the tensor-core adjoint (BF16, F = 32, summed gradient): bf16
// gradient tensors, the head gradient gL, and scratch for the per-CTA weight
// gradient partials and the per-tile bias partials.
struct TcBwdTensors {
  void* gvs[40];   // masked stream gradient of V_i
  void* ghp[40];   // masked gradient of Hp_i
  void* gcatm;
  void* gt;
  void* gvp;
  float* gl;
  float* part;
  float* bpart;
  int64_t bytes;
};

static int64_t tc_bwd_layout(const NetLayout& L, int64_t batch, char* base, TcBwdTensors* T) {
  const int64_t tiles = (batch + kTile - 1) / kTile;
  const int64_t tb = tiles * L.P * (int64_t)kTile * L.F * 2;
  int64_t off = 0;
  auto take = [&](int64_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  TcBwdTensors tmp;
  TcBwdTensors* t = T ? T : &tmp;
  memset(t, 0, sizeof(*t));
  for (int i = 0; i < L.n_cc; ++i) {  // ring of three, as in bwd_layout
    t->gvs[i] = i < kGradRing ? take(tb) : t->gvs[i % kGradRing];
    t->ghp[i] = i < kGradRing ? take(tb) : t->ghp[i % kGradRing];
  }
  t->gcatm = take(tb);
  t->gt = take(tb);
  t->gvp = take(tb);
  t->gl = reinterpret_cast<float*>(take(tiles * L.P * (int64_t)kTile * 8 * 4));
  // weight-gradient partials: the tensor-core launches' per-CTA sums, or the
  // CUDA-core launches' per-tile sums (head, first causal conv: <= 9*1*32+32
  // or 32*4+4 per tile)
  const int64_t pf = wgrad_tc_part_floats(tiles, L.H);
  t->part = reinterpret_cast<float*>(take((pf > tiles * 320 ? pf : tiles * 320) * 4));
  t->bpart = reinterpret_cast<float*>(take(tiles * L.H * 32 * 4));
  t->bytes = off;
  return off;
}

// FK_AR2D_ENGINE=rowwise also selects the CUDA-core adjoint (for comparisons).
static bool use_tc_adjoint(const NetLayout& L) {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("FK_AR2D_ENGINE");
    v = (e && strcmp(e, "rowwise") == 0) ? 0 : 1;
  }
  return v == 1 && L.precision != FK_PRECISION_FP32 && L.F == 32 && pipe_supported(L.F, L.W);
}

// With O != NULL (per-sample rows) the data gradients still run on the
// tensor cores and every weight gradient is the CUDA-core per-sample kernel
// reading the bf16 gradient tensors (the tensor-core weight-gradient GEMM sums
// over the samples, which per-sample rows must not).
static int backward_tc(const NetLayout& L, const void* packed, const float* params, const int8_t* spins,
                       int64_t batch, const float* seeds, const Tensors& A, const TcBwdTensors& G0, float* grad,
                       float* O, cudaStream_t s, RowSink* sink = nullptr, const float* seeds1 = nullptr,
                       const TcBwdTensors* G1 = nullptr) {
  using T = tc16;
  constexpr int F = 32;
  const int64_t tiles = (batch + kTile - 1) / kTile;
  const unsigned rows = (unsigned)(tiles * L.H);
  const int last = L.n_cc - 1;
  int* err = device_error_word();
  auto wt = [&](int idx) { return static_cast<const char*>(packed) + L.conv[idx].wt_off; };
  if (!O) FK_CUDA(cudaMemsetAsync(grad, 0, (size_t)L.num_params * sizeof(float), s));
  // head and step i of one pass (seeds, gradient tensors)
  auto head = [&](const float* seeds, const TcBwdTensors& G) -> int {
    HeadBwdArgs h;
    const int io = L.n_convs - 1;
    h.hlast = A.h[last];
    h.wo = w32(L, packed, io);
    h.bo = reinterpret_cast<const float*>(static_cast<const char*>(packed) + L.conv[io].b_off);
    h.spins = spins;
    h.seeds = reinterpret_cast<const float2*>(seeds);
    h.batch = batch;
    h.gL = G.gl;
    h.ghp = G.ghp[last];
    h.updown = L.updown;
    head_bwd_kernel<F, T, T><<<rows, 128, 0, s>>>(h, L.H, L.W);
    FK_CUDA(launched());
    WgArgs w;
    memset(&w, 0, sizeof(w));
    w.ntaps = 1;
    w.X = A.h[last];
    w.cin = F;
    w.G = G.gl;
    w.gC = 8;
    w.N = 4;
    w.spins = spins;
    w.part = G.part;
    return launch_wgrad<T, float>(L, w, L.conv[io], grad, O, batch, s, sink);
  };
  // per-sample weight gradient of one conv: taps of `kind` (or one tap at
  // (dr, dc) for the 1x1 convs), input X (cin channels), gradient channels
  // [g0, g0 + n) of Gt
  auto wg_rows = [&](int kind, int dr, int dc, const void* X, int cin, const void* Gt, int g0, int n,
                     const ConvDesc& cd) -> int {
    if (cin == 32 && rows_on_tensor_cores() && wgrad_rows_tc_supported(L.H, L.W, n)) {
      WgRowsArgs r;
      memset(&r, 0, sizeof(r));
      WgArgs taps;
      memset(&taps, 0, sizeof(taps));
      if (kind >= 0) {
        tap_list(kind, taps);
      } else {
        taps.ntaps = 1;
        taps.dr[0] = dr;
        taps.dc[0] = dc;
      }
      r.X = X;
      r.G = Gt;
      r.cin = 32;
      r.g_float = 0;
      r.gC = F;
      r.g0 = g0;
      r.N = n;
      r.ntaps = taps.ntaps;
      for (int t = 0; t < taps.ntaps; ++t) {
        r.dr[t] = taps.dr[t];
        r.dc[t] = taps.dc[t];
      }
      RowsTarget tg;
      const int st = rows_target(L, cd, O, batch, s, sink, &tg);
      if (st != FK_OK) return st;
      r.O = tg.O;
      r.o_kernel = tg.o_kernel;
      r.o_bias = tg.o_bias;
      r.o_ld = tg.o_ld;
      r.o_col = tg.o_col;
      r.batch = batch;
      return launch_wgrad_rows_tc(r, L.H, L.W, err, s);
    }
    WgArgs w;
    memset(&w, 0, sizeof(w));
    w.spins = spins;
    if (kind >= 0) {
      tap_list(kind, w);
    } else {
      w.ntaps = 1;
      w.dr[0] = dr;
      w.dc[0] = dc;
    }
    w.X = X;
    w.cin = cin;
    w.G = Gt;
    w.gC = F;
    w.g0 = g0;
    w.N = n;
    return launch_wgrad<T, T>(L, w, cd, nullptr, O, batch, s, sink);
  };
  // summed weight gradients on the tensor cores (single pass)
  auto wg = [&](const void* X, int x_rows, int x_row0, const void* Gt, int g0, int n, int ntc, int dc0,
                const ConvDesc& cd) -> int {
    const TcBwdTensors& G = G0;
    WgTcArgs a;
    a.X = X;
    a.x_rows = x_rows;
    a.x_row0 = x_row0;
    a.G = Gt;
    a.g0 = g0;
    a.n = n;
    a.ntc = ntc;
    a.dc0 = dc0;
    a.part = G.part;
    // the G column block that meets every output column once, at x = its column
    a.bias_jpos = dc0 + ntc - 1;
    a.part_bias = G.part + wgrad_tc_grid(tiles, L.H) * (3 * 32 * 96);
    int r = launch_wgrad_tc(a, cd.kw, 0, grad + cd.p_kernel, grad + cd.p_bias, tiles, L.H, L.W, err, s);
    if (r != FK_OK || a.bias_jpos >= 0) return r;
    return launch_bias_sum(Gt, tiles, L.H, L.W, g0, n, batch, G.bpart, grad + cd.p_bias, s);
  };
  auto step = [&](int i, const TcBwdTensors& G) -> int {
    int st;
    const ConvDesc& cv = L.conv[conv_index(i, kConvV)];
    const ConvDesc& ch = L.conv[conv_index(i, kConvH)];
    const ConvDesc& cx = L.conv[conv_index(i, kConvX)];
    const ConvDesc& cy = L.conv[conv_index(i, kConvY)];
    const ConvDesc& cc = L.conv[conv_index(i, kConvC)];
    const int shift = (i == last) ? 1 : 0;
    {
      BwdOpArgs b;
      memset(&b, 0, sizeof(b));
      b.kind = kBwdC;
      b.in = G.ghp[i];
      b.wt = wt(conv_index(i, kConvC));
      b.wx = wt(conv_index(i, kConvX));
      b.wy = wt(conv_index(i, kConvY));
      b.cat = A.cat[i];
      b.t = A.t[i];
      b.rv = A.rv[i];
      b.gvs = (i == last) ? nullptr : G.gvs[i];
      b.shift = shift;
      b.gcatm = G.gcatm;
      b.gt = G.gt;
      b.gvp = G.gvp;
      if ((st = launch_bwd_op(b, tiles, L.H, L.W, err, s)) != FK_OK) return st;
    }
    // weight and bias gradients of the five convs of causal conv i
    if (O) {
      if ((st = wg_rows(kConvC, 0, 0, A.cat[i], F, G.ghp[i], 0, F, cc)) != FK_OK) return st;
      if ((st = wg_rows(-1, 0, -shift, A.t[i], F, G.gcatm, 0, F / 2, cx)) != FK_OK) return st;
      if ((st = wg_rows(-1, -1, 0, A.rv[i], F, G.gcatm, F / 2, F / 2, cy)) != FK_OK) return st;
      if (i > 0) {
        if ((st = wg_rows(kConvH, 0, 0, A.h[i - 1], F, G.gt, 0, F, ch)) != FK_OK) return st;
        if ((st = wg_rows(kConvV, 0, 0, A.v[i - 1], F, G.gvp, 0, F, cv)) != FK_OK) return st;
      }
    } else {
      if ((st = wg(A.cat[i], 3, -2, G.ghp[i], 0, F, 3, -2, cc)) != FK_OK) return st;
      if ((st = wg(A.t[i], 1, 0, G.gcatm, 0, F / 2, 1, -shift, cx)) != FK_OK) return st;
      if ((st = wg(A.rv[i], 1, -1, G.gcatm, F / 2, F / 2, 1, 0, cy)) != FK_OK) return st;
      if (i > 0) {
        if ((st = wg(A.h[i - 1], 1, 0, G.gt, 0, F, 3, -2, ch)) != FK_OK) return st;
        if ((st = wg(A.v[i - 1], 3, -2, G.gvp, 0, F, 3, -1, cv)) != FK_OK) return st;
      }
    }
    if (i > 0) {
      // cc i = 2b+1 is the first conv of a block whose second conv (2b+2) adds
      // the block input S_{2b} = S_{i-1} as residual
      const bool block_first = (i % 2 == 1) && (i + 1 < last);
      BwdOpArgs b;
      memset(&b, 0, sizeof(b));
      b.kind = kBwdV;
      b.in = G.gvp;
      b.wt = wt(conv_index(i, kConvV));
      b.res = block_first ? G.gvs[i + 1] : nullptr;
      b.prev = A.v[i - 1];
      b.out = G.gvs[i - 1];
      if ((st = launch_bwd_op(b, tiles, L.H, L.W, err, s)) != FK_OK) return st;
      b.kind = kBwdH;
      b.in = G.gt;
      b.wt = wt(conv_index(i, kConvH));
      b.res = block_first ? G.ghp[i + 1] : nullptr;
      b.prev = A.h[i - 1];
      b.out = G.ghp[i - 1];
      if ((st = launch_bwd_op(b, tiles, L.H, L.W, err, s)) != FK_OK) return st;
    } else {
      // first causal conv: cin = 1 (spins), CUDA cores
      WgArgs w;
      memset(&w, 0, sizeof(w));
      w.spins = spins;
      tap_list(kConvH, w);
      w.X = nullptr;
      w.cin = 1;
      w.G = G.gt;
      w.gC = F;
      w.N = F;
      w.part = G.part;
      if ((st = launch_wgrad<T, T>(L, w, ch, grad, O, batch, s, sink)) != FK_OK) return st;
      tap_list(kConvV, w);
      w.G = G.gvp;
      if ((st = launch_wgrad<T, T>(L, w, cv, grad, O, batch, s, sink)) != FK_OK) return st;
    }
    return FK_OK;
  };
  int st = run_passes(L, batch, sink, seeds, G0, seeds1, G1, head, step, s);
  if (st != FK_OK) return st;
  if (sink) return sink_flush(*sink, s);
  if (L.wn) return launch_wn(L, params, grad, O, batch, s);
  return FK_OK;
}

// Seeds of the two passes of the SR rows: (1, 0) and (0, 1) for every sample.
__global__ void sr_seeds_kernel(float* s0, float* s1, int64_t batch) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  s0[2 * b] = 1.f;
  s0[2 * b + 1] = 0.f;
  s1[2 * b] = 0.f;
  s1[2 * b + 1] = 1.f;
}

// Workspace of fk_ar2d_sr_gram: the gradient tensors of two passes and their
// seeds. Returns its size; with base != NULL also the pieces.
static int64_t sr_gram_ws(const NetLayout& L, int64_t batch, char* base, char** g0, char** g1, float** seeds) {
  const int64_t g = use_tc_adjoint(L) ? tc_bwd_layout(L, batch, nullptr, nullptr) : bwd_layout(L, batch, nullptr, nullptr);
  const int64_t ga = (g + 255) / 256 * 256;
  if (base) {
    *g0 = base;
    *g1 = base + ga;
    *seeds = reinterpret_cast<float*>(base + 2 * ga);
  }
  return 2 * ga + 4 * batch * (int64_t)sizeof(float);
}

}  // namespace FK_NS

using namespace FK_NS;

extern "C" {

#ifndef FK_TC_FP16
int64_t fk_ar2d_backward_workspace_bytes(const fk_ar2d_desc* desc, int64_t batch) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK || batch < 0) return -1;
  const int64_t b = bwd_layout(L, batch, nullptr, nullptr);
  const int64_t t = (L.precision != FK_PRECISION_FP32 && L.F == 32) ? tc_bwd_layout(L, batch, nullptr, nullptr) : 0;
  return b > t ? b : t;
}
#endif

int FK_AR2D_ENTRY(fk_ar2d_backward)(const fk_ar2d_desc* desc, const void* packed, const float* params,
                                    const int8_t* spins, int64_t batch, const float* w, const void* saved,
                                    int64_t saved_bytes, void* workspace, int64_t workspace_bytes, float* grad,
                                    float* per_sample, void* stream) {
  FK_DISPATCH_FP16(desc, fk_ar2d_backward_tc_fp16(desc, packed, params, spins, batch, w, saved, saved_bytes,
                                                  workspace, workspace_bytes, grad, per_sample, stream));
  NetLayout L;
  int st = build_layout(desc, &L);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(packed && params && spins && w && saved, "fk_ar2d_backward: NULL buffer");
  FK_CHECK_ARG(grad || per_sample, "fk_ar2d_backward: need grad or per_sample");
  if (batch == 0) return FK_OK;
  Tensors A;
  int64_t need = workspace_layout(L, batch, FK_AR2D_SAVE, static_cast<char*>(const_cast<void*>(saved)), &A);
  FK_CHECK_ARG(saved_bytes >= need, "fk_ar2d_backward: saved workspace %lld < %lld bytes", (long long)saved_bytes,
               (long long)need);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (use_tc_adjoint(L)) {
    TcBwdTensors TG;
    int64_t tneed = tc_bwd_layout(L, batch, static_cast<char*>(workspace), &TG);
    FK_CHECK_ARG(workspace && workspace_bytes >= tneed, "fk_ar2d_backward: workspace %lld < %lld bytes",
                 (long long)workspace_bytes, (long long)tneed);
    return backward_tc(L, packed, params, spins, batch, w, A, TG, per_sample ? nullptr : grad, per_sample, s);
  }
  BwdTensors G;
  int64_t gneed = bwd_layout(L, batch, static_cast<char*>(workspace), &G);
  FK_CHECK_ARG(workspace && workspace_bytes >= gneed, "fk_ar2d_backward: workspace %lld < %lld bytes",
               (long long)workspace_bytes, (long long)gneed);
  float* O = per_sample;
  float* g = per_sample ? nullptr : grad;
  const bool bf = L.precision != FK_PRECISION_FP32;
  switch (L.F) {
    case 16: return bf ? backward_impl<16, tc16>(L, packed, params, spins, batch, w, A, G, g, O, s)
                       : backward_impl<16, float>(L, packed, params, spins, batch, w, A, G, g, O, s);
    case 32: return bf ? backward_impl<32, tc16>(L, packed, params, spins, batch, w, A, G, g, O, s)
                       : backward_impl<32, float>(L, packed, params, spins, batch, w, A, G, g, O, s);
    default: return bf ? backward_impl<64, tc16>(L, packed, params, spins, batch, w, A, G, g, O, s)
                       : backward_impl<64, float>(L, packed, params, spins, batch, w, A, G, g, O, s);
  }
}

int FK_AR2D_ENTRY(fk_ar2d_sr_gram)(const fk_ar2d_desc* desc, const void* packed, const float* params,
                                   const int8_t* spins, int64_t batch, const void* saved, int64_t saved_bytes,
                                   void* workspace, int64_t workspace_bytes, float* rows, int64_t rows_floats,
                                   double* gram, int32_t tensor_cores, void* stream) {
  FK_DISPATCH_FP16(desc, fk_ar2d_sr_gram_tc_fp16(desc, packed, params, spins, batch, saved, saved_bytes, workspace,
                                                 workspace_bytes, rows, rows_floats, gram, tensor_cores, stream));
  NetLayout L;
  int st = build_layout(desc, &L);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(packed && params && spins && saved && rows && gram && workspace, "fk_ar2d_sr_gram: NULL buffer");
  FK_CHECK_ARG(batch > 0, "fk_ar2d_sr_gram: batch must be positive");
  const int64_t n = 2 * batch;
  const int64_t need_floats = sink_floats(sink_min_rows(L), n, tensor_cores != 0);
  FK_CHECK_ARG(rows_floats >= need_floats, "fk_ar2d_sr_gram: row buffer of %lld floats < %lld",
               (long long)rows_floats, (long long)need_floats);
  FK_CHECK_ARG(workspace_bytes >= sr_gram_ws(L, batch, nullptr, nullptr, nullptr, nullptr),
               "fk_ar2d_sr_gram: workspace %lld < %lld bytes", (long long)workspace_bytes,
               (long long)sr_gram_ws(L, batch, nullptr, nullptr, nullptr, nullptr));
  Tensors A;
  int64_t need = workspace_layout(L, batch, FK_AR2D_SAVE, static_cast<char*>(const_cast<void*>(saved)), &A);
  FK_CHECK_ARG(saved_bytes >= need, "fk_ar2d_sr_gram: saved workspace %lld < %lld bytes", (long long)saved_bytes,
               (long long)need);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char* g0 = nullptr;
  char* g1 = nullptr;
  float* seeds0 = nullptr;
  float* seeds1 = nullptr;
  sr_gram_ws(L, batch, static_cast<char*>(workspace), &g0, &g1, &seeds0);
  seeds1 = seeds0 + 2 * batch;
  sr_seeds_kernel<<<(unsigned)((batch + 255) / 256), 256, 0, s>>>(seeds0, seeds1, batch);
  FK_CUDA(launched());
  FK_CUDA(cudaMemsetAsync(gram, 0, (size_t)(n * n) * sizeof(double), s));
  RowSink k;
  k.L = &L;
  k.params = params;
  k.buf = rows;
  // the most rows whose floats (and split operands) fit in the buffer
  int64_t lo = 0, hi = rows_floats / n;  // sink_floats(lo) fits; sink_floats grows with the rows
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo + 1) / 2;
    if (sink_floats(mid, n, tensor_cores != 0) <= rows_floats)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int64_t cap = lo;
  k.cap = cap;
  k.split = tensor_cores ? static_cast<void*>(rows + (cap * n + 63) / 64 * 64) : nullptr;
  k.split_bytes = tensor_cores ? fk_sr_gram_split_bytes(cap, n) : 0;
  k.used = 0;
  k.ld = n;
  k.col = 0;
  k.groups = 2;
  k.tensor_cores = tensor_cores;
  k.gram = gram;
  k.n = 0;
  for (int i = 0; i < kMaxConvs; ++i) k.at[i] = -1;
  if (use_tc_adjoint(L)) {
    TcBwdTensors T0, T1;
    tc_bwd_layout(L, batch, g0, &T0);
    tc_bwd_layout(L, batch, g1, &T1);
    st = backward_tc(L, packed, params, spins, batch, seeds0, A, T0, nullptr, rows, s, &k, seeds1, &T1);
  } else {
    BwdTensors G0, G1;
    bwd_layout(L, batch, g0, &G0);
    bwd_layout(L, batch, g1, &G1);
    const bool bf = L.precision != FK_PRECISION_FP32;
#define FK_SR_ROWS(FF, TT) backward_impl<FF, TT>(L, packed, params, spins, batch, seeds0, A, G0, nullptr, rows, s, &k, \
                                                 seeds1, &G1)
    switch (L.F) {
      case 16: st = bf ? FK_SR_ROWS(16, tc16) : FK_SR_ROWS(16, float); break;
      case 32: st = bf ? FK_SR_ROWS(32, tc16) : FK_SR_ROWS(32, float); break;
      default: st = bf ? FK_SR_ROWS(64, tc16) : FK_SR_ROWS(64, float);
    }
#undef FK_SR_ROWS
  }
  return st != FK_OK ? st : fk_sr_gram_mirror(gram, n, stream);
}

#ifndef FK_TC_FP16
int64_t fk_ar2d_sr_gram_workspace_bytes(const fk_ar2d_desc* desc, int64_t batch) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK || batch <= 0) return -1;
  return sr_gram_ws(L, batch, nullptr, nullptr, nullptr, nullptr);
}

int64_t fk_ar2d_sr_gram_min_rows(const fk_ar2d_desc* desc, int64_t batch, int32_t tensor_cores) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK || batch <= 0) return -1;
  return sink_floats(sink_min_rows(L), 2 * batch, tensor_cores != 0);
}
#endif

}  // extern "C"
