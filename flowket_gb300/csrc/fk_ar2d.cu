// ConvNetAutoregressive2D forward pass, exact sampler and weight packing.
//
// Network (machines/conv_net_autoregressive_2D.py:24-74), per causal conv i:
//   V op  : Vp = conv3x3(V_i) [taps rows -2..0, cols -1..1] + b_v
//           V_{i+1} = relu(Vp [+ residual]);  RV = relu(Vp)
//           U = relu(W_y RV + b_y)  -> Cat[r+1, c][F/2:F]   (DownShift, :44-45)
//   H op  : T = relu(conv1x3(H_i) [cols -2..0] + b_h)
//           Z = relu(W_x T + b_x)   -> Cat[r, c+s][0:F/2]   (RightShift s=1 on the
//                                                            final conv, :41-43)
//   C op  : Hp = conv3x3(Cat) [rows -2..0, cols -2..0] + b_c
//           H_{i+1} = relu(Hp [+ residual]); on the final conv the 1x1 head
//           W_o relu(Hp) + b_o gives the four outputs (Re0, Re1, Im0, Im1).
// Boundary values of the shifted tensors are relu(bias) (a shifted-in zero
// through the 1x1 conv + relu), written by the ops at r == 0 / c == 0.
//
// Every op is executed per (tile of 128 samples, pixel) by one CTA of 128
// threads (thread = sample). Two engines compute the GEMMs:
//   * FP32 CUDA cores (the plain FP32 path): thread-local accumulators;
//   * BF16 tcgen05: taps and weight slices arrive by bulk copies (TMA) into
//     shared memory, one thread issues tcgen05.mma (M=128, N=F, K=16 steps)
//     into TMEM, the epilogue reads TMEM with tcgen05.ld; the chained 1x1 is
//     a second MMA on the epilogue's bf16 output staged in shared memory.
// Both engines share the epilogue, so the two precisions run the same code
// path apart from the GEMMs.
#include "fk_ar2d.cuh"

#include <math.h>
#include <stdlib.h>
#include <string.h>

namespace FK_NS {

// ============================================================== layout (host)
int build_layout(const fk_ar2d_desc* d, NetLayout* L) {
  if (!d) {
    set_error("fk_ar2d: NULL descriptor");
    return FK_ERR_ARG;
  }
  if (d->height < 1 || d->width < 1 || d->height * d->width > 4096 || d->depth < 2 || d->depth > 20 ||
      !(d->channels == 16 || d->channels == 32 || d->channels == 64) ||
      !(d->precision == FK_PRECISION_FP32 || d->precision == FK_PRECISION_BF16 ||
        d->precision == FK_PRECISION_FP16)) {
    set_error("fk_ar2d: unsupported shape (H=%d W=%d depth=%d channels=%d precision=%d); "
              "supported: depth 2..20, channels 16/32/64",
              d->height, d->width, d->depth, d->channels, d->precision);
    return FK_ERR_ARG;
  }
  memset(L, 0, sizeof(*L));
  L->H = d->height;
  L->W = d->width;
  L->P = d->height * d->width;
  L->depth = d->depth;
  L->F = d->channels;
  L->wn = d->weights_normalization ? 1 : 0;
  L->precision = d->precision;
  L->updown = d->equal_up_down_spins ? 1 : 0;
  L->n_cc = 2 * d->depth - 2;
  const int F = L->F;
  int64_t p = 0, w = 0;
  auto add = [&](int kh, int kw, int cin, int cout, bool wn) {
    ConvDesc& c = L->conv[L->n_convs++];
    c.kh = kh;
    c.kw = kw;
    c.cin = cin;
    c.cout = cout;
    c.K = kh * kw * cin;
    c.Kpad = (c.K + 15) / 16 * 16;
    c.Npad = cout < 16 ? 16 : (cout + 15) / 16 * 16;
    c.p_kernel = p;
    p += (int64_t)c.K * cout;
    c.p_bias = p;
    p += cout;
    c.p_g = -1;
    if (wn) {
      c.p_g = p;
      p += cout;
    }
    c.w_off = w;
    if (L->precision != FK_PRECISION_FP32) {
      w += ((int64_t)c.Kpad * c.Npad * 2 + 255) / 256 * 256;
    }
    c.ws_off = -1;
    c.wt_off = -1;
    if (L->precision != FK_PRECISION_FP32 && kw == 3 && cin == F && F <= 32) {
      c.ws_off = w;
      w += ((int64_t)kh * cin * 3 * cout * 2 + 255) / 256 * 256;
      c.wt_off = w;
      w += ((int64_t)kh * cout * 3 * cin * 2 + 255) / 256 * 256;
    } else if (L->precision != FK_PRECISION_FP32 && kh == 1 && kw == 1 && cin == F && cout == F / 2 && F <= 32) {
      c.wt_off = w;
      w += ((int64_t)cout * cin * 2 + 255) / 256 * 256;
    }
    c.w32_off = w;
    w += ((int64_t)c.K * cout * 4 + 255) / 256 * 256;
    c.b_off = w;
    w += ((int64_t)c.Npad * 4 + 255) / 256 * 256;
  };
  for (int i = 0; i < L->n_cc; ++i) {
    int cin = i == 0 ? 1 : F;
    add(3, 3, cin, F, L->wn);      // v
    add(1, 3, cin, F, L->wn);      // h
    add(1, 1, F, F / 2, L->wn);    // x
    add(1, 1, F, F / 2, L->wn);    // y
    add(3, 3, F, F, L->wn);        // c
  }
  add(1, 1, F, 4, false);          // out head
  L->num_params = p;
  L->packed_bytes = w;
  return FK_OK;
}

static inline int64_t esize(const NetLayout& L) { return L.precision != FK_PRECISION_FP32 ? 2 : 4; }

int64_t tensor_bytes(const NetLayout& L, int64_t tiles, int channels) {
  int64_t b = tiles * L.P * (int64_t)kTile * channels * esize(L);
  return (b + 255) / 256 * 256;
}

int64_t workspace_layout(const NetLayout& L, int64_t batch, int mode, char* base, Tensors* T) {
  int64_t tiles = (batch + kTile - 1) / kTile;
  int64_t tb = tensor_bytes(L, tiles, L.F);
  int64_t off = 0;
  auto take = [&](int64_t bytes) -> void* {
    void* ptr = base ? base + off : nullptr;
    off += (bytes + 255) / 256 * 256;
    return ptr;
  };
  if (T) memset(T, 0, sizeof(*T));
  Tensors tmp;
  Tensors* t = T ? T : &tmp;
  if (mode == FK_AR2D_INFER) {
    t->v[0] = take(tb);
    t->v[1] = take(tb);
    t->h[0] = take(tb);
    t->h[1] = take(tb);
    t->cat[0] = take(tb);
  } else {
    for (int i = 0; i < L.n_cc; ++i) {
      t->v[i] = take(tb);
      t->h[i] = take(tb);
      t->cat[i] = take(tb);
      t->t[i] = take(tb);
      t->rv[i] = take(tb);
    }
  }
  t->row_partial = static_cast<float2*>(take(tiles * L.H * kTile * sizeof(float2)));
  if (L.updown) t->updown = static_cast<uint8_t*>(take(tiles * kTile * (int64_t)L.P));
  t->bytes = off;
  return off;
}

// ============================================================== weight packing
struct PackArgs {
  const float* params;
  char* packed;
  int n_convs;
  int bf16;
  ConvDesc conv[kMaxConvs];
};

// One CTA per conv: weight-norm scale per output channel (wrappers.py:130-134:
// v * rsqrt(max(sum v^2, 1e-12)) * exp(g)), then the operand layout.
__global__ void pack_kernel(const __grid_constant__ PackArgs a) {
  const ConvDesc& c = a.conv[blockIdx.x];
  __shared__ float scale[64];
  const float* v = a.params + c.p_kernel;
  for (int n = threadIdx.x; n < c.cout; n += blockDim.x) {
    float s = 1.f;
    if (c.p_g >= 0) {
      float sq = 0.f;
      for (int k = 0; k < c.K; ++k) {
        float x = v[(int64_t)k * c.cout + n];
        sq += x * x;
      }
      s = rsqrtf(fmaxf(sq, 1e-12f)) * expf(a.params[c.p_g + n]);
    }
    scale[n] = s;
  }
  __syncthreads();
  float* bias = reinterpret_cast<float*>(a.packed + c.b_off);
  for (int n = threadIdx.x; n < c.Npad; n += blockDim.x) bias[n] = n < c.cout ? a.params[c.p_bias + n] : 0.f;
  {
    float* w = reinterpret_cast<float*>(a.packed + c.w32_off);
    int total = c.K * c.cout;
    for (int i = threadIdx.x; i < total; i += blockDim.x) w[i] = v[i] * scale[i % c.cout];
  }
  if (a.bf16) {
    tc16* w = reinterpret_cast<tc16*>(a.packed + c.w_off);
    int total = c.Kpad * c.Npad;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      // element (k, n) of the no-swizzle K-major operand at ((k/8)*Npad + n)*8 + k%8
      int kg = i / (c.Npad * 8);
      int rem = i - kg * c.Npad * 8;
      int n = rem / 8, e = rem % 8;
      int k = kg * 8 + e;
      float x = (k < c.K && n < c.cout) ? v[(int64_t)k * c.cout + n] * scale[n] : 0.f;
      w[i] = to_tc16(x);
    }
  }
  if (a.bf16 && c.ws_off >= 0) {
    // column-scatter operand: element (kernel row i, k, n = s*cout + co) at
    // ((i*(cin/8) + k/8)*3*cout + n)*8 + k%8, value W[i][2 - s][k][co]
    tc16* w = reinterpret_cast<tc16*>(a.packed + c.ws_off);
    const int n3 = 3 * c.cout;
    const int total = c.kh * c.cin * n3;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int e = i % 8;
      const int n = (i / 8) % n3;
      const int kg = i / (8 * n3);  // i*(cin/8) + k/8
      const int row = kg / (c.cin / 8);
      const int k = (kg % (c.cin / 8)) * 8 + e;
      const int s = n / c.cout, co = n % c.cout;
      const int t = row * c.kw + (2 - s);
      w[i] = to_tc16(v[((int64_t)t * c.cin + k) * c.cout + co] * scale[co]);
    }
  }
  if (a.bf16 && c.wt_off >= 0) {
    // transposed operand: element (kernel row i, k = co, n = j*cin + ci) at
    // ((i*(cout/8) + co/8)*kw*cin + n)*8 + co%8, value W[i][j][ci][co]
    tc16* w = reinterpret_cast<tc16*>(a.packed + c.wt_off);
    const int nn = c.kw * c.cin;
    const int total = c.kh * c.cout * nn;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
      const int e = i % 8;
      const int n = (i / 8) % nn;
      const int kg = i / (8 * nn);  // i*(cout/8) + co/8
      const int row = kg / (c.cout / 8);
      const int co = (kg % (c.cout / 8)) * 8 + e;
      const int j = n / c.cin, ci = n % c.cin;
      const int t = row * c.kw + j;
      w[i] = to_tc16(v[((int64_t)t * c.cin + ci) * c.cout + co] * scale[co]);
    }
  }
}

// ============================================================== GEMM engines
// ---- FP32 CUDA-core engine
template <int F>
__device__ void simt_main(const OpArgs& a, int64_t tile, int m, int r, int c, int H, int W, int P, float* acc) {
#pragma unroll
  for (int n = 0; n < F; ++n) acc[n] = 0.f;
  const float* Wm = static_cast<const float*>(a.main.w);
  const int nt = num_taps(a.kind);
  for (int t = 0; t < nt; ++t) {
    int dr, dc;
    tap_offset(a.kind, t, dr, dc);
    int rr = r + dr, cc = c + dc;
    if (rr < 0 || rr >= H || cc < 0 || cc >= W) continue;
    int pix = rr * W + cc;
    if (a.first) {
      float s = spin_at(a.spins, a.batch, P, tile * kTile + m, pix);
      const float4* w4 = reinterpret_cast<const float4*>(Wm + (int64_t)t * F);
#pragma unroll
      for (int n4 = 0; n4 < F / 4; ++n4) {
        float4 wv = __ldg(w4 + n4);
        acc[4 * n4 + 0] += s * wv.x;
        acc[4 * n4 + 1] += s * wv.y;
        acc[4 * n4 + 2] += s * wv.z;
        acc[4 * n4 + 3] += s * wv.w;
      }
    } else {
      const float* x = blk<float>(a.in, tile, P, pix, F);
      for (int g = 0; g < F / 8; ++g) {
        float v[8];
        ld8(x + ((int64_t)g * kTile + m) * 8, v);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const float4* w4 = reinterpret_cast<const float4*>(Wm + ((int64_t)t * F + g * 8 + e) * F);
#pragma unroll
          for (int n4 = 0; n4 < F / 4; ++n4) {
            float4 wv = __ldg(w4 + n4);
            acc[4 * n4 + 0] += v[e] * wv.x;
            acc[4 * n4 + 1] += v[e] * wv.y;
            acc[4 * n4 + 2] += v[e] * wv.z;
            acc[4 * n4 + 3] += v[e] * wv.w;
          }
        }
      }
    }
  }
}

// out[0..NC) = in[0..KC) x W[KC][NC] (fp32, row-major)
template <int KC, int NC>
__device__ __forceinline__ void simt_chain(const ConvW& cw, const float* in, float* out) {
  const float* Wc = static_cast<const float*>(cw.w);
#pragma unroll
  for (int n = 0; n < NC; ++n) out[n] = 0.f;
#pragma unroll 4
  for (int k = 0; k < KC; ++k) {
    float x = in[k];
#pragma unroll
    for (int n = 0; n < NC; ++n) out[n] += x * __ldg(Wc + k * NC + n);
  }
}

// ---- BF16 tcgen05 engine
struct TcSmem {
  uint32_t a, w, ca, cw;    // shared addresses of the regions
  uint8_t* a_ptr;
  uint8_t* ca_ptr;
  uint8_t* w_ptr;
  uint8_t* cw_ptr;
  uint64_t* bar_load;
  uint64_t* bar_mma;
  uint64_t* vbar;  // 7 barriers of the one-pass V row op
  uint32_t* tmem_slot;
  int taps_per_group;
};

template <int F>
struct TcCfg {
  static constexpr int kTapBytesA = kTile * F * 2;
  static constexpr int kTapBytesW = F * F * 2;
  static constexpr int kChainNpad = (F / 2) < 16 ? 16 : (F / 2);
  static constexpr int kGroupBudget = 176 * 1024;
  static constexpr int kTaps = (kGroupBudget / (kTapBytesA + kTapBytesW)) > 9 ? 9
                                                                             : (kGroupBudget / (kTapBytesA + kTapBytesW));
  static constexpr int kBytesA = kTaps * kTapBytesA;
  static constexpr int kBytesW = kTaps * kTapBytesW;
  static constexpr int kBytesCA = kTile * F * 2;
  static constexpr int kBytesCW = F * 32 * 2;
  static constexpr int kSmem = kBytesA + kBytesW + kBytesCA + kBytesCW + 128;
};

template <int F>
__device__ __forceinline__ void tc_carve(uint8_t* base, TcSmem& s) {
  using C = TcCfg<F>;
  s.a_ptr = base;
  s.w_ptr = base + C::kBytesA;
  s.ca_ptr = s.w_ptr + C::kBytesW;
  s.cw_ptr = s.ca_ptr + C::kBytesCA;
  uint8_t* bars = s.cw_ptr + C::kBytesCW;
  s.bar_load = reinterpret_cast<uint64_t*>(bars);
  s.bar_mma = reinterpret_cast<uint64_t*>(bars + 8);
  s.tmem_slot = reinterpret_cast<uint32_t*>(bars + 16);
  s.vbar = reinterpret_cast<uint64_t*>(bars + 24);
  s.a = smem_u32(s.a_ptr);
  s.w = smem_u32(s.w_ptr);
  s.ca = smem_u32(s.ca_ptr);
  s.cw = smem_u32(s.cw_ptr);
  s.taps_per_group = C::kTaps;
}

struct TcState {
  uint32_t tmem, ncols;
  uint32_t ph_load, ph_mma;
  int* err;
  bool abort;
};

constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kChainCol = 64;

// Setup: barriers + `ncols` TMEM columns (warp 0 allocates).
__device__ __forceinline__ void tc_setup(TcSmem& s, TcState& st, int* err, uint32_t ncols = kTmemCols) {
  if (threadIdx.x == 0) {
    mbar_init(s.bar_load, 1);
    mbar_init(s.bar_mma, 1);
    fence_mbar_init();
  }
  if (threadIdx.x < 32) {
    tmem_alloc(s.tmem_slot, ncols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  st.tmem = *s.tmem_slot;
  st.ncols = ncols;
  st.ph_load = 0;
  st.ph_mma = 0;
  st.err = err;
  st.abort = false;
}

__device__ __forceinline__ void tc_teardown(TcState& st) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    tmem_dealloc(st.tmem, st.ncols);
  }
}

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t& ph, TcState& st) {
  bool ok = mbar_wait(bar, ph, st.err);
  ph ^= 1u;
  if (!ok) st.abort = true;
  return ok;
}

// Loads TMEM columns [col, col+N) of this thread's lane (sample) into v.
template <int N>
__device__ __forceinline__ void tc_read(const TcState& st, uint32_t col, float* v) {
  uint32_t lane_base = (uint32_t)((threadIdx.x / 32) * 32) << 16;
#pragma unroll
  for (int q = 0; q < N / 16; ++q) tmem_ld16(st.tmem + lane_base + col + q * 16, v + q * 16);
  tmem_ld_wait();
}

// Main conv GEMM of one op at (tile, r, c) into acc[F] (pre-bias) on tensor cores.
// The chained 1x1 weights are brought in with the first load group.
template <int F>
__device__ void tc_main(const OpArgs& a, TcSmem& s, TcState& st, int64_t tile, int m, int r, int c, int H, int W,
                        int P, float* acc) {
  using C = TcCfg<F>;
  const uint32_t idesc = umma_idesc_tc16(128, F);
  const int chain_bytes = F * ((a.kind == kConvC) ? 16 : C::kChainNpad) * 2;
  const bool has_chain = !(a.kind == kConvC && !a.last);
  const char* wbase = static_cast<const char*>(a.main.w);
  if (a.first) {
    // cin = 1: thread m builds its K = 16 row (taps, zero padded) in place of the
    // im2col; weights are [2][F][8].
    float v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = 0.f;
    const int nt = num_taps(a.kind);
    for (int t = 0; t < nt; ++t) {
      int dr, dc;
      tap_offset(a.kind, t, dr, dc);
      int rr = r + dr, cc = c + dc;
      if (rr >= 0 && rr < H && cc >= 0 && cc < W) v[t] = spin_at(a.spins, a.batch, P, tile * kTile + m, rr * W + cc);
    }
    st8(reinterpret_cast<tc16*>(s.a_ptr + m * 16), v);
    st8(reinterpret_cast<tc16*>(s.a_ptr + 2048 + m * 16), v + 8);
    fence_proxy_async_smem();
    if (threadIdx.x == 0) {
      uint32_t wbytes = 2 * F * 16;
      mbar_arrive_expect_tx(s.bar_load, wbytes + (has_chain ? chain_bytes : 0));
      bulk_g2s(s.w_ptr, wbase, wbytes, s.bar_load);
      if (has_chain) bulk_g2s(s.cw_ptr, a.chain.w, chain_bytes, s.bar_load);
    }
    __syncthreads();
    if (!tc_wait(s.bar_load, st.ph_load, st)) return;
    if (threadIdx.x == 0) {
      tc_fence_after();
      uint64_t ad = umma_sdesc(s.a, 2048, 128);
      uint64_t bd = umma_sdesc(s.w, F * 16, 128);
      umma_bf16(st.tmem, ad, bd, idesc, 0u);
      umma_commit(s.bar_mma);
    }
    if (!tc_wait(s.bar_mma, st.ph_mma, st)) return;
    tc_fence_after();
  } else {
    // Taps in column-major order (tap column, then tap row): the order in
    // which the pipelined engine accumulates an output pixel, so that both
    // engines and the sampler round identically.
    int taps[9];
    int pix[9];
    int nvalid = 0;
    const int nt = num_taps(a.kind);
    for (int q = 0; q < nt; ++q) {
      const int t = tap_colmajor(a.kind, q);
      int dr, dc;
      tap_offset(a.kind, t, dr, dc);
      int rr = r + dr, cc = c + dc;
      if (rr >= 0 && rr < H && cc >= 0 && cc < W) {
        taps[nvalid] = t;
        pix[nvalid] = rr * W + cc;
        ++nvalid;
      }
    }
    const uint32_t wslice = F * F * 2;  // K-range of one tap: F/8 groups x F rows x 16 B
    for (int g0 = 0; g0 < nvalid; g0 += C::kTaps) {
      int ng = nvalid - g0 < C::kTaps ? nvalid - g0 : C::kTaps;
      if (threadIdx.x == 0) {
        uint32_t bytes = ng * (C::kTapBytesA + wslice) + ((g0 == 0 && has_chain) ? chain_bytes : 0);
        mbar_arrive_expect_tx(s.bar_load, bytes);
        for (int j = 0; j < ng; ++j) {
          const tc16* src = blk<tc16>(a.in, tile, P, pix[g0 + j], F);
          bulk_g2s(s.a_ptr + j * C::kTapBytesA, src, C::kTapBytesA, s.bar_load);
          bulk_g2s(s.w_ptr + j * wslice, wbase + (int64_t)taps[g0 + j] * wslice, wslice, s.bar_load);
        }
        if (g0 == 0 && has_chain) bulk_g2s(s.cw_ptr, a.chain.w, chain_bytes, s.bar_load);
      }
      if (!tc_wait(s.bar_load, st.ph_load, st)) return;
      if (threadIdx.x == 0) {
        tc_fence_after();
        for (int j = 0; j < ng; ++j) {
#pragma unroll
          for (int ks = 0; ks < F / 16; ++ks) {
            uint64_t ad = umma_sdesc(s.a + j * C::kTapBytesA + ks * 2 * 2048, 2048, 128);
            uint64_t bd = umma_sdesc(s.w + j * wslice + ks * 2 * F * 16, F * 16, 128);
            umma_bf16(st.tmem, ad, bd, idesc, (g0 + j + ks) > 0 ? 1u : 0u);
          }
        }
        umma_commit(s.bar_mma);
      }
      if (!tc_wait(s.bar_mma, st.ph_mma, st)) return;
      tc_fence_after();
    }
  }
  tc_read<F>(st, 0, acc);
}

// out[0..NCPAD) = in[0..KC) x Wchain on tensor cores (weights already in smem).
template <int KC, int NCPAD>
__device__ void tc_chain(TcSmem& s, TcState& st, int m, const float* in, float* out) {
  tc16* ca = reinterpret_cast<tc16*>(s.ca_ptr);
#pragma unroll
  for (int g = 0; g < KC / 8; ++g) st8(ca + ((int64_t)g * kTile + m) * 8, in + 8 * g);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    const uint32_t idesc = umma_idesc_tc16(128, NCPAD);
#pragma unroll
    for (int ks = 0; ks < KC / 16; ++ks) {
      uint64_t ad = umma_sdesc(s.ca + ks * 2 * 2048, 2048, 128);
      uint64_t bd = umma_sdesc(s.cw + ks * 2 * NCPAD * 16, NCPAD * 16, 128);
      umma_bf16(st.tmem + kChainCol, ad, bd, idesc, ks > 0 ? 1u : 0u);
    }
    umma_commit(s.bar_mma);
  }
  if (!tc_wait(s.bar_mma, st.ph_mma, st)) return;
  tc_fence_after();
  tc_read<NCPAD>(st, kChainCol, out);
}

// End of one op on the tensor-core engine: TMEM reads are done before the next
// MMA, and this op's global stores (generic proxy) are visible to the bulk
// copies (async proxy) that later ops of the same kernel issue.
__device__ __forceinline__ void tc_op_end() {
  asm volatile("fence.proxy.async;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

// ============================================================== one op (shared epilogue)
// Result of the head at one pixel: normalised (Re0, Re1, Im0, Im1).
struct HeadOut {
  float re0, re1, im0, im1;
};

// `mask` bit k: outcome k is masked by EqualUpDownSpins (layers/spins_invariants.py:13-22):
// its real part becomes -inf (LOG_ZERO in float32) before the normalisation, so
// the other outcome normalises to exactly 0.
__device__ __forceinline__ HeadOut normalise_head(const float* l, int mask = 0) {
  // abstract_machine.py:56-57, autoregressive.py:7-15 (norm_type 2)
  const float l0 = (mask & 1) ? -INFINITY : l[0], l1 = (mask & 2) ? -INFINITY : l[1];
  float a = 2.f * l0, b = 2.f * l1;
  float mx = fmaxf(a, b);
  float lse = 0.5f * (mx + logf(expf(a - mx) + expf(b - mx)));
  return HeadOut{l0 - lse, l1 - lse, l[2], l[3]};
}

// EqualUpDownSpins mask bits of every (sample, site): bit 0 when at least N/2
// earlier sites (raster order) hold +1, bit 1 when at least N/2 hold -1.
__global__ void updown_mask_kernel(const int8_t* __restrict__ spins, int64_t batch, int P, uint8_t* __restrict__ out) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  int up = 0, down = 0;
  for (int k = 0; k < P; ++k) {
    out[b * P + k] = (uint8_t)((2 * up >= P ? 1 : 0) | (2 * down >= P ? 2 : 0));
    if (spins[b * P + k] > 0)
      ++up;
    else
      ++down;
  }
}

template <int F, bool TC>
struct Engine;

template <int F>
struct Engine<F, false> {
  TcSmem* s;
  TcState* st;
  __device__ void main(const OpArgs& a, int64_t tile, int m, int r, int c, int H, int W, int P, float* acc) {
    simt_main<F>(a, tile, m, r, c, H, W, P, acc);
  }
  template <int KC, int NC, int NCPAD>
  __device__ void chain(const OpArgs& a, int m, const float* in, float* out) {
    simt_chain<KC, NC>(a.chain, in, out);
  }
  __device__ void end() {}
  __device__ bool aborted() const { return false; }
};

template <int F>
struct Engine<F, true> {
  TcSmem* s;
  TcState* st;
  __device__ void main(const OpArgs& a, int64_t tile, int m, int r, int c, int H, int W, int P, float* acc) {
    tc_main<F>(a, *s, *st, tile, m, r, c, H, W, P, acc);
  }
  template <int KC, int NC, int NCPAD>
  __device__ void chain(const OpArgs& a, int m, const float* in, float* out) {
    tc_chain<KC, NCPAD>(*s, *st, m, in, out);
  }
  __device__ void end() { tc_op_end(); }
  __device__ bool aborted() const { return st->abort; }
};

// Runs one op at pixel (r, c) of `tile`. For the final C op returns the head
// output in *head (valid for every thread).
template <int F, bool TC, typename T>
__device__ void run_op(const OpArgs& a, Engine<F, TC>& eng, int64_t tile, int r, int c, int H, int W, int P,
                       HeadOut* head, int head_mask = -1) {
  const int m = threadIdx.x;
  float acc[F];
  eng.main(a, tile, m, r, c, H, W, P, acc);
  if (eng.aborted()) return;
  const float* bm = a.main.b;
  const float* bc = a.chain.b;
  const int pix = r * W + c;
  constexpr int F2 = F / 2;
  constexpr int NC2 = F2 < 16 ? 16 : F2;
  if (a.kind == kConvV) {
#pragma unroll
    for (int n = 0; n < F; ++n) acc[n] += __ldg(bm + n);
    if (a.stream_out) {
      float o[F];
      if (a.res) {
        load_row(blk<T>(a.res, tile, P, pix, F), m, 0, F, o);
#pragma unroll
        for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
      } else {
#pragma unroll
        for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
      }
      store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, o);
    }
#pragma unroll
    for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n], 0.f);
    if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, acc);
    float u[NC2];
    eng.template chain<F, F2, NC2>(a, m, acc, u);
    if (eng.aborted()) return;
#pragma unroll
    for (int n = 0; n < F2; ++n) u[n] = fmaxf(u[n] + __ldg(bc + n), 0.f);
    if (r + 1 < H) store_row(blk<T>(a.cat, tile, P, pix + W, F), m, F2, F2, u);
    if (r == 0) {
#pragma unroll
      for (int n = 0; n < F2; ++n) u[n] = fmaxf(__ldg(bc + n), 0.f);
      store_row(blk<T>(a.cat, tile, P, c, F), m, F2, F2, u);
    }
  } else if (a.kind == kConvH) {
#pragma unroll
    for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n] + __ldg(bm + n), 0.f);
    if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, acc);
    float z[NC2];
    eng.template chain<F, F2, NC2>(a, m, acc, z);
    if (eng.aborted()) return;
#pragma unroll
    for (int n = 0; n < F2; ++n) z[n] = fmaxf(z[n] + __ldg(bc + n), 0.f);
    const int sh = a.last ? 1 : 0;
    if (c + sh < W) store_row(blk<T>(a.cat, tile, P, pix + sh, F), m, 0, F2, z);
    if (sh && c == 0) {
#pragma unroll
      for (int n = 0; n < F2; ++n) z[n] = fmaxf(__ldg(bc + n), 0.f);
      store_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F2, z);
    }
  } else {
#pragma unroll
    for (int n = 0; n < F; ++n) acc[n] += __ldg(bm + n);
    if (!a.last) {
      float o[F];
      if (a.res) {
        load_row(blk<T>(a.res, tile, P, pix, F), m, 0, F, o);
#pragma unroll
        for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
      } else {
#pragma unroll
        for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
      }
      store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, o);
    } else {
#pragma unroll
      for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n], 0.f);
      if (a.stream_out) store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, acc);
      float l[16];
      eng.template chain<F, 4, 16>(a, m, acc, l);
      if (eng.aborted()) return;
#pragma unroll
      for (int n = 0; n < 4; ++n) l[n] += __ldg(bc + n);
      if (head_mask < 0) {
        const int64_t sample = tile * kTile + m;
        head_mask = (a.updown && sample < a.batch) ? a.updown[sample * P + pix] : 0;
      }
      *head = normalise_head(l, head_mask);
    }
  }
  eng.end();
}

// ============================================================== forward kernel
// Grid: one CTA per (tile, row); the CTA walks the row's pixels.
template <int F, bool TC>
__global__ void __launch_bounds__(128) op_row_kernel(const __grid_constant__ OpArgs a, int H, int W, int* err) {
  using T = typename std::conditional<TC, tc16, float>::type;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int P = H * W;
  int64_t item = blockIdx.x;
  if (a.items) {
    if ((int)blockIdx.x >= *a.n_items) return;
    item = a.items[blockIdx.x];
  }
  const int64_t tile = item / H;
  const int r = (int)(item % H);
  TcSmem s;
  TcState st;
  if (TC) {
    tc_carve<F>(smem, s);
    tc_setup(s, st, err);
  }
  Engine<F, TC> eng{&s, &st};
  const int m = threadIdx.x;
  const int64_t sample = tile * kTile + m;
  Kahan kre, kim;
  for (int c = 0; c < W; ++c) {
    HeadOut h;
    run_op<F, TC, T>(a, eng, tile, r, c, H, W, P, &h);
    if (eng.aborted()) break;
    if (a.kind == kConvC && a.last) {
      int pix = r * W + c;
      float s0 = spin_at(a.spins, a.batch, P, sample, pix);
      bool up = s0 > 0.f;
      kre.add(up ? h.re0 : h.re1);
      kim.add(up ? h.im0 : h.im1);
      if (a.cond && sample < a.batch) {
        reinterpret_cast<float4*>(a.cond)[sample * P + pix] = make_float4(h.re0, h.re1, h.im0, h.im1);
      }
    }
  }
  if (a.kind == kConvC && a.last && !eng.aborted()) {
    a.row_partial[((int64_t)tile * H + r) * kTile + m] = make_float2(kre.s - kre.c, kim.s - kim.c);
  }
  if (TC) tc_teardown(st);
}

// log psi = compensated sum over rows of the row partials (same order in the
// forward and in the sampler, so both give bitwise the same value).
__global__ void row_reduce_kernel(const float2* __restrict__ part, int64_t batch, int H, float2* __restrict__ out) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  int64_t tile = b / kTile;
  int m = (int)(b % kTile);
  Kahan re, im;
  for (int r = 0; r < H; ++r) {
    float2 p = part[((int64_t)tile * H + r) * kTile + m];
    re.add(p.x);
    im.add(p.y);
  }
  out[b] = make_float2(re.s - re.c, im.s - im.c);
}

// ============================================================== first causal conv, one row at a time
// The V and H ops of the first causal conv (input: the spin lattice, K = taps
// <= 16) for all W pixels of one (tile, row) together: the W main MMAs are
// issued at once, then the W chained MMAs, so a row costs three round trips
// instead of three per pixel. Per pixel the MMA operands, the MMA sequence
// and the epilogue arithmetic are those of run_op on the per-pixel engine:
// the results are bitwise the same.
template <int F>
struct FirstCfg {
  static constexpr int kNC = (F / 2) < 16 ? 16 : (F / 2);  // chained N (padded)
  static int smem(int W) {
    const int a = W * 2 * kTile * 16;        // A rows [W][2][128][8]
    const int ca = W * kTile * F * 2;        // chained inputs [W][F/8][128][8] (reuse A)
    return (a > ca ? a : ca) + 2 * F * 16 + F * kNC * 2 + 64;
  }
};

template <int F>
__global__ void __launch_bounds__(128) first_row_kernel(const __grid_constant__ OpArgs a, int H, int W, int* err) {
  using C = FirstCfg<F>;
  using T = tc16;
  constexpr int F2 = F / 2;
  constexpr int NC = C::kNC;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int P = H * W;
  int64_t item = blockIdx.x;
  if (a.items) {
    if ((int)blockIdx.x >= *a.n_items) return;
    item = a.items[blockIdx.x];
  }
  const int64_t tile = item / H;
  const int r = (int)(item % H);
  const int m = threadIdx.x;
  const int ab = W * 2 * kTile * 16, cab = W * kTile * F * 2;
  uint8_t* abuf = smem;                                  // A rows, then chained inputs
  uint8_t* wsm = smem + (ab > cab ? ab : cab);           // main weights [2][F][8]
  uint8_t* cwsm = wsm + 2 * F * 16;                      // chained weights [F/8][NC][8]
  uint64_t* bar = reinterpret_cast<uint64_t*>(cwsm + F * NC * 2);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 2);
  const uint32_t wbytes = 2 * F * 16, cbytes = F * NC * 2;
  if (m == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  // TMEM: W accumulators of F columns (the chained ones reuse them), a power
  // of two >= 32 columns
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(W * F)) ncols *= 2;
  if (m < 32) {
    tmem_alloc(slot, ncols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  int* e = err;
  bool ok = true;
  if (m == 0) {
    mbar_arrive_expect_tx(&bar[0], wbytes + cbytes);
    bulk_g2s(wsm, a.main.w, wbytes, &bar[0]);
    bulk_g2s(cwsm, a.chain.w, cbytes, &bar[0]);
  }
  // thread m's K = 16 row per pixel (taps in kernel order, zero padded)
  for (int c = 0; c < W; ++c) {
    float v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = 0.f;
    const int nt = num_taps(a.kind);
    for (int t = 0; t < nt; ++t) {
      int dr, dc;
      tap_offset(a.kind, t, dr, dc);
      const int rr = r + dr, cc = c + dc;
      if (rr >= 0 && rr < H && cc >= 0 && cc < W) v[t] = spin_at(a.spins, a.batch, P, tile * kTile + m, rr * W + cc);
    }
    st8(reinterpret_cast<T*>(abuf + c * 4096 + m * 16), v);
    st8(reinterpret_cast<T*>(abuf + c * 4096 + 2048 + m * 16), v + 8);
  }
  fence_proxy_async_smem();
  __syncthreads();
  ok = mbar_wait(&bar[0], 0, e);
  if (m == 0 && ok) {
    tc_fence_after();
    const uint32_t idesc = umma_idesc_tc16(128, F);
    const uint64_t bd = umma_sdesc(smem_u32(wsm), F * 16, 128);
    for (int c = 0; c < W; ++c)
      umma_bf16(tmem + c * F, umma_sdesc(smem_u32(abuf + c * 4096), 2048, 128), bd, idesc, 0u);
    umma_commit(&bar[1]);
  }
  ok = ok && mbar_wait(&bar[1], 0, e);
  tc_fence_after();
  const float* bm = a.main.b;
  const float* bc = a.chain.b;
  // first halves; the A rows are dead, their memory holds the chained inputs
  if (ok) {
    for (int c = 0; c < W; ++c) {
      const int pix = r * W + c;
      float acc[F];
#pragma unroll
      for (int q = 0; q < F / 16; ++q) tmem_ld16(tmem + ((uint32_t)((m / 32) * 32) << 16) + c * F + q * 16, acc + q * 16);
      tmem_ld_wait();
      if (a.kind == kConvV) {
#pragma unroll
        for (int n = 0; n < F; ++n) acc[n] += __ldg(bm + n);
        if (a.stream_out) {
          float o[F];
          if (a.res) {
            load_row(blk<T>(a.res, tile, P, pix, F), m, 0, F, o);
#pragma unroll
            for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
          } else {
#pragma unroll
            for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
          }
          store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, o);
        }
#pragma unroll
        for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n], 0.f);
      } else {
#pragma unroll
        for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n] + __ldg(bm + n), 0.f);
      }
      if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, acc);
      T* ca = reinterpret_cast<T*>(abuf + c * (kTile * F * 2));
#pragma unroll
      for (int g = 0; g < F / 8; ++g) st8(ca + ((int64_t)g * kTile + m) * 8, acc + 8 * g);
    }
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (m == 0 && ok) {
    const uint32_t idesc = umma_idesc_tc16(128, NC);
    for (int c = 0; c < W; ++c) {
#pragma unroll
      for (int ks = 0; ks < F / 16; ++ks)
        umma_bf16(tmem + c * NC, umma_sdesc(smem_u32(abuf + c * (kTile * F * 2) + ks * 2 * 2048), 2048, 128),
                  umma_sdesc(smem_u32(cwsm + ks * 2 * NC * 16), NC * 16, 128), idesc, ks > 0 ? 1u : 0u);
    }
    umma_commit(&bar[1]);
  }
  ok = ok && mbar_wait(&bar[1], 1, e);
  tc_fence_after();
  if (ok) {
    for (int c = 0; c < W; ++c) {
      const int pix = r * W + c;
      float u[NC];
      tmem_ld16(tmem + ((uint32_t)((m / 32) * 32) << 16) + c * NC, u);
      tmem_ld_wait();
      if (a.kind == kConvV) {
#pragma unroll
        for (int n = 0; n < F2; ++n) u[n] = fmaxf(u[n] + __ldg(bc + n), 0.f);
        if (r + 1 < H) store_row(blk<T>(a.cat, tile, P, pix + W, F), m, F2, F2, u);
        if (r == 0) {
#pragma unroll
          for (int n = 0; n < F2; ++n) u[n] = fmaxf(__ldg(bc + n), 0.f);
          store_row(blk<T>(a.cat, tile, P, c, F), m, F2, F2, u);
        }
      } else {
#pragma unroll
        for (int n = 0; n < F2; ++n) u[n] = fmaxf(u[n] + __ldg(bc + n), 0.f);
        const int sh = a.last ? 1 : 0;
        if (c + sh < W) store_row(blk<T>(a.cat, tile, P, pix + sh, F), m, 0, F2, u);
        if (sh && c == 0) {
#pragma unroll
          for (int n = 0; n < F2; ++n) u[n] = fmaxf(__ldg(bc + n), 0.f);
          store_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F2, u);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (m < 32) {
    tc_fence_after();
    tmem_dealloc(tmem, ncols);
  }
}

// FK_ERR_ARG when the row kernel does not apply (the per-pixel engine runs).
template <int F>
static int launch_first_row(const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  if (!a.first || (a.kind != kConvV && a.kind != kConvH) || F > 32 || W * F > 512 ||
      W * FirstCfg<F>::kNC > 512)
    return FK_ERR_ARG;
  const int smem = FirstCfg<F>::smem(W);
  if (smem > 200 * 1024) return FK_ERR_ARG;
  static bool attr = false;
  if (!attr) {
    FK_CUDA(cudaFuncSetAttribute(first_row_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  first_row_kernel<F><<<(unsigned)(tiles * H), 128, smem, s>>>(a, H, W, err);
  return check_cuda(launched(), "first_row_kernel");
}

// ============================================================== op list
static ConvW convw(const NetLayout& L, const void* packed, int idx) {
  const ConvDesc& c = L.conv[idx];
  ConvW w;
  w.w = static_cast<const char*>(packed) + c.w_off;
  w.ws = c.ws_off >= 0 ? static_cast<const char*>(packed) + c.ws_off : nullptr;
  w.wt = c.wt_off >= 0 ? static_cast<const char*>(packed) + c.wt_off : nullptr;
  w.b = reinterpret_cast<const float*>(static_cast<const char*>(packed) + c.b_off);
  w.K = c.K;
  w.Npad = c.Npad;
  return w;
}

// The three ops of causal conv i with the given tensors.
static void make_ops(const NetLayout& L, const void* packed, int i, const int8_t* spins, int64_t batch,
                     const void* vin, const void* hin, const void* vres, const void* hres, void* vout, void* hout,
                     void* cat, void* t_aux, void* rv_aux, OpArgs ops[3]) {
  const bool first = i == 0, last = i == L.n_cc - 1;
  for (int k = 0; k < 3; ++k) {
    memset(&ops[k], 0, sizeof(OpArgs));
    ops[k].first = first;
    ops[k].last = last;
    ops[k].cin = first ? 1 : L.F;
    ops[k].spins = spins;
    ops[k].batch = batch;
    ops[k].cat = cat;
  }
  OpArgs& v = ops[0];
  v.kind = kConvV;
  v.in = vin;
  v.main = convw(L, packed, conv_index(i, kConvV));
  v.chain = convw(L, packed, conv_index(i, kConvY));
  v.res = vres;
  v.stream_out = last ? nullptr : vout;
  v.aux_out = rv_aux;
  OpArgs& h = ops[1];
  h.kind = kConvH;
  h.in = hin;
  h.main = convw(L, packed, conv_index(i, kConvH));
  h.chain = convw(L, packed, conv_index(i, kConvX));
  h.aux_out = t_aux;
  OpArgs& c = ops[2];
  c.kind = kConvC;
  c.first = 0;  // the combine conv always reads the F-channel concat
  c.cin = L.F;
  c.in = cat;
  c.main = convw(L, packed, conv_index(i, kConvC));
  if (last) c.chain = convw(L, packed, L.n_convs - 1);
  c.res = hres;
  c.stream_out = hout;
}

// Input/output tensors of causal conv i in the two workspace modes.
struct CCTensors {
  const void *vin, *hin, *vres, *hres;
  void *vout, *hout, *cat, *t, *rv;
};

static CCTensors cc_tensors(const NetLayout& L, const Tensors& T, int mode, int i) {
  CCTensors x;
  memset(&x, 0, sizeof(x));
  const bool last = i == L.n_cc - 1;
  // residual: the second conv of block b (i = 2b+2) adds the block input S_{2b}
  const bool second = (i >= 2) && (i % 2 == 0) && !last;
  if (mode == FK_AR2D_SAVE) {
    x.vin = i == 0 ? nullptr : T.v[i - 1];
    x.hin = i == 0 ? nullptr : T.h[i - 1];
    x.vres = second ? T.v[i - 2] : nullptr;
    x.hres = second ? T.h[i - 2] : nullptr;
    x.vout = T.v[i];
    x.hout = T.h[i];
    x.cat = T.cat[i];
    x.t = T.t[i];
    x.rv = T.rv[i];
  } else {
    // ping-pong: S_i lives in slot (i % 2) except that block outputs return to
    // the block input's slot: S_{2b+2} overwrites S_{2b} in place (residual read
    // and write happen at the same pixel by the same thread).
    auto slot = [&](int j) { return (j == 0) ? 0 : ((j % 2 == 1) ? 1 : 0); };
    x.vin = i == 0 ? nullptr : T.v[slot(i - 1)];
    x.hin = i == 0 ? nullptr : T.h[slot(i - 1)];
    x.vres = second ? T.v[slot(i - 2)] : nullptr;
    x.hres = second ? T.h[slot(i - 2)] : nullptr;
    x.vout = T.v[slot(i)];
    x.hout = last ? nullptr : T.h[slot(i)];
    x.cat = T.cat[0];
  }
  return x;
}

template <int F, bool TC>
static int launch_op(const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  size_t smem = TC ? (size_t)TcCfg<F>::kSmem : 0;
  if (TC) {
    static bool attr_set = false;
    if (!attr_set) {
      FK_CUDA(cudaFuncSetAttribute(op_row_kernel<F, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)TcCfg<F>::kSmem));
      attr_set = true;
    }
  }
  op_row_kernel<F, TC><<<(unsigned)(tiles * H), 128, smem, s>>>(a, H, W, err);
  return check_cuda(launched(), "op_row_kernel");
}

// FK_AR2D_ENGINE=rowwise selects the per-pixel engine for every op (the
// pipelined engine computes bitwise the same values; the switch lets tests
// compare the two).
static bool use_pipe_engine() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("FK_AR2D_ENGINE");
    v = (e && strcmp(e, "rowwise") == 0) ? 0 : 1;
  }
  return v == 1;
}

// One op on the fastest engine that applies: the pipelined engine (ops after
// the first conv), the row kernel (first conv), else the per-pixel engine.
template <int F, bool TC>
static int run_engine_op(const OpArgs& op, int64_t tiles, const NetLayout& L, int* err, cudaStream_t s) {
  if (TC && use_pipe_engine()) {
    if (!op.first && pipe_supported(F, L.W)) return launch_pipe_op(F, op, tiles, L.H, L.W, err, s);
    if (op.first) {
      const int st = launch_first_row<F>(op, tiles, L.H, L.W, err, s);
      if (st != FK_ERR_ARG) return st;
    }
  }
  return launch_op<F, TC>(op, tiles, L.H, L.W, err, s);
}

template <int F, bool TC>
static int forward_impl(const NetLayout& L, const void* packed, const int8_t* spins, int64_t batch,
                        float* log_psi, float* cond, const Tensors& T, int mode, cudaStream_t s) {
  int64_t tiles = (batch + kTile - 1) / kTile;
  int* err = device_error_word();
  if (L.updown) {
    updown_mask_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, s>>>(spins, batch, L.P, T.updown);
    FK_CUDA(launched());
  }
  for (int i = 0; i < L.n_cc; ++i) {
    CCTensors x = cc_tensors(L, T, mode, i);
    OpArgs ops[3];
    make_ops(L, packed, i, spins, batch, x.vin, x.hin, x.vres, x.hres, x.vout, x.hout, x.cat, x.t, x.rv, ops);
    if (i == L.n_cc - 1) {
      ops[2].row_partial = T.row_partial;
      ops[2].cond = cond;
      ops[2].updown = T.updown;
    }
    for (int k = 0; k < 3; ++k) {
      int st;
      st = run_engine_op<F, TC>(ops[k], tiles, L, err, s);
      if (st != FK_OK) return st;
    }
  }
  row_reduce_kernel<<<(unsigned)((batch + 255) / 256), 256, 0, s>>>(T.row_partial, batch, L.H,
                                                                    reinterpret_cast<float2*>(log_psi));
  return check_cuda(launched(), "row_reduce_kernel");
}

// ============================================================== sampler
// One persistent CTA per tile walks the sites in raster order:
//   start : Cat_i[0, :][F/2:F] = relu(b_y,i) for all i; Cat_last[:, 0][0:F/2] = relu(b_x,last)
//   site (r, c):  head at (r, c) -> draw s(r, c)
//                 for i < last: H op_i (r, c), C op_i (r, c);  H op_last (r, c)
//   end of row r: for every i: V op_i over (r, 0..W-1)
// Every (layer, pixel) is evaluated once, after all the sites it depends on.
// ---- exact sampler on tensor cores (F <= 32)
// Op record of the sampler, copied from the kernel parameters into shared
// memory at kernel start (the ops of a site cycle through more parameter data
// than the constant cache holds).
struct SampOp {
  const void* in;
  const void* w;    // main weights (V: the column-scatter operand)
  const void* cw;   // chained 1x1 weights
  const float* b;   // main bias
  const float* cb;  // chained bias
  void* out;        // stream output
  void* aux;        // saved activation
  void* cat;
  const void* res;
  int kind;
  int flags;  // 1: first causal conv, 2: last causal conv
  __device__ bool first() const { return flags & 1; }
  __device__ bool last() const { return (flags >> 1) & 1; }
};
static_assert(sizeof(SampOp) == 80, "sampler op record");

__device__ __forceinline__ void samp_op_from(const OpArgs& a, SampOp& o) {
  o.in = a.in;
  o.w = a.kind == kConvV ? a.main.ws : a.main.w;
  o.cw = a.chain.w;
  o.b = a.main.b;
  o.cb = a.chain.b;
  o.out = a.stream_out;
  o.aux = a.aux_out;
  o.cat = a.cat;
  o.res = a.res;
  o.kind = a.kind;
  o.flags = (a.first ? 1 : 0) | (a.last ? 2 : 0);
}

// Shared memory of the sampler kernel: a ring of 18 activation blocks (C taps
// in slots 0..8 during sites; the column ring, residual and chained inputs of
// the row-end V ops), main / chained weights, the chained-input block, the H
// buffer set, the residual block and the barriers.
template <int F>
struct SiteCfg {
  static constexpr int kBlk = kTile * F * 2;
  static constexpr int kSlice = F * F * 2;
  static constexpr int kNC = (F / 2) < 16 ? 16 : (F / 2);
  static constexpr int kRingBlocks = 18;
  static constexpr int kVSlots = kRingBlocks / 3;  // input columns of a V row op in flight
  static constexpr int kW = kRingBlocks * kBlk;     // 9 tap slices = the column-scatter operand
  static constexpr int kCW = kW + 9 * kSlice;
  static constexpr int kCA = kCW + F * 32 * 2;
  static constexpr int kAH = kCA + kBlk;
  static constexpr int kWH = kAH + 3 * kBlk;
  static constexpr int kCWH = kWH + 3 * kSlice;
  static constexpr int kRes = kCWH + F * kNC * 2;
  static constexpr int kBar = kRes + kBlk;
  static constexpr int kOps = kBar + 256;  // SampOp[3 * 40]
  static constexpr int kSmem = kOps + 3 * 40 * (int)sizeof(SampOp);
};
static_assert(SiteCfg<32>::kSmem <= 227 * 1024, "sampler shared memory");

// The V op of one causal conv (after the first) over a whole lattice row of
// one tile, inside the sampler: the column-scatter MMAs of the pipelined
// engine (input column x times the three stacked kernel columns into the
// TMEM accumulators of outputs x-1..x+1, same order: columns ascending,
// kernel rows ascending, K steps ascending), then the run_op epilogue per
// output and the chained 1x1 MMAs in groups of 9 outputs. Bitwise equal to the
// per-pixel and pipelined engines; one pass instead of W sequential ops.
// Input columns stream through a ring of kVSlots slots; TMEM columns
// [0, W*F). Barriers are initialised per call and invalidated at its end;
// every arrival on them is waited for (an MMA commit arrives on its barrier
// some time after the commit that follows it may have been observed).
template <int F>
__device__ bool v_row_op(const SampOp& a, TcSmem& s, TcState& st, int64_t tile, int r, int H, int W) {
  using T = tc16;
  using SC = SiteCfg<F>;
  constexpr int F2 = F / 2;
  constexpr int NC = SC::kNC;
  constexpr int NSL = SC::kVSlots;
  constexpr int kBlk = SC::kBlk;
  constexpr uint32_t kBlk16 = kBlk >> 4, kWRow16 = (F * 3 * F * 2) >> 4;
  constexpr uint32_t kKs16 = (2 * 2048) >> 4, kKsW16 = (2 * 3 * F * 16) >> 4;
  const int P = H * W;
  const int m = threadIdx.x;
  uint64_t* full = s.vbar;          // [NSL] column loaded
  uint64_t* mdone = s.vbar + NSL;   // [NSL] MMAs of the column in the slot done
  uint64_t* done = s.vbar + 2 * NSL;  // all MMAs done
  if (m == 0) {
    for (int i = 0; i < 2 * NSL + 1; ++i) mbar_init(&s.vbar[i], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int k_lo = 2 - r > 0 ? 2 - r : 0;
  auto load_col = [&](int x) {
    const int sl = x % NSL;
    mbar_arrive_expect_tx(&full[sl], (uint32_t)(3 - k_lo) * kBlk);
    for (int k = k_lo; k < 3; ++k)
      bulk_g2s(s.a_ptr + (sl * 3 + k) * kBlk, blk<T>(a.in, tile, P, (r - 2 + k) * W + x, F), kBlk, &full[sl]);
  };
  const uint32_t wbytes = 3 * F * 3 * F * 2, cbytes = F * NC * 2;
  if (m == 0) {
    mbar_arrive_expect_tx(s.bar_load, wbytes + cbytes);
    bulk_g2s(s.w_ptr, a.w, wbytes, s.bar_load);
    bulk_g2s(s.cw_ptr, a.cw, cbytes, s.bar_load);
    for (int x = 0; x < W && x < NSL - 1; ++x) load_col(x);
  }
  if (!tc_wait(s.bar_load, st.ph_load, st)) return false;
  const uint64_t a0 = umma_sdesc(s.a, 2048, 128);
  const uint64_t w0 = umma_sdesc(s.w, 3 * F * 16, 128);
  const uint32_t idesc1 = umma_idesc_tc16(128, F), idesc2 = umma_idesc_tc16(128, 2 * F),
                 idesc3 = umma_idesc_tc16(128, 3 * F);
  bool ok = true;
  for (int x = 0; x < W && ok && m == 0; ++x) {
    const int sl = x % NSL;
    ok = mbar_wait(&full[sl], (uint32_t)(x / NSL) & 1, st.err);
    if (ok) {
      tc_fence_after();
      const int c_lo = x - 1 < 0 ? 0 : x - 1;
      const int c_hi = x + 1 < W - 1 ? x + 1 : W - 1;
      const int c_f = x == 0 ? c_lo : (x + 1 < c_hi + 1 ? x + 1 : c_hi + 1);
      bool first = true;
      for (int k = k_lo; k < 3; ++k) {
#pragma unroll
        for (int ks = 0; ks < F / 16; ++ks) {
          const uint64_t ad = a0 + (uint32_t)(sl * 3 + k) * kBlk16 + ks * kKs16;
          const uint64_t bd = w0 + (uint32_t)k * kWRow16 + ks * kKsW16;
          auto mma = [&](int ca, int cb, uint32_t acc) {
            if (ca > cb) return;
            const int n = cb - ca + 1;
            umma_bf16(st.tmem + ca * F, ad, bd + (uint32_t)((ca - x + 1) * F),
                      n == 3 ? idesc3 : (n == 2 ? idesc2 : idesc1), acc);
          };
          if (first) {
            mma(c_lo, c_f - 1, 1u);
            mma(c_f, c_hi, 0u);
            first = false;
          } else {
            mma(c_lo, c_hi, 1u);
          }
        }
      }
      // only columns whose slot is refilled signal it: every arrival is waited for
      if (x + NSL < W) umma_commit(&mdone[sl]);
    }
    // the slot of column x+NSL-1 is free once the MMAs of column x-1 completed
    if (ok && x + NSL - 1 < W) {
      if (x >= 1) ok = mbar_wait(&mdone[(x - 1) % NSL], (uint32_t)((x - 1) / NSL) & 1, st.err);
      if (ok) load_col(x + NSL - 1);
    }
  }
  if (m == 0 && ok) umma_commit(done);
  if (__syncthreads_or(m == 0 && !ok)) {
    st.abort = true;
    return false;
  }
  uint32_t ph_done = 0;
  if (!tc_wait(done, ph_done, st)) return false;
  if (m == 0)
    for (int i = 0; i < 2 * NSL + 1; ++i) mbar_inval(&s.vbar[i]);
  tc_fence_after();
  const float* bm = a.b;
  const float* bc = a.cb;
  const bool need_res = a.out && a.res;
  // ring blocks [0, 9): residual rows of a group; [9, 18): its chained inputs
  constexpr int kChunk = 9;
  for (int c0 = 0; c0 < W; c0 += kChunk) {
    const int c1 = c0 + kChunk < W ? c0 + kChunk : W;
    if (need_res) {
      if (m == 0) {
        mbar_arrive_expect_tx(s.bar_load, (uint32_t)(c1 - c0) * kBlk);
        bulk_g2s(s.a_ptr, blk<T>(a.res, tile, P, r * W + c0, F), (uint32_t)(c1 - c0) * kBlk, s.bar_load);
      }
      if (!tc_wait(s.bar_load, st.ph_load, st)) return false;
    }
    for (int c = c0; c < c1; ++c) {
      const int pix = r * W + c;
      float acc[F];
#pragma unroll
      for (int q = 0; q < F / 16; ++q)
        tmem_ld16(st.tmem + ((uint32_t)((m / 32) * 32) << 16) + c * F + q * 16, acc + q * 16);
      tmem_ld_wait();
#pragma unroll
      for (int n = 0; n < F; ++n) acc[n] += __ldg(bm + n);
      if (a.out) {
        float o[F];
        if (a.res) {
          load_row(reinterpret_cast<const T*>(s.a_ptr + (c - c0) * kBlk), m, 0, F, o);
#pragma unroll
          for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
        } else {
#pragma unroll
          for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
        }
        store_row(blk<T>(a.out, tile, P, pix, F), m, 0, F, o);
      }
#pragma unroll
      for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n], 0.f);
      if (a.aux) store_row(blk<T>(a.aux, tile, P, pix, F), m, 0, F, acc);
      T* ca = reinterpret_cast<T*>(s.a_ptr + (kChunk + c - c0) * kBlk);
#pragma unroll
      for (int g = 0; g < F / 8; ++g) st8(ca + ((int64_t)g * kTile + m) * 8, acc + 8 * g);
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (m == 0) {
      const uint32_t idesc = umma_idesc_tc16(128, NC);
      for (int c = c0; c < c1; ++c) {
#pragma unroll
        for (int ks = 0; ks < F / 16; ++ks)
          umma_bf16(st.tmem + c * F, umma_sdesc(s.a + (kChunk + c - c0) * kBlk + ks * 2 * 2048, 2048, 128),
                    umma_sdesc(s.cw + ks * 2 * NC * 16, NC * 16, 128), idesc, ks > 0 ? 1u : 0u);
      }
      umma_commit(s.bar_mma);
    }
    if (!tc_wait(s.bar_mma, st.ph_mma, st)) return false;
    tc_fence_after();
    for (int c = c0; c < c1; ++c) {
      float u[NC];
      tmem_ld16(st.tmem + ((uint32_t)((m / 32) * 32) << 16) + c * F, u);
      tmem_ld_wait();
#pragma unroll
      for (int n = 0; n < F2; ++n) u[n] = fmaxf(u[n] + __ldg(bc + n), 0.f);
      if (r + 1 < H) store_row(blk<T>(a.cat, tile, P, (r + 1) * W + c, F), m, F2, F2, u);
      if (r == 0) {
#pragma unroll
        for (int n = 0; n < F2; ++n) u[n] = fmaxf(__ldg(bc + n), 0.f);
        store_row(blk<T>(a.cat, tile, P, c, F), m, F2, F2, u);
      }
    }
    // the ring blocks of this group are reused by the next group's copies
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
  tc_op_end();
  return true;
}

// The ops of one site: the head C of the last causal conv at (r, c), then H
// and C of causal convs 0..L-1, then H of conv L (H ops use the H buffer set,
// C ops ring slots 0..8). While op k's MMAs run, another thread copies op
// k+1's weights and its taps written at earlier sites into the other set; the
// tap op k itself produces (H: the x-half of Cat at the next C op's pixel; C:
// the stream output the next H reads at (r, c)) is written by op k's
// epilogue straight into op k+1's buffer, besides global memory, and the
// residual of a C op comes from the shared-memory block where the C op two
// convs earlier left its output. Taps sit in slot t = 3 (dr + 2) + (dc + 2)
// (H: dc + 2), so an op's own pixel is slot 8 (H: 2). MMA order and roundings
// are those of the per-pixel engine (column-major taps, K steps of 16): sampled
// configurations and log psi are bitwise equal to the forward's. Global
// stores are made visible to the copy engine once per site: no op copies a
// tap written at its own site.
struct SiteBufs {
  uint8_t* ah;   // H taps (3 blocks)
  uint8_t* wh;   // H weight slices (3)
  uint8_t* cwh;  // H chained 1x1 weights
  uint8_t* res;  // residual block
  uint64_t* bar_h;
  uint32_t ph_h;
  const int8_t* spins;
  int64_t batch;
};

// One thread: copies of op `a` at (r, c) into its buffer set, all but the
// op's own pixel (C: its y-half is copied, the x-half comes from the H op).
template <int F>
__device__ void site_prefetch(const SampOp& a, TcSmem& s, SiteBufs& b, int64_t tile, int r, int c, int H, int W,
                              bool own_full = false) {
  using SC = SiteCfg<F>;
  using T = tc16;
  const int P = H * W;
  const bool isC = a.kind == kConvC;
  uint64_t* bar = isC ? s.bar_load : b.bar_h;
  const uint32_t chain_bytes = F * (isC ? 16 : SC::kNC) * 2;
  const bool has_chain = !isC || a.last();
  if (a.first()) {
    mbar_arrive_expect_tx(bar, 2 * F * 16 + chain_bytes);
    bulk_g2s(b.wh, a.w, 2 * F * 16, bar);
    bulk_g2s(b.cwh, a.cw, chain_bytes, bar);
    return;
  }
  const int j_lo = c >= 2 ? 0 : 2 - c;  // first tap column in the lattice
  const int k_lo = isC ? (r >= 2 ? 0 : 2 - r) : 2;
  const int nk = isC ? 3 : 1;
  uint8_t* A = isC ? s.a_ptr : b.ah;
  const uint32_t full_row = (uint32_t)(3 - j_lo) * SC::kBlk;
  const uint32_t own_row = own_full ? full_row : full_row - SC::kBlk;
  uint32_t bytes = (uint32_t)nk * SC::kSlice * 3 + (has_chain ? chain_bytes : 0);
  bytes += (uint32_t)(3 - k_lo - 1) * full_row + own_row + ((isC && !own_full) ? SC::kBlk / 2 : 0);
  mbar_arrive_expect_tx(bar, bytes);
  for (int k = k_lo; k < 3; ++k) {
    const int slot = isC ? k * 3 + j_lo : j_lo;
    const T* src = blk<T>(a.in, tile, P, (r - 2 + k) * W + c - 2 + j_lo, F);
    const uint32_t n = k < 2 ? full_row : own_row;
    if (n) bulk_g2s(A + slot * SC::kBlk, src, n, bar);
  }
  if (isC && !own_full) {
    const char* own = reinterpret_cast<const char*>(blk<T>(a.in, tile, P, r * W + c, F));
    bulk_g2s(A + 8 * SC::kBlk + SC::kBlk / 2, own + SC::kBlk / 2, SC::kBlk / 2, bar);
  }
  bulk_g2s(isC ? s.w_ptr : b.wh, a.w, (uint32_t)nk * 3 * SC::kSlice, bar);
  if (has_chain) bulk_g2s(isC ? s.cw_ptr : b.cwh, a.cw, chain_bytes, bar);
}

// Chained 1x1 conv on tensor cores with its weights at shared address cw.
template <int KC, int NCPAD>
__device__ bool site_chain(TcSmem& s, TcState& st, uint32_t cw, const float* in, float* out) {
  const int m = threadIdx.x;
  tc16* ca = reinterpret_cast<tc16*>(s.ca_ptr);
#pragma unroll
  for (int g = 0; g < KC / 8; ++g) st8(ca + ((int64_t)g * kTile + m) * 8, in + 8 * g);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  if (m == 0) {
    tc_fence_after();
    const uint32_t idesc = umma_idesc_tc16(128, NCPAD);
#pragma unroll
    for (int ks = 0; ks < KC / 16; ++ks)
      umma_bf16(st.tmem + kChainCol, umma_sdesc(s.ca + ks * 2 * 2048, 2048, 128),
                umma_sdesc(cw + ks * 2 * NCPAD * 16, NCPAD * 16, 128), idesc, ks > 0 ? 1u : 0u);
    umma_commit(s.bar_mma);
  }
  if (!tc_wait(s.bar_mma, st.ph_mma, st)) return false;
  tc_fence_after();
  tc_read<NCPAD>(st, kChainCol, out);
  return true;
}

// Op `a` at (r, c) from its buffer set, the run_op epilogue, and (thread 32)
// the copies of the next op `nx` at (r, nc). keep_res: the C output is the
// residual of the C op two convs later. site_end: last op of the site.
template <int F>
__device__ bool site_op(const SampOp& a, TcSmem& s, TcState& st, SiteBufs& b, int64_t tile, int r, int c, int H,
                        int W, const SampOp* nx, int nc, bool keep_res, bool site_end, HeadOut* head,
                        int head_mask) {
  using SC = SiteCfg<F>;
  using T = tc16;
  constexpr int F2 = F / 2;
  constexpr int NC2 = SC::kNC;
  const int P = H * W;
  const int m = threadIdx.x;
  const bool isC = a.kind == kConvC;
  uint8_t* A = isC ? s.a_ptr : b.ah;
  uint8_t* Wt = isC ? s.w_ptr : b.wh;
  if (a.first()) {
    // cin = 1: the K = 16 row of spins at the H taps (zero padded)
    float v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = 0.f;
    for (int t = 0; t < 3; ++t) {
      int dr, dc;
      tap_offset(a.kind, t, dr, dc);
      const int rr = r + dr, cc = c + dc;
      if (rr >= 0 && rr < H && cc >= 0 && cc < W) v[t] = spin_at(b.spins, b.batch, P, tile * kTile + m, rr * W + cc);
    }
    st8(reinterpret_cast<T*>(A + m * 16), v);
    st8(reinterpret_cast<T*>(A + 2048 + m * 16), v + 8);
    fence_proxy_async_smem();
    __syncthreads();
  }
  if (!tc_wait(isC ? s.bar_load : b.bar_h, isC ? st.ph_load : b.ph_h, st)) return false;
  if (m == 0) {
    tc_fence_after();
    const uint64_t a0 = umma_sdesc(smem_u32(A), 2048, 128);
    const uint64_t w0 = umma_sdesc(smem_u32(Wt), F * 16, 128);
    const uint32_t idesc = umma_idesc_tc16(128, F);
    if (a.first()) {
      umma_bf16(st.tmem, a0, w0, idesc, 0u);
    } else {
      // column-major taps: tap column j outer, tap row k inner
      const int j_lo = c >= 2 ? 0 : 2 - c;
      const int k_lo = isC ? (r >= 2 ? 0 : 2 - r) : 2;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (j < j_lo || k < k_lo || (!isC && k < 2)) continue;
          const uint32_t t = isC ? (uint32_t)(k * 3 + j) : (uint32_t)j;
#pragma unroll
          for (int ks = 0; ks < F / 16; ++ks)
            umma_bf16(st.tmem, a0 + ((t * SC::kBlk + ks * 4096) >> 4), w0 + ((t * SC::kSlice + ks * 2 * F * 16) >> 4),
                      idesc, (j > j_lo || k > k_lo || ks > 0) ? 1u : 0u);
        }
      }
    }
    umma_commit(s.bar_mma);
  }
  if (m == 32 && nx) site_prefetch<F>(*nx, s, b, tile, r, nc, H, W);
  if (!tc_wait(s.bar_mma, st.ph_mma, st)) return false;
  tc_fence_after();
  float acc[F];
  tc_read<F>(st, 0, acc);
  const float* bm = a.b;
  const float* bc = a.cb;
  const int pix = r * W + c;
  if (!isC) {
#pragma unroll
    for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n] + __ldg(bm + n), 0.f);
    if (a.aux) store_row(blk<T>(a.aux, tile, P, pix, F), m, 0, F, acc);
    float z[NC2];
    if (!site_chain<F, NC2>(s, st, smem_u32(b.cwh), acc, z)) return false;
#pragma unroll
    for (int n = 0; n < F2; ++n) z[n] = fmaxf(z[n] + __ldg(bc + n), 0.f);
    const int sh = a.last() ? 1 : 0;
    if (c + sh < W) {
      store_row(blk<T>(a.cat, tile, P, pix + sh, F), m, 0, F2, z);
      // x-half of the next C op's own pixel (r, c + sh)
      store_row(reinterpret_cast<T*>(s.a_ptr + 8 * SC::kBlk), m, 0, F2, z);
    }
    if (sh && c == 0) {
#pragma unroll
      for (int n = 0; n < F2; ++n) z[n] = fmaxf(__ldg(bc + n), 0.f);
      store_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F2, z);
    }
  } else {
#pragma unroll
    for (int n = 0; n < F; ++n) acc[n] += __ldg(bm + n);
    if (!a.last()) {
      float o[F];
      if (a.res) {
        load_row(reinterpret_cast<const T*>(b.res), m, 0, F, o);
#pragma unroll
        for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
      } else {
#pragma unroll
        for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
      }
      store_row(blk<T>(a.out, tile, P, pix, F), m, 0, F, o);
      // the next H op's own pixel, and the residual of a later C op
      store_row(reinterpret_cast<T*>(b.ah + 2 * SC::kBlk), m, 0, F, o);
      if (keep_res) store_row(reinterpret_cast<T*>(b.res), m, 0, F, o);
    } else {
#pragma unroll
      for (int n = 0; n < F; ++n) acc[n] = fmaxf(acc[n], 0.f);
      if (a.out) store_row(blk<T>(a.out, tile, P, pix, F), m, 0, F, acc);
      float l[16];
      if (!site_chain<F, 16>(s, st, s.cw, acc, l)) return false;
#pragma unroll
      for (int n = 0; n < 4; ++n) l[n] += __ldg(bc + n);
      *head = normalise_head(l, head_mask);
    }
  }
  if (site_end)
    asm volatile("fence.proxy.async;" ::: "memory");
  else
    fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return true;
}

struct SampleArgs {
  OpArgs op[40][3];
  int n_cc;
  int64_t batch;
  uint32_t seed_lo, seed_hi, off_lo, off_hi;
  int8_t* spins;
  float2* row_partial;
  uint64_t keep_res;  // bit i: the C output of causal conv i is the residual of conv i + 2
  int updown;         // EqualUpDownSpins mask from the running counts of drawn spins
};

template <int F, bool TC>
__global__ void __launch_bounds__(128) sample_kernel(const __grid_constant__ SampleArgs a, int H, int W, int* err) {
  using T = typename std::conditional<TC, tc16, float>::type;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int P = H * W;
  const int64_t tile = blockIdx.x;
  const int m = threadIdx.x;
  const int64_t sample = tile * kTile + m;
  const int last = a.n_cc - 1;
  constexpr int F2 = F / 2;
  // boundary rows/columns of the shifted tensors
  for (int i = 0; i < a.n_cc; ++i) {
    const OpArgs& v = a.op[i][0];
    float u[F2];
#pragma unroll
    for (int n = 0; n < F2; ++n) u[n] = fmaxf(__ldg(v.chain.b + n), 0.f);
    for (int c = 0; c < W; ++c) store_row(blk<T>(v.cat, tile, P, c, F), m, F2, F2, u);
  }
  {
    const OpArgs& h = a.op[last][1];
    float z[F2];
#pragma unroll
    for (int n = 0; n < F2; ++n) z[n] = fmaxf(__ldg(h.chain.b + n), 0.f);
    for (int r = 0; r < H; ++r) store_row(blk<T>(h.cat, tile, P, r * W, F), m, 0, F2, z);
  }
  if (TC) asm volatile("fence.proxy.async;" ::: "memory");
  __syncthreads();
  TcSmem s;
  TcState st;
  // the V ops of a row run as one pass when the TMEM holds W accumulators
  uint32_t ncols = kTmemCols;
  const bool vrow = TC && F <= 32 && W * F <= 512;
  if (vrow)
    while (ncols < (uint32_t)(W * F)) ncols *= 2;
  constexpr bool kSite = TC && F <= 32;
  SiteBufs b;
  if constexpr (kSite) {
    using SC = SiteCfg<F>;
    s.a_ptr = smem;
    s.w_ptr = smem + SC::kW;
    s.cw_ptr = smem + SC::kCW;
    s.ca_ptr = smem + SC::kCA;
    s.bar_load = reinterpret_cast<uint64_t*>(smem + SC::kBar);
    s.bar_mma = s.bar_load + 1;
    s.tmem_slot = reinterpret_cast<uint32_t*>(s.bar_load + 2);
    s.vbar = s.bar_load + 3;  // 2 * kVSlots + 1 barriers
    s.a = smem_u32(s.a_ptr);
    s.w = smem_u32(s.w_ptr);
    s.ca = smem_u32(s.ca_ptr);
    s.cw = smem_u32(s.cw_ptr);
    s.taps_per_group = TcCfg<F>::kTaps;
    b.ah = smem + SC::kAH;
    b.wh = smem + SC::kWH;
    b.cwh = smem + SC::kCWH;
    b.res = smem + SC::kRes;
    b.bar_h = s.vbar + 2 * SC::kVSlots + 1;
    b.ph_h = 0;
    b.spins = a.spins;
    b.batch = a.batch;
    SampOp* ops = reinterpret_cast<SampOp*>(smem + SC::kOps);
    for (int i = m; i < 3 * a.n_cc; i += kTile) samp_op_from(a.op[i / 3][i % 3], ops[i]);
    if (m == 0) {
      mbar_init(b.bar_h, 1);
      fence_mbar_init();
    }
    tc_setup(s, st, err, ncols);
  } else if (TC) {
    tc_carve<F>(smem, s);
    tc_setup(s, st, err, ncols);
  }
  Engine<F, TC> eng{&s, &st};
  // op k of a site: 0 = head C of conv L, then H_0, C_0, ..., H_{L-1}, C_{L-1}, H_L
  const int nseq = 2 * a.n_cc;
  // op records (the tensor-core site path only; the other paths read the kernel parameters)
  const SampOp* ops = kSite ? reinterpret_cast<const SampOp*>(smem + SiteCfg<F <= 32 ? F : 32>::kOps) : nullptr;
  auto seq_op = [&](int k) -> const SampOp& {
    return k == 0 ? ops[3 * last + 2] : (k == nseq - 1 ? ops[3 * last + 1] : ops[3 * ((k - 1) / 2) + ((k & 1) ? 1 : 2)]);
  };
  // EqualUpDownSpins: +1 spins drawn so far and the mask of the next site
  int n_up = 0, hmask = 0;
  for (int r = 0; r < H && !eng.aborted(); ++r) {
    Kahan kre, kim;
    for (int c = 0; c < W && kSite; ++c) {
      if constexpr (kSite) {
        const int pix = r * W + c;
        if (c == 0 && m == 32) site_prefetch<F>(seq_op(0), s, b, tile, r, 0, H, W, true);
        for (int k = 0; k < nseq; ++k) {
          const SampOp* nx = k + 1 < nseq ? &seq_op(k + 1) : (c + 1 < W ? &seq_op(0) : nullptr);
          const bool keep = k >= 2 && (k & 1) == 0 && ((a.keep_res >> ((k - 2) / 2)) & 1);
          HeadOut h;
          if (!site_op<F>(seq_op(k), s, st, b, tile, r, c, H, W, nx, k + 1 < nseq ? c : c + 1, keep, k == nseq - 1,
                          &h, hmask)) {
            st.abort = true;
            break;
          }
          if (k == 0) {
            // deepar/samplers/autoregressive.py:41-43 (+1 iff p(+1) > U), drawn
            // with Philox counter (sample, site, offset).
            U4 x = philox4x32(U4{(uint32_t)sample, (uint32_t)pix, a.off_lo, a.off_hi}, a.seed_lo, a.seed_hi);
            float u = philox_uniform(x.x);
            bool up = expf(2.f * h.re0) > u;
            kre.add(up ? h.re0 : h.re1);
            kim.add(up ? h.im0 : h.im1);
            if (sample < a.batch) a.spins[sample * P + pix] = up ? (int8_t)1 : (int8_t)-1;
            n_up += up ? 1 : 0;
            hmask = a.updown ? ((2 * n_up >= P ? 1 : 0) | (2 * (pix + 1 - n_up) >= P ? 2 : 0)) : 0;
          }
        }
        if (eng.aborted()) break;
      }
    }
    for (int c = 0; c < W && !kSite; ++c) {
      const int pix = r * W + c;
      HeadOut h;
      run_op<F, TC, T>(a.op[last][2], eng, tile, r, c, H, W, P, &h, hmask);
      if (eng.aborted()) break;
      // deepar/samplers/autoregressive.py:41-43 (+1 iff p(+1) > U), drawn with
      // Philox counter (sample, site, offset).
      U4 x = philox4x32(U4{(uint32_t)sample, (uint32_t)pix, a.off_lo, a.off_hi}, a.seed_lo, a.seed_hi);
      float u = philox_uniform(x.x);
      bool up = expf(2.f * h.re0) > u;
      kre.add(up ? h.re0 : h.re1);
      kim.add(up ? h.im0 : h.im1);
      if (sample < a.batch) a.spins[sample * P + pix] = up ? (int8_t)1 : (int8_t)-1;
      n_up += up ? 1 : 0;
      hmask = a.updown ? ((2 * n_up >= P ? 1 : 0) | (2 * (pix + 1 - n_up) >= P ? 2 : 0)) : 0;
      __syncthreads();
      for (int i = 0; i < last && !eng.aborted(); ++i) {
        run_op<F, TC, T>(a.op[i][1], eng, tile, r, c, H, W, P, &h);
        __syncthreads();
        run_op<F, TC, T>(a.op[i][2], eng, tile, r, c, H, W, P, &h);
        __syncthreads();
      }
      if (eng.aborted()) break;
      run_op<F, TC, T>(a.op[last][1], eng, tile, r, c, H, W, P, &h);
      __syncthreads();
    }
    if (eng.aborted()) break;
    a.row_partial[((int64_t)tile * H + r) * kTile + m] = make_float2(kre.s - kre.c, kim.s - kim.c);
    for (int i = 0; i < a.n_cc && !eng.aborted(); ++i) {
      if (kSite && vrow && a.op[i][0].main.ws) {
        if constexpr (kSite) {
          if (!v_row_op<F>(ops[3 * i], s, st, tile, r, H, W)) st.abort = true;
        }
        continue;
      }
      for (int c = 0; c < W; ++c) {
        HeadOut h;
        run_op<F, TC, T>(a.op[i][0], eng, tile, r, c, H, W, P, &h);
        __syncthreads();
      }
    }
  }
  if (TC) tc_teardown(st);
}

template <int F, bool TC>
static int sample_impl(const NetLayout& L, const void* packed, int64_t batch, uint64_t seed, uint64_t offset,
                       int8_t* spins, float* log_psi, const Tensors& T, cudaStream_t s) {
  int64_t tiles = (batch + kTile - 1) / kTile;
  SampleArgs* a = new SampleArgs;
  memset(a, 0, sizeof(SampleArgs));
  a->n_cc = L.n_cc;
  a->updown = L.updown;
  a->batch = batch;
  a->seed_lo = (uint32_t)seed;
  a->seed_hi = (uint32_t)(seed >> 32);
  a->off_lo = (uint32_t)offset;
  a->off_hi = (uint32_t)(offset >> 32);
  a->spins = spins;
  a->row_partial = T.row_partial;
  for (int i = 0; i < L.n_cc; ++i) {
    CCTensors x = cc_tensors(L, T, FK_AR2D_SAVE, i);
    make_ops(L, packed, i, spins, batch, x.vin, x.hin, x.vres, x.hres, x.vout, x.hout, x.cat, x.t, x.rv, a->op[i]);
  }
  // the tensor-core sampler keeps a C output in shared memory for the C op
  // whose residual it is, which must be the one two causal convs later
  for (int i = 0; i < L.n_cc; ++i) {
    if (!a->op[i][2].res) continue;
    if (i < 2 || a->op[i][2].res != a->op[i - 2][2].stream_out) {
      delete a;
      return FK_ERR_ARG;
    }
    a->keep_res |= 1ull << (i - 2);
  }
  if (a->keep_res & (a->keep_res >> 1)) {  // one residual block: sources two convs apart
    delete a;
    return FK_ERR_ARG;
  }
  size_t smem = TC ? (size_t)(F <= 32 ? SiteCfg<F>::kSmem : TcCfg<F>::kSmem) : 0;
  // a CTA that holds all 512 TMEM columns keeps its SM to itself
  if (TC && F <= 32 && L.W * F > 256 && smem < 120 * 1024) smem = 120 * 1024;
  int st = FK_OK;
  if (TC) {
    st = check_cuda(cudaFuncSetAttribute(sample_kernel<F, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem),
                    "cudaFuncSetAttribute");
  }
  if (st == FK_OK) {
    sample_kernel<F, TC><<<(unsigned)tiles, 128, smem, s>>>(*a, L.H, L.W, device_error_word());
    st = check_cuda(launched(), "sample_kernel");
  }
  delete a;
  if (st != FK_OK) return st;
  row_reduce_kernel<<<(unsigned)((batch + 255) / 256), 256, 0, s>>>(T.row_partial, batch, L.H,
                                                                    reinterpret_cast<float2*>(log_psi));
  return check_cuda(launched(), "row_reduce_kernel");
}


// ============================================================== causal reuse
// Connected configurations of a sample differ from it only at their flipped
// sites. Every activation of the network at a pixel depends on spins at that
// pixel's row and above (vertical stream) or earlier in raster order
// (horizontal stream), so for a configuration whose first flipped site is on
// row rk all rows < rk of every layer equal the base sample's. The
// configurations are sorted by rk; a tile of 128 starting at rk evaluates rows
// >= rk only, takes rows rk-2..rk of the tensors its 3-row taps read from the
// base sample's saved activations, and sums the log psi partials of rows < rk
// from the base. The result is bitwise that of a full forward.

__global__ void conn_rk_kernel(const short2* __restrict__ cflips, int64_t n, int H, int W, int32_t* __restrict__ rk,
                               int32_t* __restrict__ hist) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  short2 f = cflips[j];
  int r0 = f.x >= 0 ? f.x / W : H;
  int r1 = f.y >= 0 ? f.y / W : H;
  int r = r0 < r1 ? r0 : r1;
  if (r >= H) r = 0;  // no flipped site: evaluate every row
  rk[j] = r;
  atomicAdd(&hist[r], 1);
}

__global__ void conn_bucket_kernel(const int32_t* __restrict__ hist, int H, int32_t* __restrict__ cursor) {
  int run = 0;
  for (int r = 0; r < H; ++r) {
    cursor[r] = run;
    run += hist[r];
  }
}

__global__ void conn_scatter_kernel(const int32_t* __restrict__ rk, int64_t n, int32_t* __restrict__ cursor,
                                    int32_t* __restrict__ perm, int32_t* __restrict__ srk) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int r = rk[j];
  int pos = atomicAdd(&cursor[r], 1);
  perm[pos] = (int32_t)j;
  srk[pos] = r;
}

// chunk rows [j0, j0+n): configurations and owners in sorted order
__global__ void conn_gather_configs_kernel(const int8_t* __restrict__ configs, const int32_t* __restrict__ owner,
                                           const int32_t* __restrict__ perm, int64_t j0, int64_t n, int P,
                                           int8_t* __restrict__ cfg, int32_t* __restrict__ cown) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * P) return;
  int64_t j = t / P;
  int k = (int)(t - j * P);
  int64_t src = perm[j0 + j];
  cfg[t] = configs[src * P + k];
  if (k == 0) cown[j] = owner[src];
}

// Work list of the chunk: item = tile * H + r for r >= rk_start(tile).
__global__ void conn_items_kernel(const int32_t* __restrict__ srk, int64_t j0, int64_t n, int H,
                                  int32_t* __restrict__ rk_start, int32_t* __restrict__ items,
                                  int32_t* __restrict__ n_items) {
  __shared__ int32_t part[1024];
  const int tiles = (int)((n + kTile - 1) / kTile);
  const int per = (tiles + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = lo + per < tiles ? lo + per : tiles;
  int cnt = 0;
  for (int t = lo; t < hi; ++t) {
    int r = srk[j0 + (int64_t)t * kTile];
    rk_start[t] = r;
    cnt += H - r;
  }
  part[threadIdx.x] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      int v = part[i];
      part[i] = run;
      run += v;
    }
    *n_items = run;
  }
  __syncthreads();
  int off = part[threadIdx.x];
  for (int t = lo; t < hi; ++t)
    for (int r = rk_start[t]; r < H; ++r) items[off++] = t * H + r;
}

// Rows rk-2..rk-1 of the V stream and of Cat's X half, rows rk-2..rk of Cat's
// Y half, copied from the owner's base activations. Grid: (tile, 3 rows, W).
template <typename T>
__global__ void conn_gather_rows_kernel(const int32_t* __restrict__ rk_start, const int32_t* __restrict__ cown,
                                        int64_t n, int H, int W, int F, const T* __restrict__ base_v,
                                        const T* __restrict__ base_cat, T* __restrict__ v_out, T* __restrict__ cat_out) {
  const int64_t tile = blockIdx.x;
  const int slot = blockIdx.y;  // 0, 1, 2 -> rows rk-2, rk-1, rk
  const int c = blockIdx.z;
  const int m = threadIdx.x;
  const int rk = rk_start[tile];
  const int r = rk - 2 + slot;
  if (r < 0 || r >= H) return;
  const int64_t j = tile * kTile + m;
  if (j >= n) return;
  const int64_t b = cown[j];
  const int64_t tb = b / kTile;
  const int lb = (int)(b % kTile);
  const int P = H * W, pix = r * W + c;
  const int G = F / 8;
  const T* sv = base_v ? base_v + ((tb * P + pix) * (int64_t)F) * kTile : nullptr;
  const T* sc = base_cat + ((tb * P + pix) * (int64_t)F) * kTile;
  T* dv = v_out ? v_out + ((tile * P + pix) * (int64_t)F) * kTile : nullptr;
  T* dc = cat_out + ((tile * P + pix) * (int64_t)F) * kTile;
  constexpr int E = 16 / sizeof(T);  // elements per 16 bytes
  for (int g = 0; g < G; ++g) {
    const bool y_half = g >= G / 2;
    for (int e = 0; e < 8; e += E) {
      if (r < rk || y_half) {
        *reinterpret_cast<uint4*>(dc + ((int64_t)g * kTile + m) * 8 + e) =
            *reinterpret_cast<const uint4*>(sc + ((int64_t)g * kTile + lb) * 8 + e);
      }
      if (r < rk && dv) {
        *reinterpret_cast<uint4*>(dv + ((int64_t)g * kTile + m) * 8 + e) =
            *reinterpret_cast<const uint4*>(sv + ((int64_t)g * kTile + lb) * 8 + e);
      }
    }
  }
}

__global__ void conn_reduce_kernel(const float2* __restrict__ part, const float2* __restrict__ base_part,
                                   const int32_t* __restrict__ rk_start, const int32_t* __restrict__ cown,
                                   const int32_t* __restrict__ perm, int64_t j0, int64_t n, int H,
                                   float2* __restrict__ out) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t tile = j / kTile;
  const int m = (int)(j % kTile);
  const int rk = rk_start[tile];
  const int64_t b = cown[j];
  const int64_t tb = b / kTile;
  const int lb = (int)(b % kTile);
  Kahan re, im;
  for (int r = 0; r < H; ++r) {
    float2 p = r < rk ? base_part[(tb * H + r) * kTile + lb] : part[(tile * H + r) * kTile + m];
    re.add(p.x);
    im.add(p.y);
  }
  out[perm[j0 + j]] = make_float2(re.s - re.c, im.s - im.c);
}

struct ConnScratch {
  int32_t *rk, *perm, *srk, *hist, *cursor, *cown, *rk_start, *items, *n_items;
  int8_t* cfg;
  int64_t bytes;
};

static int64_t conn_layout(const NetLayout& L, int64_t max_rows, int64_t chunk, char* base, Tensors* T,
                           ConnScratch* S) {
  int64_t off = workspace_layout(L, chunk, FK_AR2D_INFER, base, T);
  auto take = [&](int64_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  ConnScratch tmp;
  ConnScratch* s = S ? S : &tmp;
  const int64_t tiles = (chunk + kTile - 1) / kTile;
  s->rk = reinterpret_cast<int32_t*>(take(max_rows * 4));
  s->perm = reinterpret_cast<int32_t*>(take(max_rows * 4));
  s->srk = reinterpret_cast<int32_t*>(take(max_rows * 4));
  s->hist = reinterpret_cast<int32_t*>(take((L.H + 1) * 4));
  s->cursor = reinterpret_cast<int32_t*>(take((L.H + 1) * 4));
  s->cown = reinterpret_cast<int32_t*>(take(chunk * 4));
  s->rk_start = reinterpret_cast<int32_t*>(take(tiles * 4));
  s->items = reinterpret_cast<int32_t*>(take(tiles * L.H * 4));
  s->n_items = reinterpret_cast<int32_t*>(take(4));
  s->cfg = reinterpret_cast<int8_t*>(take(chunk * L.P));
  s->bytes = off;
  return off;
}

template <int F, bool TC>
static int connections_impl(const NetLayout& L, const void* packed, const int8_t* configs, const int32_t* owner,
                            const int16_t* cflips, int64_t n_rows, const Tensors& B, float* log_psi,
                            const Tensors& T, const ConnScratch& S, int64_t chunk, cudaStream_t s) {
  using Tv = typename std::conditional<TC, tc16, float>::type;
  int* err = device_error_word();
  FK_CUDA(cudaMemsetAsync(S.hist, 0, (L.H + 1) * 4, s));
  conn_rk_kernel<<<(unsigned)((n_rows + 255) / 256), 256, 0, s>>>(reinterpret_cast<const short2*>(cflips), n_rows,
                                                                  L.H, L.W, S.rk, S.hist);
  conn_bucket_kernel<<<1, 1, 0, s>>>(S.hist, L.H, S.cursor);
  conn_scatter_kernel<<<(unsigned)((n_rows + 255) / 256), 256, 0, s>>>(S.rk, n_rows, S.cursor, S.perm, S.srk);
  FK_CUDA(launched(3));
  for (int64_t j0 = 0; j0 < n_rows; j0 += chunk) {
    const int64_t n = n_rows - j0 < chunk ? n_rows - j0 : chunk;
    const int64_t tiles = (n + kTile - 1) / kTile;
    conn_gather_configs_kernel<<<(unsigned)((n * L.P + 255) / 256), 256, 0, s>>>(configs, owner, S.perm, j0, n,
                                                                                 L.P, S.cfg, S.cown);
    conn_items_kernel<<<1, 1024, 0, s>>>(S.srk, j0, n, L.H, S.rk_start, S.items, S.n_items);
    FK_CUDA(launched(2));
    if (L.updown) {
      updown_mask_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(S.cfg, n, L.P, T.updown);
      FK_CUDA(launched());
    }
    for (int i = 0; i < L.n_cc; ++i) {
      CCTensors x = cc_tensors(L, T, FK_AR2D_INFER, i);
      const bool last = i == L.n_cc - 1;
      dim3 g((unsigned)tiles, 3, (unsigned)L.W);
      conn_gather_rows_kernel<Tv><<<g, kTile, 0, s>>>(
          S.rk_start, S.cown, n, L.H, L.W, F, last ? nullptr : static_cast<const Tv*>(B.v[i]),
          static_cast<const Tv*>(B.cat[i]), last ? nullptr : static_cast<Tv*>(x.vout), static_cast<Tv*>(x.cat));
      FK_CUDA(launched());
      OpArgs ops[3];
      make_ops(L, packed, i, S.cfg, n, x.vin, x.hin, x.vres, x.hres, x.vout, x.hout, x.cat, nullptr, nullptr, ops);
      for (int k = 0; k < 3; ++k) {
        ops[k].items = S.items;
        ops[k].n_items = S.n_items;
        if (last && k == 2) {
          ops[k].row_partial = T.row_partial;
          ops[k].updown = T.updown;
        }
        int st = run_engine_op<F, TC>(ops[k], tiles, L, err, s);
        if (st != FK_OK) return st;
      }
    }
    conn_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(T.row_partial, B.row_partial, S.rk_start, S.cown,
                                                                  S.perm, j0, n, L.H,
                                                                  reinterpret_cast<float2*>(log_psi));
    FK_CUDA(launched());
  }
  return FK_OK;
}

}  // namespace FK_NS

using namespace FK_NS;

extern "C" {

#ifndef FK_TC_FP16
// Layout queries: the same for both 16-bit formats, compiled once.
int64_t fk_ar2d_num_params(const fk_ar2d_desc* desc) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK) return -1;
  return L.num_params;
}

int64_t fk_ar2d_packed_bytes(const fk_ar2d_desc* desc) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK) return -1;
  return L.packed_bytes;
}
#endif

int FK_AR2D_ENTRY(fk_ar2d_pack)(const fk_ar2d_desc* desc, const float* params, void* packed, void* stream) {
  FK_DISPATCH_FP16(desc, fk_ar2d_pack_tc_fp16(desc, params, packed, stream));
  NetLayout L;
  int st = build_layout(desc, &L);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(params && packed, "fk_ar2d_pack: NULL buffer");
  PackArgs* a = new PackArgs;
  a->params = params;
  a->packed = static_cast<char*>(packed);
  a->n_convs = L.n_convs;
  a->bf16 = L.precision != FK_PRECISION_FP32;
  memcpy(a->conv, L.conv, sizeof(L.conv));
  pack_kernel<<<L.n_convs, 256, 0, static_cast<cudaStream_t>(stream)>>>(*a);
  delete a;
  FK_CUDA(launched());
  return FK_OK;
}

#ifndef FK_TC_FP16
int64_t fk_ar2d_workspace_bytes(const fk_ar2d_desc* desc, int64_t batch, int32_t mode) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK || batch < 0) return -1;
  return workspace_layout(L, batch, mode, nullptr, nullptr);
}
#endif

int FK_AR2D_ENTRY(fk_ar2d_forward)(const fk_ar2d_desc* desc, const void* packed, const int8_t* spins, int64_t batch,
                                   float* log_psi, float* cond, void* workspace, int64_t workspace_bytes,
                                   int32_t mode, void* stream) {
  FK_DISPATCH_FP16(desc, fk_ar2d_forward_tc_fp16(desc, packed, spins, batch, log_psi, cond, workspace,
                                                 workspace_bytes, mode, stream));
  NetLayout L;
  int st = build_layout(desc, &L);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(packed && spins && log_psi && batch >= 0, "fk_ar2d_forward: NULL buffer");
  FK_CHECK_ARG(mode == FK_AR2D_INFER || mode == FK_AR2D_SAVE, "fk_ar2d_forward: bad mode %d", mode);
  if (batch == 0) return FK_OK;
  Tensors T;
  int64_t need = workspace_layout(L, batch, mode, static_cast<char*>(workspace), &T);
  FK_CHECK_ARG(workspace && workspace_bytes >= need, "fk_ar2d_forward: workspace %lld < %lld bytes",
               (long long)workspace_bytes, (long long)need);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool tc = L.precision != FK_PRECISION_FP32;
  switch (L.F) {
    case 16: return tc ? forward_impl<16, true>(L, packed, spins, batch, log_psi, cond, T, mode, s)
                       : forward_impl<16, false>(L, packed, spins, batch, log_psi, cond, T, mode, s);
    case 32: return tc ? forward_impl<32, true>(L, packed, spins, batch, log_psi, cond, T, mode, s)
                       : forward_impl<32, false>(L, packed, spins, batch, log_psi, cond, T, mode, s);
    default: return tc ? forward_impl<64, true>(L, packed, spins, batch, log_psi, cond, T, mode, s)
                       : forward_impl<64, false>(L, packed, spins, batch, log_psi, cond, T, mode, s);
  }
}

int FK_AR2D_ENTRY(fk_ar2d_sample)(const fk_ar2d_desc* desc, const void* packed, int64_t batch, uint64_t seed,
                                  uint64_t offset, int8_t* spins, float* log_psi, void* workspace,
                                  int64_t workspace_bytes, void* stream) {
  FK_DISPATCH_FP16(desc, fk_ar2d_sample_tc_fp16(desc, packed, batch, seed, offset, spins, log_psi, workspace,
                                                workspace_bytes, stream));
  NetLayout L;
  int st = build_layout(desc, &L);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(packed && spins && log_psi && batch >= 0, "fk_ar2d_sample: NULL buffer");
  if (batch == 0) return FK_OK;
  Tensors T;
  int64_t need = workspace_layout(L, batch, FK_AR2D_SAVE, static_cast<char*>(workspace), &T);
  FK_CHECK_ARG(workspace && workspace_bytes >= need, "fk_ar2d_sample: workspace %lld < %lld bytes",
               (long long)workspace_bytes, (long long)need);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool tc = L.precision != FK_PRECISION_FP32;
  switch (L.F) {
    case 16: return tc ? sample_impl<16, true>(L, packed, batch, seed, offset, spins, log_psi, T, s)
                       : sample_impl<16, false>(L, packed, batch, seed, offset, spins, log_psi, T, s);
    case 32: return tc ? sample_impl<32, true>(L, packed, batch, seed, offset, spins, log_psi, T, s)
                       : sample_impl<32, false>(L, packed, batch, seed, offset, spins, log_psi, T, s);
    default: return tc ? sample_impl<64, true>(L, packed, batch, seed, offset, spins, log_psi, T, s)
                       : sample_impl<64, false>(L, packed, batch, seed, offset, spins, log_psi, T, s);
  }
}


#ifndef FK_TC_FP16
int64_t fk_ar2d_connections_workspace_bytes(const fk_ar2d_desc* desc, int64_t max_rows, int64_t chunk) {
  NetLayout L;
  if (build_layout(desc, &L) != FK_OK || max_rows < 0 || chunk <= 0) return -1;
  return conn_layout(L, max_rows, chunk, nullptr, nullptr, nullptr);
}
#endif

int FK_AR2D_ENTRY(fk_ar2d_forward_connections)(const fk_ar2d_desc* desc, const void* packed, const int8_t* configs,
                                               const int32_t* owner, const int16_t* cflips, int64_t n_rows,
                                               const void* base_saved, int64_t base_saved_bytes, int64_t base_batch,
                                               float* log_psi, void* workspace, int64_t workspace_bytes,
                                               int64_t chunk, void* stream) {
  FK_DISPATCH_FP16(desc, fk_ar2d_forward_connections_tc_fp16(desc, packed, configs, owner, cflips, n_rows, base_saved,
                                                             base_saved_bytes, base_batch, log_psi, workspace,
                                                             workspace_bytes, chunk, stream));
  NetLayout L;
  int st = build_layout(desc, &L);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(chunk > 0 && chunk % kTile == 0, "fk_ar2d_forward_connections: chunk must be a multiple of 128");
  if (n_rows == 0) return FK_OK;
  FK_CHECK_ARG(packed && configs && owner && cflips && base_saved && log_psi && n_rows > 0 && base_batch > 0,
               "fk_ar2d_forward_connections: NULL buffer");
  Tensors B;
  int64_t need = workspace_layout(L, base_batch, FK_AR2D_SAVE, static_cast<char*>(const_cast<void*>(base_saved)), &B);
  FK_CHECK_ARG(base_saved_bytes >= need, "fk_ar2d_forward_connections: base workspace %lld < %lld bytes",
               (long long)base_saved_bytes, (long long)need);
  Tensors T;
  ConnScratch S;
  int64_t wneed = conn_layout(L, n_rows, chunk, static_cast<char*>(workspace), &T, &S);
  FK_CHECK_ARG(workspace && workspace_bytes >= wneed, "fk_ar2d_forward_connections: workspace %lld < %lld bytes",
               (long long)workspace_bytes, (long long)wneed);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool tc = L.precision != FK_PRECISION_FP32;
  switch (L.F) {
    case 16: return tc ? connections_impl<16, true>(L, packed, configs, owner, cflips, n_rows, B, log_psi, T, S, chunk, s)
                       : connections_impl<16, false>(L, packed, configs, owner, cflips, n_rows, B, log_psi, T, S, chunk, s);
    case 32: return tc ? connections_impl<32, true>(L, packed, configs, owner, cflips, n_rows, B, log_psi, T, S, chunk, s)
                       : connections_impl<32, false>(L, packed, configs, owner, cflips, n_rows, B, log_psi, T, S, chunk, s);
    default: return tc ? connections_impl<64, true>(L, packed, configs, owner, cflips, n_rows, B, log_psi, T, S, chunk, s)
                       : connections_impl<64, false>(L, packed, configs, owner, cflips, n_rows, B, log_psi, T, S, chunk, s);
  }
}

}  // extern "C"
