// Pipelined tensor-core engine for the V/H/C ops of the AR2D forward
// (causal convs after the first, F <= 32).
//
// One persistent CTA per SM walks (tile, row) items; each item is one lattice
// row of 128 samples. Six warps:
//   warp 0 (one thread): TMA producer. Loads the op's weights once, then every
//       input column (the 3 rows r-2..r -- 1 row for the H op -- of one lattice
//       column, one bulk copy per [F/8][128][8] block) into a 7-8 slot ring;
//   warp 1 (one thread): MMA issuer. Per pixel, tcgen05.mma over the in-bounds
//       taps (K = 16 steps) into one of two TMEM accumulators, commits the
//       accumulator to the epilogue and every column whose last pixel this was
//       back to the producer; then the chained 1x1 MMA of the previous pixel
//       on the epilogue's staged bf16 activations;
//   warps 2-9: epilogue in two groups of four warps taking alternate pixels
//       (thread = sample, TMEM lane quarter = warp % 4): bias, relu, residual
//       (prefetched before the accumulator wait), stream store, chained-conv
//       staging, and the second half after the chained MMA; the head's log psi
//       partials are summed in pixel order through shared memory.
// A pixel loads one new column instead of nine taps, and loads, MMAs and
// epilogues of consecutive pixels overlap. The MMA sequence of a pixel (taps
// ascending, K steps ascending) and the epilogue arithmetic are those of the
// per-pixel engine in fk_ar2d.cu, so both engines give bitwise the same result.
#include "fk_ar2d.cuh"

namespace fk {

template <int F>
struct PipeCfg {
  static constexpr int kBlk = kTile * F * 2;
  // Column ring depth: a column is requested when the column kNcol places
  // earlier is released, i.e. kNcol - 2 pixels before its first use.
  static constexpr int kNcol = F <= 16 ? 8 : 7;
  static constexpr int kRing = 3 * kNcol * kBlk;
  static constexpr int kW = 9 * F * F * 2;
  static constexpr int kCW = F * 32 * 2;
  static constexpr int kGroups = 2;                 // epilogue groups (alternate pixels)
  static constexpr int kNB = kGroups;               // TMEM / staging buffers (one per group)
  static constexpr int kCA = kNB * kTile * F * 2;   // staged chained-conv inputs
  static constexpr int kBias = 64 * 4;              // main (F) + chained (<= 32) biases
  static constexpr int kBars = 512;
  static constexpr int kMaxW = 16;                  // head partials [W][128] float2
  static constexpr int kSmemBase = kRing + kW + kCW + kCA + kBias + kBars;
  static int head_bytes(int w) { return w * kTile * 8; }
};

__device__ __forceinline__ bool pwait(uint64_t* bar, uint32_t parity, int* err, bool& abort) {
  if (abort) return false;
  if (!mbar_wait(bar, parity, err)) {
    abort = true;
    return false;
  }
  return true;
}

template <int N>
__device__ __forceinline__ void tread(uint32_t taddr_lane, uint32_t col, float* v) {
#pragma unroll
  for (int q = 0; q < N / 16; ++q) tmem_ld16(taddr_lane + col + q * 16, v + q * 16);
  tmem_ld_wait();
}

template <int F>
__global__ void __launch_bounds__(320, 1) op_pipe_kernel(const __grid_constant__ OpArgs a, int H, int W,
                                                         int64_t n_items, int* err) {
  // With a work list, n_items is an upper bound and the list's count is read
  // on the device.
  using C = PipeCfg<F>;
  using T = __nv_bfloat16;
  constexpr int F2 = F / 2;
  constexpr int NC2 = F2 < 16 ? 16 : F2;
  constexpr int NB = C::kNB;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* ring = smem;
  uint8_t* wsm = smem + C::kRing;
  uint8_t* cwsm = wsm + C::kW;
  uint8_t* casm = cwsm + C::kCW;
  float* bias_sm = reinterpret_cast<float*>(casm + C::kCA);
  uint64_t* bars = reinterpret_cast<uint64_t*>(casm + C::kCA + C::kBias);
  constexpr int NR = C::kNcol;
  uint64_t* full = bars;
  uint64_t* empty = bars + NR;
  uint64_t* wbar = bars + 2 * NR;
  uint64_t* accf = wbar + 1;
  uint64_t* acce = accf + NB;
  uint64_t* caf = acce + NB;
  uint64_t* cf = caf + NB;
  uint64_t* head_ready = cf + NB;
  uint64_t* head_free = head_ready + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(head_free + 1);
  float2* head_sm = reinterpret_cast<float2*>(smem + C::kSmemBase);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int P = H * W;
  const int kind = a.kind;
  const int nrows = kind == kConvH ? 1 : 3;
  const int dcmin = kind == kConvV ? -1 : -2;
  const int dcmax = kind == kConvV ? 1 : 0;
  const int ntaps = kind == kConvH ? 3 : 9;
  const bool has_chain = !(kind == kConvC && !a.last);
  const bool head = kind == kConvC && a.last;
  const int cnp = kind == kConvC ? 16 : NC2;
  const uint32_t chain_bytes = (uint32_t)(F * cnp * 2);
  const uint32_t wbytes = (uint32_t)(ntaps * F * F * 2);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NR; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(wbar, 1);
    for (int i = 0; i < NB; ++i) {
      mbar_init(&accf[i], 1);
      mbar_init(&acce[i], 128);
      mbar_init(&caf[i], 128);
      mbar_init(&cf[i], 1);
    }
    mbar_init(head_ready, 128);
    mbar_init(head_free, 128);
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < F; i += blockDim.x) bias_sm[i] = a.main.b[i];
  if (has_chain)
    for (int i = threadIdx.x; i < cnp; i += blockDim.x) bias_sm[32 + i] = a.chain.b[i];
  if (warp == 1) {
    tmem_alloc(tslot, 256);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool abort = false;
  if (a.items) n_items = *a.n_items;
  auto item_at = [&](int64_t k) -> int64_t { return a.items ? (int64_t)a.items[k] : k; };

  if (warp == 0) {
    if (lane == 0) {
      // ---------------------------------------------------------------- producer
      mbar_arrive_expect_tx(wbar, wbytes + (has_chain ? chain_bytes : 0));
      bulk_g2s(wsm, a.main.w, wbytes, wbar);
      if (has_chain) bulk_g2s(cwsm, a.chain.w, chain_bytes, wbar);
      uint32_t g = 0;
      for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
        const int64_t item = item_at(it);
        const int64_t tile = item / H;
        const int r = (int)(item % H);
        for (int x = 0; x < W && !abort; ++x, ++g) {
          const uint32_t slot = g % NR;
          if (g >= NR && !pwait(&empty[slot], ((g / NR) - 1) & 1, err, abort)) break;
          uint32_t bytes = 0;
          for (int k = 0; k < nrows; ++k)
            if (r - (nrows - 1) + k >= 0) bytes += C::kBlk;
          mbar_arrive_expect_tx(&full[slot], bytes);
          for (int k = 0; k < nrows; ++k) {
            const int rr = r - (nrows - 1) + k;
            if (rr < 0) continue;
            bulk_g2s(ring + (slot * 3 + k) * C::kBlk, blk<T>(a.in, tile, P, rr * W + x, F), C::kBlk, &full[slot]);
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------------------------------------------------------- MMA issuer
      // The issuing thread is the critical resource (a 128x32x16 MMA costs ~48
      // cycles, the same as a few dozen instructions), so descriptors are
      // advanced by adding (byte offset >> 4) to base descriptors, and taps
      // and ring slots are resolved without divisions.
      const uint32_t idesc = umma_idesc_bf16(128, F);
      const uint32_t idesc_c = umma_idesc_bf16(128, cnp);
      const uint64_t a0 = umma_sdesc(smem_u32(ring), 2048, 128);
      const uint64_t w0 = umma_sdesc(smem_u32(wsm), F * 16, 128);
      const uint64_t ca0 = umma_sdesc(smem_u32(casm), 2048, 128);
      const uint64_t cw0 = umma_sdesc(smem_u32(cwsm), cnp * 16, 128);
      constexpr uint32_t kBlk16 = C::kBlk >> 4;           // one ring block
      constexpr uint32_t kTap16 = (F * F * 2) >> 4;       // one tap's weight slice
      constexpr uint32_t kKs16 = (2 * 2048) >> 4;         // one K=16 step of A
      constexpr uint32_t kKsW16 = (2 * F * 16) >> 4;      // one K=16 step of B
      pwait(wbar, 0, err, abort);
      uint32_t g_wait = 0, g_base = 0, p = 0, pc = 0;
      bool pending = false;
      auto issue_chain = [&](uint32_t q) {
        const uint32_t b = q % NB;
        if (!pwait(&caf[b], (q / NB) & 1, err, abort)) return;
        tc_fence_after();
#pragma unroll
        for (int ks = 0; ks < F / 16; ++ks)
          umma_bf16(tmem + 128 + b * 32, ca0 + ((b * (kTile * F * 2) + ks * 2 * 2048) >> 4),
                    cw0 + ((ks * 2 * cnp * 16) >> 4), idesc_c, ks > 0 ? 1u : 0u);
        umma_commit(&cf[b]);
      };
      // taps of this op as (dr, dc) with the weight slice index t = position
      const int tdr0 = kind == kConvH ? 0 : -2;
      const int tdc0 = kind == kConvV ? -1 : -2;
      const int tnr = kind == kConvH ? 1 : 3;
      for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
        const int64_t item = item_at(it);
        const int r = (int)(item % H);
        // ring slot of column 0 of this item
        uint32_t slot_c = g_base % NR;
        for (int c = 0; c < W && !abort; ++c) {
          const int xmax = c + dcmax < W - 1 ? c + dcmax : W - 1;
          while (g_wait < g_base + (uint32_t)xmax + 1 && !abort) {
            pwait(&full[g_wait % NR], (g_wait / NR) & 1, err, abort);
            ++g_wait;
          }
          const uint32_t b = p % NB;
          if (p >= NB) pwait(&acce[b], ((p / NB) - 1) & 1, err, abort);
          if (abort) break;
          tc_fence_after();
          const uint32_t d = tmem + b * 32;
          uint32_t acc_flag = 0u;
          // rows dr = tdr0 .. tdr0+tnr-1, columns dc = tdc0 .. tdc0+2; t = row*3 + col
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            if (i >= tnr) break;
            const int rr = r + tdr0 + i;
            if (rr < 0) continue;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const int x = c + tdc0 + j;
              if (x < 0 || x >= W) continue;
              // slot of column x = slot_c + (tdc0 + j), wrapped into [0, NR)
              int sx = (int)slot_c + tdc0 + j;
              sx += sx < 0 ? NR : 0;
              sx -= sx >= NR ? NR : 0;
              const int krow = (tnr == 1) ? 0 : i;
              const uint32_t aoff = ((uint32_t)sx * 3 + krow) * kBlk16;
              const uint32_t woff = (uint32_t)(i * 3 + j) * kTap16;
#pragma unroll
              for (int ks = 0; ks < F / 16; ++ks) {
                umma_bf16(d, a0 + aoff + ks * kKs16, w0 + woff + ks * kKsW16, idesc, acc_flag);
                acc_flag = 1u;
              }
            }
          }
          umma_commit(&accf[b]);
          const int xr = c + dcmin;
          if (xr >= 0) umma_commit(&empty[(g_base + xr) % NR]);
          if (c == W - 1) {
            for (int x = (W + dcmin > xr + 1 ? W + dcmin : xr + 1); x < W; ++x)
              if (x >= 0) umma_commit(&empty[(g_base + x) % NR]);
          }
          if (pending) issue_chain(pc);
          pending = has_chain;
          pc = p;
          ++p;
          slot_c = slot_c + 1 == (uint32_t)NR ? 0 : slot_c + 1;
        }
        g_base += W;
      }
      if (pending && !abort) issue_chain(pc);
    }
  } else {
    // ---------------------------------------------------------------- epilogue
    // Two groups of four warps take alternate pixels; within a group the TMEM
    // lane quarter is warp % 4, so thread (warp, lane) owns sample m.
    const int grp = (warp - 2) / 4;
    const int q4 = warp % 4;
    const int m = q4 * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16);
    const float* bm = bias_sm;
    const float* bc = bias_sm + 32;
    const bool need_res = (kind == kConvV && a.stream_out && a.res) || (kind == kConvC && !a.last && a.res);
    uint32_t p = 0, it_count = 0;
    for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x, ++it_count) {
      const int64_t item = item_at(it);
      const int64_t tile = item / H;
      const int r = (int)(item % H);
      const int64_t sample = tile * kTile + m;
      if (head && grp == 1 && it_count > 0 && !pwait(head_free, (it_count - 1) & 1, err, abort)) break;
      for (int c = 0; c < W && !abort; ++c, ++p) {
        if ((int)(p % C::kGroups) != grp) continue;
        const uint32_t b = p % NB;
        const int pix = r * W + c;
        float o[F];
        if (need_res) load_row(blk<T>(a.res, tile, P, pix, F), m, 0, F, o);
        if (!pwait(&accf[b], (p / NB) & 1, err, abort)) break;
        tc_fence_after();
        float acc[F];
        tread<F>(tl, b * 32, acc);
        tc_fence_before();
        mbar_arrive(&acce[b]);
        float cin[F];
        if (kind == kConvV) {
#pragma unroll
          for (int n = 0; n < F; ++n) acc[n] += bm[n];
          if (a.stream_out) {
            if (a.res) {
#pragma unroll
              for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
            } else {
#pragma unroll
              for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
            }
            store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, o);
          }
#pragma unroll
          for (int n = 0; n < F; ++n) cin[n] = fmaxf(acc[n], 0.f);
          if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, cin);
        } else if (kind == kConvH) {
#pragma unroll
          for (int n = 0; n < F; ++n) cin[n] = fmaxf(acc[n] + bm[n], 0.f);
          if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, cin);
        } else {
#pragma unroll
          for (int n = 0; n < F; ++n) acc[n] += bm[n];
          if (!a.last) {
            if (a.res) {
#pragma unroll
              for (int n = 0; n < F; ++n) o[n] = fmaxf(o[n] + acc[n], 0.f);
            } else {
#pragma unroll
              for (int n = 0; n < F; ++n) o[n] = fmaxf(acc[n], 0.f);
            }
            store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, o);
          } else {
#pragma unroll
            for (int n = 0; n < F; ++n) cin[n] = fmaxf(acc[n], 0.f);
            if (a.stream_out) store_row(blk<T>(a.stream_out, tile, P, pix, F), m, 0, F, cin);
          }
        }
        if (!has_chain) continue;
        // stage the chained conv's input (bf16 rows, [F/8][128][8])
        T* ca = reinterpret_cast<T*>(casm + b * (kTile * F * 2));
#pragma unroll
        for (int gq = 0; gq < F / 8; ++gq) st8(ca + ((int64_t)gq * kTile + m) * 8, cin + 8 * gq);
        fence_proxy_async_smem();
        mbar_arrive(&caf[b]);
        if (!pwait(&cf[b], (p / NB) & 1, err, abort)) break;
        tc_fence_after();
        float out[32];
        if (kind == kConvC)
          tread<16>(tl, 128 + b * 32, out);
        else
          tread<NC2>(tl, 128 + b * 32, out);
        tc_fence_before();
        if (kind == kConvV) {
#pragma unroll
          for (int n = 0; n < F2; ++n) out[n] = fmaxf(out[n] + bc[n], 0.f);
          if (r + 1 < H) store_row(blk<T>(a.cat, tile, P, pix + W, F), m, F2, F2, out);
          if (r == 0) {
#pragma unroll
            for (int n = 0; n < F2; ++n) out[n] = fmaxf(bc[n], 0.f);
            store_row(blk<T>(a.cat, tile, P, c, F), m, F2, F2, out);
          }
        } else if (kind == kConvH) {
#pragma unroll
          for (int n = 0; n < F2; ++n) out[n] = fmaxf(out[n] + bc[n], 0.f);
          const int sh = a.last ? 1 : 0;
          if (c + sh < W) store_row(blk<T>(a.cat, tile, P, pix + sh, F), m, 0, F2, out);
          if (sh && c == 0) {
#pragma unroll
            for (int n = 0; n < F2; ++n) out[n] = fmaxf(bc[n], 0.f);
            store_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F2, out);
          }
        } else {
#pragma unroll
          for (int n = 0; n < 4; ++n) out[n] += bc[n];
          // abstract_machine.py:56-57 normalisation (same arithmetic as the per-pixel engine)
          float a2 = 2.f * out[0], b2 = 2.f * out[1];
          float mx = fmaxf(a2, b2);
          float lse = 0.5f * (mx + logf(expf(a2 - mx) + expf(b2 - mx)));
          float re0 = out[0] - lse, re1 = out[1] - lse;
          bool up = spin_at(a.spins, a.batch, P, sample, pix) > 0.f;
          head_sm[c * kTile + m] = make_float2(up ? re0 : re1, up ? out[2] : out[3]);
          if (a.cond && sample < a.batch)
            reinterpret_cast<float4*>(a.cond)[sample * P + pix] = make_float4(re0, re1, out[2], out[3]);
        }
      }
      if (head && !abort) {
        // ordered compensated sum over the row's pixels (the per-pixel engine's order)
        if (grp == 1) {
          mbar_arrive(head_ready);
        } else if (pwait(head_ready, it_count & 1, err, abort)) {
          Kahan kre, kim;
          for (int c = 0; c < W; ++c) {
            float2 v = head_sm[c * kTile + m];
            kre.add(v.x);
            kim.add(v.y);
          }
          a.row_partial[((int64_t)tile * H + r) * kTile + m] = make_float2(kre.s - kre.c, kim.s - kim.c);
          mbar_arrive(head_free);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 256);
  }
}

template <int F>
static int launch_pipe(const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  static int sms = 0;
  static bool attr = false;
  if (!sms) {
    int dev = 0;
    FK_CUDA(cudaGetDevice(&dev));
    FK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const bool head = a.kind == kConvC && a.last;
  if (head && W > PipeCfg<F>::kMaxW) return FK_ERR_ARG;
  const int smem = PipeCfg<F>::kSmemBase + (head ? PipeCfg<F>::head_bytes(W) : 0);
  if (!attr) {
    FK_CUDA(cudaFuncSetAttribute(op_pipe_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 PipeCfg<F>::kSmemBase + PipeCfg<F>::head_bytes(PipeCfg<F>::kMaxW)));
    attr = true;
  }
  const int64_t items = tiles * H;
  int64_t grid = (int64_t)sms;  // one CTA per SM (256 TMEM columns, 320 threads)
  if (grid > items) grid = items;
  op_pipe_kernel<F><<<(unsigned)grid, 320, smem, s>>>(a, H, W, items, err);
  return check_cuda(launched(), "op_pipe_kernel");
}

int launch_pipe_op(int F, const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  if (a.first) return FK_ERR_ARG;
  if (F == 16) return launch_pipe<16>(a, tiles, H, W, err, s);
  if (F == 32) return launch_pipe<32>(a, tiles, H, W, err, s);
  return FK_ERR_ARG;
}

bool pipe_supported(int F, int W) { return (F == 16 || F == 32) && W <= PipeCfg<32>::kMaxW; }

static_assert(PipeCfg<32>::kSmemBase + 16 * kTile * 8 <= 227 * 1024, "pipelined engine exceeds shared memory");
static_assert(PipeCfg<16>::kSmemBase + 16 * kTile * 8 <= 227 * 1024, "pipelined engine exceeds shared memory");

}  // namespace fk
