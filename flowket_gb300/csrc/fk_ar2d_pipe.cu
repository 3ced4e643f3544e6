// Pipelined tensor-core engine for the V/H/C ops of the AR2D forward
// (causal convs after the first, F <= 32).
//
// One persistent CTA per SM walks (tile, row) items; each item is one lattice
// row of 128 samples. Six warps:
//   warp 0 (one thread): TMA producer. Loads the op's weights once, then every
//       input column (the 3 rows r-2..r -- 1 row for the H op -- of one lattice
//       column, one bulk copy per [F/8][128][8] block) into a 4-slot ring;
//   warp 1 (one thread): MMA issuer. Per pixel, tcgen05.mma over the in-bounds
//       taps (K = 16 steps) into one of two TMEM accumulators, commits the
//       accumulator to the epilogue and every column whose last pixel this was
//       back to the producer; then the chained 1x1 MMA of the previous pixel
//       on the epilogue's staged bf16 activations;
//   warps 2-5: epilogue (thread = sample, TMEM lane quarter = warp % 4):
//       bias, relu, residual, stream store, chained-conv staging, and the
//       second half after the chained MMA.
// A pixel loads one new column instead of nine taps, and loads, MMAs and
// epilogues of consecutive pixels overlap. The MMA sequence of a pixel (taps
// ascending, K steps ascending) and the epilogue arithmetic are those of the
// per-pixel engine in fk_ar2d.cu, so both engines give bitwise the same result.
#include "fk_ar2d.cuh"

namespace fk {

template <int F>
struct PipeCfg {
  static constexpr int kBlk = kTile * F * 2;
  static constexpr int kNcol = 4;
  static constexpr int kRing = 3 * kNcol * kBlk;
  static constexpr int kW = 9 * F * F * 2;
  static constexpr int kCW = F * 32 * 2;
  static constexpr int kCA = 2 * kTile * F * 2;
  static constexpr int kBars = 256;
  static constexpr int kSmem = kRing + kW + kCW + kCA + kBars;
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
__global__ void __launch_bounds__(192, 1) op_pipe_kernel(const __grid_constant__ OpArgs a, int H, int W,
                                                         int64_t n_items, int* err) {
  using C = PipeCfg<F>;
  using T = __nv_bfloat16;
  constexpr int F2 = F / 2;
  constexpr int NC2 = F2 < 16 ? 16 : F2;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* ring = smem;
  uint8_t* wsm = smem + C::kRing;
  uint8_t* cwsm = wsm + C::kW;
  uint8_t* casm = cwsm + C::kCW;
  uint64_t* bars = reinterpret_cast<uint64_t*>(casm + C::kCA);
  uint64_t* full = bars;
  uint64_t* empty = bars + 4;
  uint64_t* wbar = bars + 8;
  uint64_t* accf = bars + 9;
  uint64_t* acce = bars + 11;
  uint64_t* caf = bars + 13;
  uint64_t* cf = bars + 15;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 17);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int P = H * W;
  const int kind = a.kind;
  const int nrows = kind == kConvH ? 1 : 3;
  const int dcmin = kind == kConvV ? -1 : -2;
  const int dcmax = kind == kConvV ? 1 : 0;
  const int ntaps = kind == kConvH ? 3 : 9;
  const bool has_chain = !(kind == kConvC && !a.last);
  const int cnp = kind == kConvC ? 16 : NC2;
  const uint32_t chain_bytes = (uint32_t)(F * cnp * 2);
  const uint32_t wbytes = (uint32_t)(ntaps * F * F * 2);

  if (threadIdx.x == 0) {
    for (int i = 0; i < 4; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(wbar, 1);
    for (int i = 0; i < 2; ++i) {
      mbar_init(&accf[i], 1);
      mbar_init(&acce[i], 128);
      mbar_init(&caf[i], 128);
      mbar_init(&cf[i], 1);
    }
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(tslot, 128);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool abort = false;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------------------------------------------------------- producer
      mbar_arrive_expect_tx(wbar, wbytes + (has_chain ? chain_bytes : 0));
      bulk_g2s(wsm, a.main.w, wbytes, wbar);
      if (has_chain) bulk_g2s(cwsm, a.chain.w, chain_bytes, wbar);
      uint32_t g = 0;
      for (int64_t item = blockIdx.x; item < n_items && !abort; item += gridDim.x) {
        const int64_t tile = item / H;
        const int r = (int)(item % H);
        for (int x = 0; x < W && !abort; ++x, ++g) {
          const uint32_t slot = g % 4;
          if (g >= 4 && !pwait(&empty[slot], ((g / 4) - 1) & 1, err, abort)) break;
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
      const uint32_t idesc = umma_idesc_bf16(128, F);
      const uint32_t idesc_c = umma_idesc_bf16(128, cnp);
      const uint32_t ring_a = smem_u32(ring), w_a = smem_u32(wsm), cw_a = smem_u32(cwsm), ca_a = smem_u32(casm);
      pwait(wbar, 0, err, abort);
      uint32_t g_wait = 0, g_base = 0, p = 0, pc = 0;
      bool pending = false;
      auto issue_chain = [&](uint32_t q) {
        const uint32_t b = q % 2;
        if (!pwait(&caf[b], (q / 2) & 1, err, abort)) return;
        tc_fence_after();
#pragma unroll
        for (int ks = 0; ks < F / 16; ++ks) {
          uint64_t ad = umma_sdesc(ca_a + b * (kTile * F * 2) + ks * 2 * 2048, 2048, 128);
          uint64_t bd = umma_sdesc(cw_a + ks * 2 * cnp * 16, cnp * 16, 128);
          umma_bf16(tmem + 64 + b * 32, ad, bd, idesc_c, ks > 0 ? 1u : 0u);
        }
        umma_commit(&cf[b]);
      };
      for (int64_t item = blockIdx.x; item < n_items && !abort; item += gridDim.x) {
        const int r = (int)(item % H);
        for (int c = 0; c < W && !abort; ++c) {
          const int xmax = c + dcmax < W - 1 ? c + dcmax : W - 1;
          while (g_wait < g_base + (uint32_t)xmax + 1 && !abort) {
            pwait(&full[g_wait % 4], (g_wait / 4) & 1, err, abort);
            ++g_wait;
          }
          const uint32_t b = p % 2;
          if (p >= 2) pwait(&acce[b], ((p / 2) - 1) & 1, err, abort);
          if (abort) break;
          tc_fence_after();
          bool first = true;
          for (int t = 0; t < ntaps; ++t) {
            int dr, dc;
            tap_offset(kind, t, dr, dc);
            const int rr = r + dr, x = c + dc;
            if (rr < 0 || rr >= H || x < 0 || x >= W) continue;
            const uint32_t slot = (g_base + x) % 4;
            const int k = dr + (nrows - 1);
            const uint32_t abase = ring_a + (slot * 3 + k) * C::kBlk;
            const uint32_t wb = w_a + t * (F * F * 2);
#pragma unroll
            for (int ks = 0; ks < F / 16; ++ks) {
              uint64_t ad = umma_sdesc(abase + ks * 2 * 2048, 2048, 128);
              uint64_t bd = umma_sdesc(wb + ks * 2 * F * 16, F * 16, 128);
              umma_bf16(tmem + b * F, ad, bd, idesc, first ? 0u : 1u);
              first = false;
            }
          }
          umma_commit(&accf[b]);
          const int xr = c + dcmin;
          if (xr >= 0) umma_commit(&empty[(g_base + xr) % 4]);
          if (c == W - 1) {
            for (int x = (W + dcmin > xr + 1 ? W + dcmin : xr + 1); x < W; ++x)
              if (x >= 0) umma_commit(&empty[(g_base + x) % 4]);
          }
          if (pending) issue_chain(pc);
          pending = has_chain;
          pc = p;
          ++p;
        }
        g_base += W;
      }
      if (pending && !abort) issue_chain(pc);
    }
  } else {
    // ---------------------------------------------------------------- epilogue
    const int q4 = warp % 4;
    const int m = q4 * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16);
    const float* bm = a.main.b;
    const float* bc = a.chain.b;
    uint32_t p = 0;
    for (int64_t item = blockIdx.x; item < n_items && !abort; item += gridDim.x) {
      const int64_t tile = item / H;
      const int r = (int)(item % H);
      const int64_t sample = tile * kTile + m;
      Kahan kre, kim;
      for (int c = 0; c < W && !abort; ++c, ++p) {
        const uint32_t b = p % 2;
        const int pix = r * W + c;
        if (!pwait(&accf[b], (p / 2) & 1, err, abort)) break;
        tc_fence_after();
        float acc[F];
        tread<F>(tl, b * F, acc);
        tc_fence_before();
        mbar_arrive(&acce[b]);
        float cin[F];
        if (kind == kConvV) {
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
          for (int n = 0; n < F; ++n) cin[n] = fmaxf(acc[n], 0.f);
          if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, cin);
        } else if (kind == kConvH) {
#pragma unroll
          for (int n = 0; n < F; ++n) cin[n] = fmaxf(acc[n] + __ldg(bm + n), 0.f);
          if (a.aux_out) store_row(blk<T>(a.aux_out, tile, P, pix, F), m, 0, F, cin);
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
        if (!pwait(&cf[b], (p / 2) & 1, err, abort)) break;
        tc_fence_after();
        float out[32];
        if (kind == kConvC)
          tread<16>(tl, 64 + b * 32, out);
        else
          tread<NC2>(tl, 64 + b * 32, out);
        tc_fence_before();
        if (kind == kConvV) {
#pragma unroll
          for (int n = 0; n < F2; ++n) out[n] = fmaxf(out[n] + __ldg(bc + n), 0.f);
          if (r + 1 < H) store_row(blk<T>(a.cat, tile, P, pix + W, F), m, F2, F2, out);
          if (r == 0) {
#pragma unroll
            for (int n = 0; n < F2; ++n) out[n] = fmaxf(__ldg(bc + n), 0.f);
            store_row(blk<T>(a.cat, tile, P, c, F), m, F2, F2, out);
          }
        } else if (kind == kConvH) {
#pragma unroll
          for (int n = 0; n < F2; ++n) out[n] = fmaxf(out[n] + __ldg(bc + n), 0.f);
          const int sh = a.last ? 1 : 0;
          if (c + sh < W) store_row(blk<T>(a.cat, tile, P, pix + sh, F), m, 0, F2, out);
          if (sh && c == 0) {
#pragma unroll
            for (int n = 0; n < F2; ++n) out[n] = fmaxf(__ldg(bc + n), 0.f);
            store_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F2, out);
          }
        } else {
#pragma unroll
          for (int n = 0; n < 4; ++n) out[n] += __ldg(bc + n);
          // abstract_machine.py:56-57 normalisation (same arithmetic as the per-pixel engine)
          float a2 = 2.f * out[0], b2 = 2.f * out[1];
          float mx = fmaxf(a2, b2);
          float lse = 0.5f * (mx + logf(expf(a2 - mx) + expf(b2 - mx)));
          float re0 = out[0] - lse, re1 = out[1] - lse;
          bool up = spin_at(a.spins, a.batch, P, sample, pix) > 0.f;
          kre.add(up ? re0 : re1);
          kim.add(up ? out[2] : out[3]);
          if (a.cond && sample < a.batch)
            reinterpret_cast<float4*>(a.cond)[sample * P + pix] = make_float4(re0, re1, out[2], out[3]);
        }
      }
      if (kind == kConvC && a.last && !abort)
        a.row_partial[((int64_t)tile * H + r) * kTile + m] = make_float2(kre.s - kre.c, kim.s - kim.c);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
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
  if (!attr) {
    FK_CUDA(cudaFuncSetAttribute(op_pipe_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)PipeCfg<F>::kSmem));
    attr = true;
  }
  const int64_t items = tiles * H;
  const int per_sm = (227 * 1024) / PipeCfg<F>::kSmem > 0 ? (227 * 1024) / PipeCfg<F>::kSmem : 1;
  int64_t grid = (int64_t)sms * per_sm;
  if (grid > items) grid = items;
  op_pipe_kernel<F><<<(unsigned)grid, 192, PipeCfg<F>::kSmem, s>>>(a, H, W, items, err);
  return check_cuda(launched(), "op_pipe_kernel");
}

int launch_pipe_op(int F, const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  if (a.first) return FK_ERR_ARG;
  if (F == 16) return launch_pipe<16>(a, tiles, H, W, err, s);
  if (F == 32) return launch_pipe<32>(a, tiles, H, W, err, s);
  return FK_ERR_ARG;
}

}  // namespace fk
