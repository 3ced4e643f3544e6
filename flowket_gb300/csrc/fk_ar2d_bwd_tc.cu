// Adjoint of the AR2D forward on tensor cores (BF16 path, F <= 32, summed
// gradient). Same mathematics as the CUDA-core adjoint in fk_ar2d_bwd.cu:
//
//   data gradients, per causal conv i in reverse (bwd_op_kernel, on the
//   column-scatter pipeline of fk_pipe.cuh with the transposed operands):
//     C^T : gCat = sum_taps gHp[q - tap] W_c^T, masked by [Cat > 0] -> gCatm;
//           chained: gT(r, c - s) = [T > 0] . W_x^T gCatm[0:F/2]  (s = 1 on
//           the final conv, whose column W-1 of gT is zero) and
//           gVp(r - 1, c) = [relu(Vp) > 0] . W_y^T gCatm[F/2:F] + gV-stream;
//     V^T : gV_{i-1} = [V_{i-1} > 0] . (sum_taps gVp[q - tap] W_v^T + residual)
//     H^T : gHp_{i-1} = [H_{i-1} > 0] . (sum_taps gT[q - tap] W_h^T + residual)
//   The transposed conv reads rows r..r+2 of its input gradient (anti-causal
//   taps): input column x feeds outputs x-1..x+1 (V^T) or x-2..x (C^T, H^T).
//
//   weight gradients (wgrad_tc_kernel): dW[tap][ci][co] = sum over samples
//   and pixels of X[q + tap][ci] G[q][co], a GEMM over K = samples with both
//   operands MN-major, read straight from the blocked activation layout
//   (a [C/8][128][8] block is an MN-major operand with 8-element rows along
//   the channels, LBO = 128 B along the samples, SBO = 2 KB along channels).
//   A = one input column's ring slot (the kernel rows' X blocks stacked along
//   M, 4 blocks = 128 rows), B = the window of output-gradient columns it
//   feeds (stacked along N), so one MMA accumulates all taps of a column.
//   Each CTA accumulates in TMEM over its items and writes one partial; the
//   partials are summed in a fixed order (deterministic gradients).
//
//   bias gradients: column sums of the output gradients (bias_sum_kernel).
//
// Gradients between the ops are bf16 (tcgen05 operands); every sum is fp32.
#include "fk_pipe.cuh"

#include <string.h>

#include <mutex>

namespace FK_NS {

template <int F>
struct BwdCfg {
  using C = PipeCfg<F>;
  static constexpr int kCW = 2 * (F / 2) * F * 2;   // W_x^T and W_y^T
  static constexpr int kSmem = C::kRing + C::kW + kCW + C::kCA + C::kBars;
};

template <int F>
__global__ void __launch_bounds__(kPipeThreads, 1) bwd_op_kernel(const __grid_constant__ BwdOpArgs a, int H, int W,
                                                                 int64_t n_items, int* err) {
  using C = PipeCfg<F>;
  using BC = BwdCfg<F>;
  using T = tc16;
  constexpr int F2 = F / 2;
  constexpr int NB = C::kNB;
  constexpr int NS = C::kNS;
  constexpr int NR = C::kNcol;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* ring = smem;
  uint8_t* wsm = smem + C::kRing;
  uint8_t* cwsm = wsm + C::kW;  // W_x^T then W_y^T
  uint8_t* casm = cwsm + BC::kCW;
  uint64_t* bars = reinterpret_cast<uint64_t*>(casm + C::kCA);
  uint64_t* full = bars;
  uint64_t* empty = bars + NR;
  uint64_t* wbar = bars + 2 * NR;
  uint64_t* accf = wbar + 1;
  uint64_t* acce = accf + NS;
  uint64_t* caf = acce + NS;
  uint64_t* cf = caf + NB;
  uint64_t* drain = cf + NB;  // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 2);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int P = H * W;
  const int kind = a.kind;
  const bool chain = kind == kBwdC;
  const int nrows = kind == kBwdH ? 1 : 3;
  const int o0 = kind == kBwdV ? -1 : -2;
  const uint32_t cw_half = (uint32_t)(F2 * F * 2);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NR; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(wbar, 1);
    for (int i = 0; i < NS; ++i) {
      mbar_init(&accf[i], 1);
      mbar_init(&acce[i], 4);  // one arrival per epilogue warp
    }
    for (int i = 0; i < NB; ++i) {
      mbar_init(&caf[i], 4);
      mbar_init(&cf[i], 1);
    }
    mbar_init(&drain[0], 1);
    mbar_init(&drain[1], 1);
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
  const PipeGeom geom{H, W, nrows, 0, o0, 1};
  const PipeItems items{nullptr, n_items};

  if (warp == 0) {
    if (lane == 0)
      pipe_producer<F>(geom, items, a.in, ring, full, empty, wbar,
                       WeightCopy{wsm, a.wt, (uint32_t)(nrows * C::kWRow)},
                       WeightCopy{cwsm, a.wx, chain ? cw_half : 0u},
                       WeightCopy{cwsm + cw_half, a.wy, chain ? cw_half : 0u}, err, abort);
  } else if (warp == 1) {
    pipe_issuer<F>(geom, items, ring, wsm, tmem, empty, accf, &drain[0], err, abort);
  } else if (warp == 2) {
    pipe_waiter<F>(geom, items, full, wbar, acce, err, abort);
  } else if (warp == 3) {
    // ------------------------------------------------------------------ chain issuer (C^T)
    // Two MMAs per output: x half (K = gCatm channels 0..F/2) into chain
    // accumulator 2b, y half (channels F/2..F) into 2b + 1.
    if (chain && lane == 0) {
      const uint32_t idesc_c = umma_idesc_tc16(128, F);
      const uint64_t ca0 = umma_sdesc(smem_u32(casm), 2048, 128);
      const uint64_t cw0 = umma_sdesc(smem_u32(cwsm), F * 16, 128);
      pwait(wbar, 0, err, abort);
      uint32_t q = 0;
      for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
        for (int c = 0; c < W && !abort; ++c, ++q) {
          const uint32_t b = q % NB;
          if (!pwait(&caf[b], (q / NB) & 1, err, abort)) break;
          tc_fence_after();
          const uint32_t a_b = (b * (kTile * F * 2)) >> 4;
          umma_bf16(tmem + C::kChainCol + b * 2 * F, ca0 + a_b, cw0, idesc_c, 0u);
          umma_bf16(tmem + C::kChainCol + b * 2 * F + F, ca0 + a_b + ((F2 / 8 * 2048) >> 4), cw0 + (cw_half >> 4),
                    idesc_c, 0u);
          umma_commit(&cf[b]);
        }
      }
      umma_commit(&drain[1]);
      mbar_wait(&drain[1], 0, err);
    }
  } else {
    // ---------------------------------------------------------------- epilogue
    const int grp = (warp - 4) / 4;
    const int q4 = warp % 4;
    const int m = q4 * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16);
    bool pend = false;
    uint32_t pq = 0;
    int64_t ptile = 0;
    int pr = 0, pc = 0;
    // C^T, after the chained MMAs of output (ptile, pr, pc)
    auto second_half = [&]() {
      const uint32_t b = pq % NB;
      pend = false;
      const int cx = pc - a.shift;
      // masks and stream gradient, kept as packed bf16 until used
      uint4 ttr[F / 8], rvr[F / 8], gsr[F / 8];
      if (cx >= 0) load_raw<F>(blk<T>(a.t, ptile, P, pr * W + cx, F), m, ttr);
      if (pr >= 1) {
        load_raw<F>(blk<T>(a.rv, ptile, P, (pr - 1) * W + pc, F), m, rvr);
        if (a.gvs) load_raw<F>(blk<T>(a.gvs, ptile, P, (pr - 1) * W + pc, F), m, gsr);
      }
      if (!uwait(&cf[b], (pq / NB) & 1, err, abort)) return;
      tc_fence_after();
      float gx[F];
      tread<F>(tl, C::kChainCol + b * 2 * F, gx);
      if (cx >= 0) {
        float tt[F];
        unpack_raw<F>(ttr, tt);
#pragma unroll
        for (int n = 0; n < F; ++n) gx[n] = tt[n] > 0.f ? gx[n] : 0.f;
        store_row(blk<T>(a.gt, ptile, P, pr * W + cx, F), m, 0, F, gx);
      }
      if (a.shift && pc == W - 1) {
#pragma unroll
        for (int n = 0; n < F; ++n) gx[n] = 0.f;
        store_row(blk<T>(a.gt, ptile, P, pr * W + pc, F), m, 0, F, gx);
      }
      float gy[F];
      tread<F>(tl, C::kChainCol + b * 2 * F + F, gy);
      tc_fence_before();
      if (pr >= 1) {
        float rv[F];
        unpack_raw<F>(rvr, rv);
#pragma unroll
        for (int n = 0; n < F; ++n) gy[n] = rv[n] > 0.f ? gy[n] : 0.f;
        if (a.gvs) {
          float gs[F];
          unpack_raw<F>(gsr, gs);
#pragma unroll
          for (int n = 0; n < F; ++n) gy[n] += gs[n];
        }
        store_row(blk<T>(a.gvp, ptile, P, (pr - 1) * W + pc, F), m, 0, F, gy);
      }
      if (pr == H - 1) {
        float gs[F];
        if (a.gvs) {
          load_row(blk<T>(a.gvs, ptile, P, pr * W + pc, F), m, 0, F, gs);
        } else {
#pragma unroll
          for (int n = 0; n < F; ++n) gs[n] = 0.f;
        }
        store_row(blk<T>(a.gvp, ptile, P, pr * W + pc, F), m, 0, F, gs);
      }
    };
    uint32_t p = 0;
    for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
      const int64_t tile = it / H;
      const int r = (int)(it % H);
      for (int c = 0; c < W && !abort; ++c, ++p) {
        if ((int)(p % C::kGroups) != grp) continue;
        const uint32_t sl = p % NS;
        const int pix = r * W + c;
        float mk[F], rs[F];
        if (chain) {
          load_row(blk<T>(a.cat, tile, P, pix, F), m, 0, F, mk);
        } else {
          load_row(blk<T>(a.prev, tile, P, pix, F), m, 0, F, mk);
          if (a.res) load_row(blk<T>(a.res, tile, P, pix, F), m, 0, F, rs);
        }
        if (!uwait(&accf[sl], (p / NS) & 1, err, abort)) break;
        tc_fence_after();
        float g[F];
        tread<F>(tl, sl * F, g);
        tc_fence_before();
        warp_arrive(&acce[sl]);
        if (!chain) {
          if (a.res) {
#pragma unroll
            for (int n = 0; n < F; ++n) g[n] += rs[n];
          }
#pragma unroll
          for (int n = 0; n < F; ++n) g[n] = mk[n] > 0.f ? g[n] : 0.f;
          store_row(blk<T>(a.out, tile, P, pix, F), m, 0, F, g);
          continue;
        }
#pragma unroll
        for (int n = 0; n < F; ++n) g[n] = mk[n] > 0.f ? g[n] : 0.f;
        store_row(blk<T>(a.gcatm, tile, P, pix, F), m, 0, F, g);
        const uint32_t b = p % NB;
        T* ca = reinterpret_cast<T*>(casm + b * (kTile * F * 2));
#pragma unroll
        for (int gq = 0; gq < F / 8; ++gq) st8(ca + ((int64_t)gq * kTile + m) * 8, g + 8 * gq);
        fence_proxy_async_smem();
        warp_arrive(&caf[b]);
        if (pend) second_half();
        pend = true;
        pq = p;
        ptile = tile;
        pr = r;
        pc = c;
      }
    }
    if (pend && !abort) second_half();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ============================================================== weight gradients
template <int F>
struct WgCfg {
  static constexpr int kBlk = kTile * F * 2;
  static constexpr int kNX = 3;                  // X column slots (4 blocks each: kernel rows + spare)
  static constexpr int kNG = 4;                  // G column slots (+2 mirrors)
  static constexpr int kSmem = kNX * 4 * kBlk + (kNG + 2) * kBlk + 512;
};

constexpr int kWgThreads = 256;  // producer, issuer, waiter, idle, 4 readers

// One zero block (largest F) for kernel rows above the lattice.
static __device__ __align__(128) uint8_t g_zero_block[kTile * 32 * 2];

template <int F>
__global__ void __launch_bounds__(kWgThreads, 1) wgrad_tc_kernel(const __grid_constant__ WgTcArgs a, int H, int W,
                                                                 int64_t n_items, int* err) {
  using C = WgCfg<F>;
  static_assert(F == 32, "the stacked-row MMA needs 4 blocks of 32 channels (M = 128)");
  using T = tc16;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* xr = smem;                            // [kNX][4][kBlk]
  uint8_t* gr = smem + C::kNX * 4 * C::kBlk;     // [kNG + 2][kBlk]
  uint64_t* bars = reinterpret_cast<uint64_t*>(gr + (C::kNG + 2) * C::kBlk);
  uint64_t* xfull = bars;
  uint64_t* xempty = bars + C::kNX;
  uint64_t* gfull = bars + 2 * C::kNX;
  uint64_t* gempty = gfull + C::kNG;
  uint64_t* done = gempty + C::kNG;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int P = H * W;
  const int ntc = a.ntc, dc0 = a.dc0, n = a.n;
  // G columns of an item: y_min..W-1; column y is used by input columns
  // x in [y + dc0, y + dc0 + ntc - 1] (clipped to the lattice)
  const int y_min = -dc0 - ntc + 1 > 0 ? -dc0 - ntc + 1 : 0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < C::kNX; ++i) {
      mbar_init(&xfull[i], 1);
      mbar_init(&xempty[i], 1);
    }
    for (int i = 0; i < C::kNG; ++i) {
      mbar_init(&gfull[i], 1);
      mbar_init(&gempty[i], 1);
    }
    mbar_init(done, 1);
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
  // zero the accumulator (rows = lanes, 96 columns); the spare fourth block
  // of every X slot holds ones, so accumulator rows 96..127 collect the
  // column sums of G over the samples: the bias gradient (see a.bias).
  if (warp >= 4) {
    const uint32_t tl = tmem + ((uint32_t)((warp % 4) * 32) << 16);
    for (int c0 = 0; c0 < 96; c0 += 16) tmem_zero16(tl + c0);
    tmem_st_wait();
    const uint4 one8 = make_uint4(kTcOnePair, kTcOnePair, kTcOnePair, kTcOnePair);  // 1.0 x 8 in the 16-bit format
    for (int i = threadIdx.x - 128; i < C::kNX * (C::kBlk / 16); i += 128) {
      const int slot = i / (C::kBlk / 16), e = i % (C::kBlk / 16);
      reinterpret_cast<uint4*>(xr + (slot * 4 + 3) * C::kBlk)[e] = one8;
    }
    fence_proxy_async_smem();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  bool abort = false;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------------------------------------------------------- producer
      uint32_t gx = 0, gg = 0;
      for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
        const int64_t tile = it / H;
        const int r = (int)(it % H);
        for (int x = 0; x < W && !abort; ++x, ++gx) {
          // X column x: ring rows k hold X rows r + x_row0 + k (zero above the lattice)
          const uint32_t xs = gx % C::kNX;
          if (gx >= C::kNX && !pwait(&xempty[xs], ((gx / C::kNX) - 1) & 1, err, abort)) break;
          mbar_arrive_expect_tx(&xfull[xs], (uint32_t)a.x_rows * C::kBlk);
          for (int k = 0; k < a.x_rows; ++k) {
            const int rr = r + a.x_row0 + k;
            const void* src = rr >= 0 ? (const void*)blk<T>(a.X, tile, P, rr * W + x, F) : (const void*)g_zero_block;
            bulk_g2s(xr + (xs * 4 + k) * C::kBlk, src, C::kBlk, &xfull[xs]);
          }
          // G columns first needed by input column x
          const int y_lo = x == 0 ? y_min : x - dc0;
          const int y_hi = x == 0 ? (-dc0 < W - 1 ? -dc0 : W - 1) : (x - dc0 < W - 1 ? x - dc0 : W - 1);
          for (int y = y_lo; y <= y_hi && !abort; ++y, ++gg) {
            const uint32_t s = gg % C::kNG;
            if (gg >= C::kNG && !pwait(&gempty[s], ((gg / C::kNG) - 1) & 1, err, abort)) break;
            const bool mirror = s < 2 && ntc > 1;
            mbar_arrive_expect_tx(&gfull[s], (mirror ? 2u : 1u) * C::kBlk);
            const T* src = blk<T>(a.G, tile, P, r * W + y, F);
            bulk_g2s(gr + s * C::kBlk, src, C::kBlk, &gfull[s]);
            if (mirror) bulk_g2s(gr + (C::kNG + s) * C::kBlk, src, C::kBlk, &gfull[s]);
          }
        }
      }
    }
  } else if (warp == 2) {
    // ------------------------------------------------------------------ waiter
    uint32_t gx = 0, gg = 0;
    bool stop = false;
    for (int64_t it = blockIdx.x; it < n_items && !stop; it += gridDim.x) {
      for (int x = 0; x < W; ++x, ++gx) {
        pwait(&xfull[gx % C::kNX], (gx / C::kNX) & 1, err, abort);
        const int y_lo = x == 0 ? y_min : x - dc0;
        const int y_hi = x == 0 ? (-dc0 < W - 1 ? -dc0 : W - 1) : (x - dc0 < W - 1 ? x - dc0 : W - 1);
        for (int y = y_lo; y <= y_hi; ++y, ++gg) pwait(&gfull[gg % C::kNG], (gg / C::kNG) & 1, err, abort);
        stop = step_rendezvous(abort);
        if (stop) break;
      }
    }
    abort = stop || abort;
  } else if (warp == 1) {
    // ------------------------------------------------------------------ issuer
    const uint64_t xa0 = umma_sdesc(smem_u32(xr), 128, 2048);
    const uint64_t gb0 = umma_sdesc(smem_u32(gr), 128, 2048);
    constexpr uint32_t kBlk16 = C::kBlk >> 4;
    const uint32_t g_off16 = (uint32_t)(a.g0 / 8) * (2048 >> 4);
    uint32_t gx = 0;
    uint32_t gbase = 0;  // G load count at the item's column y_min
    for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
      for (int x = 0; x < W; ++x, ++gx) {
        abort = step_rendezvous(false);
        if (abort) break;
        tc_fence_after();
        if (lane == 0) {
          // window of G columns fed by X column x: c = x - dc, jpos = c - (x - dc0 - ntc + 1)
          const int wlo = x - dc0 - ntc + 1;
          const int ca = wlo > y_min ? wlo : y_min;
          const int cb = x - dc0 < W - 1 ? x - dc0 : W - 1;
          if (ca <= cb) {
            const uint32_t gs = (gbase + (uint32_t)(ca - y_min)) % C::kNG;
            const uint32_t idesc = umma_idesc_tc16_mn(128, (cb - ca + 1) * n);
            const uint32_t d = tmem + (uint32_t)((ca - wlo) * n);
            const uint32_t xs = gx % C::kNX;
#pragma unroll
            for (int ks = 0; ks < kTile / 16; ++ks)
              umma_bf16(d, xa0 + xs * 4 * kBlk16 + ks * 16, gb0 + gs * kBlk16 + g_off16 + ks * 16, idesc, 1u);
          }
          umma_commit(&xempty[gx % C::kNX]);
          // G columns whose last input column is x
          const int r_lo = x == W - 1 ? (W - 1 - dc0 - ntc + 1 > y_min ? W - 1 - dc0 - ntc + 1 : y_min)
                                      : x - dc0 - ntc + 1;
          const int r_hi = x == W - 1 ? W - 1 : x - dc0 - ntc + 1;
          for (int y = r_lo; y <= r_hi; ++y)
            if (y >= y_min) umma_commit(&gempty[(gbase + (uint32_t)(y - y_min)) % C::kNG]);
        }
        __syncwarp();
      }
      gbase += (uint32_t)(W - y_min);
    }
    if (lane == 0) umma_commit(done);
  } else if (warp >= 4) {
    // ------------------------------------------------------------------ readers
    const int q4 = warp % 4;  // lane quarter = stacked row block = kernel row of ring row q4
    uwait(done, 0, err, abort);
    tc_fence_after();
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16);
    if (!abort && q4 < a.x_rows) {
      float* dst = a.part + ((int64_t)blockIdx.x * a.x_rows * 32 + q4 * 32 + lane) * (ntc * n);
      for (int c0 = 0; c0 < ntc * n; c0 += 16) {
        float v[16];
        tmem_ld16(tl + c0, v);
        tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 16; ++j) dst[c0 + j] = v[j];
      }
    }
    if (!abort && q4 == 3 && a.bias_jpos >= 0) {
      // row 96 (all rows of the ones block are equal): column block bias_jpos
      // meets every G column exactly once, at input column x = its column
      float* dst = a.part_bias + (int64_t)blockIdx.x * n;
      for (int c0 = 0; c0 < n; c0 += 16) {
        float v[16];
        tmem_ld16(tl + a.bias_jpos * n + c0, v);
        tmem_ld_wait();
        if (lane == 0)
#pragma unroll
          for (int j = 0; j < 16; ++j) dst[c0 + j] = v[j];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
  }
}

// Sums the per-CTA partials in CTA order into the raw kernel gradient
// dW[((i*kw + j)*cin + ci)*n + co] (i = kernel row, j = kernel column).
// Sums the per-CTA partials in a fixed order: block = 32 elements x 8 lanes
// of partials; lane group pg sums partials pg, pg + 8, ...; the 8 sums are
// then added in order pg = 0..7.
__global__ void __launch_bounds__(256) wgrad_reduce_kernel(const float* part, int parts, int x_rows, int ntc, int n,
                                                           int kw, int kcol0, float* dW, const float* part_bias,
                                                           float* db) {
  __shared__ float acc[8][33];
  const int per = x_rows * 32 * ntc * n;
  const int eg = threadIdx.x % 32, pg = threadIdx.x / 32;
  const int e = blockIdx.x * 32 + eg;
  const bool bias = e >= per;
  float s = 0.f;
  if (!bias) {
#pragma unroll 4
    for (int b = pg; b < parts; b += 8) s += part[(int64_t)b * per + e];
  } else if (db && e < per + n) {
#pragma unroll 4
    for (int b = pg; b < parts; b += 8) s += part_bias[(int64_t)b * n + (e - per)];
  }
  acc[pg][eg] = s;
  __syncthreads();
  if (pg != 0) return;
  float t = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) t += acc[q][eg];
  if (bias) {
    if (db && e < per + n) db[e - per] = t;
    return;
  }
  const int row = e / (ntc * n), col = e % (ntc * n);
  const int i = row / 32, ci = row % 32;
  const int jpos = col / n, co = col % n;
  const int j = kcol0 + (ntc - 1 - jpos);
  dW[((int64_t)(i * kw + j) * 32 + ci) * n + co] = t;
}

// Bias gradient, step 1: per tile (one CTA, thread = sample) the sum over
// pixels of G[.., g0 + co], reduced over the tile's samples; step 2 sums the
// tiles in order.
__global__ void __launch_bounds__(128) bias_tile_kernel(const tc16* G, int P, int W, int g0, int n,
                                                        int64_t batch, float* part) {
  constexpr int F = 32;
  __shared__ float red[4][32];
  const int H = P / W;
  const int64_t tile = blockIdx.x / H;
  const int r = (int)(blockIdx.x % H);
  const int m = threadIdx.x;
  float s[F];
#pragma unroll
  for (int c = 0; c < F; ++c) s[c] = 0.f;
  if (tile * kTile + m < batch) {
    for (int pix = r * W; pix < (r + 1) * W; ++pix) {
      float v[F];
      load_row(blk<tc16>(G, tile, P, pix, F), m, 0, F, v);
#pragma unroll
      for (int c = 0; c < F; ++c) s[c] += v[c];
    }
  }
  const int lane = m % 32, warp = m / 32;
#pragma unroll
  for (int c = 0; c < F; ++c) {
    float v = s[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    s[c] = v;
  }
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < F; ++c) red[warp][c] = s[c];
  __syncthreads();
  if (m < n) part[(int64_t)blockIdx.x * n + m] = red[0][g0 + m] + red[1][g0 + m] + red[2][g0 + m] + red[3][g0 + m];
}

__global__ void bias_reduce_kernel(const float* part, int64_t tiles, int n, float* db) {
  const int co = threadIdx.x;
  if (co >= n) return;
  float s = 0.f;
  for (int64_t t = 0; t < tiles; ++t) s += part[t * n + co];
  db[co] = s;
}

// ============================================================== per-sample rows
// Per-sample weight gradients of a 32-input-channel conv as tensor-core
// products, one sample at a time: with K = the sample's pixels (padded to a
// multiple of 16), A = its input activations shifted by each tap (M = taps x
// 32 channels: four taps per M = 128 tile, one more 8-row group of ones whose
// products are the bias gradient), B = its output gradients (N = 16 or 32):
// D_b[(tap, ci)][n] = sum_pix X_b[pix + tap][ci] G_b[pix][n]. Both operands
// MN-major in shared memory ([8-channel group][pixel][8 channels], LBO 128 B
// along the pixels, SBO = K * 16 B along the channels), staged from the
// blocked layouts by 8 warps (zero outside the lattice); one thread issues
// the K/16 MMAs of each sample into its own N columns of a TMEM buffer that
// holds 8 samples; 4 drain warps (TMEM lane quarter = tap slot, lane = input
// channel) write each (row, n) as 8 consecutive samples (32 bytes) of the
// parameter-major rows. Work item = (8 samples, M tile); two 8-sample TMEM
// buffers and two staging stages of S samples (2, or 1 on lattices whose
// operands would not fit) overlap staging, MMAs and writes. Every wait is
// bounded.
namespace wgrows {
constexpr int kStageWarps = 8, kIssuer = 8, kThreads = 32 * 13;
constexpr int kGroupRows = 16;  // A: 16 groups of 8 rows (M = 128)
__host__ __device__ inline int ksteps(int H, int W) { return (H * W + 15) / 16; }
inline int stage_bytes(int S, int H, int W, int N) { return S * (kGroupRows + N / 8) * ksteps(H, W) * 16 * 16; }
// two samples per stage when their operands fit in shared memory and one
// staging thread per (pixel, sample) remains
inline int samples_per_stage(int H, int W, int N) {
  return 2 * stage_bytes(2, H, W, N) + 256 <= 200 * 1024 && ksteps(H, W) * 32 <= kStageWarps * 32 ? 2 : 1;
}
}  // namespace wgrows

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 gradient values of a (pixel, sample, 8-channel group) as one 16-byte
// operand row: 16-bit gradients as they are, float gradients rounded.
__device__ __forceinline__ uint4 grad_row(const tc16* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }
__device__ __forceinline__ uint4 grad_row(const float* p) {
  const float4 x = __ldg(reinterpret_cast<const float4*>(p));
  const float4 y = __ldg(reinterpret_cast<const float4*>(p) + 1);
  return make_uint4(pack_tc16x2(x.x, x.y), pack_tc16x2(x.z, x.w), pack_tc16x2(y.x, y.y), pack_tc16x2(y.z, y.w));
}

// CIN input channels (32: four taps per M tile, 64: two), N output channels,
// TG the gradients' type (16-bit, or float from the CUDA-core adjoint). A
// work item is SPB = 256 / N samples (one TMEM buffer of 256 columns).
template <int CIN, int N, typename TG>
__global__ void __launch_bounds__(wgrows::kThreads, 1) wgrad_rows_tc_kernel(const __grid_constant__ WgRowsArgs a,
                                                                             int H, int W, int S, int* err) {
  using namespace wgrows;
  using T = tc16;
  constexpr int NG = N / 8;
  constexpr int TPM = 128 / CIN;  // taps per M tile
  constexpr int GPT = CIN / 8;    // 8-channel groups per tap
  constexpr int SPB = 256 / N;    // samples per TMEM buffer (work item)
  extern __shared__ __align__(1024) uint8_t smem[];
  const int P = H * W;
  const int KS = ksteps(H, W), Qk = KS * 16;
  const int stage = S * (kGroupRows + NG) * Qk * 16;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 2 * stage);
  uint64_t* full = bars;          // [2] staged (8 warp arrivals)
  uint64_t* empty = bars + 2;     // [2] MMAs done with a stage (commit)
  uint64_t* accfull = bars + 4;   // [2] a work item's products complete (commit)
  uint64_t* accempty = bars + 6;  // [2] written out (4 warp arrivals)
  uint64_t* drain = bars + 8;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 9);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int ntiles_m = (a.ntaps + 1 + TPM - 1) / TPM;  // taps and the ones slot
  const int64_t groups = (a.batch + SPB - 1) / SPB;
  const int64_t items = groups * ntiles_m;
  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(&full[i], kStageWarps);
      mbar_init(&empty[i], 1);
      mbar_init(&accfull[i], 1);
      mbar_init(&accempty[i], 4);
    }
    mbar_init(drain, 1);
    fence_mbar_init();
  }
  if (warp == kIssuer) {
    tmem_alloc(tslot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool abort = false;
  const int subs = SPB / S;

  if (warp < kStageWarps) {
    // ---------------------------------------------------------------- staging
    const int tid = threadIdx.x;
    uint32_t gc = 0;
    for (int64_t it = blockIdx.x; it < items && !abort; it += gridDim.x) {
      const int64_t grp = it / ntiles_m;
      const int mt = (int)(it % ntiles_m);
      for (int sub = 0; sub < subs && !abort; ++sub, ++gc) {
        const uint32_t st = gc % 2;
        if (gc >= 2 && !mbar_wait(&empty[st], ((gc / 2) - 1) & 1, err)) {
          abort = true;
          break;
        }
        uint8_t* base = smem + st * stage;
        // thread = (pixel p, sample s) of the stage, s fastest (the S samples of
        // a (pixel, group) are adjacent in the blocked layout); it stages that
        // pixel's 16 A groups (taps x channel groups) and NG B groups, every
        // load issued before the first store.
        if (tid < Qk * S) {
          const int s = tid % S;
          const int p = tid / S;
          const int64_t b = grp * SPB + sub * S + s;
          const int64_t tile = b / kTile;
          const int m = (int)(b % kTile);
          const int r0 = p / W, cq = p - (p / W) * W;
          const bool live = p < P;
          uint8_t* arow = base + ((int64_t)s * kGroupRows * Qk + p) * 16;
          uint8_t* brow = base + ((int64_t)S * kGroupRows * Qk + (int64_t)s * NG * Qk + p) * 16;
          const uint4* src[TPM];
#pragma unroll
          for (int k = 0; k < TPM; ++k) {
            const int t = TPM * mt + k;
            src[k] = nullptr;
            if (live && t < a.ntaps) {
              const int r = r0 + a.dr[t], cc = cq + a.dc[t];
              if (r >= 0 && r < H && cc >= 0 && cc < W)
                src[k] = reinterpret_cast<const uint4*>(blk<T>(a.X, tile, P, r * W + cc, CIN) + m * 8);
            }
          }
          const TG* gsrc = live ? blk<TG>(a.G, tile, P, p, a.gC) + ((int64_t)(a.g0 / 8) * kTile + m) * 8 : nullptr;
          const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
          uint4 va[kGroupRows], vb[NG];
#pragma unroll
          for (int k = 0; k < TPM; ++k)
#pragma unroll
            for (int g = 0; g < GPT; ++g) va[GPT * k + g] = src[k] ? __ldg(src[k] + g * kTile) : zero;
#pragma unroll
          for (int g = 0; g < NG; ++g) vb[g] = gsrc ? grad_row(gsrc + (int64_t)g * kTile * 8) : zero;
#pragma unroll
          for (int k = 0; k < TPM; ++k)
            if (live && TPM * mt + k == a.ntaps) va[GPT * k] = make_uint4(kTcOnePair, kTcOnePair, kTcOnePair, kTcOnePair);
#pragma unroll
          for (int i = 0; i < kGroupRows; ++i) *reinterpret_cast<uint4*>(arow + (int64_t)i * Qk * 16) = va[i];
#pragma unroll
          for (int g = 0; g < NG; ++g) *reinterpret_cast<uint4*>(brow + (int64_t)g * Qk * 16) = vb[g];
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&full[st]);
      }
    }
  } else if (warp == kIssuer) {
    // ---------------------------------------------------------------- issuer
    const uint32_t idesc = umma_idesc_tc16_mn(128, N);
    uint32_t gc = 0, li = 0;
    for (int64_t it = blockIdx.x; it < items && !abort; it += gridDim.x, ++li) {
      const uint32_t buf = li % 2;
      if (li >= 2 && !mbar_wait(&accempty[buf], ((li / 2) - 1) & 1, err)) {
        abort = true;
        break;
      }
      tc_fence_after();
      for (int sub = 0; sub < subs; ++sub, ++gc) {
        const uint32_t st = gc % 2;
        if (!mbar_wait(&full[st], (gc / 2) & 1, err)) {
          abort = true;
          break;
        }
        tc_fence_after();
        if (lane == 0) {
          const uint32_t base = smem_u32(smem + st * stage);
          for (int s = 0; s < S; ++s) {
            const uint32_t d = tmem + buf * 256 + (uint32_t)((sub * S + s) * N);
            const uint32_t ab = base + (uint32_t)(s * kGroupRows * Qk * 16);
            const uint32_t bb = base + (uint32_t)((S * kGroupRows + s * NG) * Qk * 16);
            for (int ks = 0; ks < KS; ++ks)
              umma_bf16(d, umma_sdesc(ab + ks * 256, 128, Qk * 16), umma_sdesc(bb + ks * 256, 128, Qk * 16), idesc,
                        ks > 0 ? 1u : 0u);
          }
          umma_commit(&empty[st]);
        }
        __syncwarp();
      }
      if (abort) break;
      if (lane == 0) umma_commit(&accfull[buf]);
      __syncwarp();
    }
    if (lane == 0) {
      umma_commit(drain);
      mbar_wait(drain, 0, err);
    }
    __syncwarp();
  } else {
    // ---------------------------------------------------------------- drain
    // warp 9..12 -> TMEM lane quarter 1, 2, 3, 0; M row R = quarter * 32 + lane
    // is input channel R % CIN of tap slot R / CIN
    const int q4 = warp % 4;
    const int R = q4 * 32 + lane;
    const int k = R / CIN, ci = R % CIN;
    const bool vec = (a.o_ld % 4) == 0 && (a.o_col % 4) == 0;
    constexpr int JB = SPB < 8 ? SPB : 8;  // samples written per store group
    uint32_t li = 0;
    for (int64_t it = blockIdx.x; it < items && !abort; it += gridDim.x, ++li) {
      const int64_t grp = it / ntiles_m;
      const int mt = (int)(it % ntiles_m);
      const uint32_t buf = li % 2;
      bool ok = mbar_wait(&accfull[buf], (li / 2) & 1, err);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        abort = true;
        break;
      }
      tc_fence_after();
      const int t = TPM * mt + k;
      const int64_t b0 = grp * SPB;
      const int nb = a.batch - b0 < SPB ? (int)(a.batch - b0) : SPB;
      const uint32_t tl = tmem + buf * 256 + ((uint32_t)(q4 * 32) << 16);
      // slot k is warp-uniform when CIN >= 32
      if (t <= a.ntaps) {
        for (int nc = 0; nc < NG; ++nc) {
          for (int j0 = 0; j0 < SPB; j0 += JB) {
            float v[JB][8];
#pragma unroll
            for (int j = 0; j < JB; ++j) tmem_ld8(tl + (uint32_t)((j0 + j) * N + nc * 8), v[j]);
            tmem_ld_wait();
            if (t < a.ntaps || ci == 0) {
#pragma unroll
              for (int n = 0; n < 8; ++n) {
                const int64_t row = t < a.ntaps ? a.o_kernel + ((int64_t)(t * CIN + ci) * N + nc * 8 + n)
                                                : a.o_bias + nc * 8 + n;
                float* dst = a.O + row * a.o_ld + a.o_col + b0 + j0;
                const int nj = nb - j0;
                if (vec && nj >= JB && JB % 4 == 0) {
#pragma unroll
                  for (int q = 0; q < JB / 4; ++q)
                    reinterpret_cast<float4*>(dst)[q] =
                        make_float4(v[4 * q][n], v[4 * q + 1][n], v[4 * q + 2][n], v[4 * q + 3][n]);
                } else {
#pragma unroll
                  for (int j = 0; j < JB; ++j)
                    if (j < nj) dst[j] = v[j][n];
                }
              }
            }
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
  if (warp == kIssuer) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ============================================================== launchers
template <int F>
static int set_smem(const void* fn, int bytes) {
  return check_cuda(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                    "cudaFuncSetAttribute");
}

static int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 148;
  }
  return sms;
}

int launch_bwd_op(const BwdOpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    int st = set_smem<32>((const void*)bwd_op_kernel<32>, BwdCfg<32>::kSmem);
    if (st != FK_OK) return st;
    attr = true;
  }
  const int64_t items = tiles * H;
  int64_t grid = sm_count();
  if (grid > items) grid = items;
  // shared memory above half an SM keeps one CTA (512 TMEM columns) per SM
  bwd_op_kernel<32><<<(unsigned)grid, kPipeThreads, BwdCfg<32>::kSmem, s>>>(a, H, W, items, err);
  return check_cuda(launched(), "bwd_op_kernel");
}

int64_t wgrad_tc_grid(int64_t tiles, int H) {
  int64_t grid = sm_count();
  return grid < tiles * H ? grid : tiles * H;
}

int64_t wgrad_tc_part_floats(int64_t tiles, int H) { return wgrad_tc_grid(tiles, H) * (3 * 32 * 96 + 32); }

int launch_wgrad_tc(const WgTcArgs& a, int kw, int kcol0, float* dW, float* db, int64_t tiles, int H, int W,
                    int* err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    int st = set_smem<32>((const void*)wgrad_tc_kernel<32>, WgCfg<32>::kSmem);
    if (st != FK_OK) return st;
    attr = true;
  }
  const int64_t items = tiles * H;
  const int64_t grid = wgrad_tc_grid(tiles, H);
  wgrad_tc_kernel<32><<<(unsigned)grid, kWgThreads, WgCfg<32>::kSmem, s>>>(a, H, W, items, err);
  FK_CUDA(launched());
  const int per = a.x_rows * 32 * a.ntc * a.n + (a.bias_jpos >= 0 ? a.n : 0);
  wgrad_reduce_kernel<<<(per + 31) / 32, 256, 0, s>>>(a.part, (int)grid, a.x_rows, a.ntc, a.n, kw, kcol0, dW,
                                                      a.part_bias, a.bias_jpos >= 0 ? db : nullptr);
  return check_cuda(launched(), "wgrad_reduce_kernel");
}

bool wgrad_rows_tc_supported(int H, int W, int N) {
  const int S = wgrows::samples_per_stage(H, W, N);
  return (N == 16 || N == 32 || N == 64) && 2 * wgrows::stage_bytes(S, H, W, N) + 256 <= 220 * 1024 &&
         wgrows::ksteps(H, W) * 16 * S <= wgrows::kStageWarps * 32;
}

template <int CIN, int N, typename TG>
static int rows_launch(const WgRowsArgs& a, int H, int W, int* err, cudaStream_t s) {
  static std::once_flag once;
  static int attr = FK_OK;
  std::call_once(once, [] {
    attr = set_smem<32>((const void*)wgrad_rows_tc_kernel<CIN, N, TG>, 220 * 1024);
  });
  if (attr != FK_OK) return attr;
  const int S = wgrows::samples_per_stage(H, W, N);
  const int smem = 2 * wgrows::stage_bytes(S, H, W, N) + 256;
  const int64_t items = (a.batch + 256 / N - 1) / (256 / N) * ((a.ntaps + 128 / CIN) / (128 / CIN));
  int64_t grid = sm_count();
  if (grid > items) grid = items;
  wgrad_rows_tc_kernel<CIN, N, TG><<<(unsigned)grid, wgrows::kThreads, smem, s>>>(a, H, W, S, err);
  return check_cuda(launched(), "wgrad_rows_tc_kernel");
}

int launch_wgrad_rows_tc(const WgRowsArgs& a, int H, int W, int* err, cudaStream_t s) {
  if (!wgrad_rows_tc_supported(H, W, a.N) || a.ntaps < 1 || a.ntaps > 9) return FK_ERR_ARG;
  if (a.cin == 32 && !a.g_float && a.N == 16) return rows_launch<32, 16, tc16>(a, H, W, err, s);
  if (a.cin == 32 && !a.g_float && a.N == 32) return rows_launch<32, 32, tc16>(a, H, W, err, s);
  if (a.cin == 64 && a.g_float && a.N == 32) return rows_launch<64, 32, float>(a, H, W, err, s);
  if (a.cin == 64 && a.g_float && a.N == 64) return rows_launch<64, 64, float>(a, H, W, err, s);
  return FK_ERR_ARG;
}

int launch_bias_sum(const void* G, int64_t tiles, int H, int W, int g0, int n, int64_t batch, float* part, float* db,
                    cudaStream_t s) {
  bias_tile_kernel<<<(unsigned)(tiles * H), 128, 0, s>>>(static_cast<const tc16*>(G), H * W, W, g0, n, batch,
                                                         part);
  FK_CUDA(launched());
  bias_reduce_kernel<<<1, 32, 0, s>>>(part, tiles * H, n, db);
  return check_cuda(launched(), "bias_reduce_kernel");
}

}  // namespace FK_NS
