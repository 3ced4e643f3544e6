// Pipelined column-scatter tensor-core engine for the V/H/C ops of the AR2D
// forward (causal convs after the first, F <= 32), on the pipeline of
// fk_pipe.cuh. Twelve warps per CTA (one CTA per SM):
//   warp 0: producer; warp 1: MMA issuer; warp 2: waiter (fk_pipe.cuh);
//   warp 3: chain issuer -- the chained 1x1 MMA of each output (y conv for
//       the V op, x conv for the H op, the head for the last C op) on the
//       epilogue's staged bf16 activations, into one of four accumulators;
//   warps 4-11: epilogue in two groups of four warps taking alternate outputs
//       (thread = sample, TMEM lane quarter = warp % 4): bias, relu, residual
//       (prefetched before the accumulator wait), stream store and
//       chained-conv staging; the part after the chained MMA (Cat halves, or
//       the head's normalised log psi partials, summed in pixel order through
//       shared memory) runs after the group's next output, which hides the
//       chained MMA's round trip.
// Compared with gathering nine taps per output (18 MMAs of N = F per pixel)
// this issues 6-7 MMAs of N = 3F per pixel.
//
// Each output accumulates its taps in column-major order (tap column outer,
// tap row inner, K steps innermost), the order of the per-pixel engine in
// fk_ar2d.cu, and the epilogue arithmetic is the same, so both engines give
// bitwise the same result.
#include "fk_pipe.cuh"

namespace FK_NS {

// Forward-specific shared memory on top of the pipeline's ring and weights.
template <int F>
struct FwdCfg {
  using C = PipeCfg<F>;
  static constexpr int kCW = F * 32 * 2;            // chained 1x1 weights
  static constexpr int kBias = 64 * 4;              // main (F) + chained (<= 32) biases
  static constexpr int kMaxW = 16;                  // head partials [W][128] float2
  static constexpr int kSmemBase = C::kRing + C::kW + kCW + C::kCA + kBias + C::kBars;
  // TMEM: a ring of kNS accumulator slots of F columns, then the kNB chained
  // accumulators (32 columns each) -- a deeper ring than the adjoint's, whose
  // chained accumulators take 2F columns each
  static constexpr int kNS = (512 - C::kNB * 32) / F;
  static constexpr uint32_t kChainCol = (uint32_t)(kNS * F);
  static int head_bytes(int w) { return w * kTile * 8; }
};

// RES: the op adds a residual to its stream output (its own instantiation, so
// that ops without one compile without the residual prefetch).
template <int F, bool RES>
__global__ void __launch_bounds__(kPipeThreads, 1) op_pipe_kernel(const __grid_constant__ OpArgs a, int H, int W,
                                                                  int64_t n_items, int* err) {
  // With a work list, n_items is an upper bound and the list's count is read
  // on the device.
  using C = PipeCfg<F>;
  using FC = FwdCfg<F>;
  using T = tc16;
  constexpr int F2 = F / 2;
  constexpr int NC2 = F2 < 16 ? 16 : F2;
  constexpr int NB = C::kNB;
  constexpr int NS = FC::kNS;
  constexpr int NR = C::kNcol;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* ring = smem;
  uint8_t* wsm = smem + C::kRing;
  uint8_t* cwsm = wsm + C::kW;
  uint8_t* casm = cwsm + FC::kCW;
  float* bias_sm = reinterpret_cast<float*>(casm + C::kCA);
  uint64_t* bars = reinterpret_cast<uint64_t*>(casm + C::kCA + FC::kBias);
  uint64_t* full = bars;
  uint64_t* empty = bars + NR;
  uint64_t* wbar = bars + 2 * NR;
  uint64_t* accf = wbar + 1;
  uint64_t* acce = accf + NS;
  uint64_t* caf = acce + NS;
  uint64_t* cf = caf + NB;
  uint64_t* head_ready = cf + NB;
  uint64_t* head_free = head_ready + 1;
  uint64_t* drain = head_free + 1;  // [2]: MMA completion before teardown (issuer, chain issuer)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 2);
  float2* head_sm = reinterpret_cast<float2*>(smem + FC::kSmemBase);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int P = H * W;
  const int kind = a.kind;
  const int nrows = kind == kConvH ? 1 : 3;
  const bool has_chain = !(kind == kConvC && !a.last);
  const bool head = kind == kConvC && a.last;
  const int cnp = kind == kConvC ? 16 : NC2;
  const uint32_t chain_bytes = (uint32_t)(F * cnp * 2);
  const uint32_t wbytes = (uint32_t)(nrows * C::kWRow);
  // outputs x + o0 .. x + o0 + 2 receive input column x; output c is complete
  // after input column min(c - o0, W - 1)
  const int o0 = kind == kConvV ? -1 : 0;

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
    mbar_init(head_ready, 4);
    mbar_init(head_free, 4);
    mbar_init(&drain[0], 1);
    mbar_init(&drain[1], 1);
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < F; i += blockDim.x) bias_sm[i] = a.main.b[i];
  if (has_chain)
    for (int i = threadIdx.x; i < cnp; i += blockDim.x) bias_sm[32 + i] = a.chain.b[i];
  if (warp == 1) {
    tmem_alloc(tslot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  bool abort = false;
  if (a.items) n_items = *a.n_items;
  auto item_at = [&](int64_t k) -> int64_t { return a.items ? (int64_t)a.items[k] : k; };

  const PipeGeom geom{H, W, nrows, kind == kConvH ? 0 : -2, o0, 0};
  const PipeItems items{a.items, n_items};
  if (warp == 0) {
    if (lane == 0)
      pipe_producer<F>(geom, items, a.in, ring, full, empty, wbar, WeightCopy{wsm, a.main.ws, wbytes},
                       WeightCopy{cwsm, a.chain.w, has_chain ? chain_bytes : 0u}, WeightCopy{nullptr, nullptr, 0u},
                       err, abort);
  } else if (warp == 1) {
    pipe_issuer<F, NS>(geom, items, ring, wsm, tmem, empty, accf, &drain[0], err, abort);
  } else if (warp == 2) {
    pipe_waiter<F, NS>(geom, items, full, wbar, acce, err, abort);
  } else if (warp == 3) {
    // ------------------------------------------------------------------ chain issuer
    // The chained 1x1 MMA of each output, on the epilogue's staged bf16
    // activations, into one of NB chained accumulators.
    if (has_chain && lane == 0) {
      const uint32_t idesc_c = umma_idesc_tc16(128, cnp);
      const uint64_t ca0 = umma_sdesc(smem_u32(casm), 2048, 128);
      const uint64_t cw0 = umma_sdesc(smem_u32(cwsm), cnp * 16, 128);
      pwait(wbar, 0, err, abort);
      uint32_t q = 0;
      for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
        for (int c = 0; c < W && !abort; ++c, ++q) {
          const uint32_t b = q % NB;
          if (!pwait(&caf[b], (q / NB) & 1, err, abort)) break;
          tc_fence_after();
#pragma unroll
          for (int ks = 0; ks < F / 16; ++ks)
            umma_bf16(tmem + FC::kChainCol + b * 32, ca0 + ((b * (kTile * F * 2) + ks * 2 * 2048) >> 4),
                      cw0 + ((ks * 2 * cnp * 16) >> 4), idesc_c, ks > 0 ? 1u : 0u);
          umma_commit(&cf[b]);
        }
      }
      umma_commit(&drain[1]);
      mbar_wait(&drain[1], 0, err);
    }
  } else {
    // ---------------------------------------------------------------- epilogue
    // Two groups of four warps take alternate outputs; within a group the TMEM
    // lane quarter is warp % 4, so thread (warp, lane) owns sample m. The part
    // after the chained MMA of an output runs after the first part of the
    // group's next output, which hides the chained MMA's round trip.
    const int grp = (warp - 4) / 4;
    const int q4 = warp % 4;
    const int m = q4 * 32 + lane;
    const uint32_t tl = tmem + ((uint32_t)(q4 * 32) << 16);
    const float* bm = bias_sm;
    const float* bc = bias_sm + 32;
    constexpr bool need_res = RES;
    // deferred second half: output index, tile, row, column
    bool pend = false;
    uint32_t pq = 0;
    int64_t ptile = 0;
    int pr = 0, pc = 0;
    auto second_half = [&]() {
      const uint32_t b = pq % NB;
      pend = false;
      if (!uwait(&cf[b], (pq / NB) & 1, err, abort)) return;
      tc_fence_after();
      float out[32];
      if (kind == kConvC)
        tread<16>(tl, FC::kChainCol + b * 32, out);
      else
        tread<NC2>(tl, FC::kChainCol + b * 32, out);
      tc_fence_before();
      const int pix = pr * W + pc;
      if (kind == kConvV) {
#pragma unroll
        for (int n = 0; n < F2; ++n) out[n] = fmaxf(out[n] + bc[n], 0.f);
        if (pr + 1 < H) store_row(blk<T>(a.cat, ptile, P, pix + W, F), m, F2, F2, out);
        if (pr == 0) {
#pragma unroll
          for (int n = 0; n < F2; ++n) out[n] = fmaxf(bc[n], 0.f);
          store_row(blk<T>(a.cat, ptile, P, pc, F), m, F2, F2, out);
        }
      } else if (kind == kConvH) {
#pragma unroll
        for (int n = 0; n < F2; ++n) out[n] = fmaxf(out[n] + bc[n], 0.f);
        const int sh = a.last ? 1 : 0;
        if (pc + sh < W) store_row(blk<T>(a.cat, ptile, P, pix + sh, F), m, 0, F2, out);
        if (sh && pc == 0) {
#pragma unroll
          for (int n = 0; n < F2; ++n) out[n] = fmaxf(bc[n], 0.f);
          store_row(blk<T>(a.cat, ptile, P, pix, F), m, 0, F2, out);
        }
      } else {
#pragma unroll
        for (int n = 0; n < 4; ++n) out[n] += bc[n];
        const int64_t sample = ptile * kTile + m;
        if (a.updown && sample < a.batch) {
          // EqualUpDownSpins (layers/spins_invariants.py:13-22)
          const int mk = a.updown[sample * P + pix];
          if (mk & 1) out[0] = -INFINITY;
          if (mk & 2) out[1] = -INFINITY;
        }
        // abstract_machine.py:56-57 normalisation (same arithmetic as the per-pixel engine)
        float a2 = 2.f * out[0], b2 = 2.f * out[1];
        float mx = fmaxf(a2, b2);
        float lse = 0.5f * (mx + logf(expf(a2 - mx) + expf(b2 - mx)));
        float re0 = out[0] - lse, re1 = out[1] - lse;
        bool up = spin_at(a.spins, a.batch, P, sample, pix) > 0.f;
        head_sm[pc * kTile + m] = make_float2(up ? re0 : re1, up ? out[2] : out[3]);
        if (a.cond && sample < a.batch)
          reinterpret_cast<float4*>(a.cond)[sample * P + pix] = make_float4(re0, re1, out[2], out[3]);
      }
    };
    // residual rows (raw bf16) of the group's next output in the same row,
    // loaded while the current output is processed
    uint4 rraw[F / 8];
    bool have_raw = false;
    uint32_t p = 0, it_count = 0;
    for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x, ++it_count) {
      const int64_t item = item_at(it);
      const int64_t tile = item / H;
      const int r = (int)(item % H);
      if (head && grp == 1 && it_count > 0 && !uwait(head_free, (it_count - 1) & 1, err, abort)) break;
      for (int c = 0; c < W && !abort; ++c, ++p) {
        if ((int)(p % C::kGroups) != grp) continue;
        const uint32_t b = p % NB;
        const uint32_t sl = p % NS;
        const int pix = r * W + c;
        float o[F];
        if (need_res && !have_raw) load_raw<F>(blk<T>(a.res, tile, P, pix, F), m, rraw);
        if (!uwait(&accf[sl], (p / NS) & 1, err, abort)) break;
        tc_fence_after();
        float acc[F];
        tread<F>(tl, sl * F, acc);
        tc_fence_before();
        warp_arrive(&acce[sl]);
        if (need_res) {
          unpack_raw<F>(rraw, o);
          have_raw = c + C::kGroups < W;
          if (have_raw) load_raw<F>(blk<T>(a.res, tile, P, pix + C::kGroups, F), m, rraw);
        }
        float cin[F];
        if (kind == kConvV) {
#pragma unroll
          for (int n = 0; n < F; ++n) acc[n] += bm[n];
          if (a.stream_out) {
            if (need_res) {
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
            if (need_res) {
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
        warp_arrive(&caf[b]);
        if (pend) second_half();
        pend = true;
        pq = p;
        ptile = tile;
        pr = r;
        pc = c;
      }
      if (head && !abort) {
        if (pend) second_half();
        // ordered compensated sum over the row's pixels (the per-pixel engine's order)
        if (grp == 1) {
          warp_arrive(head_ready);
        } else if (uwait(head_ready, it_count & 1, err, abort)) {
          Kahan kre, kim;
          for (int c = 0; c < W; ++c) {
            float2 v = head_sm[c * kTile + m];
            kre.add(v.x);
            kim.add(v.y);
          }
          a.row_partial[((int64_t)tile * H + r) * kTile + m] = make_float2(kre.s - kre.c, kim.s - kim.c);
          warp_arrive(head_free);
        }
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

constexpr int kMinSmem = 120 * 1024;

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
  if (head && W > FwdCfg<F>::kMaxW) return FK_ERR_ARG;
  if (!a.main.ws) return FK_ERR_ARG;
  // At least half of an SM's shared memory, so that one CTA (holding all 512
  // TMEM columns) runs per SM.
  int smem = FwdCfg<F>::kSmemBase + (head ? FwdCfg<F>::head_bytes(W) : 0);
  if (smem < kMinSmem) smem = kMinSmem;
  if (!attr) {
    const int most = FwdCfg<F>::kSmemBase + FwdCfg<F>::head_bytes(FwdCfg<F>::kMaxW);
    FK_CUDA(cudaFuncSetAttribute(op_pipe_kernel<F, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 most > kMinSmem ? most : kMinSmem));
    FK_CUDA(cudaFuncSetAttribute(op_pipe_kernel<F, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 most > kMinSmem ? most : kMinSmem));
    attr = true;
  }
  const int64_t items = tiles * H;
  int64_t grid = (int64_t)sms;  // one CTA per SM (512 TMEM columns)
  if (grid > items) grid = items;
  const bool res = (a.kind == kConvV && a.stream_out && a.res) || (a.kind == kConvC && !a.last && a.res);
  if (res)
    op_pipe_kernel<F, true><<<(unsigned)grid, kPipeThreads, smem, s>>>(a, H, W, items, err);
  else
    op_pipe_kernel<F, false><<<(unsigned)grid, kPipeThreads, smem, s>>>(a, H, W, items, err);
  return check_cuda(launched(), "op_pipe_kernel");
}

int launch_pipe_op(int F, const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  if (a.first) return FK_ERR_ARG;
  if (F == 16) return launch_pipe<16>(a, tiles, H, W, err, s);
  if (F == 32) return launch_pipe<32>(a, tiles, H, W, err, s);
  return FK_ERR_ARG;
}

bool pipe_supported(int F, int W) { return (F == 16 || F == 32) && W >= 2 && W <= FwdCfg<32>::kMaxW; }

static_assert(FwdCfg<32>::kSmemBase + 16 * kTile * 8 <= 227 * 1024, "pipelined engine exceeds shared memory");
static_assert(FwdCfg<16>::kSmemBase + 16 * kTile * 8 <= 227 * 1024, "pipelined engine exceeds shared memory");
static_assert(FwdCfg<32>::kChainCol + PipeCfg<32>::kNB * 32 <= 512 &&
                  FwdCfg<16>::kChainCol + PipeCfg<16>::kNB * 32 <= 512 && FwdCfg<32>::kNS >= 6,
              "TMEM layout");

}  // namespace FK_NS
