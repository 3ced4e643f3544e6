// Pipelined column-scatter tensor-core engine for the V/H/C ops of the AR2D
// forward (causal convs after the first, F <= 32).
//
// One persistent CTA per SM walks (tile, row) items; each item is one lattice
// row of 128 samples. Ten warps:
//   warp 0 (one thread): TMA producer. Loads the op's column-scatter weights
//       once, then every input column (the rows r-2..r -- only row r for the
//       H op -- of one lattice column, one bulk copy per [F/8][128][8] block)
//       into a ring of column slots;
//   warp 1 (one thread): MMA issuer. Input column x is multiplied once per
//       kernel row i by the three kernel columns stacked along N (N = 3F):
//       the product holds x's contributions to the three output columns it
//       feeds (x-1..x+1 for the V op, x..x+2 for the H and C ops), which
//       accumulate in three consecutive TMEM slots of a ring. An output is
//       committed to the epilogue after its last input column; the chained
//       1x1 MMA of an output is issued one output later, on the epilogue's
//       staged bf16 activations;
//   warps 2-9: epilogue in two groups of four warps taking alternate outputs
//       (thread = sample, TMEM lane quarter = warp % 4): bias, relu, residual
//       (prefetched before the accumulator wait), stream store, chained-conv
//       staging, and the second half after the chained MMA; the head's log psi
//       partials are summed in pixel order through shared memory.
// Compared with gathering nine taps per output (18 MMAs of N = F per pixel)
// this issues 6-7 MMAs of N = 3F per pixel: the single issuing thread, not the
// tensor pipe, bounds small-N MMA streams.
//
// Each output accumulates its taps in column-major order (tap column outer,
// tap row inner, K steps innermost), the order of the per-pixel engine in
// fk_ar2d.cu, and the epilogue arithmetic is the same, so both engines give
// bitwise the same result.
#include "fk_ar2d.cuh"

namespace fk {

template <int F>
struct PipeCfg {
  static constexpr int kBlk = kTile * F * 2;        // one [F/8][128][8] bf16 block
  static constexpr int kNcol = F <= 16 ? 8 : 6;     // input column slots
  static constexpr int kRing = 3 * kNcol * kBlk;
  static constexpr int kWRow = F * 3 * F * 2;       // one kernel row of the scatter operand
  static constexpr int kW = 3 * kWRow;
  static constexpr int kCW = F * 32 * 2;
  static constexpr int kGroups = 2;                 // epilogue groups (alternate outputs)
  static constexpr int kNB = 2 * kGroups;           // chained-conv staging buffers / accumulators
  static constexpr int kCA = kNB * kTile * F * 2;
  static constexpr int kBias = 64 * 4;              // main (F) + chained (<= 32) biases
  static constexpr int kNS = 256 / F;               // TMEM accumulator slots (F columns each)
  static constexpr uint32_t kChainCol = 256;        // chained accumulators: 256 + b * 32 (b < kNB)
  static constexpr int kBars = 1024;
  static constexpr int kMaxW = 16;                  // head partials [W][128] float2
  static constexpr int kSmemBase = kRing + kW + kCW + kCA + kBias + kBars;
  static int head_bytes(int w) { return w * kTile * 8; }
};

constexpr int kPipeThreads = 384;  // 12 warps: producer, issuer, waiter, chain issuer, 8 epilogue

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

// Barrier 1 of the CTA: rendezvous of the waiter warp and the issuer warp,
// one per input column, returning the OR of both warps' abort flags.
__device__ __forceinline__ bool step_rendezvous(bool abort) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "barrier.cta.red.or.pred q, 1, 64, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)abort)
      : "memory");
  return r != 0;
}

template <int F>
__global__ void __launch_bounds__(kPipeThreads, 1) op_pipe_kernel(const __grid_constant__ OpArgs a, int H, int W,
                                                                  int64_t n_items, int* err) {
  // With a work list, n_items is an upper bound and the list's count is read
  // on the device.
  using C = PipeCfg<F>;
  using T = __nv_bfloat16;
  constexpr int F2 = F / 2;
  constexpr int NC2 = F2 < 16 ? 16 : F2;
  constexpr int NB = C::kNB;
  constexpr int NS = C::kNS;
  constexpr int NR = C::kNcol;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* ring = smem;
  uint8_t* wsm = smem + C::kRing;
  uint8_t* cwsm = wsm + C::kW;
  uint8_t* casm = cwsm + C::kCW;
  float* bias_sm = reinterpret_cast<float*>(casm + C::kCA);
  uint64_t* bars = reinterpret_cast<uint64_t*>(casm + C::kCA + C::kBias);
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
  float2* head_sm = reinterpret_cast<float2*>(smem + C::kSmemBase);

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
      mbar_init(&acce[i], 128);
    }
    for (int i = 0; i < NB; ++i) {
      mbar_init(&caf[i], 128);
      mbar_init(&cf[i], 1);
    }
    mbar_init(head_ready, 128);
    mbar_init(head_free, 128);
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

  if (warp == 0) {
    if (lane == 0) {
      // ---------------------------------------------------------------- producer
      mbar_arrive_expect_tx(wbar, wbytes + (has_chain ? chain_bytes : 0));
      bulk_g2s(wsm, a.main.ws, wbytes, wbar);
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
    // ------------------------------------------------------------------ MMA issuer
    // The whole warp runs the loop and lane 0 issues. This thread performs no
    // memory load while MMAs stream (a load, mbarrier waits included, stalls
    // the tensor pipe for hundreds of cycles): the waiter warp observes every
    // barrier and releases each input column through barrier 1.
    const uint32_t idesc1 = umma_idesc_bf16(128, F);
    const uint32_t idesc2 = umma_idesc_bf16(128, 2 * F);
    const uint32_t idesc3 = umma_idesc_bf16(128, 3 * F);
    const uint64_t a0 = umma_sdesc(smem_u32(ring), 2048, 128);
    const uint64_t w0 = umma_sdesc(smem_u32(wsm), 3 * F * 16, 128);
    constexpr uint32_t kBlk16 = C::kBlk >> 4;           // one ring block
    constexpr uint32_t kRow16 = C::kWRow >> 4;          // one kernel row of the scatter operand
    constexpr uint32_t kKs16 = (2 * 2048) >> 4;         // one K=16 step of A
    constexpr uint32_t kKsW16 = (2 * 3 * F * 16) >> 4;  // one K=16 step of B
    uint32_t gx = 0;     // input columns consumed (ring position)
    uint32_t cs = 0;     // ring slot of column gx
    uint32_t gbase = 0;  // global index of output column 0 of the current item
    int64_t next_item = blockIdx.x < n_items ? item_at(blockIdx.x) : 0;
    for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x) {
      const int r = (int)(next_item % H);
      if (it + gridDim.x < n_items) next_item = item_at(it + gridDim.x);  // consumed one item later
      const int k0 = (nrows - 1) - r > 0 ? (nrows - 1) - r : 0;        // first in-lattice kernel row
      for (int x = 0; x < W; ++x, ++gx) {
        abort = step_rendezvous(false);
        if (abort) break;
        tc_fence_after();
        const int c_lo = x + o0 < 0 ? 0 : x + o0;
        const int c_hi = x + o0 + 2 < W - 1 ? x + o0 + 2 : W - 1;
        // outputs first reached by this column, [c_f, c_hi]: all of them at
        // x == 0, else output x + o0 + 2 if it exists
        const int c_f = x == 0 ? c_lo : (x + o0 + 2 < c_hi + 1 ? x + o0 + 2 : c_hi + 1);
        if (lane == 0) {
          // One MMA per (kernel row, K step) over outputs [ca, cb], split where
          // the TMEM slot ring wraps.
          auto mma = [&](int ca, int cb, uint32_t aoff, uint32_t boff, uint32_t acc) {
            while (ca <= cb) {
              const uint32_t s = (gbase + (uint32_t)ca) % NS;
              int n = cb - ca + 1;
              if (n > NS - (int)s) n = NS - (int)s;
              const uint32_t id = n == 3 ? idesc3 : (n == 2 ? idesc2 : idesc1);
              umma_bf16(tmem + s * F, a0 + aoff, w0 + boff + (uint32_t)((ca - x - o0) * F), id, acc);
              ca += n;
            }
          };
          bool first = true;
          for (int k = k0; k < nrows; ++k) {
#pragma unroll
            for (int ks = 0; ks < F / 16; ++ks) {
              const uint32_t aoff = (cs * 3 + (uint32_t)k) * kBlk16 + ks * kKs16;
              const uint32_t boff = (uint32_t)k * kRow16 + ks * kKsW16;
              if (first) {
                if (c_f > c_lo) mma(c_lo, c_f - 1, aoff, boff, 1u);
                mma(c_f, c_hi, aoff, boff, 0u);
                first = false;
              } else {
                mma(c_lo, c_hi, aoff, boff, 1u);
              }
            }
          }
          umma_commit(&empty[cs]);
          // outputs completed by this column
          const int d_lo = x + o0 < 0 ? 0 : x + o0;
          const int d_hi = x == W - 1 ? W - 1 : x + o0;
          for (int c = d_lo; c <= d_hi; ++c) umma_commit(&accf[(gbase + (uint32_t)c) % NS]);
        }
        __syncwarp();
        cs = cs + 1 == (uint32_t)NR ? 0 : cs + 1;
      }
      gbase += (uint32_t)W;
    }
    if (lane == 0) {
      umma_commit(&drain[0]);
      mbar_wait(&drain[0], 0, err);
    }
  } else if (warp == 2) {
    // ------------------------------------------------------------------ waiter
    // Observes the barriers each input column needs (column loaded, TMEM slots
    // of the outputs it starts released by the epilogue), then releases the
    // column to the issuer through barrier 1.
    pwait(wbar, 0, err, abort);
    uint32_t gx = 0, gbase = 0;
    bool stop = false;
    for (int64_t it = blockIdx.x; it < n_items && !stop; it += gridDim.x) {
      for (int x = 0; x < W; ++x, ++gx) {
        pwait(&full[gx % NR], (gx / NR) & 1, err, abort);
        const int c_hi = x + o0 + 2 < W - 1 ? x + o0 + 2 : W - 1;
        const int c_f = x == 0 ? (x + o0 < 0 ? 0 : x + o0) : (x + o0 + 2 < c_hi + 1 ? x + o0 + 2 : c_hi + 1);
        for (int c = c_f; c <= c_hi; ++c) {
          const uint32_t p = gbase + (uint32_t)c;
          if (p >= (uint32_t)NS) pwait(&acce[p % NS], ((p / NS) - 1) & 1, err, abort);
        }
        stop = step_rendezvous(abort);
        if (stop) break;
      }
      gbase += (uint32_t)W;
    }
    abort = stop;
  } else if (warp == 3) {
    // ------------------------------------------------------------------ chain issuer
    // The chained 1x1 MMA of each output, on the epilogue's staged bf16
    // activations, into one of NB chained accumulators.
    if (has_chain && lane == 0) {
      const uint32_t idesc_c = umma_idesc_bf16(128, cnp);
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
            umma_bf16(tmem + C::kChainCol + b * 32, ca0 + ((b * (kTile * F * 2) + ks * 2 * 2048) >> 4),
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
    const bool need_res = (kind == kConvV && a.stream_out && a.res) || (kind == kConvC && !a.last && a.res);
    // deferred second half: output index, tile, row, column
    bool pend = false;
    uint32_t pq = 0;
    int64_t ptile = 0;
    int pr = 0, pc = 0;
    auto second_half = [&]() {
      const uint32_t b = pq % NB;
      pend = false;
      if (!pwait(&cf[b], (pq / NB) & 1, err, abort)) return;
      tc_fence_after();
      float out[32];
      if (kind == kConvC)
        tread<16>(tl, C::kChainCol + b * 32, out);
      else
        tread<NC2>(tl, C::kChainCol + b * 32, out);
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
        // abstract_machine.py:56-57 normalisation (same arithmetic as the per-pixel engine)
        float a2 = 2.f * out[0], b2 = 2.f * out[1];
        float mx = fmaxf(a2, b2);
        float lse = 0.5f * (mx + logf(expf(a2 - mx) + expf(b2 - mx)));
        float re0 = out[0] - lse, re1 = out[1] - lse;
        const int64_t sample = ptile * kTile + m;
        bool up = spin_at(a.spins, a.batch, P, sample, pix) > 0.f;
        head_sm[pc * kTile + m] = make_float2(up ? re0 : re1, up ? out[2] : out[3]);
        if (a.cond && sample < a.batch)
          reinterpret_cast<float4*>(a.cond)[sample * P + pix] = make_float4(re0, re1, out[2], out[3]);
      }
    };
    uint32_t p = 0, it_count = 0;
    for (int64_t it = blockIdx.x; it < n_items && !abort; it += gridDim.x, ++it_count) {
      const int64_t item = item_at(it);
      const int64_t tile = item / H;
      const int r = (int)(item % H);
      if (head && grp == 1 && it_count > 0 && !pwait(head_free, (it_count - 1) & 1, err, abort)) break;
      for (int c = 0; c < W && !abort; ++c, ++p) {
        if ((int)(p % C::kGroups) != grp) continue;
        const uint32_t b = p % NB;
        const uint32_t sl = p % NS;
        const int pix = r * W + c;
        float o[F];
        if (need_res) load_row(blk<T>(a.res, tile, P, pix, F), m, 0, F, o);
        if (!pwait(&accf[sl], (p / NS) & 1, err, abort)) break;
        tc_fence_after();
        float acc[F];
        tread<F>(tl, sl * F, acc);
        tc_fence_before();
        mbar_arrive(&acce[sl]);
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
  if (head && W > PipeCfg<F>::kMaxW) return FK_ERR_ARG;
  if (!a.main.ws) return FK_ERR_ARG;
  // At least half of an SM's shared memory, so that one CTA (holding all 512
  // TMEM columns) runs per SM.
  int smem = PipeCfg<F>::kSmemBase + (head ? PipeCfg<F>::head_bytes(W) : 0);
  if (smem < kMinSmem) smem = kMinSmem;
  if (!attr) {
    const int most = PipeCfg<F>::kSmemBase + PipeCfg<F>::head_bytes(PipeCfg<F>::kMaxW);
    FK_CUDA(cudaFuncSetAttribute(op_pipe_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 most > kMinSmem ? most : kMinSmem));
    attr = true;
  }
  const int64_t items = tiles * H;
  int64_t grid = (int64_t)sms;  // one CTA per SM (512 TMEM columns)
  if (grid > items) grid = items;
  op_pipe_kernel<F><<<(unsigned)grid, kPipeThreads, smem, s>>>(a, H, W, items, err);
  return check_cuda(launched(), "op_pipe_kernel");
}

int launch_pipe_op(int F, const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s) {
  if (a.first) return FK_ERR_ARG;
  if (F == 16) return launch_pipe<16>(a, tiles, H, W, err, s);
  if (F == 32) return launch_pipe<32>(a, tiles, H, W, err, s);
  return FK_ERR_ARG;
}

bool pipe_supported(int F, int W) { return (F == 16 || F == 32) && W >= 2 && W <= PipeCfg<32>::kMaxW; }

static_assert(PipeCfg<32>::kSmemBase + 16 * kTile * 8 <= 227 * 1024, "pipelined engine exceeds shared memory");
static_assert(PipeCfg<16>::kSmemBase + 16 * kTile * 8 <= 227 * 1024, "pipelined engine exceeds shared memory");
static_assert(3 * 32 <= 256 && PipeCfg<16>::kNS * 16 <= 256, "TMEM layout");

}  // namespace fk
