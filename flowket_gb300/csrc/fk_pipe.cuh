// Column-scatter pipeline shared by the AR2D forward ops (fk_ar2d_pipe.cu)
// and the data-gradient ops of the adjoint (fk_ar2d_bwd_tc.cu).
//
// One persistent CTA per SM walks (tile, row) items; each item is one lattice
// row of 128 samples. Input column x of an item (nrows lattice rows, one
// [F/8][128][8] bf16 block each) is multiplied once per kernel row by the
// three kernel columns stacked along N (N = 3F): the product holds x's
// contributions to the three output columns x + o0 .. x + o0 + 2, which
// accumulate in three consecutive F-column slots of a TMEM ring. Output c is
// complete after input column min(c - o0, W - 1).
//
// Roles (warps of the CTA):
//   producer (one thread): bulk copies of the weights once, then of every
//       input column into a ring of column slots;
//   waiter (whole warp): observes the barriers each column needs (column
//       loaded, TMEM slots of the outputs it starts released by the
//       epilogue), then releases the column to the issuer through named
//       barrier 1, which also carries an abort flag;
//   issuer (whole warp, lane 0 issues): tcgen05.mma over the column and
//       commits. This thread performs no memory load while MMAs stream: a
//       load in the issuing thread -- an mbarrier wait included -- stalls the
//       tensor pipe for hundreds of cycles.
// The accumulation order of an output is: input columns ascending, kernel
// rows ascending in ring order, K steps ascending.
#pragma once

#include "fk_ar2d.cuh"

namespace FK_NS {

template <int F>
struct PipeCfg {
  static constexpr int kBlk = kTile * F * 2;        // one [F/8][128][8] bf16 block
  static constexpr int kNcol = F <= 16 ? 8 : 6;     // input column slots
  static constexpr int kRing = 3 * kNcol * kBlk;
  static constexpr int kWRow = F * 3 * F * 2;       // one kernel row of the scatter operand
  static constexpr int kW = 3 * kWRow;
  static constexpr int kGroups = 2;                 // epilogue groups (alternate outputs)
  static constexpr int kNB = 2 * kGroups;           // chained-conv staging buffers
  static constexpr int kCA = kNB * kTile * F * 2;
  static constexpr int kNS = 256 / F;               // TMEM accumulator slots (F columns each)
  static constexpr uint32_t kChainCol = 256;        // chained accumulators start here
  static constexpr int kBars = 1024;
};

constexpr int kPipeThreads = 384;  // 12 warps: producer, issuer, waiter, chain issuer, 8 epilogue

// Geometry of one op: ring row k of an item at lattice row r holds input row
// r + row0 + k (k < nrows); its kernel row is k, or nrows - 1 - k when rev.
struct PipeGeom {
  int H, W;
  int nrows, row0, o0;
  int rev;
};

__device__ __forceinline__ bool pwait(uint64_t* bar, uint32_t parity, int* err, bool& abort) {
  if (abort) return false;
  if (!mbar_wait(bar, parity, err)) {
    abort = true;
    return false;
  }
  return true;
}

// pwait for code that all 32 lanes run converged (barrier counts of one
// arrival per warp, named barriers): a timeout on any lane aborts the whole
// warp, so the lanes never part at a later warp-wide step.
__device__ __forceinline__ bool uwait(uint64_t* bar, uint32_t parity, int* err, bool& abort) {
  pwait(bar, parity, err, abort);
  abort = __any_sync(0xffffffffu, abort);
  return !abort;
}

// Warp-wide arrival (one arrival per warp): the warp synchronisation orders
// every lane's earlier accesses before lane 0's release.
__device__ __forceinline__ void warp_arrive(uint64_t* bar) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) mbar_arrive(bar);
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

struct PipeItems {
  const int32_t* items;  // work list (NULL: item k = k)
  int64_t n;
  __device__ __forceinline__ int64_t at(int64_t k) const { return items ? (int64_t)items[k] : k; }
};

// In-lattice ring rows [k_lo, k_hi] of an item at row r.
__device__ __forceinline__ void ring_rows(const PipeGeom& g, int r, int& k_lo, int& k_hi) {
  k_lo = -(r + g.row0) > 0 ? -(r + g.row0) : 0;
  k_hi = g.H - 1 - r - g.row0 < g.nrows - 1 ? g.H - 1 - r - g.row0 : g.nrows - 1;
}

// A weight region copied once into shared memory.
struct WeightCopy {
  uint8_t* dst;
  const void* src;
  uint32_t bytes;  // 0: none
};

// Producer (one thread): up to three weight regions once, then every input
// column of every item into the ring.
template <int F>
__device__ void pipe_producer(const PipeGeom& g, const PipeItems& items, const void* in, uint8_t* ring,
                              uint64_t* full, uint64_t* empty, uint64_t* wbar, WeightCopy w1, WeightCopy w2,
                              WeightCopy w3, int* err, bool& abort) {
  using C = PipeCfg<F>;
  constexpr int NR = C::kNcol;
  mbar_arrive_expect_tx(wbar, w1.bytes + w2.bytes + w3.bytes);
  if (w1.bytes) bulk_g2s(w1.dst, w1.src, w1.bytes, wbar);
  if (w2.bytes) bulk_g2s(w2.dst, w2.src, w2.bytes, wbar);
  if (w3.bytes) bulk_g2s(w3.dst, w3.src, w3.bytes, wbar);
  const int P = g.H * g.W;
  uint32_t gc = 0;
  for (int64_t it = blockIdx.x; it < items.n && !abort; it += gridDim.x) {
    const int64_t item = items.at(it);
    const int64_t tile = item / g.H;
    const int r = (int)(item % g.H);
    int k_lo, k_hi;
    ring_rows(g, r, k_lo, k_hi);
    for (int x = 0; x < g.W && !abort; ++x, ++gc) {
      const uint32_t slot = gc % NR;
      if (gc >= NR && !pwait(&empty[slot], ((gc / NR) - 1) & 1, err, abort)) break;
      mbar_arrive_expect_tx(&full[slot], (uint32_t)(k_hi - k_lo + 1) * C::kBlk);
      for (int k = k_lo; k <= k_hi; ++k)
        bulk_g2s(ring + (slot * 3 + k) * C::kBlk,
                 blk<tc16>(in, tile, P, (r + g.row0 + k) * g.W + x, F), C::kBlk, &full[slot]);
    }
  }
}

// Input columns released to the issuer per rendezvous: the issuer issues
// their MMAs back to back (same MMAs, same order, so results are unchanged),
// and the rendezvous cost is shared. The ring (>= 6 slots) and the TMEM
// accumulator slots (>= 8) hold the columns and outputs of a step.
constexpr int kColsPerStep = 2;

// Waiter (whole warp).
template <int F, int NS = PipeCfg<F>::kNS>
__device__ void pipe_waiter(const PipeGeom& g, const PipeItems& items, uint64_t* full, uint64_t* wbar,
                            uint64_t* acce, int* err, bool& abort) {
  using C = PipeCfg<F>;
  constexpr int NR = C::kNcol;
  static_assert(NR >= 2 * kColsPerStep && NS >= 3 + kColsPerStep + 1, "ring or TMEM slots too few for a step");
  pwait(wbar, 0, err, abort);
  uint32_t gx = 0, gbase = 0;
  bool stop = false;
  for (int64_t it = blockIdx.x; it < items.n && !stop; it += gridDim.x) {
    for (int x0 = 0; x0 < g.W; x0 += kColsPerStep) {
      const int x1 = x0 + kColsPerStep < g.W ? x0 + kColsPerStep : g.W;
      for (int x = x0; x < x1; ++x, ++gx) {
        pwait(&full[gx % NR], (gx / NR) & 1, err, abort);
        const int c_lo = x + g.o0 < 0 ? 0 : x + g.o0;
        const int c_hi = x + g.o0 + 2 < g.W - 1 ? x + g.o0 + 2 : g.W - 1;
        const int c_f = x == 0 ? c_lo : (x + g.o0 + 2 < c_hi + 1 ? x + g.o0 + 2 : c_hi + 1);
        for (int c = c_f; c <= c_hi; ++c) {
          const uint32_t p = gbase + (uint32_t)c;
          if (p >= (uint32_t)NS) pwait(&acce[p % NS], ((p / NS) - 1) & 1, err, abort);
        }
      }
      stop = step_rendezvous(abort);
      if (stop) break;
    }
    gbase += (uint32_t)g.W;
  }
  abort = stop || abort;
}

// Lane 0's MMAs of a column without TMEM ring wrap, ring rows KLO..KHI:
// operands computed by the whole warp before the branch that selects lane 0,
// compile-time offsets inside, so that the issuing thread only issues.
template <int F, int KLO, int KHI>
__device__ __forceinline__ void issue_plain(uint64_t a_col, uint64_t b_live, uint64_t b_fresh, uint32_t d_live,
                                            uint32_t d_fresh, uint32_t id_tot, uint32_t id_live, uint32_t id_fresh,
                                            int n_live, int n_tot, int rev) {
  constexpr uint32_t kBlk16 = PipeCfg<F>::kBlk >> 4;
  constexpr uint32_t kRow16 = PipeCfg<F>::kWRow >> 4;
  constexpr uint32_t kKs16 = (2 * 2048) >> 4;
  constexpr uint32_t kKsW16 = (2 * 3 * F * 16) >> 4;
#pragma unroll
  for (int k = KLO; k <= KHI; ++k) {
#pragma unroll
    for (int ks = 0; ks < F / 16; ++ks) {
      const uint32_t aoff = (uint32_t)k * kBlk16 + ks * kKs16;
      const uint32_t boff = (rev ? (uint32_t)(KHI - k + KLO) : (uint32_t)k) * kRow16 + ks * kKsW16;
      if (k == KLO && ks == 0) {
        if (n_live > 0) umma_bf16(d_live, a_col + aoff, b_live + boff, id_live, 1u);
        if (n_tot > n_live) umma_bf16(d_fresh, a_col + aoff, b_fresh + boff, id_fresh, 0u);
      } else {
        umma_bf16(d_live, a_col + aoff, b_live + boff, id_tot, 1u);
      }
    }
  }
}

// Reversed (adjoint) op near the bottom edge: ring rows 0..KHI, kernel row
// 2 - k.
template <int F, int KHI>
__device__ __forceinline__ void issue_rev_partial(uint64_t a_col, uint64_t b_live, uint64_t b_fresh, uint32_t d_live,
                                                  uint32_t d_fresh, uint32_t id_tot, uint32_t id_live,
                                                  uint32_t id_fresh, int n_live, int n_tot) {
  constexpr uint32_t kBlk16 = PipeCfg<F>::kBlk >> 4;
  constexpr uint32_t kRow16 = PipeCfg<F>::kWRow >> 4;
  constexpr uint32_t kKs16 = (2 * 2048) >> 4;
  constexpr uint32_t kKsW16 = (2 * 3 * F * 16) >> 4;
#pragma unroll
  for (int k = 0; k <= KHI; ++k) {
#pragma unroll
    for (int ks = 0; ks < F / 16; ++ks) {
      const uint32_t aoff = (uint32_t)k * kBlk16 + ks * kKs16;
      const uint32_t boff = (uint32_t)(2 - k) * kRow16 + ks * kKsW16;
      if (k == 0 && ks == 0) {
        if (n_live > 0) umma_bf16(d_live, a_col + aoff, b_live + boff, id_live, 1u);
        if (n_tot > n_live) umma_bf16(d_fresh, a_col + aoff, b_fresh + boff, id_fresh, 0u);
      } else {
        umma_bf16(d_live, a_col + aoff, b_live + boff, id_tot, 1u);
      }
    }
  }
}

// Issuer (whole warp; lane 0 issues). `w0` is the descriptor of kernel row 0
// of the scatter operand ([F/8][3F][8] per kernel row).
template <int F, int NS = PipeCfg<F>::kNS>
__device__ void pipe_issuer(const PipeGeom& g, const PipeItems& items, uint8_t* ring, uint8_t* wsm,
                            uint32_t tmem, uint64_t* empty, uint64_t* accf, uint64_t* drain, int* err,
                            bool& abort) {
  using C = PipeCfg<F>;
  constexpr int NR = C::kNcol;
  const int lane = threadIdx.x % 32;
  const uint32_t idesc1 = umma_idesc_tc16(128, F);
  const uint32_t idesc2 = umma_idesc_tc16(128, 2 * F);
  const uint32_t idesc3 = umma_idesc_tc16(128, 3 * F);
  const uint64_t a0 = umma_sdesc(smem_u32(ring), 2048, 128);
  const uint64_t w0 = umma_sdesc(smem_u32(wsm), 3 * F * 16, 128);
  constexpr uint32_t kBlk16 = C::kBlk >> 4;  // one ring block
  const int W = g.W, o0 = g.o0;
  uint32_t cs = 0;     // ring slot of the current column
  uint32_t gbase = 0;  // global index of output column 0 of the current item
  int64_t next_item = blockIdx.x < items.n ? items.at(blockIdx.x) : 0;
  for (int64_t it = blockIdx.x; it < items.n && !abort; it += gridDim.x) {
    const int r = (int)(next_item % g.H);
    if (it + gridDim.x < items.n) next_item = items.at(it + gridDim.x);  // used one item later
    int k_lo, k_hi;
    ring_rows(g, r, k_lo, k_hi);
    for (int x = 0; x < W; ++x) {
      if (x % kColsPerStep == 0) {
        abort = step_rendezvous(false);
        if (abort) break;
        tc_fence_after();
      }
      const int c_lo = x + o0 < 0 ? 0 : x + o0;
      const int c_hi = x + o0 + 2 < W - 1 ? x + o0 + 2 : W - 1;
      // outputs first reached by this column, [c_f, c_hi]: all of them at
      // x == 0, else output x + o0 + 2 if it exists
      const int c_f = x == 0 ? c_lo : (x + o0 + 2 < c_hi + 1 ? x + o0 + 2 : c_hi + 1);
      // The column's outputs [c_lo, c_hi] in one part, or in two where the
      // TMEM slot ring wraps ([c_lo, c_s) at slot s_lo.., [c_s, c_hi] at
      // slot 0..); each part is issued as straight-line MMAs on operands
      // computed here by the whole warp, so that the issuing thread only
      // issues. An output lies in one part, so its accumulation order is
      // unchanged by the split.
      const uint32_t s_lo = (gbase + (uint32_t)c_lo) % NS;
      const int c_s = c_lo + (NS - (int)s_lo) < c_hi + 1 ? c_lo + (NS - (int)s_lo) : c_hi + 1;
      const uint64_t a_col = a0 + cs * 3 * kBlk16;
      auto part = [&](int pa, int pb, uint32_t slot) {  // outputs [pa, pb], pa at TMEM slot `slot`
        const int n_tot = pb - pa + 1;
        const int f0 = c_f > pa ? c_f : pa;                       // first fresh output of the part
        const int n_live = (f0 < pb + 1 ? f0 : pb + 1) - pa;
        const uint32_t d_live = tmem + slot * F;
        const uint32_t d_fresh = d_live + (uint32_t)(n_live * F);
        const uint32_t id_tot = n_tot == 3 ? idesc3 : (n_tot == 2 ? idesc2 : idesc1);
        const uint32_t id_live = n_live == 2 ? idesc2 : idesc1;
        const uint32_t id_fresh = n_tot - n_live == 3 ? idesc3 : (n_tot - n_live == 2 ? idesc2 : idesc1);
        const uint64_t b_live = w0 + (uint32_t)((pa - x - o0) * F);
        const uint64_t b_fresh = w0 + (uint32_t)((f0 - x - o0) * F);
        if (lane == 0) {
          // in-lattice ring rows: all (k_lo, k_hi) = (0, 2); forward ops near
          // the top edge (1, 2), (2, 2); reversed ops near the bottom edge
          // (0, 1), (0, 0); 1-row ops (0, 0)
          if (g.nrows == 1)
            issue_plain<F, 0, 0>(a_col, b_live, b_fresh, d_live, d_fresh, id_tot, id_live, id_fresh, n_live, n_tot, 0);
          else if (k_lo == 0 && k_hi == 2)
            issue_plain<F, 0, 2>(a_col, b_live, b_fresh, d_live, d_fresh, id_tot, id_live, id_fresh, n_live, n_tot,
                                 g.rev);
          else if (!g.rev && k_lo == 1)
            issue_plain<F, 1, 2>(a_col, b_live, b_fresh, d_live, d_fresh, id_tot, id_live, id_fresh, n_live, n_tot, 0);
          else if (!g.rev)
            issue_plain<F, 2, 2>(a_col, b_live, b_fresh, d_live, d_fresh, id_tot, id_live, id_fresh, n_live, n_tot, 0);
          else if (k_hi == 1)
            issue_rev_partial<F, 1>(a_col, b_live, b_fresh, d_live, d_fresh, id_tot, id_live, id_fresh, n_live, n_tot);
          else
            issue_rev_partial<F, 0>(a_col, b_live, b_fresh, d_live, d_fresh, id_tot, id_live, id_fresh, n_live, n_tot);
        }
      };
      part(c_lo, c_s - 1, s_lo);
      if (c_s <= c_hi) part(c_s, c_hi, 0u);
      if (lane == 0) {
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
    umma_commit(drain);
    mbar_wait(drain, 0, err);
  }
}

}  // namespace FK_NS
