// ConvNetAutoregressive2D on GB300: shared declarations of the forward,
// sampling and adjoint kernels.
//
// Activation layout ("sample-major blocked"): a tensor with C channels is
// stored per tile of 128 samples and per lattice pixel as a block
// [C/8][128][8] of elements, blocks ordered (tile, pixel). One block is
// exactly the no-swizzle K-major operand layout of a tcgen05 MMA with
// M = 128 samples and K = C channels (rows 16 B apart, K-groups 2 KB apart),
// so a convolution tap is one contiguous bulk copy and the implicit GEMM needs
// no im2col: a 3x3 causal conv at pixel (r, c) is the sum over the in-bounds
// taps of [128 x C] x [C x F] products. Out-of-lattice taps are skipped (the
// reference's ZeroPadding2D).
#pragma once

#include <cuda_fp16.h>

#include "fk_common.cuh"

// The 16-bit operand format of the tensor-core path. Every translation unit of
// the AR2D machine is compiled twice: as is (BF16 operands, namespace fk,
// entry points fk_ar2d_*) and with FK_TC_FP16 defined (FP16 operands,
// namespace fk16, entry points fk_ar2d_*_tc_fp16, which the BF16 build's
// entry points call for FK_PRECISION_FP16). Both formats feed the same
// kind::f16 MMAs with FP32 accumulation at the same rate; FP16 keeps 10
// mantissa bits of every stored activation instead of 7.
#ifdef FK_TC_FP16
#define FK_NS fk16
#define FK_AR2D_ENTRY(name) name##_tc_fp16
#else
#define FK_NS fk
#define FK_AR2D_ENTRY(name) name
#endif

namespace FK_NS {

using namespace ::fk;

#ifdef FK_TC_FP16
using tc16 = __half;
constexpr uint32_t kTcFormatBits = 0u;           // A and B: F16
constexpr uint32_t kTcOnePair = 0x3C003C00u;     // two fp16 1.0
__device__ __forceinline__ uint32_t pack_tc16x2(float a, float b) {
  __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ void unpack_tc16x8(uint4 u, float* f) {
  const __half2* h = reinterpret_cast<const __half2*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 t = __half22float2(h[i]);
    f[2 * i] = t.x;
    f[2 * i + 1] = t.y;
  }
}
__device__ __forceinline__ tc16 to_tc16(float x) { return __float2half_rn(x); }
#else
using tc16 = __nv_bfloat16;
constexpr uint32_t kTcFormatBits = (1u << 7) | (1u << 10);  // A and B: BF16
constexpr uint32_t kTcOnePair = 0x3F803F80u;                // two bf16 1.0
__device__ __forceinline__ uint32_t pack_tc16x2(float a, float b) { return pack_bf16x2(a, b); }
__device__ __forceinline__ void unpack_tc16x8(uint4 u, float* f) { unpack_bf16x8(u, f); }
__device__ __forceinline__ tc16 to_tc16(float x) { return __float2bfloat16_rn(x); }
#endif

// Instruction descriptor of tcgen05.mma kind::f16 for this build's operand
// format: D fp32, both operands K-major, shape M x N (x K=16).
__host__ __device__ constexpr uint32_t umma_idesc_tc16(int m, int n) {
  return (1u << 4) | kTcFormatBits | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
// Same with both operands MN-major.
__host__ __device__ constexpr uint32_t umma_idesc_tc16_mn(int m, int n) {
  return umma_idesc_tc16(m, n) | (1u << 15) | (1u << 16);
}

constexpr int kTile = 128;  // samples per tile = MMA M

enum ConvKind { kConvV = 0, kConvH = 1, kConvX = 2, kConvY = 3, kConvC = 4 };

// One conv of the network (kernel, bias, optional weight-norm gain).
struct ConvDesc {
  int64_t p_kernel, p_bias, p_g;  // float offsets into the flat parameter vector (p_g < 0: none)
  int64_t w_off, b_off;           // byte offsets into the packed buffer (weights, fp32 bias)
  int64_t w32_off;                // byte offset of the fp32 [K][cout] effective kernel (== w_off on fp32)
  int64_t ws_off;                 // byte offset of the column-scatter operand (-1: none), see below
  int64_t wt_off;                 // byte offset of the transposed operand of the adjoint (-1: none)
  int kh, kw, cin, cout;
  int K, Kpad, Npad;              // GEMM K (taps*cin), padded K / N for the bf16 operand
};

constexpr int kMaxConvs = 5 * 38 + 1;

struct NetLayout {
  int H, W, P, depth, F, wn, precision, n_cc;
  int updown;  // EqualUpDownSpins mask
  int n_convs;
  int64_t num_params;
  int64_t packed_bytes;
  ConvDesc conv[kMaxConvs];
};

int build_layout(const fk_ar2d_desc* d, NetLayout* L);

inline int conv_index(int cc, int kind) { return cc * 5 + kind; }

// Packed weights as seen by one op.
//
// Column-scatter operand (bf16, convs with 3 kernel columns reading F <= 32
// channels): per kernel row i a no-swizzle K-major block [cin/8][3*cout][8]
// whose row n = s*cout + co holds W[i][2 - s][:, co]. One MMA of an input
// column against kernel row i then yields the contributions to the three
// output columns it feeds, output x + o + s in TMEM slot order (o = -1 for the
// V op, 0 for the H and C ops).
//
// Transposed operand (bf16, adjoint on tensor cores): for the 3-column convs
// per kernel row i a block [cout/8][3*cin][8] whose row n = j*cin + ci holds
// W[i][j][ci][:] (K = output channel), so that one MMA of an output-gradient
// column against kernel row i yields its contributions to three input-gradient
// columns; for the 1x1 convs one block [cout/8][cin][8] holding W^T.
struct ConvW {
  const void* w;    // fp32 [K][N] or bf16 [Kpad/8][Npad][8]
  const void* ws;   // column-scatter operand or NULL
  const void* wt;   // transposed operand of the adjoint or NULL
  const float* b;   // bias [N]
  int K, Npad;
};

struct OpArgs {
  int kind;          // kConvV, kConvH or kConvC
  int first;         // input is the spin lattice (cin = 1)
  int last;          // op of the final causal conv (H: right shift; C: output head)
  int cin;
  const int8_t* spins;  // [batch][P] +-1 (first-layer ops, head spin lookup)
  const void* in;       // input tensor, blocked, cin channels
  ConvW main, chain;    // main conv; chained 1x1 (y for V, x for H, head for the last C)
  const void* res;      // residual for the stream output (NULL: none)
  void* stream_out;     // V/H stream output (last C: relu(Hp) when saving)
  void* aux_out;        // V: relu(Vp) when saving; H: relu(conv_h) when saving
  void* cat;            // concat tensor (F channels): H writes [0,F/2), V writes [F/2,F)
  float2* row_partial;  // last C: [tiles][H][128] log psi partial per row
  float* cond;          // last C: [batch][P][4] normalised conditionals (optional)
  const uint8_t* updown;  // last C: [batch][P] EqualUpDownSpins mask bits (1: outcome +1, 2: -1) or NULL
  int64_t batch;
  // Optional work list: item k = tile * H + row for k < *n_items (row-suffix
  // evaluation of connected configurations); NULL = every (tile, row).
  const int32_t* items;
  const int32_t* n_items;
};

// Workspace tensors of one forward.
struct Tensors {
  // FK_AR2D_INFER: v[0..1], h[0..1], cat[0]; FK_AR2D_SAVE: one set per causal conv.
  void* v[40];
  void* h[40];
  void* cat[40];
  void* t[40];
  void* rv[40];
  float2* row_partial;
  uint8_t* updown;  // [batch][P] mask bits (EqualUpDownSpins) or NULL
  int64_t bytes;
};

// ---------------------------------------------------------------- device helpers
template <typename T>
__device__ __forceinline__ T* blk(const void* base, int64_t tile, int P, int pix, int C) {
  return reinterpret_cast<T*>(const_cast<void*>(base)) + ((tile * P + pix) * (int64_t)C) * kTile;
}

__device__ __forceinline__ void ld8(const float* p, float* v) {
  float4 a = reinterpret_cast<const float4*>(p)[0];
  float4 b = reinterpret_cast<const float4*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void ld8(const tc16* p, float* v) {
  unpack_tc16x8(*reinterpret_cast<const uint4*>(p), v);
}
__device__ __forceinline__ void st8(float* p, const float* v) {
  reinterpret_cast<float4*>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
  reinterpret_cast<float4*>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
}
__device__ __forceinline__ void st8(tc16* p, const float* v) {
  uint4 u;
  u.x = pack_tc16x2(v[0], v[1]);
  u.y = pack_tc16x2(v[2], v[3]);
  u.z = pack_tc16x2(v[4], v[5]);
  u.w = pack_tc16x2(v[6], v[7]);
  *reinterpret_cast<uint4*>(p) = u;
}

// Store `n` channels (multiple of 8) of thread row m into a block at channel offset c0.
template <typename T>
__device__ __forceinline__ void store_row(T* block, int m, int c0, int n, const float* v) {
  for (int g = 0; g < n / 8; ++g) st8(block + ((int64_t)((c0 / 8) + g) * kTile + m) * 8, v + 8 * g);
}
template <typename T>
__device__ __forceinline__ void load_row(const T* block, int m, int c0, int n, float* v) {
  for (int g = 0; g < n / 8; ++g) ld8(block + ((int64_t)((c0 / 8) + g) * kTile + m) * 8, v + 8 * g);
}

// Raw 16-byte chunks of thread row m's n channels (bf16), unpacked later.
template <int N>
__device__ __forceinline__ void load_raw(const tc16* block, int m, uint4* r) {
#pragma unroll
  for (int g = 0; g < N / 8; ++g) r[g] = *reinterpret_cast<const uint4*>(block + ((int64_t)g * kTile + m) * 8);
}
template <int N>
__device__ __forceinline__ void unpack_raw(const uint4* r, float* v) {
#pragma unroll
  for (int g = 0; g < N / 8; ++g) unpack_tc16x8(r[g], v + 8 * g);
}

// Tap offsets of the three ops (kernel element t = i*kw + j).
__device__ __forceinline__ void tap_offset(int kind, int t, int& dr, int& dc) {
  if (kind == kConvV) {
    dr = t / 3 - 2;
    dc = t % 3 - 1;
  } else if (kind == kConvH) {
    dr = 0;
    dc = t - 2;
  } else {
    dr = t / 3 - 2;
    dc = t % 3 - 2;
  }
}
__device__ __forceinline__ int num_taps(int kind) { return kind == kConvH ? 3 : 9; }
// q-th tap in column-major order (kernel column j outer, kernel row i inner).
__device__ __forceinline__ int tap_colmajor(int kind, int q) { return kind == kConvH ? q : (q % 3) * 3 + q / 3; }

__device__ __forceinline__ float spin_at(const int8_t* spins, int64_t batch, int P, int64_t sample, int pix) {
  return sample < batch ? (float)spins[sample * P + pix] : 1.f;
}

int64_t tensor_bytes(const NetLayout& L, int64_t tiles, int channels);
// Pipelined persistent tensor-core engine (fk_ar2d_pipe.cu) for the ops after
// the first layer with F <= 32; FK_ERR_ARG when the op is not supported.
int launch_pipe_op(int F, const OpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s);
bool pipe_supported(int F, int W);
int64_t workspace_layout(const NetLayout& L, int64_t batch, int mode, char* base, Tensors* T);

// ---------------------------------------------------------------- adjoint on tensor cores (F = 32)
enum BwdKind { kBwdC = 0, kBwdV = 1, kBwdH = 2 };

struct BwdOpArgs {
  int kind;
  const void* in;        // input gradient: gHp (C^T), gVp (V^T), gT (H^T)
  const void* wt;        // transposed scatter operand of the conv
  const void* wx;        // C^T: transposed operand of the x conv ([F/16][F][8])
  const void* wy;        // C^T: transposed operand of the y conv
  const void* cat;       // C^T: saved Cat (mask)
  const void* t;         // C^T: saved T (mask of gT)
  const void* rv;        // C^T: saved relu(Vp) (mask of gVp)
  const void* gvs;       // C^T: stream gradient of V added into gVp (NULL on the final conv)
  int shift;             // C^T: 1 on the final conv
  void* gcatm;           // C^T out
  void* gt;              // C^T out
  void* gvp;             // C^T out
  const void* res;       // V^T / H^T: residual gradient (NULL: none)
  const void* prev;      // V^T / H^T: saved V_{i-1} / H_{i-1} (mask)
  void* out;             // V^T / H^T out
};

struct WgTcArgs {
  const void* X;      // activations (bf16 blocked, F channels)
  int x_rows;         // ring rows of X: 3 (rows r-2..r) or 1
  int x_row0;         // X row of ring row 0 relative to the item row
  const void* G;      // output gradient (bf16 blocked, F channels)
  int g0;             // first gradient channel used (multiple of 8)
  int n;              // output channels of the conv (16 or 32)
  int ntc;            // kernel columns: 3 or 1
  int dc0;            // column offset of kernel column 0
  float* part;        // [gridDim.x][x_rows * 32][ntc * n] per-CTA partial dW
  int bias_jpos;      // column block whose ones-row sum is the bias gradient (-1: none)
  float* part_bias;   // [gridDim.x][n] per-CTA partial bias gradient
};

int launch_bwd_op(const BwdOpArgs& a, int64_t tiles, int H, int W, int* err, cudaStream_t s);
int64_t wgrad_tc_grid(int64_t tiles, int H);        // CTAs (and partials) of a weight-gradient launch
int64_t wgrad_tc_part_floats(int64_t tiles, int H);  // partial dW (3*32*96 per CTA) then partial bias (32 per CTA)
// dW: raw kernel gradient of the conv ([kh*kw*32][n]); kcol0: first kernel
// column the launch covers (1x1 convs: 0).
// db: bias gradient when a.bias_jpos >= 0.
int launch_wgrad_tc(const WgTcArgs& a, int kw, int kcol0, float* dW, float* db, int64_t tiles, int H, int W,
                    int* err, cudaStream_t s);
// part: >= tiles * H * n floats of scratch
int launch_bias_sum(const void* G, int64_t tiles, int H, int W, int g0, int n, int64_t batch, float* part, float* db,
                    cudaStream_t s);

// Per-sample weight and bias gradients of one conv on the tensor cores
// (wgrad_rows_tc_kernel): for every sample b,
// dW_b[tap][ci][n] = sum_pix X_b[pix + tap][ci] G_b[pix][g0 + n] and
// db_b[n] = sum_pix G_b[pix][g0 + n], written to
// O[(o_kernel + (tap * cin + ci) * N + n) * o_ld + o_col + b] and
// O[(o_bias + n) * o_ld + o_col + b]. cin = 32 with 16-bit gradients (N = 16
// or 32), or cin = 64 with float gradients rounded to the operand format
// (N = 32 or 64).
struct WgRowsArgs {
  const void* X;   // activations (16-bit blocked, cin channels)
  const void* G;   // gradients (blocked, gC channels; float when g_float)
  int cin, g_float;
  int gC, g0, N;
  int ntaps;
  int dr[9], dc[9];
  float* O;
  int64_t o_kernel, o_bias, o_ld, o_col;
  int64_t batch;
};
// False when the lattice is too large for the kernel's shared memory.
bool wgrad_rows_tc_supported(int H, int W, int N);
int launch_wgrad_rows_tc(const WgRowsArgs& a, int H, int W, int* err, cudaStream_t s);

}  // namespace FK_NS

#ifndef FK_TC_FP16
// The FP16-operand build of the entry points (FK_PRECISION_FP16), called by
// the entry points of this build; not part of the public header.
extern "C" {
int fk_ar2d_pack_tc_fp16(const fk_ar2d_desc* desc, const float* params, void* packed, void* stream);
int fk_ar2d_forward_tc_fp16(const fk_ar2d_desc* desc, const void* packed, const int8_t* spins, int64_t batch,
                            float* log_psi, float* cond, void* workspace, int64_t workspace_bytes, int32_t mode,
                            void* stream);
int fk_ar2d_sample_tc_fp16(const fk_ar2d_desc* desc, const void* packed, int64_t batch, uint64_t seed,
                           uint64_t offset, int8_t* spins, float* log_psi, void* workspace, int64_t workspace_bytes,
                           void* stream);
int fk_ar2d_forward_connections_tc_fp16(const fk_ar2d_desc* desc, const void* packed, const int8_t* configs,
                                        const int32_t* owner, const int16_t* cflips, int64_t n_rows,
                                        const void* base_saved, int64_t base_saved_bytes, int64_t base_batch,
                                        float* log_psi, void* workspace, int64_t workspace_bytes, int64_t chunk,
                                        void* stream);
int fk_ar2d_backward_tc_fp16(const fk_ar2d_desc* desc, const void* packed, const float* params, const int8_t* spins,
                             int64_t batch, const float* w, const void* saved, int64_t saved_bytes, void* workspace,
                             int64_t workspace_bytes, float* grad, float* per_sample, void* stream);
int fk_ar2d_sr_gram_tc_fp16(const fk_ar2d_desc* desc, const void* packed, const float* params, const int8_t* spins,
                            int64_t batch, const void* saved, int64_t saved_bytes, void* workspace,
                            int64_t workspace_bytes, float* rows, int64_t rows_floats, double* gram,
                            int32_t tensor_cores, void* stream);
}
#define FK_DISPATCH_FP16(desc, call) \
  do {                                \
    if ((desc) && (desc)->precision == FK_PRECISION_FP16) return call; \
  } while (0)
#else
#define FK_DISPATCH_FP16(desc, call) \
  do {                                \
  } while (0)
#endif

