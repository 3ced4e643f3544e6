// Complex-parameter machines (the RBM family): tied parameters and the loss
// gradient from per-sample log-derivatives.
//
// * Tied parameters. RBMSym (machines/rbm.py:51-65) trains a bare kernel of
//   shape lattice + (alpha,), one hidden bias per feature and one visible bias;
//   the network evaluates the dense RBM whose every parameter is a copy of
//   one bare parameter (layers/complex/dense.py:53-85: kernel column f*T + t
//   is the bare kernel rolled by translation t, the bias repeated per
//   translation). fk_gather_complex expands bare -> dense through the index map;
//   fk_segment_sum_rows reduces dense per-sample rows O to the bare
//   parameters (d/d bare = sum of d/d its copies), in a fixed order.
// * Loss gradient. For a holomorphic log psi and a complex parameter
//   theta = u + i v with O = d log psi / d theta:
//     d Re log psi / du = Re O,  d Re log psi / dv = -Im O,
//     d Im log psi / du = Im O,  d Im log psi / dv =  Re O,
//   so the gradient of sum_b (w_re Re log psi_b + w_im Im log psi_b) with
//   respect to the stored (u, v) pairs is
//     g_u = sum_b (w_re Re O + w_im Im O),  g_v = sum_b (w_im Re O - w_re Im O)
//   (fk_complex_param_gradient), the Keras gradient of
//   optimization/loss.py:4-5 through the complex layers' (re, im) weights.
#include "fk_common.cuh"

namespace fk {

__global__ void gather_complex_kernel(const float2* __restrict__ src, const int32_t* __restrict__ index, int64_t n,
                                      float2* __restrict__ dst) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) dst[i] = src[index[i]];
}

// out[k][c] = sum_{q in [off[k], off[k+1])} in[rows[q]][c], q ascending.
// Block: 256 threads over columns; grid.x over column tiles, grid.y over k.
__global__ void segment_sum_rows_kernel(const float* __restrict__ in, const int64_t* __restrict__ off,
                                        const int32_t* __restrict__ rows, int64_t cols, float* __restrict__ out) {
  const int64_t k = blockIdx.y;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int64_t q0 = off[k], q1 = off[k + 1];
  float acc = 0.f;
  for (int64_t q = q0; q < q1; ++q) acc += in[(int64_t)rows[q] * cols + c];
  out[k * cols + c] = acc;
}

// One block per complex parameter row: fixed-order partial sums over the
// samples (strided by thread, then a shared-memory tree), FP64 accumulation.
__global__ void __launch_bounds__(256) complex_grad_kernel(const float* __restrict__ o_re,
                                                           const float* __restrict__ o_im, int64_t P, int64_t B,
                                                           const float2* __restrict__ w, float2* __restrict__ grad) {
  __shared__ double su[256], sv[256];
  const int64_t k = blockIdx.x;
  if (k >= P) return;
  const float* ar = o_re + k * B;
  const float* ai = o_im + k * B;
  double gu = 0.0, gv = 0.0;
  for (int64_t b = threadIdx.x; b < B; b += blockDim.x) {
    float2 wb = w[b];
    double r = ar[b], i = ai[b];
    gu += (double)wb.x * r + (double)wb.y * i;
    gv += (double)wb.y * r - (double)wb.x * i;
  }
  su[threadIdx.x] = gu;
  sv[threadIdx.x] = gv;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      su[threadIdx.x] += su[threadIdx.x + o];
      sv[threadIdx.x] += sv[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) grad[k] = make_float2((float)su[0], (float)sv[0]);
}

}  // namespace fk

using namespace fk;

extern "C" {

int fk_gather_complex(const float* src, const int32_t* index, int64_t n, float* dst, void* stream) {
  FK_CHECK_ARG(src && index && dst && n >= 0, "fk_gather_complex: bad arguments");
  if (n == 0) return FK_OK;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  gather_complex_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<const float2*>(src), index, n, reinterpret_cast<float2*>(dst));
  FK_CUDA(launched());
  return FK_OK;
}

int fk_segment_sum_rows(const float* in, const int64_t* offsets, const int32_t* rows, int64_t n_out, int64_t cols,
                        float* out, void* stream) {
  FK_CHECK_ARG(in && offsets && rows && out && n_out >= 0 && cols >= 0, "fk_segment_sum_rows: bad arguments");
  FK_CHECK_ARG(n_out <= 65535, "fk_segment_sum_rows: at most 65535 output rows (got %lld)", (long long)n_out);
  if (n_out == 0 || cols == 0) return FK_OK;
  dim3 grid((unsigned)((cols + 255) / 256), (unsigned)n_out);
  segment_sum_rows_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(in, offsets, rows, cols, out);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_complex_param_gradient(const float* o_re, const float* o_im, int64_t n_params, int64_t batch, const float* w,
                              float* grad, void* stream) {
  FK_CHECK_ARG(o_re && o_im && w && grad && n_params >= 0 && batch > 0, "fk_complex_param_gradient: bad arguments");
  FK_CHECK_ARG(n_params <= 0x7fffffffLL, "fk_complex_param_gradient: too many parameters");
  if (n_params == 0) return FK_OK;
  complex_grad_kernel<<<(unsigned)n_params, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      o_re, o_im, n_params, batch, reinterpret_cast<const float2*>(w), reinterpret_cast<float2*>(grad));
  FK_CUDA(launched());
  return FK_OK;
}

}  // extern "C"
