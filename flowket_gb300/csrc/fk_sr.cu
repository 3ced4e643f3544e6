// Kernel set (d): stochastic reconfiguration in sample space.
//
// The reference solves (S + lambda I) x = F in parameter space with
// S = O_c^H O_c / B and F = O_c^H (E - Ebar) / B
// (optimizers/stochastic_reconfiguration/optimizer.py:55-124). With the P x 2B
// matrix Y = [Re O_c | Im O_c] (parameter-major rows of the per-sample
// log-derivatives) the push-through identity
//     (X^T X + lambda I)^-1 X^T e = X^T (X X^T + lambda I)^-1 e
// moves the solve to the 2B x 2B Gram T = Y^T Y / B:
//   1. centre every row of O over the samples (fk_center_columns);
//   2. T = Y^T Y: FP32 products accumulated in FP32 over chunks of K, chunk
//      sums reduced in FP64 (fk_sr_gram), upper-triangle tiles only;
//   3. (T/B + lambda I) alpha = eps solved by FP64 conjugate gradients with the
//      reference's stopping rule ||r|| <= tol ||eps|| (linear_equations.py:34-137)
//      (fk_sr_solve);
//   4. x = Y alpha / B and theta <- theta - lr x (fk_sr_backmap).
// For real parameters (the AR network) eps = [Re(E - Ebar); Im(E - Ebar)] and
// the update solves the real SR system S = Re<O_c^* O_c>, F = Re<O_c^* E_c>.
#include <mutex>

#include "fk_common.cuh"

namespace fk {

// ---------------------------------------------------------------- centring
__global__ void center_kernel(float* __restrict__ y, int64_t rows, int64_t cols, float* __restrict__ mean) {
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= rows) return;
  float* r = y + row * cols;
  double s = 0.0;
  for (int64_t j = lane; j < cols; j += 32) s += r[j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  float mu = (float)(s / (double)cols);
  for (int64_t j = lane; j < cols; j += 32) r[j] -= mu;
  if (mean && lane == 0) mean[row] = mu;
}

// ---------------------------------------------------------------- Gram
// T[i][j] = sum_p Y[p][i] Y[p][j], Y columns: [0,B) from A (row stride B),
// [B,2B) from Bm. 64x64 output tile per CTA (256 threads, 4x4 each), K split
// over blockIdx.z; per CTA the K range is walked in chunks whose FP32 partial
// sums are added into FP64 registers, then atomically into T (FP64).
constexpr int kGT = 64;
constexpr int kGK = 16;
constexpr int kChunk = 2048;

__device__ __forceinline__ float ycol(const float* __restrict__ a, const float* __restrict__ b, int64_t bsz,
                                      int64_t p, int64_t j) {
  return j < bsz ? a[p * bsz + j] : b[p * bsz + (j - bsz)];
}

__global__ void __launch_bounds__(256) gram_kernel(const float* __restrict__ a, const float* __restrict__ b,
                                                   int64_t P, int64_t bsz, int64_t n, int64_t k_per_cta,
                                                   double* __restrict__ t) {
  // upper-triangle tile index -> (ti, tj)
  int64_t ntile = (n + kGT - 1) / kGT;
  int64_t idx = blockIdx.x, ti = 0;
  while (idx >= ntile - ti) {
    idx -= ntile - ti;
    ++ti;
  }
  int64_t tj = ti + idx;
  const int64_t i0 = ti * kGT, j0 = tj * kGT;
  const int64_t k_begin = (int64_t)blockIdx.z * k_per_cta;
  const int64_t k_end = min(P, k_begin + k_per_cta);
  __shared__ float si[kGK][kGT];
  __shared__ float sj[kGK][kGT];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc64[4][4];
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc64[u][v] = 0.0;
  for (int64_t c0 = k_begin; c0 < k_end; c0 += kChunk) {
    const int64_t c1 = min(k_end, c0 + kChunk);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    for (int64_t k0 = c0; k0 < c1; k0 += kGK) {
      for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
        int kk = e / kGT, col = e % kGT;
        int64_t p = k0 + kk;
        bool ok = p < c1;
        si[kk][col] = (ok && i0 + col < n) ? ycol(a, b, bsz, p, i0 + col) : 0.f;
        sj[kk][col] = (ok && j0 + col < n) ? ycol(a, b, bsz, p, j0 + col) : 0.f;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kGK; ++kk) {
        float xi[4], xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          xi[u] = si[kk][ty * 4 + u];
          xj[u] = sj[kk][tx * 4 + u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] += xi[u] * xj[v];
      }
      __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc64[u][v] += (double)acc[u][v];
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      int64_t i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
      if (i < n && j < n && j >= i) atomicAdd(&t[i * n + j], acc64[u][v]);
    }
  }
}

__global__ void mirror_kernel(double* t, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  int64_t i = idx / n, j = idx % n;
  if (j < i) t[i * n + j] = t[j * n + i];
}

// ---------------------------------------------------------------- FP64 CG
// State: x, r, p, q (n each) + scalars s[0]=rr, s[1]=pq, s[2]=rr_new, s[3]=stop
// (1 when converged), s[4]=tol^2 * ||b||^2, s[5]=iterations.
__global__ void cg_init_kernel(const double* __restrict__ rhs, int64_t n, double* x, double* r, double* p,
                               double* s, double tol) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double v = rhs[i];
    x[i] = 0.0;
    r[i] = v;
    p[i] = v;
    acc += v * v;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s[0] = red[0];
    s[1] = 0.0;
    s[2] = 0.0;
    s[3] = red[0] == 0.0 ? 1.0 : 0.0;
    s[4] = tol * tol * red[0];
    s[5] = 0.0;
  }
}

// q = (scale T + shift I) p ; s[1] += p.q   (a warp per row)
__global__ void cg_matvec_kernel(const double* __restrict__ t, int64_t n, double scale, double shift,
                                 const double* __restrict__ p, double* __restrict__ q, double* s) {
  if (s[3] != 0.0) return;
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= n) return;
  const double* tr = t + row * n;
  double acc = 0.0;
  for (int64_t j = lane; j < n; j += 32) acc += tr[j] * p[j];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    double v = scale * acc + shift * p[row];
    q[row] = v;
    atomicAdd(&s[1], v * p[row]);
  }
}

// x += alpha p, r -= alpha q, s[2] += r.r
__global__ void cg_update_kernel(int64_t n, double* x, double* r, const double* p, const double* q, double* s) {
  if (s[3] != 0.0) return;
  __shared__ double red[256];
  double alpha = s[0] / s[1];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    double ri = r[i] - alpha * q[i];
    r[i] = ri;
    acc += ri * ri;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(&s[2], red[0]);
}

// p = r + beta p; roll the scalars; stop when ||r||^2 <= tol^2 ||b||^2
__global__ void cg_direction_kernel(int64_t n, const double* r, double* p, double* s, int last) {
  if (s[3] != 0.0) return;
  double beta = s[2] / s[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = r[i] + beta * p[i];
}

__global__ void cg_roll_kernel(double* s) {
  if (s[3] != 0.0) return;
  s[5] += 1.0;
  s[0] = s[2];
  s[1] = 0.0;
  s[2] = 0.0;
  if (s[0] <= s[4]) s[3] = 1.0;
}

// ---------------------------------------------------------------- back-map
// params[p] -= lr * scale * sum_j Y[p][j] alpha[j]   (a warp per row)
__global__ void backmap_kernel(const float* __restrict__ a, const float* __restrict__ b, int64_t P, int64_t bsz,
                               int64_t n, const double* __restrict__ alpha, double scale, float lr,
                               float* __restrict__ params, float* __restrict__ x_out) {
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= P) return;
  double acc = 0.0;
  for (int64_t j = lane; j < n; j += 32) acc += (double)ycol(a, b, bsz, row, j) * alpha[j];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) {
    float xv = (float)(scale * acc);
    if (x_out) x_out[row] = xv;
    if (params) params[row] -= lr * xv;
  }
}

// ---------------------------------------------------------------- complex parameters
// For complex parameters (the RBM family) the SR system is Hermitian:
// S = O_c^H O_c / B, F = O_c^H E_c / B (optimizer.py:94-114). With
// O_c = A + iC (A, C real, stored parameter-major [P][B] as o_re, o_im) the
// push-through identity gives x = O_c^H (T/B + lambda I)^-1 E_c / B with the
// B x B Hermitian T = O_c O_c^H = (A^T A + C^T C) + i (C^T A - A^T C) (samples
// as rows here). The 2B x 2B real Gram G of [A | C] holds these blocks:
// Tr = G11 + G22, Ti = G21 - G12. The Hermitian system T z = e is solved as
// the real symmetric positive (semi)definite embedding
//     [[Tr, -Ti], [Ti, Tr]] [zr; zi] = [er; ei],
// written over G in place: each thread owns the four entries (i, j),
// (i, n+j), (n+i, j), (n+i, n+j) of one (i, j), reads them and writes them.
__global__ void hermitian_embed_kernel(double* g, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const int64_t i = idx / n, j = idx % n, m = 2 * n;
  const double g11 = g[i * m + j], g12 = g[i * m + n + j];
  const double g21 = g[(n + i) * m + j], g22 = g[(n + i) * m + n + j];
  const double tr = g11 + g22, ti = g21 - g12;
  g[i * m + j] = tr;
  g[i * m + n + j] = -ti;
  g[(n + i) * m + j] = ti;
  g[(n + i) * m + n + j] = tr;
}

// x = scale * O_c^H z = scale * [(A zr + C zi) + i (A zi - C zr)] per parameter
// (A, C parameter-major rows); params (interleaved re, im) -= lr * x when
// params != NULL, x (interleaved) written to x_out when != NULL. Warp per row.
__global__ void complex_backmap_kernel(const float* __restrict__ a, const float* __restrict__ c, int64_t P,
                                       int64_t bsz, const double* __restrict__ z, double scale, float lr,
                                       float2* __restrict__ params, float2* __restrict__ x_out) {
  int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= P) return;
  const float* ar = a + row * bsz;
  const float* cr = c + row * bsz;
  double xr = 0.0, xi = 0.0;
  for (int64_t j = lane; j < bsz; j += 32) {
    double av = ar[j], cv = cr[j], zr = z[j], zi = z[bsz + j];
    xr += av * zr + cv * zi;
    xi += av * zi - cv * zr;
  }
  for (int o = 16; o > 0; o >>= 1) {
    xr += __shfl_xor_sync(0xffffffffu, xr, o);
    xi += __shfl_xor_sync(0xffffffffu, xi, o);
  }
  if (lane == 0) {
    float2 xv = make_float2((float)(scale * xr), (float)(scale * xi));
    if (x_out) x_out[row] = xv;
    if (params) {
      float2 p = params[row];
      params[row] = make_float2(p.x - lr * xv.x, p.y - lr * xv.y);
    }
  }
}

}  // namespace fk

using namespace fk;

extern "C" {

int fk_sr_hermitian_embed(double* gram, int64_t n_samples, void* stream) {
  FK_CHECK_ARG(gram && n_samples > 0, "fk_sr_hermitian_embed: bad arguments");
  int64_t nn = n_samples * n_samples;
  hermitian_embed_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(gram,
                                                                                                     n_samples);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_sr_complex_backmap(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples,
                          const double* z, double scale, float lr, float* params, float* x_out, void* stream) {
  FK_CHECK_ARG(o_re && o_im && z && n_params > 0 && n_samples > 0 && (params || x_out),
               "fk_sr_complex_backmap: bad arguments");
  int64_t threads = n_params * 32;
  complex_backmap_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      o_re, o_im, n_params, n_samples, z, scale, lr, reinterpret_cast<float2*>(params),
      reinterpret_cast<float2*>(x_out));
  FK_CUDA(launched());
  return FK_OK;
}

int fk_center_columns(float* y, int64_t rows, int64_t cols, float* mean, void* stream) {
  FK_CHECK_ARG(y && rows >= 0 && cols > 0, "fk_center_columns: bad arguments");
  if (rows == 0) return FK_OK;
  int64_t threads = rows * 32;
  center_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(y, rows, cols,
                                                                                                 mean);
  FK_CUDA(launched());
  return FK_OK;
}

int64_t fk_sr_gram_workspace_bytes(int64_t n_params, int64_t n_samples) {
  (void)n_params;
  (void)n_samples;
  return 0;
}

int fk_sr_gram(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, double* gram,
               int64_t gram_elems, void* stream) {
  FK_CHECK_ARG(o_re && gram && n_params > 0 && n_samples > 0, "fk_sr_gram: bad arguments");
  int64_t n = o_im ? 2 * n_samples : n_samples;
  FK_CHECK_ARG(gram_elems >= n * n, "fk_sr_gram: gram buffer too small (%lld < %lld)", (long long)gram_elems,
               (long long)(n * n));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FK_CUDA(cudaMemsetAsync(gram, 0, (size_t)(n * n) * sizeof(double), s));
  int64_t ntile = (n + kGT - 1) / kGT;
  int64_t tiles = ntile * (ntile + 1) / 2;
  // enough K splits to fill the GPU ~4 times over
  int64_t splits = (4 * 152 + tiles - 1) / tiles;
  int64_t kmax = (n_params + kGK - 1) / kGK;
  if (splits > kmax) splits = kmax;
  if (splits < 1) splits = 1;
  int64_t kper = (n_params + splits - 1) / splits;
  kper = (kper + kGK - 1) / kGK * kGK;
  dim3 grid((unsigned)tiles, 1, (unsigned)splits);
  gram_kernel<<<grid, 256, 0, s>>>(o_re, o_im ? o_im : o_re, n_params, n_samples, n, kper, gram);
  FK_CUDA(launched());
  mirror_kernel<<<(unsigned)((n * n + 255) / 256), 256, 0, s>>>(gram, n);
  FK_CUDA(launched());
  return FK_OK;
}

int64_t fk_sr_solve_workspace_bytes(int64_t n) { return (3 * n + 8) * (int64_t)sizeof(double); }

int fk_sr_solve(const double* gram, int64_t n, double scale, double shift, const double* rhs, double tol,
                int32_t max_iter, double* x, double* stats, void* workspace, int64_t workspace_bytes,
                void* stream) {
  FK_CHECK_ARG(gram && rhs && x && n > 0 && max_iter > 0, "fk_sr_solve: bad arguments");
  FK_CHECK_ARG(workspace && workspace_bytes >= fk_sr_solve_workspace_bytes(n), "fk_sr_solve: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* r = static_cast<double*>(workspace);
  double* p = r + n;
  double* q = p + n;
  double* sc = q + n;
  cg_init_kernel<<<1, 1024, 0, st>>>(rhs, n, x, r, p, sc, tol);
  FK_CUDA(launched());
  const unsigned mv_blocks = (unsigned)((n * 32 + 255) / 256);
  const unsigned vec_blocks = (unsigned)((n + 255) / 256 < 152 ? (n + 255) / 256 : 152);
  // Every iteration is launched; once converged the kernels return at once
  // (no host synchronisation inside the solve).
  for (int it = 0; it < max_iter; ++it) {
    cg_matvec_kernel<<<mv_blocks, 256, 0, st>>>(gram, n, scale, shift, p, q, sc);
    cg_update_kernel<<<vec_blocks, 256, 0, st>>>(n, x, r, p, q, sc);
    cg_direction_kernel<<<vec_blocks, 256, 0, st>>>(n, r, p, sc, 0);
    cg_roll_kernel<<<1, 1, 0, st>>>(sc);
    FK_CUDA(launched(4));
  }
  if (stats) {
    // stats = {iterations, ||r||^2, tol^2 ||b||^2}
    FK_CUDA(cudaMemcpyAsync(stats, sc + 5, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 1, sc + 0, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 2, sc + 4, sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  return FK_OK;
}

int fk_sr_backmap(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, const double* alpha,
                  double scale, float lr, float* params, float* x_out, void* stream) {
  FK_CHECK_ARG(o_re && alpha && n_params > 0 && n_samples > 0 && (params || x_out), "fk_sr_backmap: bad arguments");
  int64_t n = o_im ? 2 * n_samples : n_samples;
  int64_t threads = n_params * 32;
  backmap_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      o_re, o_im ? o_im : o_re, n_params, n_samples, n, alpha, scale, lr, params, x_out);
  FK_CUDA(launched());
  return FK_OK;
}


}  // extern "C"

// ---------------------------------------------------------------- no-allocation solve
// Some hosts cannot hand this library a workspace: their device memory is
// owned by another allocator (a framework that reserves nearly all of the GPU
// at start-up, so a cudaMalloc would fail), or their policy forbids
// cudaMalloc/cudaFree on the solve path because those calls synchronise the
// device. fk_sr_solve_noalloc serves them with the scratch of the conjugate
// gradients (three vectors of length n plus eight scalars) in a file-scope
// device array of fixed size. The array exists once per device that loads the
// library and stays reserved until the process exits.
namespace fk {

constexpr int64_t kNoAllocMaxN = 8192;  // largest n: 196,672 bytes of scratch
static __device__ __align__(256) double g_sr_noalloc_scratch[3 * kNoAllocMaxN + 8];

// Device address of the scratch array on the current device, looked up once
// per device with that device current (the host-side name is not a device
// pointer and must never be handed to a kernel).
// std::call_once makes the per-device set-up safe when several host threads
// make their first call on a device at the same time. The address belongs to
// the device's current context: after cudaDeviceReset the library must be
// reloaded before this entry point is called again on that device.
constexpr int kNoAllocMaxDevices = 64;

static double* noalloc_scratch() {
  int dev = 0;
  if (check_cuda(cudaGetDevice(&dev), "cudaGetDevice") != FK_OK) return nullptr;
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("fk_sr_solve_noalloc: device index %d out of range", dev);
    return nullptr;
  }
  static std::once_flag once[kNoAllocMaxDevices];
  static double* cached[kNoAllocMaxDevices] = {nullptr};
  static cudaError_t lookup[kNoAllocMaxDevices];
  std::call_once(once[dev], [dev] {
    void* p = nullptr;
    lookup[dev] = cudaGetSymbolAddress(&p, g_sr_noalloc_scratch);
    if (lookup[dev] == cudaSuccess) cached[dev] = static_cast<double*>(p);
  });
  if (check_cuda(lookup[dev], "cudaGetSymbolAddress") != FK_OK) return nullptr;
  return cached[dev];
}

}  // namespace fk

extern "C" int fk_sr_solve_noalloc(const double* gram, int64_t n, double scale, double shift, const double* rhs,
                                   double tol, int32_t max_iter, double* x, double* stats, void* stream) {
  FK_CHECK_ARG(gram && rhs && x && n > 0 && max_iter > 0, "fk_sr_solve_noalloc: bad arguments");
  FK_CHECK_ARG(n <= fk::kNoAllocMaxN,
               "fk_sr_solve_noalloc: n = %lld exceeds the built-in scratch (n <= %lld); use fk_sr_solve with a "
               "workspace",
               (long long)n, (long long)fk::kNoAllocMaxN);
  double* ws = fk::noalloc_scratch();
  if (!ws) return FK_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* r = ws;
  double* p = r + n;
  double* q = p + n;
  double* sc = q + n;
  // cg_init rewrites x, r, p and every scalar before any of them is read, so
  // nothing left in the shared array by an earlier call is ever used.
  fk::cg_init_kernel<<<1, 1024, 0, st>>>(rhs, n, x, r, p, sc, tol);
  FK_CUDA(fk::launched());
  const unsigned mv_blocks = (unsigned)((n * 32 + 255) / 256);
  const unsigned vec_blocks = (unsigned)((n + 255) / 256 < 152 ? (n + 255) / 256 : 152);
  for (int it = 0; it < max_iter; ++it) {
    fk::cg_matvec_kernel<<<mv_blocks, 256, 0, st>>>(gram, n, scale, shift, p, q, sc);
    fk::cg_update_kernel<<<vec_blocks, 256, 0, st>>>(n, x, r, p, q, sc);
    fk::cg_direction_kernel<<<vec_blocks, 256, 0, st>>>(n, r, p, sc, 0);
    fk::cg_roll_kernel<<<1, 1, 0, st>>>(sc);
    FK_CUDA(fk::launched(4));
  }
  if (stats) {
    FK_CUDA(cudaMemcpyAsync(stats, sc + 5, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 1, sc + 0, sizeof(double), cudaMemcpyDeviceToDevice, st));
    FK_CUDA(cudaMemcpyAsync(stats + 2, sc + 4, sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  return FK_OK;
}
