// Host-side plumbing shared by every entry point: error strings, the device
// error word written by bounded waits, the build string, and the Adam step.
#include <stdarg.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "fk_common.cuh"

namespace fk {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FK_OK;
  set_error("%s failed: %s", what, cudaGetErrorString(e));
  return FK_ERR_CUDA;
}

// One error word per device. Bounded waits OR 1 into it; it lives in a
// file-scope __device__ variable, so reading its address allocates nothing.
__device__ int g_device_error;

static std::atomic<long long> g_launches{0};

cudaError_t launched(int n) {
  g_launches.fetch_add(n, std::memory_order_relaxed);
  return cudaGetLastError();
}

// Looked up once per device (std::call_once: safe when several host threads
// make their first call together). The address belongs to the device's
// current context; after cudaDeviceReset the library must be reloaded.
int* device_error_word() {
  constexpr int kMaxDevices = 64;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  if (dev < 0 || dev >= kMaxDevices) return nullptr;
  static std::once_flag once[kMaxDevices];
  static int* cached[kMaxDevices] = {nullptr};
  std::call_once(once[dev], [dev] {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_error) == cudaSuccess) cached[dev] = static_cast<int*>(p);
  });
  return cached[dev];
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr_t, float b1, float b2, float eps) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr_t * mi / (sqrtf(vi) + eps);
  }
}

// Self-test of the bounded-wait mechanism: waits on an mbarrier that nothing
// arrives at, `limit` polls at most, so the wait runs out, sets the timeout bit
// of the error word and the kernel returns normally.
__global__ void selftest_wait_kernel(int* err, uint32_t limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  mbar_wait_limit(&bar, 0, err, limit);
  mbar_inval(&bar);
}

__global__ void axpy_kernel(int64_t n, float a, const float* __restrict__ x, float* __restrict__ y) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) y[i] += a * x[i];
}

}  // namespace fk

extern "C" {

int fk_axpy(int64_t n, float a, const float* x, float* y, void* stream) {
  FK_CHECK_ARG(x && y && n >= 0, "fk_axpy: bad arguments");
  if (n == 0) return FK_OK;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  fk::axpy_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(n, a, x, y);
  FK_CUDA(fk::launched());
  return FK_OK;
}

const char* fk_last_error(void) { return fk::g_last_error; }

int64_t fk_kernel_launches(void) { return fk::g_launches.load(); }

const char* fk_version(void) { return "flowket_gb300 0.1 sm_103a (tcgen05 + bulk-copy TMA)"; }

int fk_device_status(int* status, int clear, void* stream) {
  FK_CHECK_ARG(status != nullptr, "fk_device_status: status is NULL");
  int* word = fk::device_error_word();
  if (!word) {
    fk::set_error("fk_device_status: no device error word");
    return FK_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FK_CUDA(cudaMemcpyAsync(status, word, sizeof(int), cudaMemcpyDeviceToHost, s));
  FK_CUDA(cudaStreamSynchronize(s));
  if (clear) FK_CUDA(cudaMemsetAsync(word, 0, sizeof(int), s));
  return FK_OK;
}

int fk_selftest_wait_timeout(int32_t polls, void* stream) {
  FK_CHECK_ARG(polls >= 1 && polls <= (1 << 20), "fk_selftest_wait_timeout: polls must be in [1, 2^20]");
  int* word = fk::device_error_word();
  if (!word) {
    fk::set_error("fk_selftest_wait_timeout: no device error word");
    return FK_ERR_CUDA;
  }
  fk::selftest_wait_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(word, (uint32_t)polls);
  FK_CUDA(fk::launched());
  return FK_OK;
}

int fk_adam_step(float* params, const float* grad, float* m, float* v, int64_t n, int64_t step, float lr,
                 float beta1, float beta2, float epsilon, void* stream) {
  FK_CHECK_ARG(params && grad && m && v && n >= 0 && step >= 1, "fk_adam_step: bad arguments");
  if (n == 0) return FK_OK;
  double t = (double)step;
  float lr_t = (float)(lr * sqrt(1.0 - pow((double)beta2, t)) / (1.0 - pow((double)beta1, t)));
  int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  if (blocks > 152 * 16) blocks = 152 * 16;
  fk::adam_kernel<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(params, grad, m, v, n,
                                                                                        lr_t, beta1, beta2,
                                                                                        epsilon);
  FK_CUDA(fk::launched());
  return FK_OK;
}

}  // extern "C"
