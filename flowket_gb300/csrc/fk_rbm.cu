// RBM machines and Metropolis-Hastings chains (the MCMC path).
//
// log psi(s) = sum_i a_i s_i + sum_j lncosh(theta_j),  theta_j = b_j + sum_i W_ij s_i
// (machines/rbm.py:35-48, layers/complex/dense.py:11-50), complex64 parameters
// stored as interleaved (re, im) floats [a (N) | b (M) | W (N x M row-major)].
// lncosh(z) = |Re z| - ln 2 + log(e^{z-|Re z|} + e^{-z-|Re z|})
// (layers/complex/tensorflow_ops.py:79-85).
//
// One warp owns one chain or sample: lane l holds theta_j for j = l, l+32, ...
// Proposals and acceptance follow samplers/metropolis_hastings.py:99-145:
// Local flips one site, Exchange swaps a site with a neighbour at offset in
// {-1,0,1} (wrap); accept iff 2 dRe log psi >= 0 or exp(2 dRe log psi) > U.
// The random words come from Philox4x32-10 with counter
// (chain, sweep_lo, sweep_hi, 0x4D48), the same as the oracle's.
#include "fk_common.cuh"

namespace fk {

struct Cplx {
  float re, im;
};
__device__ __forceinline__ Cplx cadd(Cplx a, Cplx b) { return Cplx{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Cplx cscale(Cplx a, float s) { return Cplx{a.re * s, a.im * s}; }

// lncosh(z) with the reference's overflow-safe form.
__device__ __forceinline__ Cplx lncosh(Cplx z) {
  float a = fabsf(z.re);
  // e^{z - a} + e^{-z - a}
  float e1 = expf(z.re - a), e2 = expf(-z.re - a);
  float s, c;
  sincosf(z.im, &s, &c);
  float wr = e1 * c + e2 * c;
  float wi = e1 * s - e2 * s;
  return Cplx{a - 0.69314718055994531f + 0.5f * logf(wr * wr + wi * wi), atan2f(wi, wr)};
}

__device__ __forceinline__ Cplx warp_sum(Cplx v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  return v;
}

struct RbmView {
  const Cplx* a;
  const Cplx* b;
  const Cplx* w;
  int n, m;
};

__device__ __forceinline__ RbmView rbm_view(const float* params, int n, int m) {
  const Cplx* p = reinterpret_cast<const Cplx*>(params);
  return RbmView{p, p + n, p + n + m, n, m};
}

constexpr int kMaxHiddenPerLane = 32;  // M <= 1024

// theta (per lane) and log psi of spins s (int8, length n) for one warp.
__device__ __forceinline__ Cplx rbm_theta_logpsi(const RbmView& v, const int8_t* s, Cplx* th, int lane) {
  const int per = (v.m + 31) / 32;
  for (int q = 0; q < per; ++q) {
    int j = lane + 32 * q;
    th[q] = j < v.m ? v.b[j] : Cplx{0.f, 0.f};
  }
  Cplx vis{0.f, 0.f};
  for (int i = 0; i < v.n; ++i) {
    float si = (float)s[i];
    if (lane == 0) vis = cadd(vis, cscale(v.a[i], si));
    const Cplx* wr = v.w + (int64_t)i * v.m;
    for (int q = 0; q < per; ++q) {
      int j = lane + 32 * q;
      if (j < v.m) th[q] = cadd(th[q], cscale(wr[j], si));
    }
  }
  Cplx acc = vis;
  for (int q = 0; q < per; ++q) {
    int j = lane + 32 * q;
    if (j < v.m) acc = cadd(acc, lncosh(th[q]));
  }
  return warp_sum(acc);
}

// log psi(s') - log psi(s) for flipping the sites f0, f1 (f1 < 0: one site),
// with theta of s in th. Optionally writes theta' into thn.
__device__ __forceinline__ Cplx rbm_delta(const RbmView& v, const Cplx* th, int f0, float s0, int f1, float s1,
                                          Cplx* thn, int lane) {
  const int per = (v.m + 31) / 32;
  Cplx acc{0.f, 0.f};
  if (lane == 0) {
    acc = cscale(v.a[f0], -2.f * s0);
    if (f1 >= 0) acc = cadd(acc, cscale(v.a[f1], -2.f * s1));
  }
  const Cplx* w0 = v.w + (int64_t)f0 * v.m;
  const Cplx* w1 = f1 >= 0 ? v.w + (int64_t)f1 * v.m : nullptr;
  for (int q = 0; q < per; ++q) {
    int j = lane + 32 * q;
    if (j >= v.m) continue;
    Cplx t = cadd(th[q], cscale(w0[j], -2.f * s0));
    if (w1) t = cadd(t, cscale(w1[j], -2.f * s1));
    Cplx d = lncosh(t);
    Cplx o = lncosh(th[q]);
    acc = cadd(acc, Cplx{d.re - o.re, d.im - o.im});
    if (thn) thn[q] = t;
  }
  return warp_sum(acc);
}

__global__ void rbm_logpsi_kernel(const float* __restrict__ params, int n, int m, const int8_t* __restrict__ spins,
                                  int64_t batch, float2* __restrict__ out) {
  int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= batch) return;
  RbmView v = rbm_view(params, n, m);
  Cplx th[kMaxHiddenPerLane];
  Cplx lp = rbm_theta_logpsi(v, spins + w * n, th, lane);
  if (lane == 0) out[w] = make_float2(lp.re, lp.im);
}

// E_loc(s) = mel_0 + sum_{used slots} mel_c exp(log psi(s_c) - log psi(s)),
// connections given by the operator enumeration (flip pairs), ratios from theta.
__global__ void rbm_local_energy_kernel(const float* __restrict__ params, int n, int m,
                                        const int8_t* __restrict__ spins, int64_t batch, const short2* __restrict__ flips,
                                        const double* __restrict__ mel, const uint8_t* __restrict__ use, int n_slots,
                                        double2* __restrict__ local) {
  int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= batch) return;
  RbmView v = rbm_view(params, n, m);
  const int8_t* s = spins + w * n;
  Cplx th[kMaxHiddenPerLane];
  rbm_theta_logpsi(v, s, th, lane);
  Kahan re, im;
  for (int c = 1; c < n_slots; ++c) {
    int64_t o = (int64_t)c * batch + w;
    if (!use[o]) continue;
    short2 f = flips[o];
    float s0 = (float)s[f.x];
    float s1 = f.y >= 0 ? (float)s[f.y] : 0.f;
    Cplx d = rbm_delta(v, th, f.x, s0, f.y, s1, nullptr, lane);
    float e = expf(d.re), sn, cs;
    sincosf(d.im, &sn, &cs);
    float mm = (float)mel[o];
    re.add(mm * e * cs);
    im.add(mm * e * sn);
  }
  if (lane == 0) local[w] = make_double2((double)(re.s - re.c) + mel[w], (double)(im.s - im.c));
}

// O_k = d log psi / d p_k (complex, holomorphic): a -> s_i, b -> tanh(theta_j),
// W -> s_i tanh(theta_j). Output parameter-major, split re/im: [P][batch].
__global__ void rbm_logder_kernel(const float* __restrict__ params, int n, int m, const int8_t* __restrict__ spins,
                                  int64_t batch, float* __restrict__ o_re, float* __restrict__ o_im) {
  int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= batch) return;
  RbmView v = rbm_view(params, n, m);
  const int8_t* s = spins + w * n;
  Cplx th[kMaxHiddenPerLane];
  rbm_theta_logpsi(v, s, th, lane);
  const int per = (m + 31) / 32;
  for (int i = lane; i < n; i += 32) {
    o_re[(int64_t)i * batch + w] = (float)s[i];
    o_im[(int64_t)i * batch + w] = 0.f;
  }
  for (int q = 0; q < per; ++q) {
    int j = lane + 32 * q;
    if (j >= m) continue;
    // tanh of a complex number: (sinh 2x + i sin 2y) / (cosh 2x + cos 2y)
    float x2 = 2.f * th[q].re, y2 = 2.f * th[q].im;
    float den = coshf(x2) + cosf(y2);
    Cplx t = Cplx{sinhf(x2) / den, sinf(y2) / den};
    if (fabsf(x2) > 40.f) t = Cplx{x2 > 0 ? 1.f : -1.f, 0.f};
    o_re[(int64_t)(n + j) * batch + w] = t.re;
    o_im[(int64_t)(n + j) * batch + w] = t.im;
    for (int i = 0; i < n; ++i) {
      float si = (float)s[i];
      int64_t p = n + m + (int64_t)i * m + j;
      o_re[p * batch + w] = si * t.re;
      o_im[p * batch + w] = si * t.im;
    }
  }
}

// Persistent Metropolis-Hastings: one warp per chain, all sweeps in one launch.
// Records the chain after every (unused + 1) sweeps once warm-up is done
// (metropolis_hastings.py:51-65). theta is recomputed from scratch at every
// recorded sample to keep incremental rounding from accumulating.
struct MhArgs {
  const float* params;
  int n, m, hh, ww;  // lattice hh x ww (chain: hh = n, ww = 1)
  int kind;          // 0 = local, 1 = exchange
  int8_t* chains;    // [C][n] in/out
  float2* logpsi;    // [C] in/out
  int64_t n_chains;
  int64_t warmup_sweeps;
  int32_t samples_per_chain;
  int32_t unused;
  uint32_t k0, k1;
  uint64_t sweep0;
  int8_t* samples;   // [C][samples_per_chain][n]
  unsigned long long* accepted;
};

__global__ void __launch_bounds__(128) rbm_mh_kernel(const __grid_constant__ MhArgs a) {
  extern __shared__ int8_t sh_spins[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t chain = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (chain >= a.n_chains) return;
  int8_t* s = sh_spins + warp * a.n;
  for (int i = lane; i < a.n; i += 32) s[i] = a.chains[chain * a.n + i];
  __syncwarp();
  RbmView v = rbm_view(a.params, a.n, a.m);
  Cplx th[kMaxHiddenPerLane], thn[kMaxHiddenPerLane];
  Cplx lp = rbm_theta_logpsi(v, s, th, lane);
  uint64_t sweep = a.sweep0;
  unsigned long long acc_count = 0;
  const int64_t total = a.warmup_sweeps + (int64_t)a.samples_per_chain * (a.unused + 1);
  const int per = (a.m + 31) / 32;
  for (int64_t t = 0; t < total; ++t, ++sweep) {
    U4 x = philox4x32(U4{(uint32_t)chain, (uint32_t)sweep, (uint32_t)(sweep >> 32), 0x4D48u}, a.k0, a.k1);
    int f0, f1 = -1;
    if (a.ww == 1) {
      int i = (int)(x.x % (uint32_t)a.n);
      f0 = i;
      if (a.kind == 1) f1 = (int)((i + (int)(x.y % 3u) - 1 + a.n) % a.n);
    } else {
      int r = (int)(x.x % (uint32_t)a.hh), q = (int)(x.w % (uint32_t)a.ww);
      f0 = r * a.ww + q;
      if (a.kind == 1) {
        int r2 = (r + (int)(x.y % 3u) - 1 + a.hh) % a.hh;
        int q2 = (q + (int)((x.y / 3u) % 3u) - 1 + a.ww) % a.ww;
        f1 = r2 * a.ww + q2;
      }
    }
    bool moved = true;
    if (a.kind == 1) {
      // a swap of equal spins (or of a site with itself) leaves the chain unchanged
      if (f1 == f0 || s[f0] == s[f1]) moved = false;
    }
    float u = philox_uniform(x.z);
    if (moved) {
      Cplx d = rbm_delta(v, th, f0, (float)s[f0], f1, f1 >= 0 ? (float)s[f1] : 0.f, thn, lane);
      float dd = 2.f * d.re;
      bool acc = dd >= 0.f || expf(dd) > u;
      if (acc) {
        for (int q = 0; q < per; ++q) th[q] = thn[q];
        lp = cadd(lp, d);
        __syncwarp();
        if (lane == 0) {
          s[f0] = (int8_t)-s[f0];
          if (f1 >= 0) s[f1] = (int8_t)-s[f1];
        }
        __syncwarp();
        if (t >= a.warmup_sweeps) ++acc_count;  // warm-up moves are not counted (metropolis_hastings.py:58-64)
      }
    } else if (t >= a.warmup_sweeps) {
      ++acc_count;  // the unchanged candidate is accepted (exp(0) > U)
    }
    if (t >= a.warmup_sweeps) {
      int64_t k = t - a.warmup_sweeps;
      if ((k + 1) % (a.unused + 1) == 0) {
        int64_t idx = k / (a.unused + 1);
        int8_t* out = a.samples + (chain * a.samples_per_chain + idx) * a.n;
        for (int i = lane; i < a.n; i += 32) out[i] = s[i];
        lp = rbm_theta_logpsi(v, s, th, lane);
      }
    }
  }
  for (int i = lane; i < a.n; i += 32) a.chains[chain * a.n + i] = s[i];
  if (lane == 0) {
    a.logpsi[chain] = make_float2(lp.re, lp.im);
    atomicAdd(a.accepted, acc_count);
  }
}

// Independent-proposal Metropolis-Hastings step (the learned proposal):
// accept s' with min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s'))), log q = 2 Re log psi_q.
__global__ void mh_independent_kernel(int8_t* __restrict__ chains, float2* __restrict__ lp_chain,
                                      float2* __restrict__ lq_chain, const int8_t* __restrict__ cand,
                                      const float2* __restrict__ lp_cand, const float2* __restrict__ lq_cand,
                                      int64_t n_chains, int n, uint32_t k0, uint32_t k1, uint64_t step,
                                      unsigned long long* accepted) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chains) return;
  U4 x = philox4x32(U4{(uint32_t)c, (uint32_t)step, (uint32_t)(step >> 32), 0x1D4Du}, k0, k1);
  float u = philox_uniform(x.x);
  float d = 2.f * (lp_cand[c].x - lp_chain[c].x) + 2.f * (lq_chain[c].x - lq_cand[c].x);
  bool acc = d >= 0.f || expf(d) > u;
  if (acc) {
    for (int i = 0; i < n; ++i) chains[c * n + i] = cand[c * n + i];
    lp_chain[c] = lp_cand[c];
    lq_chain[c] = lq_cand[c];
    atomicAdd(accepted, 1ull);
  }
}

// Metropolis-Hastings with Hamiltonian proposals (metropolis_hastings.py:170-195):
// the candidate is one of the chain's used connections of the operator (in
// find_conn slot order), drawn uniformly with Philox word 0 of counter
// (chain, sweep_lo, sweep_hi, 0x484D); it is accepted with
// min(1, |psi(s')|^2 n(s) / (|psi(s)|^2 n(s'))), n = number of used
// connections, against word 2 of the same counter.
__global__ void mh_ham_propose_kernel(const int8_t* __restrict__ chains, const short2* __restrict__ flips,
                                      const uint8_t* __restrict__ use, int n_slots, int64_t n_chains, int n,
                                      uint32_t k0, uint32_t k1, uint64_t sweep, int8_t* __restrict__ cand,
                                      int32_t* __restrict__ n_conn) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chains) return;
  int cnt = 0;
  for (int q = 0; q < n_slots; ++q) cnt += use[(int64_t)q * n_chains + c] != 0;
  U4 x = philox4x32(U4{(uint32_t)c, (uint32_t)sweep, (uint32_t)(sweep >> 32), 0x484Du}, k0, k1);
  int f0 = -1, f1 = -1;
  if (cnt > 0) {
    int k = (int)(philox_uniform(x.x) * (float)cnt);
    if (k >= cnt) k = cnt - 1;
    for (int q = 0; q < n_slots; ++q) {
      if (!use[(int64_t)q * n_chains + c]) continue;
      if (k-- == 0) {
        short2 f = flips[(int64_t)q * n_chains + c];
        f0 = f.x;
        f1 = f.y;
        break;
      }
    }
  }
  for (int i = 0; i < n; ++i) {
    int8_t v = chains[c * n + i];
    cand[c * n + i] = (i == f0 || i == f1) ? (int8_t)-v : v;
  }
  n_conn[c] = cnt > 0 ? cnt : 1;
}

__global__ void mh_ham_accept_kernel(int8_t* __restrict__ chains, float2* __restrict__ lp_chain,
                                     const int8_t* __restrict__ cand, const float2* __restrict__ lp_cand,
                                     const int32_t* __restrict__ n_conn, const uint8_t* __restrict__ use_cand,
                                     int n_slots, int64_t n_chains, int n, uint32_t k0, uint32_t k1, uint64_t sweep,
                                     unsigned long long* accepted) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chains) return;
  int nc = 0;
  for (int q = 0; q < n_slots; ++q) nc += use_cand[(int64_t)q * n_chains + c] != 0;
  if (nc == 0) nc = 1;
  U4 x = philox4x32(U4{(uint32_t)c, (uint32_t)sweep, (uint32_t)(sweep >> 32), 0x484Du}, k0, k1);
  const float u = philox_uniform(x.z);
  const float d = 2.f * (lp_cand[c].x - lp_chain[c].x) + logf((float)n_conn[c] / (float)nc);
  if (d >= 0.f || expf(d) > u) {
    for (int i = 0; i < n; ++i) chains[c * n + i] = cand[c * n + i];
    lp_chain[c] = lp_cand[c];
    if (accepted) atomicAdd(accepted, 1ull);
  }
}

}  // namespace fk

using namespace fk;

static int rbm_check(int n, int m) {
  if (n < 1 || n > 4096 || m < 1 || m > 32 * kMaxHiddenPerLane) {
    set_error("fk_rbm: unsupported size (visible %d, hidden %d; hidden <= %d)", n, m, 32 * kMaxHiddenPerLane);
    return FK_ERR_ARG;
  }
  return FK_OK;
}

extern "C" {

int fk_rbm_log_psi(const float* params, int32_t n_visible, int32_t n_hidden, const int8_t* spins, int64_t batch,
                   float* log_psi, void* stream) {
  int st = rbm_check(n_visible, n_hidden);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(params && spins && log_psi && batch >= 0, "fk_rbm_log_psi: NULL buffer");
  if (batch == 0) return FK_OK;
  int64_t threads = batch * 32;
  rbm_logpsi_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      params, n_visible, n_hidden, spins, batch, reinterpret_cast<float2*>(log_psi));
  FK_CUDA(launched());
  return FK_OK;
}

int fk_rbm_local_energy(const float* params, int32_t n_visible, int32_t n_hidden, const int8_t* spins, int64_t batch,
                        const int16_t* flips, const double* mel, const uint8_t* use, int32_t n_slots, double* local,
                        void* stream) {
  int st = rbm_check(n_visible, n_hidden);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(params && spins && flips && mel && use && local && batch >= 0, "fk_rbm_local_energy: NULL buffer");
  if (batch == 0) return FK_OK;
  int64_t threads = batch * 32;
  rbm_local_energy_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      params, n_visible, n_hidden, spins, batch, reinterpret_cast<const short2*>(flips), mel, use, n_slots,
      reinterpret_cast<double2*>(local));
  FK_CUDA(launched());
  return FK_OK;
}

int fk_rbm_log_derivatives(const float* params, int32_t n_visible, int32_t n_hidden, const int8_t* spins,
                           int64_t batch, float* o_re, float* o_im, void* stream) {
  int st = rbm_check(n_visible, n_hidden);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(params && spins && o_re && o_im && batch >= 0, "fk_rbm_log_derivatives: NULL buffer");
  if (batch == 0) return FK_OK;
  int64_t threads = batch * 32;
  rbm_logder_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      params, n_visible, n_hidden, spins, batch, o_re, o_im);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_rbm_mh_sweeps(const float* params, int32_t n_visible, int32_t n_hidden, int32_t height, int32_t width,
                     int32_t kind, int8_t* chains, float* log_psi, int64_t n_chains, int64_t warmup_sweeps,
                     int32_t samples_per_chain, int32_t unused, uint64_t seed, uint64_t sweep_offset, int8_t* samples,
                     unsigned long long* accepted, void* stream) {
  int st = rbm_check(n_visible, n_hidden);
  if (st != FK_OK) return st;
  FK_CHECK_ARG(params && chains && log_psi && samples && accepted && n_chains > 0 && samples_per_chain >= 0 &&
                   unused >= 0 && warmup_sweeps >= 0,
               "fk_rbm_mh_sweeps: bad arguments");
  FK_CHECK_ARG(height * width == n_visible, "fk_rbm_mh_sweeps: lattice %dx%d != %d visible", height, width,
               n_visible);
  FK_CHECK_ARG(kind == 0 || kind == 1, "fk_rbm_mh_sweeps: kind must be 0 (local) or 1 (exchange)");
  MhArgs a;
  a.params = params;
  a.n = n_visible;
  a.m = n_hidden;
  a.hh = height;
  a.ww = width;
  a.kind = kind;
  a.chains = chains;
  a.logpsi = reinterpret_cast<float2*>(log_psi);
  a.n_chains = n_chains;
  a.warmup_sweeps = warmup_sweeps;
  a.samples_per_chain = samples_per_chain;
  a.unused = unused;
  a.k0 = (uint32_t)seed;
  a.k1 = (uint32_t)(seed >> 32);
  a.sweep0 = sweep_offset;
  a.samples = samples;
  a.accepted = accepted;
  const int warps = 4;
  size_t smem = (size_t)warps * n_visible;
  rbm_mh_kernel<<<(unsigned)((n_chains + warps - 1) / warps), 32 * warps, smem, static_cast<cudaStream_t>(stream)>>>(
      a);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_mh_independent_step(int8_t* chains, float* lp_chain, float* lq_chain, const int8_t* candidates,
                           const float* lp_cand, const float* lq_cand, int64_t n_chains, int32_t n_visible,
                           uint64_t seed, uint64_t step, unsigned long long* accepted, void* stream) {
  FK_CHECK_ARG(chains && lp_chain && lq_chain && candidates && lp_cand && lq_cand && accepted && n_chains > 0,
               "fk_mh_independent_step: NULL buffer");
  mh_independent_kernel<<<(unsigned)((n_chains + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, reinterpret_cast<float2*>(lp_chain), reinterpret_cast<float2*>(lq_chain), candidates,
      reinterpret_cast<const float2*>(lp_cand), reinterpret_cast<const float2*>(lq_cand), n_chains, n_visible,
      (uint32_t)seed, (uint32_t)(seed >> 32), step, accepted);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_mh_hamiltonian_propose(const int8_t* chains, const int16_t* flips, const uint8_t* use, int32_t n_slots,
                              int64_t n_chains, int32_t n_sites, uint64_t seed, uint64_t sweep, int8_t* candidates,
                              int32_t* n_conn, void* stream) {
  FK_CHECK_ARG(chains && flips && use && candidates && n_conn && n_slots > 0 && n_chains > 0 && n_sites > 0,
               "fk_mh_hamiltonian_propose: bad arguments");
  mh_ham_propose_kernel<<<(unsigned)((n_chains + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, reinterpret_cast<const short2*>(flips), use, n_slots, n_chains, n_sites, (uint32_t)seed,
      (uint32_t)(seed >> 32), sweep, candidates, n_conn);
  FK_CUDA(launched());
  return FK_OK;
}

int fk_mh_hamiltonian_accept(int8_t* chains, float* lp_chain, const int8_t* candidates, const float* lp_cand,
                             const int32_t* n_conn, const uint8_t* use_cand, int32_t n_slots, int64_t n_chains,
                             int32_t n_sites, uint64_t seed, uint64_t sweep, unsigned long long* accepted,
                             void* stream) {
  FK_CHECK_ARG(chains && lp_chain && candidates && lp_cand && n_conn && use_cand && n_slots > 0 && n_chains > 0 &&
                   n_sites > 0,
               "fk_mh_hamiltonian_accept: bad arguments");
  mh_ham_accept_kernel<<<(unsigned)((n_chains + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, reinterpret_cast<float2*>(lp_chain), candidates, reinterpret_cast<const float2*>(lp_cand), n_conn,
      use_cand, n_slots, n_chains, n_sites, (uint32_t)seed, (uint32_t)(seed >> 32), sweep, accepted);
  FK_CUDA(launched());
  return FK_OK;
}

}  // extern "C"
