/*
 * flowket_gb300 -- C ABI of the GB300 (sm_103a) variational Monte Carlo hot path.
 *
 * Conventions
 *   - Every entry point returns an int status: FK_OK (0) or a negative FK_ERR_*;
 *     fk_last_error() returns the message of the last failure on this thread.
 *   - All device buffers are caller owned. Scratch memory is passed in as a
 *     workspace whose size comes from the matching *_bytes() query; the library
 *     allocates nothing on these paths and never synchronises the stream.
 *   - `stream` is a cudaStream_t passed as void*.
 *   - Spins are int8 +-1 at the boundary, row-major [batch][H*W]; complex
 *     numbers are interleaved (re, im) pairs.
 *   - Citations name the reference (FlowKet) interface each entry point replaces,
 *     as path:line within the FlowKet source tree.
 */
#ifndef FLOWKET_GB300_H
#define FLOWKET_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FK_OK 0
#define FK_ERR_ARG (-1)         /* bad argument or unsupported shape */
#define FK_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define FK_ERR_TIMEOUT (-3)     /* a device-side wait gave up (see fk_device_status) */
#define FK_ERR_NONFINITE (-4)   /* a non-finite value where the reference raises */

#define FK_PRECISION_FP32 0     /* plain FP32 CUDA-core path */
#define FK_PRECISION_BF16 1     /* BF16 tcgen05 tensor-core path, FP32 accumulate */
#define FK_PRECISION_FP16 2     /* the same tensor-core path with FP16 operands and stored
                                   activations (10 mantissa bits instead of 7), FP32 accumulate */

#define FK_AR2D_INFER 0         /* forward keeps only a rolling set of activations */
#define FK_AR2D_SAVE 1          /* forward keeps every activation for the adjoint */

const char* fk_last_error(void);
/* Device error word: bits set by kernels instead of faulting or hanging. */
#define FK_STATUS_TIMEOUT 1     /* a bounded device-side wait gave up (the kernel unwound) */
#define FK_STATUS_NONFINITE 2   /* a non-finite energy statistic (the reference raises on a
                                   non-finite wave function, samplers/metropolis_hastings.py:103-105) */
/* Reads (and optionally clears) the device error word of the current device:
 * synchronises `stream` and writes the FK_STATUS_* bits set since the last clear. */
int fk_device_status(int* status, int clear, void* stream);
/* Self-test of the failure detection (no reference counterpart): one kernel
 * waits on an mbarrier that nothing arrives at, at most `polls` polls
 * (1..2^20), so the wait runs out, FK_STATUS_TIMEOUT is set in the device
 * error word and the kernel returns normally; the context stays usable. */
int fk_selftest_wait_timeout(int32_t polls, void* stream);
/* Library build string (arch, version). */
const char* fk_version(void);
/* Number of kernel launches this library has issued in this process. */
int64_t fk_kernel_launches(void);

/* ------------------------------------------------------------------ operators
 * Connected-configuration enumeration (kernel c). For every sample b and slot c
 * (slot 0 = the sample itself) writes:
 *   flips[c][b][2]  int16 sites exchanged/flipped by slot c (-1 = none),
 *   mel[c][b]       float64 matrix element,
 *   use[c][b]       uint8 1 iff the slot is a real connection,
 *   conn[c][b][N]   int8 connected configuration (optional, may be NULL).
 * Slot order and values are those of the reference operator.
 */
/* operators/heisenberg.py:47-121 (HeisenbergFindConn.find_conn); slots = N*dim+1,
 * dim = number of lattice axes (1 for a chain, 2 for H x W). */
int fk_find_conn_heisenberg(const int8_t* spins, int64_t batch, int32_t height, int32_t width, int32_t dim,
                            int32_t pbc, int32_t unitary_rotation, int16_t* flips, double* mel, uint8_t* use,
                            int8_t* conn, void* stream);
/* operators/ising.py:17-46 (Ising.find_conn); slots = N+1. */
int fk_find_conn_ising(const int8_t* spins, int64_t batch, int32_t height, int32_t width, double h, double j,
                       int32_t pbc, int16_t* flips, double* mel, uint8_t* use, int8_t* conn, void* stream);
/* operators/j1j2.py:7-69 via operators/netket_operator.py:46-66; slots = 4N+1,
 * exchange connections packed in edge order, unused slots zero. */
int fk_find_conn_j1j2(const int8_t* spins, int64_t batch, int32_t height, int32_t width, double j2, int32_t pbc,
                      int16_t* flips, double* mel, uint8_t* use, int8_t* conn, void* stream);

/* Compaction of the used slots (observables/monte_carlo/operator.py:6-10):
 * offsets[b] .. offsets[b+1] are the rows of sample b in the compact list
 * (offsets int64 [B+1]); owner[row] = b; cmel[row] = matrix element;
 * cflips[row][2] = the slot's flip pair; configs[row][N] = the connected
 * configuration (optional, may be NULL). Slot 0 is skipped when skip_self != 0.
 * *n_rows (device int64) receives the row count; rows beyond max_rows are
 * counted but not written. Workspace: fk_compact_workspace_bytes(batch). */
int64_t fk_compact_workspace_bytes(int64_t batch);
int fk_compact_connections(const int8_t* spins, int64_t batch, int32_t n_sites, int32_t n_slots,
                           const int16_t* flips, const double* mel, const uint8_t* use, int32_t skip_self,
                           int8_t* configs, int32_t* owner, double* cmel, int16_t* cflips, int64_t* offsets,
                           int64_t max_rows, int64_t* n_rows, void* workspace, int64_t workspace_bytes,
                           void* stream);

/* E_loc(b) = mel_self[b] + sum over rows of b of cmel * exp(logpsi_row - logpsi_b)
 * (observables/monte_carlo/operator.py:20-42): the ratio in FP32 as the
 * reference's complex64, Kahan-compensated FP32 sum, diagonal added in FP64.
 * log psi arrays are [.][2] float32; local [B][2] float64. */
int fk_local_energy_reduce(const float* log_psi_self, const double* mel_self, int64_t batch,
                           const float* log_psi_rows, const int64_t* offsets, const double* cmel, double* local,
                           void* stream);
/* Mean and variance of the local energies (observables/monte_carlo/observable.py:10-14)
 * and the loss weights w[b] = (2 Re y, -2 Im y) / B with y = conj(E - Ebar)/B
 * (optimization/variational_monte_carlo.py:38-40, optimization/loss.py:4-5).
 * stats = {Re mean, Im mean, var(Re)} float64; w float32 [B][2]. */
int fk_energy_stats(const double* local, int64_t batch, double* stats, float* w, void* stream);

/* ------------------------------------------------------------------ AR2D machine */
typedef struct fk_ar2d_desc {
  int32_t height;                /* lattice rows (1 for a chain) */
  int32_t width;                 /* lattice columns */
  int32_t depth;                 /* ConvNetAutoregressive2D depth, >= 2 */
  int32_t channels;              /* num_of_channels: 16, 32 or 64 */
  int32_t weights_normalization; /* 1 = WeightNormalization(exponential_norm=True) */
  int32_t precision;             /* FK_PRECISION_FP32, FK_PRECISION_BF16 or FK_PRECISION_FP16 */
  int32_t equal_up_down_spins;   /* 1 = EqualUpDownSpins mask before the normalisation
                                    (abstract_machine.py:52-53, layers/spins_invariants.py:13-22):
                                    outcome k of a site gets log-amplitude -inf once N/2 earlier
                                    sites (raster order) hold it, so the distribution lives on the
                                    Sz = 0 sector */
} fk_ar2d_desc;

/* Flat FP32 parameter vector in Keras layer order: per causal conv i and conv
 * x in (v, h, x, y, c): kernel (kh,kw,cin,cout), bias (cout), g (cout, only
 * with weight normalisation); then out.kernel (1,1,F,4), out.bias (4).
 * machines/conv_net_autoregressive_2D.py:24-74. */
int64_t fk_ar2d_num_params(const fk_ar2d_desc* desc);
int64_t fk_ar2d_packed_bytes(const fk_ar2d_desc* desc);
/* Weight normalisation (deepar/layers/wrappers.py:123-134) and packing into the
 * kernels' operand layouts. */
int fk_ar2d_pack(const fk_ar2d_desc* desc, const float* params, void* packed, void* stream);
int64_t fk_ar2d_workspace_bytes(const fk_ar2d_desc* desc, int64_t batch, int32_t mode);
/* log psi (machines/abstract_machine.py:31-71, model.predict): log_psi [B][2];
 * cond [B][N][4] = (Re0, Re1, Im0, Im1) normalised conditionals, optional.
 * Index 0 of the last axis pair is spin +1 (deepar/layers/one_hot.py:7-9). */
int fk_ar2d_forward(const fk_ar2d_desc* desc, const void* packed, const int8_t* spins, int64_t batch,
                    float* log_psi, float* cond, void* workspace, int64_t workspace_bytes, int32_t mode,
                    void* stream);
/* Exact autoregressive sampling in raster order (deepar/samplers/fast_autoregressive.py:13-76,
 * samplers/fast_autoregressive/__init__.py:8): one persistent CTA per 128
 * samples walks the sites, evaluates each (layer, site) once and draws the
 * site with Philox4x32-10 (counter = sample, site, offset). Writes spins [B][N],
 * log_psi [B][2], and leaves the activations in `workspace` (FK_AR2D_SAVE
 * layout) for fk_ar2d_backward. */
int fk_ar2d_sample(const fk_ar2d_desc* desc, const void* packed, int64_t batch, uint64_t seed, uint64_t offset,
                   int8_t* spins, float* log_psi, void* workspace, int64_t workspace_bytes, void* stream);
/* log psi of connected configurations with causal reuse (the batched
 * wave-function evaluation of observables/monte_carlo/operator.py:20-34).
 * configs [n_rows][N], owner[row] = base sample, cflips[row][2] = flipped
 * sites (the compact list of fk_compact_connections). base_saved is the
 * FK_AR2D_SAVE workspace of the sampler/forward that evaluated the base_batch
 * base samples with these weights. Rows are sorted by the row rk of their first
 * flipped site; only lattice rows >= rk are evaluated, rows rk-2..rk of the
 * tensors the causal taps read and the log psi of rows < rk come from the base.
 * Bitwise equal to fk_ar2d_forward on the same configurations. log_psi [n_rows][2]
 * in the input order. chunk (a multiple of 128) bounds the rows in flight. */
int64_t fk_ar2d_connections_workspace_bytes(const fk_ar2d_desc* desc, int64_t max_rows, int64_t chunk);
int fk_ar2d_forward_connections(const fk_ar2d_desc* desc, const void* packed, const int8_t* configs,
                                const int32_t* owner, const int16_t* cflips, int64_t n_rows, const void* base_saved,
                                int64_t base_saved_bytes, int64_t base_batch, float* log_psi, void* workspace,
                                int64_t workspace_bytes, int64_t chunk, void* stream);
/* Adjoint of log psi through the masked convolutions. Seeds w [B][2] weight
 * Re and Im log psi of each sample. grad [num_params] = d/dtheta sum_b
 * (w_re Re log psi_b + w_im Im log psi_b) (the Keras loss gradient of
 * optimization/loss.py:4-5; utils/jacobian.py:114-127 per example). When
 * per_sample != NULL it receives the per-sample rows instead of the sum,
 * parameter-major: per_sample[p * B + b].
 * `saved` is the FK_AR2D_SAVE workspace of the forward/sample that produced
 * the activations of these spins. */
int64_t fk_ar2d_backward_workspace_bytes(const fk_ar2d_desc* desc, int64_t batch);
int fk_ar2d_backward(const fk_ar2d_desc* desc, const void* packed, const float* params, const int8_t* spins,
                     int64_t batch, const float* w, const void* saved, int64_t saved_bytes, void* workspace,
                     int64_t workspace_bytes, float* grad, float* per_sample, void* stream);
/* The SR Gram of the per-sample rows without storing them (the S matrix of
 * optimizers/stochastic_reconfiguration/optimizer.py:94-114 in sample space,
 * for networks whose [num_params][B] rows do not fit in memory): gram
 * [2B][2B] = Y^T Y with Y = [Re O_c | Im O_c] (num_params x 2B, each half
 * centred over its samples), the matrix fk_sr_gram builds from the stored
 * rows of fk_ar2d_backward with seeds (1, 0) and (0, 1). Both per-sample
 * adjoints run together over the one set of activations in `saved`; each
 * conv's rows go, as they are produced, to a row buffer of rows_floats
 * floats (at least fk_ar2d_sr_gram_min_rows with the same tensor_cores).
 * When the next step's convs do not fit, and at the end, the buffered rows
 * get the weight-norm chain rule and Y^T Y of the buffer is added into gram:
 * tensor_cores = 0: centred (fk_center_columns) and fk_sr_gram_accumulate on
 * the CUDA cores; 1: centred and split in one pass (fk_sr_center_split, the
 * split operands kept in the same buffer after the rows) and
 * fk_sr_gram_split_accumulate on the tensor cores. */
int64_t fk_ar2d_sr_gram_workspace_bytes(const fk_ar2d_desc* desc, int64_t batch);
int64_t fk_ar2d_sr_gram_min_rows(const fk_ar2d_desc* desc, int64_t batch, int32_t tensor_cores);
int fk_ar2d_sr_gram(const fk_ar2d_desc* desc, const void* packed, const float* params, const int8_t* spins,
                    int64_t batch, const void* saved, int64_t saved_bytes, void* workspace, int64_t workspace_bytes,
                    float* rows, int64_t rows_floats, double* gram, int32_t tensor_cores, void* stream);

/* ------------------------------------------------------------------ optimisers */
/* tf.keras Adam (TF 1.x): lr_t = lr sqrt(1-b2^t)/(1-b1^t), epsilon 1e-7.
 * m, v, params, grad float32 [n]; `step` is t (1-based). */
int fk_adam_step(float* params, const float* grad, float* m, float* v, int64_t n, int64_t step, float lr,
                 float beta1, float beta2, float epsilon, void* stream);
/* y += a x (float32): the SR parameter update W <- W - lr x
 * (optimizers/complex_values_optimizer.py:48-58). */
int fk_axpy(int64_t n, float a, const float* x, float* y, void* stream);

/* ------------------------------------------------------------------ RBM + Metropolis-Hastings
 * Complex RBM parameters as interleaved float32 (re, im):
 * [a (n_visible) | b (n_hidden) | W (n_visible x n_hidden, row-major)].
 * log psi = a.s + sum_j lncosh(b_j + W_j.s) (machines/rbm.py:35-48). */
int fk_rbm_log_psi(const float* params, int32_t n_visible, int32_t n_hidden, const int8_t* spins, int64_t batch,
                   float* log_psi, void* stream);
/* Local energy from an operator enumeration (flips/mel/use as written by the
 * fk_find_conn_* entry points), ratios from incremental theta updates
 * (observables/monte_carlo/operator.py:13-53 with the RBM as wave function). */
int fk_rbm_local_energy(const float* params, int32_t n_visible, int32_t n_hidden, const int8_t* spins, int64_t batch,
                        const int16_t* flips, const double* mel, const uint8_t* use, int32_t n_slots, double* local,
                        void* stream);
/* Per-sample complex O_k (layers/complex/base_layer.py:18-35 convention:
 * holomorphic derivative), parameter-major float32 [P][batch] re and im. */
int fk_rbm_log_derivatives(const float* params, int32_t n_visible, int32_t n_hidden, const int8_t* spins,
                           int64_t batch, float* o_re, float* o_im, void* stream);
/* Persistent Metropolis-Hastings (samplers/metropolis_hastings.py:51-145):
 * kind 0 = Local, 1 = Exchange; chains [n_chains][n_visible] and log_psi [n_chains][2]
 * in/out; warmup_sweeps unrecorded sweeps, then samples_per_chain records every
 * unused+1 sweeps into samples [n_chains][samples_per_chain][n_visible];
 * *accepted (device) += accepted proposals. Philox counter (chain, sweep, 0x4D48). */
int fk_rbm_mh_sweeps(const float* params, int32_t n_visible, int32_t n_hidden, int32_t height, int32_t width,
                     int32_t kind, int8_t* chains, float* log_psi, int64_t n_chains, int64_t warmup_sweeps,
                     int32_t samples_per_chain, int32_t unused, uint64_t seed, uint64_t sweep_offset, int8_t* samples,
                     unsigned long long* accepted, void* stream);
/* Independent-proposal step: accept candidates with
 * min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s'))), log q = 2 Re log psi_q. The
 * symmetric-proposal rule of MetropolisHastingsGlobal (metropolis_hastings.py:148-157)
 * with the proposal ratio added, so any proposal leaves |psi|^2 invariant. */
int fk_mh_independent_step(int8_t* chains, float* lp_chain, float* lq_chain, const int8_t* candidates,
                           const float* lp_cand, const float* lq_cand, int64_t n_chains, int32_t n_visible,
                           uint64_t seed, uint64_t step, unsigned long long* accepted, void* stream);

/* Hamiltonian-proposal Metropolis-Hastings (MetropolisHastingsHamiltonian,
 * samplers/metropolis_hastings.py:170-195), one sweep as propose -> the
 * caller enumerates the candidates' connections and evaluates their log psi
 * -> accept. Propose: the candidate of chain c is its used connection number
 * floor(U * n(c)) (find_conn slot order; flips/use as fk_find_conn_* give them,
 * [n_slots][n_chains]); n_conn[c] = n(c), the chain's number of used
 * connections. Accept: min(1, |psi(s')|^2 n(s) / (|psi(s)|^2 n(s'))), with
 * use_cand the candidates' use flags; accepted chains take the candidate and
 * its log psi; `accepted` (may be NULL) counts acceptances. Both draw from
 * the Philox counter (chain, sweep_lo, sweep_hi, 0x484D): word 0 proposes,
 * word 2 accepts. */
int fk_mh_hamiltonian_propose(const int8_t* chains, const int16_t* flips, const uint8_t* use, int32_t n_slots,
                              int64_t n_chains, int32_t n_sites, uint64_t seed, uint64_t sweep, int8_t* candidates,
                              int32_t* n_conn, void* stream);
int fk_mh_hamiltonian_accept(int8_t* chains, float* lp_chain, const int8_t* candidates, const float* lp_cand,
                             const int32_t* n_conn, const uint8_t* use_cand, int32_t n_slots, int64_t n_chains,
                             int32_t n_sites, uint64_t seed, uint64_t sweep, unsigned long long* accepted,
                             void* stream);

/* Tied complex parameters (RBMSym, machines/rbm.py:51-65 with
 * layers/complex/dense.py:53-85): dst[i] = src[index[i]] over interleaved
 * complex values (bare -> dense expansion). */
int fk_gather_complex(const float* src, const int32_t* index, int64_t n, float* dst, void* stream);
/* out[k][c] = sum_{q = offsets[k]}^{offsets[k+1]-1} in[rows[q]][c] (float32,
 * fixed order): per-sample log-derivative rows of the dense copies summed
 * into the bare parameter they copy. n_out <= 65535. */
int fk_segment_sum_rows(const float* in, const int64_t* offsets, const int32_t* rows, int64_t n_out, int64_t cols,
                        float* out, void* stream);
/* Loss gradient for complex parameters stored as (re, im) pairs
 * (optimization/loss.py:4-5 through layers/complex/base_layer.py:18-35):
 * from per-sample O = d log psi / d theta, parameter-major [P][batch] re and im,
 * and the seeds w [batch][2] of sum_b (w_re Re log psi_b + w_im Im log psi_b):
 * grad[k] = (sum_b w_re Re O + w_im Im O, sum_b w_im Re O - w_re Im O). */
int fk_complex_param_gradient(const float* o_re, const float* o_im, int64_t n_params, int64_t batch, const float* w,
                              float* grad, void* stream);

/* ------------------------------------------------------------------ SR (kernel d)
 * Sample-space stochastic reconfiguration
 * (optimizers/stochastic_reconfiguration/optimizer.py:33-124): per-sample
 * log-derivative rows O are parameter-major float32 [n_params][n_samples]. */
/* Subtracts the mean over the columns from every row (J - mean(J), optimizer.py:111-114). */
int fk_center_columns(float* y, int64_t rows, int64_t cols, float* mean, void* stream);
/* gram (n x n float64, n = n_samples or 2 n_samples when o_im != NULL) =
 * Y^T Y with Y = [o_re | o_im]: FP32 products, FP32 chunk sums reduced in FP64. */
int64_t fk_sr_gram_workspace_bytes(int64_t n_params, int64_t n_samples);
int fk_sr_gram(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, double* gram,
               int64_t gram_elems, void* stream);
/* The same Gram on the tensor cores (tcgen05, kind::f16): every float32 value
 * is split into bf16 hi + lo and each product taken as hi*hi + hi*lo + lo*hi
 * with float32 accumulation in TMEM over ranges of at most 4096 parameters,
 * float64 sums across ranges (relative error of an entry against
 * sqrt(T_ii T_jj): ~2e-7 off the diagonal, up to ~2e-5 on it). n_samples a
 * multiple of 8, o_re / o_im 16-byte aligned, n <= 65536. */
int fk_sr_gram_tc(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, double* gram,
                  int64_t gram_elems, void* stream);
/* Adds the upper triangle (j >= i) of Y^T Y into gram (n x n float64), Y
 * [rows][n] float32 row-major: the Gram of a block of parameter rows, for
 * Grams accumulated block by block (fk_sr_gram's arithmetic with
 * tensor_cores = 0, fk_sr_gram_tc's with 1, which needs n a multiple of 8 and
 * y 16-byte aligned). The lower triangle is left as it is. */
int fk_sr_gram_accumulate(const float* y, int64_t rows, int64_t n, double* gram, int32_t tensor_cores,
                          void* stream);
/* Copies the upper triangle of gram (n x n) into the lower one. */
int fk_sr_gram_mirror(double* gram, int64_t n, void* stream);
/* The tensor-core Gram (the S matrix of
 * optimizers/stochastic_reconfiguration/optimizer.py:94-114 in sample space)
 * in two stages, for Grams that read each value many times (n / 128 +
 * n / 256 tiles per value): fk_sr_gram_split writes Y (rows
 * x n, column c from a[p * ld + c] when c < bsz, else b[p * ld + c - bsz];
 * b = NULL: all from a) once as bf16 hi + lo in the blocked operand layout
 * (fk_sr_gram_split_bytes(rows, n) bytes, 16-byte aligned), and
 * fk_sr_gram_split_accumulate adds the upper triangle of Y^T Y into gram
 * (n x n float64, n <= 65536) from it, streaming the operands with bulk
 * copies: the products and accuracy of fk_sr_gram_tc, any n. */
int64_t fk_sr_gram_split_bytes(int64_t rows, int64_t n);
int fk_sr_gram_split(const float* a, const float* b, int64_t ld, int64_t bsz, int64_t rows, int64_t n, void* split,
                     int64_t split_bytes, void* stream);
int fk_sr_gram_split_accumulate(const void* split, int64_t rows, int64_t n, double* gram, void* stream);
/* fk_center_columns and fk_sr_gram_split in one pass over the rows: every
 * row of Y (columns [0, bsz) from a, [bsz, n) from b, row stride ld) centred
 * within those two column groups with fk_center_columns' arithmetic,
 * written back in place when write_back != 0, and split into `split`. */
int fk_sr_center_split(float* a, float* b, int64_t ld, int64_t bsz, int64_t rows, int64_t n, int32_t write_back,
                       void* split, int64_t split_bytes, void* stream);
/* FP64 conjugate gradients on (scale * gram + shift I) x = rhs, stopping at
 * ||r|| <= tol ||rhs|| or max_iter (linear_equations.py:34-137); stats (device,
 * optional) = {iterations, ||r||^2, tol^2 ||rhs||^2}. No host synchronisation. */
int64_t fk_sr_solve_workspace_bytes(int64_t n);
int fk_sr_solve(const double* gram, int64_t n, double scale, double shift, const double* rhs, double tol,
                int32_t max_iter, double* x, double* stats, void* workspace, int64_t workspace_bytes,
                void* stream);
/* fk_sr_solve without a workspace, for callers that cannot allocate device
 * memory (their GPU memory belongs to another allocator, or cudaMalloc is not
 * allowed on their solve path). No counterpart in the reference. The CG
 * scratch lives in a fixed device array inside the library, so n is limited to
 * 8192; larger n is rejected with FK_ERR_ARG. The first call on a device looks
 * the array up (cudaGetSymbolAddress) and should come before any stream
 * capture. All calls share the array: calls that overlap on the GPU (other
 * streams, other threads) race and must be serialised by the caller. Nothing
 * from an earlier call is read; results equal fk_sr_solve's. */
int fk_sr_solve_noalloc(const double* gram, int64_t n, double scale, double shift, const double* rhs, double tol,
                        int32_t max_iter, double* x, double* stats, void* stream);
/* Complex-parameter SR (optimizer.py:94-114 with complex_values_optimizer.py:28-82):
 * turns the 2n x 2n Gram of [Re O_c | Im O_c] (fk_sr_gram with o_im, n =
 * n_samples) in place into the real symmetric embedding [[Tr, -Ti], [Ti, Tr]]
 * of the Hermitian sample-space Gram T = O_c O_c^H, so that fk_sr_solve on it
 * with rhs [Re e; Im e] solves T z = e. */
int fk_sr_hermitian_embed(double* gram, int64_t n_samples, void* stream);
/* x = scale * O_c^H z for complex parameters (z = [Re z; Im z], 2 n_samples):
 * x interleaved (re, im) [n_params][2]; params (interleaved) -= lr x when
 * params != NULL, x written to x_out when != NULL. */
int fk_sr_complex_backmap(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples,
                          const double* z, double scale, float lr, float* params, float* x_out, void* stream);
/* x = scale * Y alpha (complex_values_optimizer.py:48-58 update direction);
 * params -= lr * x when params != NULL; x written to x_out when != NULL. */
int fk_sr_backmap(const float* o_re, const float* o_im, int64_t n_params, int64_t n_samples, const double* alpha,
                  double scale, float lr, float* params, float* x_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FLOWKET_GB300_H */
