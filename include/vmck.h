/*
 * vmck.h - C ABI of the GB300-native VMC hot loop (libvmck.so).
 *
 * One function per hot-path kernel.  Every pointer argument is a DEVICE pointer
 * unless stated otherwise; the caller owns all input and output buffers.  Calls
 * are stream-ordered on the given stream (a cudaStream_t passed as void*; NULL is
 * the legacy default stream) and return a host status code (VMCK_OK == 0).
 * Conditions found on the device (non-finite values, a failed factorisation)
 * are OR-ed into an optional int32 device status word, read by the host once per
 * step.  No kernel traps.
 *
 * Spin configurations are int8 values in {+1, -1} (NetKet's Spin(1/2) states,
 * netket/hilbert/spin.py:167-172).  RBM parameters are one flat buffer in NetKet's
 * ravel order: [Dense.bias (M) | Dense.kernel (N*M, row-major) | visible_bias (N)]
 * (netket/models/rbm.py:57-81 under jax.flatten_util.ravel_pytree).
 */
#ifndef VMCK_H
#define VMCK_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VMCK_ABI_VERSION 1

/* host status codes */
#define VMCK_OK 0
#define VMCK_ERR_ARG 1         /* null pointer, bad size */
#define VMCK_ERR_UNSUPPORTED 2 /* dtype / shape outside what the kernel handles */
#define VMCK_ERR_CUDA 3        /* a CUDA runtime call or launch failed */
#define VMCK_ERR_LIBRARY 4     /* cuBLAS / cuSOLVER failure */
#define VMCK_ERR_NOMEM 5       /* workspace allocation failed */

/* device status bits */
#define VMCK_DEV_NONFINITE 1   /* NaN or Inf in a solver input or output */
#define VMCK_DEV_NOT_SPD 2     /* Cholesky info != 0 */
#define VMCK_DEV_NO_CONVERGE 4 /* iterative refinement did not reach tolerance */
#define VMCK_DEV_TIMEOUT 8     /* a bounded device-side wait ran out (kernel wound down) */
#define VMCK_DEV_INTERNAL 16   /* a kernel's internal consistency check failed (work skipped) */

/* element types */
#define VMCK_F64 0
#define VMCK_F32 1
#define VMCK_BF16 2

typedef void *vmck_stream; /* cudaStream_t */
typedef struct vmck_ctx vmck_ctx;

int vmck_abi_version(void);
const char *vmck_error_string(int code);
/* Last CUDA / library error text recorded by this thread (host string). */
const char *vmck_last_error(void);
/* Number of kernels this library has launched in this process (diagnostic;
 * cuBLAS / cuSOLVER launches are not included). */
int64_t vmck_launch_count(void);
/* Wall-time limit (ns, default 2e9) of the device-side waits for work: the
 * tensor-core kernels' pipeline waits and the waits between CTAs of the
 * persistent triangular solves.  A wait that runs out sets VMCK_DEV_TIMEOUT in
 * the call's status word and the kernel winds down; copies and MMAs already
 * issued are still waited for with the fixed 2 s limit, so no CTA exits with
 * work in flight.  No counterpart in the reference (XLA's kernels have no
 * device-side waits); the tests shorten it to make a wait run out. */
int vmck_set_wait_limit_ns(uint64_t ns);
uint64_t vmck_wait_limit_ns(void);

/* Library context: owns cuBLAS / cuSOLVER handles and the solver workspace.
 * Replaces the XLA-managed handles behind jax.scipy.linalg.cho_factor
 * (netket/optimizer/solver/solvers.py:242-271). */
int vmck_ctx_create(vmck_ctx **out);
int vmck_ctx_destroy(vmck_ctx *ctx);

/* ---------------------------------------------------------------- a1
 * Random spin states.  n_down < 0: every site +1/-1 uniformly
 * (netket/hilbert/random/homogeneous.py:37-47); n_down >= 0: a uniformly random
 * arrangement of exactly n_down down spins (the Sz-constrained permutation draw,
 * netket/hilbert/random/fock.py:92-101).  Philox4x32-10 keyed by seed. */
int vmck_random_states(vmck_stream s, int8_t *out, int64_t n_batches, int32_t N,
                       int32_t n_down, uint64_t seed, uint64_t stream_id);

/* ---------------------------------------------------------------- a7
 * IsingJax.get_conn_padded (netket/operator/_ising/jax.py:82-88, 125-165).
 * x (n, N) -> xp (n, K, N), mels (n, K) with K = N+1 (K = 1 when h_is_zero).
 * Row 0: x, mel J * sum_e (2 [x_u == x_v] - 1).  Row k: x with site k-1 flipped,
 * mel -h.  n_conn (nullable, int32 (n,)): IsingJax.n_conn (jax.py:168-175). */
int vmck_get_conn_ising(vmck_stream s, const int8_t *x, int64_t n, int32_t N,
                        const int32_t *edges, int32_t n_edges, double h, double J,
                        int32_t h_is_zero, int8_t *xp, double *mels, int32_t *n_conn);

/* ---------------------------------------------------------------- a8
 * Packed LocalOperator for spin-1/2 terms acting on <= 4 sites, the device form
 * of pack_internals_jax (netket/operator/_local_operator/compile_helpers.py:
 * 29-218).  Terms are stored in output order: grouped by acting size
 * (ascending), insertion order inside a group.  All pointers are device
 * pointers.  Row index of a term = sum_s idx(x[acting_on[s]]) * 2^(size-1-s)
 * with idx(+1) = 0, idx(-1) = 1. */
typedef struct {
  int32_t n_sites;          /* N */
  int32_t n_terms;          /* T */
  int32_t max_sites;        /* S: stride of acting_on / x_prime (<= 4) */
  int32_t max_rows;         /* R = 2^S */
  int32_t max_conns;        /* C: stride of mels / x_prime */
  int32_t max_conn_size;    /* K: padded output width */
  int32_t nonzero_diagonal; /* the diagonal candidate exists */
  int32_t n_groups;         /* number of acting-size groups */
  double constant;          /* identity shift */
  double mel_cutoff;        /* keep an entry only if |mel| > mel_cutoff */
  const int32_t *acting_on; /* [T][S] */
  const int32_t *acting_size; /* [T] */
  const int32_t *group_end; /* [n_groups] exclusive end term index of each group */
  const double *diag_mels;  /* [T][R] */
  const int32_t *n_conns;   /* [T][R] */
  const double *mels;       /* [T][R][C] */
  const int8_t *x_prime;    /* [T][R][C][S] new spin values (+1/-1) */
} vmck_local_op;

/* ---------------------------------------------------------------- f3b
 * PauliStrings on spin-1/2 states (netket/operator/_pauli_strings/jax.py), as
 * bitmasks.  Slot f (one per distinct flip set, in PauliStringsJax's order:
 * by the number of strings sharing the flip set, then first appearance) maps x
 * to x with the sites of flip_mask[f] flipped, with
 *   mel_f(x) = sum_{s = string_offset[f]}^{string_offset[f+1]-1}
 *              weight[s] * (-1)^popcount(z_mask[s] & down(x)),
 * down(x) bit i set where x_i = -1.  A string's weight already carries the
 * (-i)^(#Y) factor; only real weights are supported (an even number of Y per
 * string).  z_mask holds the sites a string reads with Z or Y.  Words are
 * 32-bit, bit i of word w is site 32 w + i.  All pointers are device pointers. */
typedef struct {
  int32_t n_sites;               /* N */
  int32_t n_words;               /* W = (N + 31) / 32 */
  int32_t n_flips;               /* F: slots (max_conn_size) */
  int32_t n_strings;             /* strings after dropping |weight| <= cutoff */
  double cutoff;                 /* drop a slot where |mel| <= cutoff */
  const uint32_t *flip_mask;     /* [F][W] */
  const int32_t *flip_offset;    /* [F+1] CSR into flip_site */
  const int32_t *flip_site;      /* flipped sites of each slot, ascending */
  const int32_t *string_offset;  /* [F+1] CSR into z_mask / weight */
  const uint32_t *z_mask;        /* [n_strings][W] */
  const double *weight;          /* [n_strings] */
} vmck_pauli_strings;

/* PauliStringsJax.get_conn_padded (jax.py:240-269, 342-355): xp (n, F, N),
 * mels (n, F) with dropped slots holding (x, 0.0); n_conn (nullable, int32
 * (n,)) = the number of nonzero slots (PauliStringsJax.n_conn, jax.py:256-269,
 * 331-340). */
int vmck_get_conn_pauli(vmck_stream s, const vmck_pauli_strings *op, const int8_t *x,
                        int64_t n, int8_t *xp, double *mels, int32_t *n_conn);

/* LocalOperatorJax.get_conn_padded (netket/operator/_local_operator/jax.py:
 * 74-201, 256-288): candidates [diagonal] + per term, per stored column; those
 * with |mel| > mel_cutoff are compacted to the front; the rest of the K slots
 * hold (x, 0.0).  n_conn (nullable) receives the number kept. */
int vmck_get_conn_local(vmck_stream s, const vmck_local_op *op, const int8_t *x,
                        int64_t n, int8_t *xp, double *mels, int32_t *n_conn);

/* ---------------------------------------------------------------- a5
 * RBM.__call__ (netket/models/rbm.py:57-81) with log_cosh
 * (netket/nn/activation.py:78-84): logpsi(x) = sum_j log_cosh(theta_j) + a.x,
 * theta = b + x W.  dtype VMCK_F64 or VMCK_F32 (params and outputs in dtype).
 * theta_out / tanh_out (nullable): (n, M) in dtype. */
int vmck_rbm_logpsi(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                    int32_t M, const int8_t *x, int64_t n, void *logpsi,
                    void *theta_out, void *tanh_out);
/* The same for FP32 parameters with x W on the tensor cores (tcgen05; W split
 * into FP16 hi + lo, x exact; FP32 accumulation drained every 64 sites), then
 * one pass for b, tanh and the log_cosh row sums.  workspace: caller-owned
 * device bytes, at least vmck_rbm_logpsi_tc_workspace_size(N, M, n,
 * theta_out != NULL).  status (device, nullable): VMCK_DEV_TIMEOUT if a
 * bounded wait ran out. */
int64_t vmck_rbm_logpsi_tc_workspace_size(int32_t N, int32_t M, int64_t n,
                                          int32_t with_theta_out);
int vmck_rbm_logpsi_tc(vmck_stream s, const float *params, int32_t N, int32_t M,
                       const int8_t *x, int64_t n, float *logpsi, float *theta_out,
                       float *tanh_out, void *workspace, int64_t workspace_bytes,
                       int32_t *status);

/* ---------------------------------------------------------------- a9 (plain)
 * local_value_kernel_jax reduction (netket/vqs/mc/kernels.py:62-71) from
 * precomputed log-amplitudes: eloc[i] = sum_k mels[i,k] exp(lp_conn[i,k] - lp[i]).
 * lp / lp_conn in dtype (F64 or F32); eloc is FP64. */
int vmck_eloc_from_logpsi(vmck_stream s, int32_t dtype, const void *lp,
                          const void *lp_conn, const double *mels, int64_t n,
                          int32_t K, double *eloc);

/* ---------------------------------------------------------------- a6 + a9 (fused)
 * Local energies without materialising connected states: for each sample the
 * RBM log-ratio of every connected element is formed from theta and the rows of
 * W of the changed sites.  Replaces get_conn_padded + logpsi on every row +
 * the reduction (netket/vqs/mc/kernels.py:62-71).  logpsi_out nullable. */
int vmck_rbm_eloc_ising(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                        int32_t M, const int8_t *x, int64_t n, const int32_t *edges,
                        int32_t n_edges, double h, double J, double *eloc,
                        void *logpsi_out);
int vmck_rbm_eloc_local(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                        int32_t M, const int8_t *x, int64_t n, const vmck_local_op *op,
                        double *eloc, void *logpsi_out);
/* The same for PauliStrings: slot f's log-ratio flips the sites of
 * flip_site[flip_offset[f] : flip_offset[f+1]]; slots with an empty flip set
 * add their mel directly. */
int vmck_rbm_eloc_pauli(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                        int32_t M, const int8_t *x, int64_t n, const vmck_pauli_strings *op,
                        double *eloc, void *logpsi_out);

/* ---------------------------------------------------------------- a2 - a4
 * MetropolisSampler sweep (netket/sampler/metropolis.py:416-505) with the RBM
 * log-amplitude updated incrementally.  rule 0: LocalRule (rules/local.py:40-49);
 * rule 1: ExchangeRule (rules/exchange.py:143-218) over clusters (C, 2).
 * Runs n_discard + chain_length sweeps of sweep_size proposals per chain and
 * stores the state after each of the last chain_length sweeps:
 * samples (B, chain_length, N).  sigma (B, N) is read and written; log_prob (B,)
 * FP64 receives 2 Re logpsi of the final state; n_accepted (B,) is incremented.
 * The random stream is Philox4x32-10 with key = seed and counter =
 * (proposal index counter + k, chain, 0); callers advance counter by
 * (n_discard + chain_length) * sweep_size between calls. */
int vmck_metropolis_sample(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                           int32_t M, int8_t *sigma, double *log_prob,
                           int64_t *n_accepted, int32_t B, int32_t sweep_size,
                           int32_t n_discard, int32_t chain_length, int8_t *samples,
                           uint64_t seed, uint64_t counter, int32_t rule,
                           const int32_t *clusters, int32_t n_clusters);

/* ---------------------------------------------------------------- f3
 * MetropolisSampler with the Hamiltonian rule (netket/sampler/metropolis.py:
 * 686-735, rules/hamiltonian.py:99-213) for the RBM: every proposal picks one of
 * the n(x) entries of x's operator row uniformly,
 *   n(x) = [diagonal slot] + sum_t #{stored off-diagonal columns of term t's
 *          row with |mel| > mel_cutoff},
 * the diagonal slot proposing x itself, and corrects the acceptance by
 * log n(x) - log n(x').  diag_rule: 0 = no diagonal slot, 1 = a slot whenever
 * the operator has a diagonal (LocalOperator n_conn, _local_operator/jax.py:
 * 107-112), 2 = a slot only where |diagonal element| > mel_cutoff (IsingJax
 * n_conn, _ising/jax.py:168-175; pass Ising as its LocalOperator tables).
 * Arguments, samples, random stream and bookkeeping as vmck_metropolis_sample.
 * status (device int32) gets VMCK_DEV_INTERNAL if a chain's counts ever
 * disagree with its row (not expected; the proposal is skipped). */
int vmck_metropolis_hamiltonian(vmck_stream s, int32_t dtype, const void *params, int32_t N,
                                int32_t M, const vmck_local_op *op, int32_t diag_rule,
                                int8_t *sigma, double *log_prob, int64_t *n_accepted, int32_t B,
                                int32_t sweep_size, int32_t n_discard, int32_t chain_length,
                                int8_t *samples, uint64_t seed, uint64_t counter,
                                int32_t *status);

/* The Hamiltonian rule for PauliStrings: n(x) = the number of slots with
 * |mel| > cutoff (PauliStringsJax.n_conn, _pauli_strings/jax.py:256-269); a
 * kept slot with an empty flip set proposes x itself.  Otherwise as
 * vmck_metropolis_hamiltonian. */
int vmck_metropolis_hamiltonian_pauli(vmck_stream s, int32_t dtype, const void *params,
                                      int32_t N, int32_t M, const vmck_pauli_strings *op,
                                      int8_t *sigma, double *log_prob, int64_t *n_accepted,
                                      int32_t B, int32_t sweep_size, int32_t n_discard,
                                      int32_t chain_length, int8_t *samples, uint64_t seed,
                                      uint64_t counter, int32_t *status);

/* ---------------------------------------------------------------- batched (C3)
 * Many independent problems of uneven size in one persistent launch.  Each
 * instance's chains run exactly as vmck_metropolis_sample would run them
 * (same per-chain code, same Philox stream keyed by the instance seed and the
 * chain index), so an instance's samples are identical alone and in a batch.
 * The instance table and the work list live in device memory; work holds
 * (instance, first chain) pairs of chains_per_item chains each, ordered by the
 * caller (largest cost first); queue is a device int32 the call resets.
 * Persistent CTAs (n_ctas of them, chains_per_item warps each) take items from
 * the queue with an atomic counter.  Each instance's counter is advanced by
 * (n_discard + chain_length) * sweep_size at the end of the call.  Local rule
 * only.  No counterpart function in the reference: it batches
 * MetropolisSampler._sample_chain (netket/sampler/metropolis.py:466-505) over
 * independent samplers. */
typedef struct {
  const void *params;  /* flat RBM parameters of the instance, in dtype */
  int8_t *sigma;       /* (n_chains, N) chain states, read and written */
  double *log_prob;    /* (n_chains,) */
  int64_t *n_accepted; /* (n_chains,) incremented */
  int8_t *samples;     /* (n_chains, chain_length, N) */
  uint64_t seed;       /* Philox key */
  uint64_t counter;    /* proposal counter, advanced by the call */
  int32_t N, M, n_chains, sweep_size;
} vmck_batch_chains;

int vmck_batched_metropolis_local(vmck_stream s, int32_t dtype, vmck_batch_chains *inst,
                                  int32_t n_inst, const int32_t *work, int32_t n_items,
                                  int32_t chains_per_item, int32_t *queue, int32_t n_discard,
                                  int32_t chain_length, int32_t max_N, int32_t max_M,
                                  int32_t n_ctas);

/* Batched fused Ising local energies (vmck_rbm_eloc_ising per instance, in one
 * persistent launch): work holds (instance, first sample) pairs of
 * samples_per_item samples each. */
typedef struct {
  const void *params;
  const int8_t *x;      /* (n, N) */
  double *eloc;         /* (n,) */
  const int32_t *edges; /* (n_edges, 2) */
  int64_t n;
  double h, J;
  int32_t N, M, n_edges, pad;
} vmck_batch_ising;

int vmck_batched_eloc_ising(vmck_stream s, int32_t dtype, const vmck_batch_ising *inst,
                            int32_t n_inst, const int32_t *work, int32_t n_items,
                            int32_t samples_per_item, int32_t *queue, int32_t max_N,
                            int32_t max_M, int32_t n_ctas);

/* ---------------------------------------------------------------- a10
 * netket.stats.statistics, blocking estimator (netket/stats/mc_stats_old.py:
 * 88-196) in FP64 over data (n_chains, chain_length):
 * out5 = [mean, error_of_mean, variance, tau_corr, R_hat].
 * workspace: vmck_stats_workspace_size() doubles. */
int64_t vmck_stats_workspace_size(int32_t n_chains, int32_t chain_length);
int vmck_stats_f64(vmck_stream s, const double *data, int32_t n_chains,
                   int32_t chain_length, int32_t plain_rhat, double *out5,
                   double *workspace, int64_t workspace_len);

/* Allocation-free form of vmck_stats_f64.  It has no counterpart in the
 * reference: it exists for callers that cannot allocate device memory while
 * they run -- an XLA custom call / FFI handler, or a host runtime whose memory
 * pool owns the device -- where a cudaMalloc / cudaFree would synchronise the
 * device or fail.  The caller still provides data and out5.  The scratch is a
 * fixed array of VMCK_STATS_NOALLOC_MAX_DOUBLES doubles (2 MiB) compiled into
 * the library; every GPU that loads the library holds it until the process
 * exits.  Sizes needing more scratch than that
 * (vmck_stats_workspace_size(n_chains, chain_length) > the maximum, roughly
 * n_chains > 3900 for long chains) are rejected with VMCK_ERR_ARG.
 * The first call on a device looks up the array's device address (set-up, no
 * allocation); make that first call before any stream capture.  All calls share
 * the one array and it keeps the last call's contents (each call overwrites what
 * it reads, so nothing needs clearing); calls that overlap on the GPU (other
 * streams, other host threads) race on it and must be serialised by the caller. */
#define VMCK_STATS_NOALLOC_MAX_DOUBLES 262144
int vmck_stats_f64_noalloc(vmck_stream s, const double *data, int32_t n_chains,
                           int32_t chain_length, int32_t plain_rhat, double *out5);

/* ---------------------------------------------------------------- f4
 * Streaming statistics: the update of netket.stats.OnlineStats
 * (netket/_src/stats/online_stats/kernels.py:123-190, called from
 * accumulator.py:160-223) on the device.  The state of n_chains chains is
 * FP64 device arrays, row-major:
 *   count, mean, M2          (n_chains)              per-chain Welford state
 *   cross, m1, m2, pair      (n_chains, max_lag + 1) sums of x_t x_{t-k},
 *                                                    x_{t-k}, x_t and pair counts
 *   buf                      (n_chains, max_lag)     the last max_lag samples,
 *                                                    newest last
 * (the ACF arrays may be NULL when max_lag == 0).  data is (n_chains, n_batch)
 * FP64.  buf_len = how many buffer entries are valid before this call
 * (min(samples seen so far per chain, max_lag)); the caller advances it to
 * min(buf_len + n_batch, max_lag).  decay in [0, 1] multiplies the old counts
 * and sums first (1 = the reference's decay=None).  mean_f32 != 0 rounds the
 * stored per-chain means to float after the merge (float32 input data). */
#define VMCK_ONLINE_STATS_MAX_LAG 4096
typedef struct vmck_online_stats {
  double *count, *mean, *M2;
  double *cross, *m1, *m2, *pair;
  double *buf;
} vmck_online_stats;
int vmck_online_stats_update(vmck_stream s, const double *data, int32_t n_chains,
                             int32_t n_batch, int32_t max_lag, int32_t buf_len,
                             double decay, int32_t mean_f32,
                             const vmck_online_stats *state);

/* ---------------------------------------------------------------- a11 / a12 / a14
 * out = O^T v for the RBM Jacobian O (n, P) without materialising it
 * (the VJP of netket/vqs/mc/mc_state/expect_forces.py:99-106 and the
 * O_L^T aux contraction of netket/_src/ngd/srt.py:83-84):
 *   out[bias_j] = sum_s t_sj v_s, out[kernel_ij] = sum_s x_si t_sj v_s,
 *   out[visible_i] = sum_s x_si v_s,  t = tanh(theta) (n, M) in dtype.
 * v (n,) and out (P,) are FP64.  workspace: vmck_ot_v_workspace_size() doubles. */
/* out = O v (n,) for the RBM Jacobian O (n, P) without materialising it: the
 * JVP behind QGTOnTheFly's mat-vec (netket/optimizer/qgt/qgt_onthefly_logic.py:
 * 43-56):  out[s] = t_s . (v_bias + x_s^T V) + x_s . v_visible, V = v_kernel
 * (N x M).  v (P,) and out (n,) FP64; FP64 accumulation. */
int vmck_rbm_o_v(vmck_stream s, int32_t dtype, const void *tanh_theta, const int8_t *x,
                 int32_t N, int32_t M, int64_t n, const double *v, double *out);
int64_t vmck_ot_v_workspace_size(int32_t N, int32_t M, int64_t n);
int vmck_rbm_ot_v(vmck_stream s, int32_t dtype, const void *tanh_theta,
                  const int8_t *x, int32_t N, int32_t M, int64_t n, const double *v,
                  double *out, double *workspace, int64_t workspace_len);
/* O^T v for FP32 tanh(theta) on the tensor cores: one GEMM of v (.) [t, 1]
 * (split into FP16 hi + lo) with [x, 1] over the samples (split into chunks,
 * partial sums added in FP64 in chunk order) gives the kernel, hidden-bias and
 * visible-bias parts at once.  workspace: caller-owned device bytes, at least
 * vmck_rbm_ot_v_tc_workspace_size(N, M, n).  status as vmck_rbm_logpsi_tc. */
int64_t vmck_rbm_ot_v_tc_workspace_size(int32_t N, int32_t M, int64_t n);
int vmck_rbm_ot_v_tc(vmck_stream s, const float *tanh_theta, const int8_t *x, int32_t N,
                     int32_t M, int64_t n, const double *v, double *out, void *workspace,
                     int64_t workspace_bytes, int32_t *status);

/* Dense centred, scaled Jacobian O_L = (O - mean O) * scale, (n, P) in out_dtype,
 * from tanh(theta) (dtype) and the column means (FP64, P) -- nkjax.jacobian
 * (netket/jax/_jacobian/logic.py:48-384, center=True) followed by
 * _prepare_input (netket/_src/ngd/sr_srt_common.py:45-101). */
int vmck_rbm_jacobian(vmck_stream s, int32_t dtype, const void *tanh_theta,
                      const int8_t *x, int32_t N, int32_t M, int64_t n,
                      const double *col_mean, double scale, int32_t out_dtype, void *O);

/* ---------------------------------------------------------------- a14 (structured)
 * minSR matrix T = O_L O_L^T + diag_shift I for the RBM without O:
 *   O(s).O(s') = (t_s.t_s')(1 + x_s.x_s') + x_s.x_s',
 *   T = (G - g 1^T - 1 g^T + c 11^T) / n + diag_shift I, g = O obar, c = |obar|^2.
 * obar (P, FP64): column means.  Only the lower triangle (row >= col) is written;
 * T64 (n, n) FP64 row-major; T32 (nullable) receives an FP32 copy.
 * mode 0: FP64 contraction (CUDA cores); 1: FP32 contraction (CUDA cores);
 * 2: tensor cores (tcgen05, TMA) on t rounded to hi + lo BF16 pairs (all four
 * products, FP32 accumulation); 3: tensor cores on t rounded to one BF16;
 * 4: tensor cores on t - fp32(tbar) rounded to a multiple of 2^-19 and split
 * into fixed-point FP16 hi + lo (all four products): every 64-wide slab of the
 * hi * hi products sums exactly, the slabs add in FP32 registers (mode 2's
 * accumulation error grows with the MMA chain and lost positive definiteness
 * at M = 2048), and a separate assembly pass adds the exact terms.
 * Modes 1-4 take tanh_theta in FP32 and contract the shifted c = t - fp32(tbar)
 * (tbar = obar[0:M]), adding the shift back exactly in a double-float epilogue,
 * so T is the exact Gram matrix of the contracted Jacobian (positive
 * definite) with no cancellation against the mean.  status (nullable device int32) receives
 * VMCK_DEV_TIMEOUT if a tensor-core CTA's bounded wait ran out. */
int64_t vmck_gram_workspace_size(int32_t N, int32_t M, int64_t n);

int vmck_rbm_gram(vmck_ctx *ctx, vmck_stream s, int32_t mode, int32_t dtype,
                  const void *tanh_theta, const int8_t *x, int32_t N, int32_t M,
                  int64_t n, const double *obar, double diag_shift, double *T64,
                  float *T32, double *workspace, int64_t workspace_len, int32_t *status);

/* Dense T = O_L O_L^T + diag_shift I (lower triangle) or S = O_L^T O_L + shift I
 * (transpose = 1) with cuBLAS, from a materialised O_L (rows, cols) in dtype
 * (netket/_src/ngd/srt.py:53-60, netket/_src/ngd/sr.py:54-60). */
int vmck_gram_dense(vmck_ctx *ctx, vmck_stream s, int32_t dtype, const void *O_L,
                    int64_t rows, int64_t cols, int32_t transpose, double diag_shift,
                    void *out);

/* ---------------------------------------------------------------- a15
 * cholesky (netket/optimizer/solver/solvers.py:242-271): solve A x = b for SPD A
 * (n, n) whose LOWER triangle is read (row-major; A is preserved).  dtype F64 or
 * F32.  On info != 0 or a non-finite x, VMCK_DEV_NOT_SPD / VMCK_DEV_NONFINITE is
 * OR-ed into *status; the caller then takes the pinv_smooth fallback
 * (solvers.py:305-340, netket/_src/solvers/nan_fallback.py:22-45). */
int vmck_cholesky_solve(vmck_ctx *ctx, vmck_stream s, int32_t dtype, const void *A,
                        const void *b, void *x, int64_t n, int32_t *status);
/* FP32 Cholesky factor of A32 (lower triangle, overwritten) refined against the
 * FP64 matrix A64 (lower triangle): max_iter correction solves, each from the
 * FP64 residual b - A64 x; the final relative residual goes to residual_out
 * (device, nullable) and VMCK_DEV_NO_CONVERGE is raised if it exceeds tol.
 * The residual is evaluated in double-float arithmetic (~2^-46 per term).
 * factor_mode 0: cuSOLVER SPOTRF; 1: cuSOLVER SPOTRF with FP32-accurate BF16x9
 * tensor-core emulation; 2: recursive Cholesky whose TRSM / SYRK are recursive
 * GEMMs on BF16x9-emulated tensor cores (cuSOLVER / cuBLAS at <= 1024 leaves);
 * 3: blocked right-looking Cholesky (512-row panels, this library's 128 x 128
 * leaf kernel, emulated-GEMM panel solves and trailing updates). */
int vmck_cholesky_solve_refined(vmck_ctx *ctx, vmck_stream s, const double *A64,
                                float *A32, const double *b, double *x, int64_t n,
                                int32_t max_iter, double tol, int32_t factor_mode,
                                int32_t *status, double *residual_out);
/* The solution of the FP64 Cholesky solve (netket/optimizer/solver/solvers.py
 * cholesky, the minSR solve of netket/_src/ngd/srt.py:76-79) when the FP32
 * factor of A fails (cond(A) beyond FP32): A + mu I is factored on the tensor
 * cores, mu = shift_rel trace(A) (x16 per failed attempt, at most six), and
 * preconditions flexible conjugate gradients against A64 (FP64 products) until
 * ||b - A x|| <= tol ||b|| or max_iter iterations.  A32 (nullable: context
 * workspace) is overwritten by the factor.  status (device) gets NOT_SPD when
 * CG meets non-positive curvature (A not positive definite) or every factor
 * failed, NO_CONVERGE when tol is not reached, NONFINITE.  residual_out
 * (device, nullable) receives the final relative FP64 residual, *shift_out
 * (host, nullable) the shift used.  Synchronises the stream. */
int vmck_cholesky_solve_pcg(vmck_ctx *ctx, vmck_stream s, const double *A64,
                            float *A32, const double *b, double *x, int64_t n,
                            int32_t max_iter, double tol, double shift_rel,
                            int32_t *status, double *residual_out, double *shift_out);
/* pinv_smooth (solvers.py:33-139) via a symmetric eigendecomposition (FP64). */
int vmck_pinv_smooth_solve(vmck_ctx *ctx, vmck_stream s, const double *A,
                           const double *b, double *x, int64_t n, double rtol,
                           double rtol_smooth);

/* ---------------------------------------------------------------- a14 helpers
 * dv = 2 (e - mean) * scale with mean = *mean_dev (netket/_src/ngd/
 * sr_srt_common.py:86-88); all FP64. */
int vmck_center_scale(vmck_stream s, const double *e, const double *mean_dev,
                      int64_t n, double factor, double *out);
/* update = scale * (raw - obar * sum(aux)) with sum(aux) computed on the device:
 * turns O^T aux into O_L^T aux for the centred Jacobian (srt.py:83-84). */
int vmck_center_update(vmck_stream s, const double *raw, const double *obar,
                       const double *aux, int64_t n, int64_t P, double scale,
                       double *update);

/* ---------------------------------------------------------------- a16
 * optax.sgd step (netket/optimizer/__init__.py:33-60 via
 * netket/_src/driver/abstract_optimization_driver.py:86-92):
 * p64 -= lr * update; p32 (nullable) receives the FP32 copy. */
int vmck_sgd(vmck_stream s, double *p64, const double *update, int64_t P, double lr,
             float *p32);
/* Cast FP64 -> FP32 (n elements). */
int vmck_cast_f64_f32(vmck_stream s, const double *in, float *out, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* VMCK_H */
